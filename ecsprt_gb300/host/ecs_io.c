/*
 * Output files of the GB300 ECSPRT host.
 *
 * Particles: OutputSwarmBinary (src/file-io.c:103-161) writes positions and
 * velocities with VecView to a PETSc binary viewer: int32 class id 1211214,
 * int32 length, then the FP64 values, all big-endian.  ecs_write_petsc_vec
 * writes that format byte for byte.
 * Fluid: OutputFluidHDF5 (src/file-io.c:164-222) writes the datasets
 * "density", "x flux", "y flux", "z flux", "rhs", "potential".  HDF5 is not
 * available to this build, so ecs_write_fluid writes the same six vectors, in
 * that order, as consecutive PETSc binary Vecs.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ecs_host.h"

#define VEC_FILE_CLASSID 1211214

static void put_be32(unsigned char *b, uint32_t v) {
  b[0] = (unsigned char)(v >> 24);
  b[1] = (unsigned char)(v >> 16);
  b[2] = (unsigned char)(v >> 8);
  b[3] = (unsigned char)v;
}
static uint32_t get_be32(const unsigned char *b) {
  return ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | (uint32_t)b[3];
}

static int write_vec(FILE *f, const double *v, int64_t n) {
  unsigned char hdr[8];
  if (n < 0 || n > INT32_MAX) return ECS_ERR_INVALID;
  put_be32(hdr, VEC_FILE_CLASSID);
  put_be32(hdr + 4, (uint32_t)n);
  if (fwrite(hdr, 1, 8, f) != 8) return ECS_ERR_INVALID;
  unsigned char buf[8 * 1024];
  int64_t i = 0;
  while (i < n) {
    int64_t m = n - i < 1024 ? n - i : 1024;
    for (int64_t q = 0; q < m; q++) {
      uint64_t u;
      memcpy(&u, &v[i + q], 8);
      for (int b = 0; b < 8; b++) buf[8 * q + b] = (unsigned char)(u >> (56 - 8 * b));
    }
    if (fwrite(buf, 1, (size_t)(8 * m), f) != (size_t)(8 * m)) return ECS_ERR_INVALID;
    i += m;
  }
  return ECS_OK;
}

int ecs_write_petsc_vec(const char *path, const double *v, int64_t n) {
  FILE *f = fopen(path, "wb");
  if (!f) return ECS_ERR_INVALID;
  int rc = write_vec(f, v, n);
  fclose(f);
  return rc;
}

int ecs_read_petsc_vec(const char *path, double *v, int64_t n) {
  FILE *f = fopen(path, "rb");
  if (!f) return ECS_ERR_INVALID;
  unsigned char hdr[8];
  int rc = ECS_OK;
  if (fread(hdr, 1, 8, f) != 8 || get_be32(hdr) != VEC_FILE_CLASSID || (int64_t)get_be32(hdr + 4) != n) {
    rc = ECS_ERR_INVALID;
  } else {
    for (int64_t i = 0; i < n && rc == ECS_OK; i++) {
      unsigned char b[8];
      if (fread(b, 1, 8, f) != 8) {
        rc = ECS_ERR_INVALID;
        break;
      }
      uint64_t u = 0;
      for (int q = 0; q < 8; q++) u = (u << 8) | b[q];
      memcpy(&v[i], &u, 8);
    }
  }
  fclose(f);
  return rc;
}

int ecs_write_fluid(const char *path, const double *moments, const double *rhs, const double *phi,
                    int64_t ncell) {
  FILE *f = fopen(path, "wb");
  if (!f) return ECS_ERR_INVALID;
  double *tmp = malloc(sizeof(double) * (size_t)(ncell > 0 ? ncell : 1));
  int rc = tmp ? ECS_OK : ECS_ERR_NOMEM;
  for (int d = 0; d < 4 && rc == ECS_OK; d++) {
    for (int64_t c = 0; c < ncell; c++) tmp[c] = moments[4 * c + d];
    rc = write_vec(f, tmp, ncell);
  }
  if (rc == ECS_OK) rc = write_vec(f, rhs, ncell);
  if (rc == ECS_OK) rc = write_vec(f, phi, ncell);
  free(tmp);
  fclose(f);
  return rc;
}
