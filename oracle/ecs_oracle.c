/*
 * ECSPRT hot-path ORACLE: a plain-C, FP64 restatement of the reference's
 * per-timestep algorithm, used only as a checker.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load this library.  The product (libecsgpu) never
 * links or calls it.
 *
 * Every function states the reference lines it follows (paths relative to the
 * reference project).  Arithmetic is written operand-for-operand in the
 * reference's evaluation order and the file is compiled with
 * -ffp-contract=off, so results agree bit for bit with the reference's own
 * sources compiled against the PETSc-API shim (oracle/ref_shim).
 *
 * Grid conventions: node arrays are [Nz][Ny][Nx] with x fastest, moments are
 * [Nz][Ny][Nx][4] = (n, Gx, Gy, Gz), particles are AoS pos[ip*3+d],
 * vel[ip*3+d].  Boundary kinds: 0 = periodic, 1 = reflecting (z only; the
 * reference has no reflecting behaviour, see orc_apply_bc).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* Parameter block, filled by the Python host from the derived context. */
typedef struct {
  int Nx, Ny, Nz;
  int bc[3];           /* 0 periodic, 1 reflecting */
  double dx, dy, dz;
  double x0, y0, z0;   /* lower bounds (0 when dx is given: src/setup.c:319-342) */
  double x1, y1, z1;   /* upper bounds */
  double Lx, Ly, Lz;
  double qi, mi, B0, E0;
  double nui;          /* ion-neutral collision frequency */
  double viT;          /* ion thermal-speed magnitude (src/setup.c:250-252) */
  double vi0[3];
  double mn;           /* neutral mass; 0 disables collisions */
  double vnT;          /* neutral thermal speed (src/setup.c:268) */
  double vn0[3];
  double vn0mag;
  double kappa_e;      /* electron magnetisation (src/setup.c:226) */
  double scale;        /* 1/(1+kappa_e^2) (src/setup.c:230) */
  double cth;          /* gammaT*KB*Te/Q (src/rhs.c:291) */
  double cG;           /* (1+kappa^2)*me*nue/Q (src/rhs.c:292) */
  double n0;           /* background density (-n0) */
  int lhs_type;        /* LHSType src/global.h: 0 identity, 1 laplacian, 2 full */
  int rhs_type;        /* RHSType: 0 constant, 1 sinusoidal, 2 full */
  int ndim;            /* 2 or 3; a 2-D grid is [1][Ny][Nx] */
} OrcParams;

static inline int wrapi(int i, int n) { return ((i % n) + n) % n; }

/* Value of a node array through the ghost semantics of the reference's DMDA:
   periodic dimensions wrap, non-periodic (ghosted) dimensions read 0. */
static inline double node_val(const OrcParams *p, const double *F, int k, int j, int i) {
  if (i < 0 || i >= p->Nx) { if (p->bc[0]) return 0.0; i = wrapi(i, p->Nx); }
  if (j < 0 || j >= p->Ny) { if (p->bc[1]) return 0.0; j = wrapi(j, p->Ny); }
  if (k < 0 || k >= p->Nz) { if (p->bc[2]) return 0.0; k = wrapi(k, p->Nz); }
  return F[((size_t)k * p->Ny + j) * p->Nx + i];
}

/* ------------------------------------------------------------------------ */
/* E-field difference vector: src/vector-math.c:596-722 (DifferenceVector3D) */
/* ------------------------------------------------------------------------ */

/* Second-order difference numerator of F along `axis` at the node whose
   index along that axis is `h` (other two indices fixed).  `low` selects the
   rule used for the low node: central unless the index is negative (forward,
   src/vector-math.c:625-631).  For the high node the rule is central unless
   the index equals N (backward, src/vector-math.c:638-644) -- this is applied
   even on periodic grids (reference behaviour kept). */
static double diff_num(const OrcParams *p, const double *F, int axis, int k, int j, int i,
                       int low) {
  int N = axis == 0 ? p->Nx : (axis == 1 ? p->Ny : p->Nz);
  int h = axis == 0 ? i : (axis == 1 ? j : k);
#define AT(o) (axis == 0 ? node_val(p, F, k, j, i + (o)) : \
               (axis == 1 ? node_val(p, F, k, j + (o), i) : node_val(p, F, k + (o), j, i)))
  if (low) {
    if (h >= 0) return AT(1) - AT(-1);
    return -1.0 * AT(2) + 4.0 * AT(1) - 3.0 * AT(0);
  }
  if (h < N) return AT(1) - AT(-1);
  return +3.0 * AT(0) - 4.0 * AT(-1) + 1.0 * AT(-2);
#undef AT
}

/* Interpolated difference vector at fractional grid position (x,y,z).
   Interpolation order and weights follow src/vector-math.c:645-651: first
   along y with wyh, then across the z pair with wxh, then across the x pair
   with wzh (the x and z weights are exchanged in the reference). */
static void difference_vector(const OrcParams *p, const double *F, double x, double y,
                              double z, double f[3]) {
  int ixl = (int)x, iyl = (int)y, izl = (int)z;
  int ixh = ixl + 1, iyh = iyl + 1, izh = izl + 1;
  double wxh = x - (double)ixl;
  double wyh = y - (double)iyl;
  double wzh = z - (double)izl;
  int ix[2] = {ixl, ixh}, iy[2] = {iyl, iyh}, iz[2] = {izl, izh};
  for (int axis = 0; axis < 3; axis++) {
    double D[2][2][2]; /* [zb][yb][xb] */
    for (int zb = 0; zb < 2; zb++)
      for (int yb = 0; yb < 2; yb++)
        for (int xb = 0; xb < 2; xb++) {
          int low = axis == 0 ? (xb == 0) : (axis == 1 ? (yb == 0) : (zb == 0));
          D[zb][yb][xb] = diff_num(p, F, axis, iz[zb], iy[yb], ix[xb], low);
        }
    double a[2][2]; /* [zb][xb] */
    for (int zb = 0; zb < 2; zb++)
      for (int xb = 0; xb < 2; xb++)
        a[zb][xb] = D[zb][0][xb] + wyh * (D[zb][1][xb] - D[zb][0][xb]);
    double c[2]; /* [xb] */
    for (int xb = 0; xb < 2; xb++) c[xb] = a[0][xb] + wxh * (a[1][xb] - a[0][xb]);
    f[axis] = c[0] + wzh * (c[1] - c[0]);
  }
}

/* ------------------------------------------------------------------------ */
/* Boris push, B along z: src/velocities.c:281-371 (BorisMoverBz3D)          */
/* Only the first half E-kick is applied; vz keeps v^- (src/velocities.c:     */
/* 347-356).  Positions are divided by the cell widths with no x0 offset     */
/* (src/velocities.c:342-344).                                                */
/* ------------------------------------------------------------------------ */
int orc_push(const OrcParams *p, int np, const double *pos, double *vel, const double *phi,
             double dt) {
  double tscale = 0.5 * (p->qi / p->mi) * dt;
  double t = tscale * p->B0;
  double s = 2.0 * t / (1 + t * t);
  double h[3] = {1.0 / p->dx, 1.0 / p->dy, 1.0 / p->dz};
  double Escale[3];
  for (int d = 0; d < 3; d++) Escale[d] = -0.5 * h[d] * tscale;
#pragma omp parallel for schedule(static)
  for (int ip = 0; ip < np; ip++) {
    double E[3];
    double x = pos[ip * 3 + 0] / p->dx;
    double y = pos[ip * 3 + 1] / p->dy;
    double z = pos[ip * 3 + 2] / p->dz;
    difference_vector(p, phi, x, y, z, E);
    double vxm = vel[ip * 3 + 0] + Escale[0] * E[0];
    double vym = vel[ip * 3 + 1] + Escale[1] * E[1];
    double vz = vel[ip * 3 + 2] + Escale[2] * E[2];
    double vxt = vxm + vym * t;
    double vyp = vym - vxt * s;
    double vxp = vxt + vyp * t;
    vel[ip * 3 + 0] = vxp;
    vel[ip * 3 + 1] = vyp;
    vel[ip * 3 + 2] = vz;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Position advance + boundary: src/positions.c:455-459, src/boundaries.c:   */
/* 19-31 (one periodic wrap per call).  Reflecting z is defined here (the     */
/* reference names BC_INJECT_REFLECT but does not implement it): specular     */
/* reflection z -> 2 z1 - z (or 2 z0 - z) with vz -> -vz.                     */
/* ------------------------------------------------------------------------ */
int orc_move(const OrcParams *p, int np, double *pos, double *vel, double dt) {
  double r0[3] = {p->x0, p->y0, p->z0};
  double r1v[3] = {p->x1, p->y1, p->z1};
  double L[3] = {p->Lx, p->Ly, p->Lz};
#pragma omp parallel for schedule(static)
  for (int ip = 0; ip < np; ip++) {
    for (int d = 0; d < 3; d++) pos[ip * 3 + d] += vel[ip * 3 + d] * dt;
    for (int d = 0; d < 3; d++) {
      double r = pos[ip * 3 + d];
      double r1 = r1v[d];
      if (p->bc[d] == 0) {
        if (r < r0[d]) r += L[d];
        if (r >= r1) r -= L[d];
      } else {
        if (r < r0[d]) { r = 2.0 * r0[d] - r; vel[ip * 3 + d] = -vel[ip * 3 + d]; }
        if (r >= r1) { r = 2.0 * r1 - r; vel[ip * 3 + d] = -vel[ip * 3 + d]; }
      }
      pos[ip * 3 + d] = r;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* CIC moments: src/moments.c:108-226 (Collect3DFluidMoments)                */
/* Accumulates in particle order into a ghosted (width 1) local array, then   */
/* folds ghosts into owners in local-array order, as DMLocalToGlobal(ADD)     */
/* does.  out is [Nz][Ny][Nx][4].                                             */
/* ------------------------------------------------------------------------ */
static void cic_weights(double x, double y, double z, int idx[3], double w[8]) {
  int ixl = (int)x, iyl = (int)y, izl = (int)z;
  double wxh = x - (double)ixl, wxl = 1.0 - wxh;
  double wyh = y - (double)iyl, wyl = 1.0 - wyh;
  double wzh = z - (double)izl, wzl = 1.0 - wzh;
  idx[0] = ixl; idx[1] = iyl; idx[2] = izl;
  /* corner order b = zb*4 + yb*2 + xb */
  w[7] = wzh * wyh * wxh;
  w[6] = wzh * wyh * wxl;
  w[5] = wzh * wyl * wxh;
  w[4] = wzh * wyl * wxl;
  w[3] = wzl * wyh * wxh;
  w[2] = wzl * wyh * wxl;
  w[1] = wzl * wyl * wxh;
  w[0] = wzl * wyl * wxl;
}

int orc_collect(const OrcParams *p, int np, const double *pos, const double *vel,
                double *out) {
  int gx = p->Nx + 2, gy = p->Ny + 2, gz = p->Nz + 2;
  double *loc = calloc((size_t)gx * gy * gz * 4, sizeof(double));
  if (!loc) return -1;
  for (int ip = 0; ip < np; ip++) {
    int idx[3];
    double w[8];
    cic_weights(pos[ip * 3 + 0] / p->dx, pos[ip * 3 + 1] / p->dy, pos[ip * 3 + 2] / p->dz,
                idx, w);
    /* local index with ghost offset 1; cells beyond the ghost layer are
       outside the reference's defined behaviour and are skipped here */
    for (int b = 0; b < 8; b++) {
      int i = idx[0] + (b & 1) + 1, j = idx[1] + ((b >> 1) & 1) + 1, k = idx[2] + (b >> 2) + 1;
      if (i < 0 || i >= gx || j < 0 || j >= gy || k < 0 || k >= gz) continue;
      double *node = loc + (((size_t)k * gy + j) * gx + i) * 4;
      node[0] += w[b];
    }
    for (int d = 0; d < 3; d++) {
      double v = vel[ip * 3 + d];
      for (int b = 0; b < 8; b++) {
        int i = idx[0] + (b & 1) + 1, j = idx[1] + ((b >> 1) & 1) + 1, k = idx[2] + (b >> 2) + 1;
        if (i < 0 || i >= gx || j < 0 || j >= gy || k < 0 || k >= gz) continue;
        double *node = loc + (((size_t)k * gy + j) * gx + i) * 4;
        node[1 + d] += v * w[b];
      }
    }
  }
  memset(out, 0, sizeof(double) * (size_t)p->Nx * p->Ny * p->Nz * 4);
  for (int kk = 0; kk < gz; kk++) {
    int k = kk - 1;
    if (k < 0 || k >= p->Nz) { if (p->bc[2]) continue; k = wrapi(k, p->Nz); }
    for (int jj = 0; jj < gy; jj++) {
      int j = jj - 1;
      if (j < 0 || j >= p->Ny) { if (p->bc[1]) continue; j = wrapi(j, p->Ny); }
      for (int ii = 0; ii < gx; ii++) {
        int i = ii - 1;
        if (i < 0 || i >= p->Nx) { if (p->bc[0]) continue; i = wrapi(i, p->Nx); }
        const double *src = loc + (((size_t)kk * gy + jj) * gx + ii) * 4;
        double *dst = out + (((size_t)k * p->Ny + j) * p->Nx + i) * 4;
        for (int c = 0; c < 4; c++) dst[c] += src[c];
      }
    }
  }
  free(loc);
  return 0;
}

/* Fixed-point CIC deposit: the same weights as orc_collect, each density
   contribution rounded to an integer multiple of 2^-Sn and each flux
   contribution to a multiple of 2^-Sf (round to nearest even), summed exactly
   in int64, then converted once to FP64.  This is the order-independent
   deposition the GPU library performs; it is exact integer work, so the GPU
   must reproduce it bit for bit.  out is [Nz][Ny][Nx][4] FP64; acc (optional)
   receives the raw int64 sums. */
int orc_collect_fixed(const OrcParams *p, int np, const double *pos, const double *vel,
                      int Sn, int Sf, double *out, int64_t *acc_out) {
  size_t ncell = (size_t)p->Nx * p->Ny * p->Nz;
  int64_t *acc = calloc(ncell * 4, sizeof(int64_t));
  if (!acc) return -1;
  double sc = ldexp(1.0, Sn), scf = ldexp(1.0, Sf);
  for (int ip = 0; ip < np; ip++) {
    int idx[3];
    double w[8];
    cic_weights(pos[ip * 3 + 0] / p->dx, pos[ip * 3 + 1] / p->dy, pos[ip * 3 + 2] / p->dz,
                idx, w);
    for (int b = 0; b < 8; b++) {
      int i = idx[0] + (b & 1), j = idx[1] + ((b >> 1) & 1), k = idx[2] + (b >> 2);
      if (i < 0 || i >= p->Nx) { if (p->bc[0]) continue; i = wrapi(i, p->Nx); }
      if (j < 0 || j >= p->Ny) { if (p->bc[1]) continue; j = wrapi(j, p->Ny); }
      if (k < 0 || k >= p->Nz) { if (p->bc[2]) continue; k = wrapi(k, p->Nz); }
      int64_t *node = acc + (((size_t)k * p->Ny + j) * p->Nx + i) * 4;
      node[0] += (int64_t)llrint(w[b] * sc);
      for (int d = 0; d < 3; d++) node[1 + d] += (int64_t)llrint((vel[ip * 3 + d] * w[b]) * scf);
    }
  }
  double isc = ldexp(1.0, -Sn), iscf = ldexp(1.0, -Sf);
  for (size_t e = 0; e < ncell * 4; e++) out[e] = (double)acc[e] * ((e % 4) == 0 ? isc : iscf);
  if (acc_out) memcpy(acc_out, acc, sizeof(int64_t) * ncell * 4);
  free(acc);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* 2-D particle phase (-ndim 2): positions and velocities are [np][2].       */
/* ------------------------------------------------------------------------ */
/* DifferenceVector2D src/vector-math.c:529-593: bilinear, no weight swap,   */
/* the backward difference at index N as in 3-D.                             */
static void difference_vector2d(const OrcParams *p, const double *F, double x0, double y0, double f[2]) {
  int Nx = p->Nx, Ny = p->Ny;
  int ixl = (int)x0, ixh = ixl + 1, iyl = (int)y0, iyh = iyl + 1;
  double wxh = x0 - (double)ixl, wyh = y0 - (double)iyl;
  double hh, lh, hl, ll, Ewh, Ewl;
#define PHI2(j, i) node_val(p, F, 0, (j), (i))
  if (ixl >= 0) {
    hl = PHI2(iyh, ixl + 1) - PHI2(iyh, ixl - 1);
    ll = PHI2(iyl, ixl + 1) - PHI2(iyl, ixl - 1);
  } else {
    hl = -1.0 * PHI2(iyh, ixl + 2) + 4.0 * PHI2(iyh, ixl + 1) - 3.0 * PHI2(iyh, ixl);
    ll = -1.0 * PHI2(iyl, ixl + 2) + 4.0 * PHI2(iyl, ixl + 1) - 3.0 * PHI2(iyl, ixl);
  }
  if (ixh < Nx) {
    hh = PHI2(iyh, ixh + 1) - PHI2(iyh, ixh - 1);
    lh = PHI2(iyl, ixh + 1) - PHI2(iyl, ixh - 1);
  } else {
    hh = +3.0 * PHI2(iyh, ixh) - 4.0 * PHI2(iyh, ixh - 1) + 1.0 * PHI2(iyh, ixh - 2);
    lh = +3.0 * PHI2(iyl, ixh) - 4.0 * PHI2(iyl, ixh - 1) + 1.0 * PHI2(iyl, ixh - 2);
  }
  Ewh = lh + wyh * (hh - lh);
  Ewl = ll + wyh * (hl - ll);
  f[0] = Ewl + wxh * (Ewh - Ewl);
  if (iyl >= 0) {
    lh = PHI2(iyl + 1, ixh) - PHI2(iyl - 1, ixh);
    ll = PHI2(iyl + 1, ixl) - PHI2(iyl - 1, ixl);
  } else {
    lh = -1.0 * PHI2(iyl + 2, ixh) + 4.0 * PHI2(iyl + 1, ixh) - 3.0 * PHI2(iyl, ixh);
    ll = -1.0 * PHI2(iyl + 2, ixl) + 4.0 * PHI2(iyl + 1, ixl) - 3.0 * PHI2(iyl, ixl);
  }
  if (iyh < Ny) {
    hh = PHI2(iyh + 1, ixh) - PHI2(iyh - 1, ixh);
    hl = PHI2(iyh + 1, ixl) - PHI2(iyh - 1, ixl);
  } else {
    hh = +3.0 * PHI2(iyh, ixh) - 4.0 * PHI2(iyh - 1, ixh) + 1.0 * PHI2(iyh - 2, ixh);
    hl = +3.0 * PHI2(iyh, ixl) - 4.0 * PHI2(iyh - 1, ixl) + 1.0 * PHI2(iyh - 2, ixl);
  }
#undef PHI2
  Ewh = lh + wyh * (hh - lh);
  Ewl = ll + wyh * (hl - ll);
  f[1] = Ewl + wxh * (Ewh - Ewl);
}

/* BorisMoverBz2D src/velocities.c:186-277 (the half E-kick as in 3-D). */
int orc_push2d(const OrcParams *p, int np, const double *pos, double *vel, const double *phi, double dt) {
  double tscale = 0.5 * (p->qi / p->mi) * dt;
  double t = tscale * p->B0;
  double s = 2.0 * t / (1 + t * t);
  double h[2] = {1.0 / p->dx, 1.0 / p->dy};
  double Escale[2];
  for (int d = 0; d < 2; d++) Escale[d] = -0.5 * h[d] * tscale;
  for (int ip = 0; ip < np; ip++) {
    double E[2];
    double x = pos[ip * 2 + 0] / p->dx, y = pos[ip * 2 + 1] / p->dy;
    difference_vector2d(p, phi, x, y, E);
    double vxm = vel[ip * 2 + 0] + Escale[0] * E[0];
    double vym = vel[ip * 2 + 1] + Escale[1] * E[1];
    double vxt = vxm + vym * t;
    double vyp = vym - vxt * s;
    double vxp = vxt + vyp * t;
    vel[ip * 2 + 0] = vxp;
    vel[ip * 2 + 1] = vyp;
  }
  return 0;
}

/* UpdatePositions + Apply2DBC (src/positions.c:455-459, src/boundaries.c:   */
/* 35-40): periodic x and y.                                                  */
int orc_move2d(const OrcParams *p, int np, double *pos, double *vel, double dt) {
  double r0[2] = {p->x0, p->y0}, r1v[2] = {p->x1, p->y1}, L[2] = {p->Lx, p->Ly};
  for (int ip = 0; ip < np; ip++) {
    for (int d = 0; d < 2; d++) pos[ip * 2 + d] += vel[ip * 2 + d] * dt;
    for (int d = 0; d < 2; d++) {
      double r = pos[ip * 2 + d];
      if (r < r0[d]) r += L[d];
      if (r >= r1v[d]) r -= L[d];
      pos[ip * 2 + d] = r;
    }
  }
  return 0;
}

/* Bilinear weights of Collect2DFluidMoments src/moments.c:59-78, corners    */
/* b = yb*2 + xb.                                                             */
static void cic_weights2d(double x, double y, int idx[2], double w[4]) {
  int ixl = (int)x, iyl = (int)y;
  double wxh = x - (double)ixl, wxl = 1.0 - wxh;
  double wyh = y - (double)iyl, wyl = 1.0 - wyh;
  idx[0] = ixl; idx[1] = iyl;
  w[3] = wyh * wxh;
  w[1] = wyl * wxh;
  w[2] = wyh * wxl;
  w[0] = wyl * wxl;
}

/* Collect2DFluidMoments src/moments.c:5-105: particle-order sums into the    */
/* ghosted local array, ghost fold in local-array order; out [1][Ny][Nx][4]   */
/* with Gz = 0.                                                               */
int orc_collect2d(const OrcParams *p, int np, const double *pos, const double *vel, double *out) {
  int gx = p->Nx + 2, gy = p->Ny + 2;
  double *loc = calloc((size_t)gx * gy * 4, sizeof(double));
  if (!loc) return -1;
  static const int order[4] = {3, 1, 2, 0}; /* hh, lh, hl, ll */
  for (int ip = 0; ip < np; ip++) {
    int idx[2];
    double w[4];
    cic_weights2d(pos[ip * 2 + 0] / p->dx, pos[ip * 2 + 1] / p->dy, idx, w);
    for (int q = 0; q < 4; q++) {
      int b = order[q];
      int i = idx[0] + (b & 1) + 1, j = idx[1] + (b >> 1) + 1;
      if (i < 0 || i >= gx || j < 0 || j >= gy) continue;
      loc[((size_t)j * gx + i) * 4] += w[b];
    }
    for (int d = 0; d < 2; d++) {
      double v = vel[ip * 2 + d];
      for (int q = 0; q < 4; q++) {
        int b = order[q];
        int i = idx[0] + (b & 1) + 1, j = idx[1] + (b >> 1) + 1;
        if (i < 0 || i >= gx || j < 0 || j >= gy) continue;
        loc[((size_t)j * gx + i) * 4 + 1 + d] += v * w[b];
      }
    }
  }
  memset(out, 0, sizeof(double) * (size_t)p->Nx * p->Ny * 4);
  for (int jj = 0; jj < gy; jj++) {
    int j = jj - 1;
    if (j < 0 || j >= p->Ny) { if (p->bc[1]) continue; j = wrapi(j, p->Ny); }
    for (int ii = 0; ii < gx; ii++) {
      int i = ii - 1;
      if (i < 0 || i >= p->Nx) { if (p->bc[0]) continue; i = wrapi(i, p->Nx); }
      const double *src = loc + ((size_t)jj * gx + ii) * 4;
      double *dst = out + ((size_t)j * p->Nx + i) * 4;
      for (int c = 0; c < 4; c++) dst[c] += src[c];
    }
  }
  free(loc);
  return 0;
}

/* The fixed-point deposit of orc_collect_fixed for 2-D ions. */
int orc_collect2d_fixed(const OrcParams *p, int np, const double *pos, const double *vel, int Sn, int Sf,
                        double *out) {
  size_t ncell = (size_t)p->Nx * p->Ny;
  int64_t *acc = calloc(ncell * 4, sizeof(int64_t));
  if (!acc) return -1;
  double sc = ldexp(1.0, Sn), scf = ldexp(1.0, Sf);
  for (int ip = 0; ip < np; ip++) {
    int idx[2];
    double w[4];
    cic_weights2d(pos[ip * 2 + 0] / p->dx, pos[ip * 2 + 1] / p->dy, idx, w);
    for (int b = 0; b < 4; b++) {
      int i = wrapi(idx[0] + (b & 1), p->Nx), j = wrapi(idx[1] + (b >> 1), p->Ny);
      int64_t *node = acc + ((size_t)j * p->Nx + i) * 4;
      node[0] += (int64_t)llrint(w[b] * sc);
      for (int d = 0; d < 2; d++) node[1 + d] += (int64_t)llrint((vel[ip * 2 + d] * w[b]) * scf);
    }
  }
  double isc = ldexp(1.0, -Sn), iscf = ldexp(1.0, -Sf);
  for (size_t e = 0; e < ncell * 4; e++) out[e] = (double)acc[e] * ((e % 4) == 0 ? isc : iscf);
  free(acc);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* RHS: src/rhs.c:259-373 (ComputeFullRHS3D), mean removed as                */
/* MatNullSpaceRemove does (sequential sum, then subtract the mean).          */
/* ------------------------------------------------------------------------ */
static inline double mom(const OrcParams *p, const double *m, int k, int j, int i, int c) {
  if (i < 0 || i >= p->Nx) { if (p->bc[0]) return 0.0; i = wrapi(i, p->Nx); }
  if (j < 0 || j >= p->Ny) { if (p->bc[1]) return 0.0; j = wrapi(j, p->Ny); }
  if (k < 0 || k >= p->Nz) { if (p->bc[2]) return 0.0; k = wrapi(k, p->Nz); }
  return m[(((size_t)k * p->Ny + j) * p->Nx + i) * 4 + c];
}

/* Mean removal of MatNullSpaceRemove with the constant null space: b - sum/n. */
static void null_space_remove(double *b, size_t n) {
  double s = 0.0;
  for (size_t e = 0; e < n; e++) s += b[e];
  s = s / (double)n;
  for (size_t e = 0; e < n; e++) b[e] -= s;
}

/* -rhs constant, ComputeConstantRHS src/rhs.c:6-23: b = n0 * scale. */
static void rhs_constant(const OrcParams *p, double *b) {
  size_t n = (size_t)p->Nx * p->Ny * p->Nz;
  double val = p->n0 * p->scale;
  for (size_t e = 0; e < n; e++) b[e] = val;
}

/* -rhs sinusoidal, ComputeSinusoidalRHS3D src/rhs.c:82-148: at the cell
   centres x = (i + 0.5) dx (grid units), b = n0 cos(2 pi x) cos(2 pi y)
   cos(2 pi z) scale, then the constant null space removed. */
static void rhs_sinusoidal(const OrcParams *p, double *b) {
  const double PI = 3.141592653589793238462643383279502884;
  if (p->ndim == 2) {  /* ComputeSinusoidalRHS2D src/rhs.c:26-79 */
    for (int j = 0; j < p->Ny; j++)
      for (int i = 0; i < p->Nx; i++) {
        double x = ((double)i + 0.5) * p->dx, y = ((double)j + 0.5) * p->dy;
        double Cx = cos(2 * PI * x), Cy = cos(2 * PI * y);
        double val = Cx * Cy;
        b[(size_t)j * p->Nx + i] = p->n0 * val * p->scale;
      }
    null_space_remove(b, (size_t)p->Nx * p->Ny);
    return;
  }
  for (int k = 0; k < p->Nz; k++)
    for (int j = 0; j < p->Ny; j++)
      for (int i = 0; i < p->Nx; i++) {
        double x = ((double)i + 0.5) * p->dx, y = ((double)j + 0.5) * p->dy, z = ((double)k + 0.5) * p->dz;
        double Cx = cos(2 * PI * x), Cy = cos(2 * PI * y), Cz = cos(2 * PI * z);
        double val = Cx * Cy * Cz;
        b[((size_t)k * p->Ny + j) * p->Nx + i] = p->n0 * val * p->scale;
      }
  null_space_remove(b, (size_t)p->Nx * p->Ny * p->Nz);
}

static int rhs_full(const OrcParams *p, const double *m, double *b);

/* RHS by -rhs type (the ctx->potential.rhs binding of src/setup.c:63-90). */
int orc_rhs(const OrcParams *p, const double *m, double *b) {
  if (p->rhs_type == 0) { rhs_constant(p, b); return 0; }
  if (p->rhs_type == 1) { rhs_sinusoidal(p, b); return 0; }
  return rhs_full(p, m, b);
}

/* ComputeFullRHS2D src/rhs.c:151-258 */
static int rhs_full2d(const OrcParams *p, const double *m, double *b) {
  double kappa = p->kappa_e;
  double hx = 1.0 / (2.0 * p->dx), hy = 1.0 / (2.0 * p->dy);
  double hxx = 1.0 / (p->dx * p->dx), hyy = 1.0 / (p->dy * p->dy);
  size_t n = (size_t)p->Nx * p->Ny;
  for (int j = 0; j < p->Ny; j++)
    for (int i = 0; i < p->Nx; i++) {
      double nijk = mom(p, m, 0, j, i, 0);
      double npjk = mom(p, m, 0, j, i + 1, 0), nmjk = mom(p, m, 0, j, i - 1, 0);
      double nipk = mom(p, m, 0, j + 1, i, 0), nimk = mom(p, m, 0, j - 1, i, 0);
      double dndx = hx * (npjk - nmjk);
      double dndy = hy * (nipk - nimk);
      double d2ndxx = hxx * (npjk - 2 * nijk + nmjk);
      double d2ndyy = hyy * (nipk - 2 * nijk + nimk);
      double dGxdx = hx * (mom(p, m, 0, j, i + 1, 1) - mom(p, m, 0, j, i - 1, 1));
      double dGydy = hy * (mom(p, m, 0, j + 1, i, 2) - mom(p, m, 0, j - 1, i, 2));
      double Eterm = (dndy - kappa * dndx) * p->E0;
      double Pterm = p->cth * (d2ndxx + d2ndyy);
      double Gterm = p->cG * (dGxdx + dGydy);
      b[(size_t)j * p->Nx + i] = p->scale * (Eterm + Pterm + Gterm);
    }
  double s = 0.0;
  for (size_t e = 0; e < n; e++) s += b[e];
  s = s / (-(double)n);
  for (size_t e = 0; e < n; e++) b[e] += s;
  return 0;
}

static int rhs_full(const OrcParams *p, const double *m, double *b) {
  if (p->ndim == 2) return rhs_full2d(p, m, b);
  double kappa = p->kappa_e;
  double hx = 1.0 / (2.0 * p->dx), hy = 1.0 / (2.0 * p->dy), hz = 1.0 / (2.0 * p->dz);
  double hxx = 1.0 / (p->dx * p->dx), hyy = 1.0 / (p->dy * p->dy), hzz = 1.0 / (p->dz * p->dz);
  size_t n = (size_t)p->Nx * p->Ny * p->Nz;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < p->Nz; k++)
    for (int j = 0; j < p->Ny; j++)
      for (int i = 0; i < p->Nx; i++) {
        double nijk = mom(p, m, k, j, i, 0);
        double npjk = mom(p, m, k, j, i + 1, 0), nmjk = mom(p, m, k, j, i - 1, 0);
        double nipk = mom(p, m, k, j + 1, i, 0), nimk = mom(p, m, k, j - 1, i, 0);
        double nijp = mom(p, m, k + 1, j, i, 0), nijm = mom(p, m, k - 1, j, i, 0);
        double dndx = hx * (npjk - nmjk);
        double dndy = hy * (nipk - nimk);
        double d2ndxx = hxx * (npjk - 2 * nijk + nmjk);
        double d2ndyy = hyy * (nipk - 2 * nijk + nimk);
        double d2ndzz = hzz * (nijp - 2 * nijk + nijm);
        double dGxdx = hx * (mom(p, m, k, j, i + 1, 1) - mom(p, m, k, j, i - 1, 1));
        double dGydy = hy * (mom(p, m, k, j + 1, i, 2) - mom(p, m, k, j - 1, i, 2));
        double dGzdz = hz * (mom(p, m, k + 1, j, i, 3) - mom(p, m, k - 1, j, i, 3));
        double Eterm = (dndy - kappa * dndx) * p->E0;
        double Pterm = p->cth * (d2ndxx + d2ndyy + (1 + kappa * kappa) * d2ndzz);
        double Gterm = p->cG * (dGxdx + dGydy + dGzdz);
        b[((size_t)k * p->Ny + j) * p->Nx + i] = p->scale * (Eterm + Pterm + Gterm);
      }
  double s = 0.0;
  for (size_t e = 0; e < n; e++) s += b[e];
  s = s / (-(double)n);
  for (size_t e = 0; e < n; e++) b[e] += s;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Operator: src/lhs.c:337-505 (ComputeFullLHS3D).  The 11 coefficients of   */
/* row (k,j,i) in the reference's insertion order: x+, x-, y+, y-, z+, z-,    */
/* (x+,y+), (x+,y-), (x-,y+), (x-,y-), centre.                                */
/* ------------------------------------------------------------------------ */
static const int k_off[11][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1},
                                 {0, 0, -1}, {1, 1, 0}, {1, -1, 0}, {-1, 1, 0}, {-1, -1, 0},
                                 {0, 0, 0}}; /* (di, dj, dk) */

static inline double dens(const OrcParams *p, const double *n, int k, int j, int i) {
  return node_val(p, n, k, j, i);
}

/* Rows of -lhs identity (ComputeIdentityLHS src/lhs.c:11-23: A = I) and
   -lhs laplacian (ComputeLaplacianLHS3D src/lhs.c:101-191: 1/h^2 off the
   diagonal, the diagonal minus their sum in insertion order) in the 11-entry
   layout; the corner entries stay 0. */
static int lhs_row_simple(const OrcParams *p, double v[11]) {
  for (int e = 0; e < 11; e++) v[e] = 0.0;
  if (p->lhs_type == 0) { v[10] = 1.0; return 1; }
  if (p->lhs_type != 1) return 0;
  double vpjk = 1.0 / (p->dx * p->dx), vmjk = 1.0 / (p->dx * p->dx);
  double vipk = 1.0 / (p->dy * p->dy), vimk = 1.0 / (p->dy * p->dy);
  v[0] = vpjk; v[1] = vmjk; v[2] = vipk; v[3] = vimk;
  if (p->ndim == 2) {  /* ComputeLaplacianLHS2D src/lhs.c:26-97 */
    v[10] = -(vpjk + vipk + vmjk + vimk);
    return 1;
  }
  double vijp = 1.0 / (p->dz * p->dz), vijm = 1.0 / (p->dz * p->dz);
  v[4] = vijp; v[5] = vijm;
  v[10] = -(vpjk + vipk + vijp + vmjk + vimk + vijm);
  return 1;
}

void orc_lhs_row(const OrcParams *p, const double *n, int k, int j, int i, double v[11]) {
  if (lhs_row_simple(p, v)) return;
  double kappa = p->kappa_e, scale = p->scale;
  double hxx = 1.0 / (2.0 * p->dx * p->dx);
  double hyy = 1.0 / (2.0 * p->dy * p->dy);
  double hzz = 1.0 / (2.0 * p->dz * p->dz);
  double hod = 1.0 / (8.0 * p->dy * p->dx);
  double sxx = scale * hxx, syy = scale * hyy;
  double szz = scale * (1 + kappa * kappa) * hzz;
  double sod = scale * kappa * hod;
  double nijk = dens(p, n, k, j, i);
  double nmjk = dens(p, n, k, j, i - 1), npjk = dens(p, n, k, j, i + 1);
  double nimk = dens(p, n, k, j - 1, i), nipk = dens(p, n, k, j + 1, i);
  double nijm = dens(p, n, k - 1, j, i), nijp = dens(p, n, k + 1, j, i);
  if (p->ndim == 2) {  /* ComputeFullLHS2D src/lhs.c:194-335: the in-plane 9 entries */
    v[6] = sod * (nipk - npjk);
    v[7] = sod * (npjk - nimk);
    v[8] = sod * (nmjk - nipk);
    v[9] = sod * (nimk - nmjk);
    v[0] = sxx * (npjk + nijk) + sod * (nipk - nimk);
    v[1] = sxx * (nijk + nmjk) - sod * (nipk - nimk);
    v[2] = syy * (nipk + nijk) - sod * (npjk - nmjk);
    v[3] = syy * (nijk + nimk) + sod * (npjk - nmjk);
    v[4] = v[5] = 0.0;
    v[10] = -(sxx * (npjk + 2 * nijk + nmjk) + syy * (nipk + 2 * nijk + nimk));
    return;
  }
  v[6] = sod * (nipk - npjk);
  v[7] = sod * (npjk - nimk);
  v[8] = sod * (nmjk - nipk);
  v[9] = sod * (nimk - nmjk);
  v[0] = sxx * (npjk + nijk) + sod * (nipk - nimk);
  v[1] = sxx * (nijk + nmjk) - sod * (nipk - nimk);
  v[2] = syy * (nipk + nijk) - sod * (npjk - nmjk);
  v[3] = syy * (nijk + nimk) + sod * (npjk - nmjk);
  v[4] = szz * (nijp + nijk);
  v[5] = szz * (nijk + nijm);
  v[10] = -(sxx * (npjk + 2 * nijk + nmjk) + syy * (nipk + 2 * nijk + nimk) +
            szz * (nijp + 2 * nijk + nijm));
}

/* Dense operator (small grids only); out-of-range columns of non-periodic
   dimensions are dropped, as MatSetValuesStencil does for ghosted DMDAs. */
int orc_lhs_dense(const OrcParams *p, const double *n, double *A) {
  int N = p->Nx * p->Ny * p->Nz;
  memset(A, 0, sizeof(double) * (size_t)N * N);
  for (int k = 0; k < p->Nz; k++)
    for (int j = 0; j < p->Ny; j++)
      for (int i = 0; i < p->Nx; i++) {
        double v[11];
        int row = (k * p->Ny + j) * p->Nx + i;
        orc_lhs_row(p, n, k, j, i, v);
        for (int e = 0; e < 11; e++) {
          int ci = i + k_off[e][0], cj = j + k_off[e][1], ck = k + k_off[e][2];
          if (ci < 0 || ci >= p->Nx) { if (p->bc[0]) continue; ci = wrapi(ci, p->Nx); }
          if (cj < 0 || cj >= p->Ny) { if (p->bc[1]) continue; cj = wrapi(cj, p->Ny); }
          if (ck < 0 || ck >= p->Nz) { if (p->bc[2]) continue; ck = wrapi(ck, p->Nz); }
          A[(size_t)row * N + (ck * p->Ny + cj) * p->Nx + ci] = v[e];
        }
      }
  return 0;
}

/* y = A x, matrix free, entries summed in insertion order. */
int orc_lhs_apply(const OrcParams *p, const double *n, const double *x, double *y) {
#pragma omp parallel for schedule(static)
  for (int k = 0; k < p->Nz; k++)
    for (int j = 0; j < p->Ny; j++)
      for (int i = 0; i < p->Nx; i++) {
        double v[11], s = 0.0;
        orc_lhs_row(p, n, k, j, i, v);
        for (int e = 0; e < 11; e++)
          s += v[e] * node_val(p, x, k + k_off[e][2], j + k_off[e][1], i + k_off[e][0]);
        y[((size_t)k * p->Ny + j) * p->Nx + i] = s;
      }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Potential solve (stand-in for PETSc KSPSolve, src/potential.c:6-15):      */
/* restarted GMRES(m) with modified Gram-Schmidt and Givens rotations, zero   */
/* initial guess (src/potential.c:20-29), stopping on ||b-Ax||/||b|| <= rtol; */
/* the constant null space is projected out of the iterate at every restart   */
/* and at exit.  Returns the iteration count, or -1 on allocation failure.    */
/* ------------------------------------------------------------------------ */
static double dotv(const double *a, const double *b, size_t n) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (size_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}
static void remove_mean(const OrcParams *p, double *x, size_t n) {
  if (p->bc[0] || p->bc[1] || p->bc[2]) return; /* nonsingular when not fully periodic */
  double s = 0.0;
  for (size_t i = 0; i < n; i++) s += x[i];
  s /= (double)n;
  for (size_t i = 0; i < n; i++) x[i] -= s;
}

int orc_gmres(const OrcParams *p, const double *dens_n, const double *b, double *x,
              double rtol, int maxit, int m, double *relres_out) {
  size_t n = (size_t)p->Nx * p->Ny * p->Nz;
  double *V = malloc(sizeof(double) * n * (size_t)(m + 1));
  double *w = malloc(sizeof(double) * n);
  double *H = calloc((size_t)(m + 1) * m, sizeof(double));
  double *cs = malloc(sizeof(double) * m), *sn = malloc(sizeof(double) * m);
  double *g = malloc(sizeof(double) * (m + 1)), *yv = malloc(sizeof(double) * m);
  if (!V || !w || !H || !cs || !sn || !g || !yv) return -1;
  double bnorm = sqrt(dotv(b, b, n));
  int it = 0;
  double relres = 0.0;
  memset(x, 0, sizeof(double) * n);
  if (bnorm == 0.0) {
    if (relres_out) *relres_out = 0.0;
    goto done;
  }
  for (;;) {
    orc_lhs_apply(p, dens_n, x, w);
    for (size_t i = 0; i < n; i++) V[i] = b[i] - w[i];
    double beta = sqrt(dotv(V, V, n));
    relres = beta / bnorm;
    if (relres <= rtol || it >= maxit) break;
    for (size_t i = 0; i < n; i++) V[i] /= beta;
    memset(g, 0, sizeof(double) * (m + 1));
    g[0] = beta;
    int jj;
    for (jj = 0; jj < m && it < maxit; jj++, it++) {
      double *vj = V + (size_t)jj * n, *vn = V + (size_t)(jj + 1) * n;
      orc_lhs_apply(p, dens_n, vj, vn);
      for (int q = 0; q <= jj; q++) {
        double hq = dotv(vn, V + (size_t)q * n, n);
        H[q * m + jj] = hq;
        for (size_t i = 0; i < n; i++) vn[i] -= hq * V[(size_t)q * n + i];
      }
      double hn = sqrt(dotv(vn, vn, n));
      H[(jj + 1) * m + jj] = hn;
      if (hn > 0) for (size_t i = 0; i < n; i++) vn[i] /= hn;
      for (int q = 0; q < jj; q++) {
        double a = H[q * m + jj], c = H[(q + 1) * m + jj];
        H[q * m + jj] = cs[q] * a + sn[q] * c;
        H[(q + 1) * m + jj] = -sn[q] * a + cs[q] * c;
      }
      double a = H[jj * m + jj], c = H[(jj + 1) * m + jj];
      double r = sqrt(a * a + c * c);
      cs[jj] = r > 0 ? a / r : 1.0;
      sn[jj] = r > 0 ? c / r : 0.0;
      H[jj * m + jj] = r;
      H[(jj + 1) * m + jj] = 0.0;
      g[jj + 1] = -sn[jj] * g[jj];
      g[jj] = cs[jj] * g[jj];
      if (fabs(g[jj + 1]) / bnorm <= rtol * 0.5) { jj++; it++; break; }
    }
    for (int q = jj - 1; q >= 0; q--) {
      double s = g[q];
      for (int r2 = q + 1; r2 < jj; r2++) s -= H[q * m + r2] * yv[r2];
      yv[q] = s / H[q * m + q];
    }
    for (int q = 0; q < jj; q++)
      for (size_t i = 0; i < n; i++) x[i] += yv[q] * V[(size_t)q * n + i];
    remove_mean(p, x, n);
  }
  remove_mean(p, x, n);
  if (relres_out) *relres_out = relres;
done:
  free(V); free(w); free(H); free(cs); free(sn); free(g); free(yv);
  return it;
}

/* ------------------------------------------------------------------------ */
/* Random numbers with the reference's process-global state.                 */
/*   ran1   (src/random.c:24-72): Park-Miller minimal standard generator      */
/*          (a = 16807, m = 2^31-1, Schrage factorisation) behind a 32-entry   */
/*          Bays-Durham shuffle, 8 warm-up draws, float output capped below 1. */
/*   ran3   (src/random.c:94-154): Knuth's subtractive generator (modulus 1e9, */
/*          55-entry lagged table, lag 24), re-seeded whenever *idum < 0.      */
/*   gasdev (src/random.c:172-204): Marsaglia polar method on ran1, caching    */
/*          the second deviate; *idum < 0 drops the cache.                     */
/* ------------------------------------------------------------------------ */
static long r1_iy = 0;
static long r1_iv[32];
static int r3_inext, r3_inextp, r3_iff = 0;
static long r3_ma[56];
static int gd_iset = 0;
static float gd_gset;

void orc_rng_reset(void) {
  r1_iy = 0;
  memset(r1_iv, 0, sizeof r1_iv);
  r3_iff = 0;
  gd_iset = 0;
  gd_gset = 0.0f;
}

float orc_ran1(long *idum) {
  const long A = 16807, M = 2147483647, Qd = 127773, Rm = 2836;
  const long NDIV = 1 + (M - 1) / 32;
  const double AM = 1.0 / M, RNMX = 1.0 - 2.2204460492503131e-16;
  long k;
  if (*idum <= 0 || !r1_iy) {
    *idum = (-(*idum) < 1) ? 1 : -(*idum);
    for (int j = 32 + 7; j >= 0; j--) {
      k = *idum / Qd;
      *idum = A * (*idum - k * Qd) - Rm * k;
      if (*idum < 0) *idum += M;
      if (j < 32) r1_iv[j] = *idum;
    }
    r1_iy = r1_iv[0];
  }
  k = *idum / Qd;
  *idum = A * (*idum - k * Qd) - Rm * k;
  if (*idum < 0) *idum += M;
  int j = (int)(r1_iy / NDIV);
  r1_iy = r1_iv[j];
  r1_iv[j] = *idum;
  float temp = AM * r1_iy;
  return (temp > RNMX) ? RNMX : temp;
}

float orc_ran3(long *idum) {
  const long MBIG = 1000000000, MSEED = 161803398;
  long mj, mk;
  if (*idum < 0 || r3_iff == 0) {
    r3_iff = 1;
    mj = labs(MSEED - labs(*idum)) % MBIG;
    r3_ma[55] = mj;
    mk = 1;
    for (int i = 1; i <= 54; i++) {
      int ii = (21 * i) % 55;
      r3_ma[ii] = mk;
      mk = mj - mk;
      if (mk < 0) mk += MBIG;
      mj = r3_ma[ii];
    }
    for (int k = 1; k <= 4; k++)
      for (int i = 1; i <= 55; i++) {
        r3_ma[i] -= r3_ma[1 + (i + 30) % 55];
        if (r3_ma[i] < 0) r3_ma[i] += MBIG;
      }
    r3_inext = 0;
    r3_inextp = 31;
    *idum = 1;
  }
  if (++r3_inext == 56) r3_inext = 1;
  if (++r3_inextp == 56) r3_inextp = 1;
  mj = r3_ma[r3_inext] - r3_ma[r3_inextp];
  if (mj < 0) mj += MBIG;
  r3_ma[r3_inext] = mj;
  return mj * (1.0 / MBIG);
}

float orc_gasdev(long *idum) {
  float fac, rsq, v1, v2;
  if (*idum < 0) gd_iset = 0;
  if (gd_iset == 0) {
    do {
      v1 = 2.0 * orc_ran1(idum) - 1.0;
      v2 = 2.0 * orc_ran1(idum) - 1.0;
      rsq = v1 * v1 + v2 * v2;
    } while (rsq >= 1.0 || rsq == 0.0);
    fac = sqrt(-2.0 * log(rsq) / rsq);
    gd_gset = v1 * fac;
    gd_iset = 1;
    return v2 * fac;
  }
  gd_iset = 0;
  return gd_gset;
}

/* Batch access for tests. */
int orc_ran1_n(long *idum, int n, float *out) { for (int i = 0; i < n; i++) out[i] = orc_ran1(idum); return 0; }
int orc_ran3_n(long *idum, int n, float *out) { for (int i = 0; i < n; i++) out[i] = orc_ran3(idum); return 0; }
int orc_gasdev_n(long *idum, int n, float *out) { for (int i = 0; i < n; i++) out[i] = orc_gasdev(idum); return 0; }

/* ------------------------------------------------------------------------ */
/* Sobol points (src/random.c:233-289, src/positions.c:139-233): Bratley-Fox */
/* Gray-code generator, 30 bits, first 6 dimensions with the primitive        */
/* polynomials (degree mdeg, interior coefficients ip) and initial direction  */
/* numbers of the published algorithm, restarted at index 0 (the state of a   */
/* freshly started reference process).  pos[ip*3+d] = x_d * L_d.             */
/* Reference behaviour kept: the recurrence for the higher direction numbers  */
/* XORs v[j-1] where the published method uses v[j-l] (src/random.c:264), so  */
/* dimensions whose polynomial has degree >= 3 (z here) differ from textbook  */
/* Sobol points.                                                              */
/* ------------------------------------------------------------------------ */
int orc_sobol(const OrcParams *p, int np, double *pos) {
  enum { MAXBIT = 30, MAXDIM = 6 };
  static const unsigned long mdeg[MAXDIM + 1] = {0, 1, 2, 3, 3, 4, 4};
  static const unsigned long ipoly[MAXDIM + 1] = {0, 0, 1, 1, 2, 1, 4};
  static const unsigned long init[4][MAXDIM + 1] = {
      {0, 1, 1, 1, 1, 1, 1}, {0, 3, 1, 3, 3, 1, 1}, {0, 5, 7, 7, 3, 3, 5}, {0, 15, 11, 5, 15, 13, 9}};
  unsigned long v[MAXBIT + 1][MAXDIM + 1];
  unsigned long x[MAXDIM + 1] = {0};
  memset(v, 0, sizeof v);
  for (int k = 1; k <= MAXDIM; k++) {
    for (unsigned long j = 1; j <= mdeg[k]; j++) v[j][k] = init[j - 1][k] << (MAXBIT - j);
    for (unsigned long j = mdeg[k] + 1; j <= MAXBIT; j++) {
      unsigned long ipp = ipoly[k];
      unsigned long i = v[j - mdeg[k]][k];
      i ^= (i >> mdeg[k]);
      for (long l = (long)mdeg[k] - 1; l >= 1; l--) {
        if (ipp & 1) i ^= v[j - 1][k];
        ipp >>= 1;
      }
      v[j][k] = i;
    }
  }
  double fac = 1.0 / (double)(1L << MAXBIT);
  double L[3] = {p->Lx, p->Ly, p->Lz};
  for (long n = 0; n < np; n++) {
    unsigned long im = (unsigned long)n;
    int j;
    for (j = 1; j <= MAXBIT; j++) {
      if (!(im & 1)) break;
      im >>= 1;
    }
    if (j > MAXBIT) return -1;
    for (int k = 1; k <= 3; k++) {
      x[k] ^= v[j][k];
      pos[n * 3 + (k - 1)] = (x[k] * fac) * L[k - 1];
    }
  }
  return 0;
}

/* Maxwellian velocities (src/velocities.c:14-47): v_d = vT_d*gasdev + v0_d
   with the rank-0 seed -12345 (src/random.c:292-295). */
int orc_normal_velocities(const double vT[3], const double v0[3], int np, double *vel) {
  long seed = -12345;
  for (int ip = 0; ip < np; ip++)
    for (int d = 0; d < 3; d++) {
      double dv = (double)orc_gasdev(&seed);
      vel[ip * 3 + d] = vT[d] * dv + v0[d];
    }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Elastic ion-neutral collisions: src/collisions.c:9-167 (ScatterElastic).  */
/* Reference behaviour kept: the local seed restarts at -12345 every call, so */
/* ran3 is re-seeded and repeats its stream each step; the acceptance draw    */
/* PetscSqr(ran3(&seed)) expands to the product of two ran3 draws computed in */
/* float; the ion index np*ran3 is formed in float.  Returns the number of    */
/* accepted collisions, or -(10+Nf) when 10 results were refused (where the   */
/* reference aborts).  stats[0..2] = attempts, accepted, refused.             */
/* ------------------------------------------------------------------------ */
int orc_collide(const OrcParams *p, int np, double *vel, double dt, long *stats) {
  double fc = p->nui * dt, viT = p->viT, vnT = p->vnT;
  double mi = p->mi, mn = p->mn, M = mn + mi;
  double tmp = 0.0;
  for (int d = 0; d < 3; d++) tmp += (p->vi0[d] - p->vn0[d]) * (p->vi0[d] - p->vn0[d]);
  double vrm = 4.0 * viT + sqrt(tmp);
  int Nc = (int)(((double)np * fc * vrm) / ((vnT + p->vn0mag) * sqrt(mn / mi)));
  if (Nc > np) Nc = np;
  else if (Nc < 0) Nc = 0;
  long seed = -12345;
  int Ns = 0, Nf = 0;
  long attempts = 0;
  while (Ns < Nc) {
    int ip = (int)(np * orc_ran3(&seed));
    if (ip >= np) ip = np - 1; /* float product can round to np; the reference would index past the end */
    attempts++;
    double vi[3], vn[3], vr[3], vc[3];
    tmp = 0.0;
    for (int d = 0; d < 3; d++) {
      vi[d] = vel[ip * 3 + d];
      vn[d] = orc_gasdev(&seed) * vnT + p->vn0[d];
      vr[d] = vi[d] - vn[d];
      tmp += vr[d] * vr[d];
    }
    double vrr = sqrt(tmp);
    float u1 = orc_ran3(&seed);
    float u2 = orc_ran3(&seed);
    if (u1 * u2 < (vrr * vrr) / (vrm * vrm)) {
      tmp = 0.0;
      for (int d = 0; d < 3; d++) {
        vc[d] = (vi[d] * mi + vn[d] * mn) / M;
        tmp += (vi[d] - vc[d]) * (vi[d] - vc[d]);
      }
      double vcr = sqrt(tmp);
      double u0z = 2.0 * orc_ran3(&seed) - 1.0;
      double uperp = sqrt(1.0 - u0z * u0z);
      double uphi = 2 * 3.14159265358979323846264338327950288419716939937510582 * orc_ran3(&seed);
      double u0x = uperp * cos(uphi);
      double u0y = uperp * sin(uphi);
      double costht = vr[2] / vrr;
      double sintht = sqrt(1.0 - costht * costht);
      double cosphi = vr[0] / (vrr * sintht);
      double sinphi = vr[1] / (vrr * sintht);
      double u1x = u0z * sintht + u0x * costht;
      double u1y = u0y;
      double u1z = u0z * costht - u0x * sintht;
      double u2v[3] = {u1x * cosphi - u1y * sinphi, u1x * sinphi + u1y * cosphi, u1z};
      double vf[3];
      tmp = 0.0;
      for (int d = 0; d < 3; d++) {
        vf[d] = vc[d] + vcr * u2v[d];
        tmp += vf[d] * vf[d];
      }
      double ratio = sqrt(tmp) / viT;
      if (ratio > 10) {
        Nf++;
        if (Nf >= 10) {
          if (stats) { stats[0] = attempts; stats[1] = Ns; stats[2] = Nf; }
          return -(10 + Nf);
        }
      } else {
        for (int d = 0; d < 3; d++) vel[ip * 3 + d] = vf[d];
        Ns++;
      }
    }
  }
  if (stats) { stats[0] = attempts; stats[1] = Ns; stats[2] = Nf; }
  return Ns;
}

/* Number of collisions the reference attempts to complete per call
   (src/collisions.c:58-63). */
int orc_collision_count(const OrcParams *p, int np, double dt) {
  double tmp = 0.0;
  for (int d = 0; d < 3; d++) tmp += (p->vi0[d] - p->vn0[d]) * (p->vi0[d] - p->vn0[d]);
  double vrm = 4.0 * p->viT + sqrt(tmp);
  int Nc = (int)(((double)np * (p->nui * dt) * vrm) / ((p->vnT + p->vn0mag) * sqrt(p->mn / p->mi)));
  if (Nc > np) Nc = np;
  else if (Nc < 0) Nc = 0;
  return Nc;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Multi-threaded CIC deposit for timing the CPU baseline on all host cores.
   The grid is split into z slabs, one per OpenMP thread, as the reference's
   ranks split the domain (each rank deposits into its subdomain plus a ghost
   layer and adds the ghosts to their owners, src/moments.c:108-226 with
   DMLocalToGlobal(ADD)): thread t deposits the ions whose base cell lies in
   its slab, into the slab's planes and a private copy of the plane above,
   which is then added to the plane's owner.  Same weights as orc_collect;
   only the summation order differs. */
int orc_collect_mt(const OrcParams *p, int np, const double *pos, const double *vel, double *out) {
  int nt = orc_num_threads();
  if (nt > p->Nz) nt = p->Nz;
  if (nt < 1) nt = 1;
  const size_t plane = (size_t)p->Nx * p->Ny * 4;
  memset(out, 0, sizeof(double) * plane * (size_t)p->Nz);
  double *top = calloc(plane * (size_t)nt, sizeof(double)); /* the plane above each slab */
  if (!top) return -1;
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    const int t = omp_get_thread_num();
#else
    const int t = 0;
#endif
    const int k0 = (int)((long long)p->Nz * t / nt), k1 = (int)((long long)p->Nz * (t + 1) / nt);
    double *T = top + plane * (size_t)t;
    for (int ip = 0; ip < np; ip++) {
      const double z = pos[ip * 3 + 2] / p->dz;
      const int izl = (int)z;
      if (izl < k0 || izl >= k1) continue;
      int idx[3];
      double w[8];
      cic_weights(pos[ip * 3 + 0] / p->dx, pos[ip * 3 + 1] / p->dy, z, idx, w);
      for (int b = 0; b < 8; b++) {
        int i = idx[0] + (b & 1), j = idx[1] + ((b >> 1) & 1);
        const int k = idx[2] + (b >> 2);
        if (i < 0 || i >= p->Nx) { if (p->bc[0]) continue; i = wrapi(i, p->Nx); }
        if (j < 0 || j >= p->Ny) { if (p->bc[1]) continue; j = wrapi(j, p->Ny); }
        double *node;
        if (k < k1) {
          node = out + (((size_t)k * p->Ny + j) * p->Nx + i) * 4;
        } else {
          if (k >= p->Nz && p->bc[2]) continue; /* past a ghosted z edge: dropped */
          node = T + ((size_t)j * p->Nx + i) * 4;
        }
        node[0] += w[b];
        node[1] += vel[ip * 3 + 0] * w[b];
        node[2] += vel[ip * 3 + 1] * w[b];
        node[3] += vel[ip * 3 + 2] * w[b];
      }
    }
  }
  for (int t = 0; t < nt; t++) { /* each slab's upper plane to its owner */
    int k = (int)((long long)p->Nz * (t + 1) / nt);
    if (k >= p->Nz) {
      if (p->bc[2]) continue;
      k -= p->Nz;
    }
    double *dst = out + plane * (size_t)k;
    const double *src = top + plane * (size_t)t;
    for (size_t e = 0; e < plane; e++) dst[e] += src[e];
  }
  free(top);
  return 0;
}
