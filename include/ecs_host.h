/*
 * ecs_host.h -- host-side C of the GB300 ECSPRT path (libecshost): options
 * database, parameter derivation and output files.  No CUDA, no PETSc.
 *
 * Reference behaviour replaced (paths relative to the reference project):
 *   PetscInitialize options file (argv[1] or petsc.ini)  src/common.c:16-22
 *                                          -> ecs_options_load_file / _parse
 *   ProcessOptions (names and defaults)    src/parameters.c:25-346
 *   SetUpContext + NormalizeGrid           src/setup.c:13-277, 296-346
 *                                          -> ecs_params_from_options
 *   ProcessPICOptions                      src/pic.c:32-115 -> ecs_pic_app_from_options
 *   ProcessSolverOptions                   src/solver.c:29-74 -> ecs_solver_app_from_options
 *   EchoOptions (options.log)              src/parameters.c:354-433 -> ecs_echo_options
 *   OutputSwarmBinary (PETSc binary Vec)   src/file-io.c:103-161 -> ecs_write_petsc_vec
 *   OutputFluidHDF5 datasets               src/file-io.c:164-222 -> ecs_write_fluid
 */
#ifndef ECS_HOST_H
#define ECS_HOST_H

#include <stdint.h>

#include "ecsgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct EcsOptions EcsOptions;

EcsOptions *ecs_options_create(void);
void ecs_options_destroy(EcsOptions *o);
/* "-key value" tokens (PETSc options-file syntax; '#' starts a comment).
   Later occurrences override earlier ones. */
int ecs_options_parse(EcsOptions *o, const char *text);
int ecs_options_load_file(EcsOptions *o, const char *path);
/* Value of an option (NULL if absent or given without value); *found set. */
const char *ecs_options_get(const EcsOptions *o, const char *key, int *found);

/* ProcessOptions + SetUpContext + NormalizeGrid.  Returns ECS_OK or
   ECS_ERR_INVALID with a message in err. */
int ecs_params_from_options(const EcsOptions *o, EcsParams *p, char *err, int errlen);

/* Position distributions, src/pic.h:7-14 (PDistTypes order). */
enum { ECS_PDIST_SOBOL = 0, ECS_PDIST_REVERSE, ECS_PDIST_NORMAL, ECS_PDIST_UNIFORM,
       ECS_PDIST_SINUSOIDAL, ECS_PDIST_GAUSSIAN };

typedef struct EcsPicApp {
  int32_t Nt;              /* -Nt, default 1 */
  double dt;               /* -dt, default 1/nui */
  int32_t every;           /* --every, default 1 */
  int64_t Np;              /* total ions: -Np > 0 total, < 0 per cell, default one per cell */
  int32_t pdist;           /* --position-dist, default sobol */
  int32_t vdist;           /* --velocity-dist, default normal (0) */
  int32_t output_particles;/* --output-particles */
} EcsPicApp;
int ecs_pic_app_from_options(const EcsOptions *o, const EcsParams *p, EcsPicApp *app, char *err,
                             int errlen);

typedef struct EcsSolverApp {
  char input[4096];        /* --input */
  double flux_scale[3];    /* --flux-scale, --{x,y,z}-flux-scale, default 1 */
  int32_t view_lhs;        /* --view-lhs */
} EcsSolverApp;
int ecs_solver_app_from_options(const EcsOptions *o, EcsSolverApp *app);

/* options.log as EchoOptions writes it. */
int ecs_echo_options(const char *path, const EcsOptions *o, const EcsParams *p);

/* PETSc binary Vec: int32 class id 1211214, int32 length, FP64 values, all
   big-endian (the format VecView writes to a binary viewer). */
int ecs_write_petsc_vec(const char *path, const double *v, int64_t n);
int ecs_read_petsc_vec(const char *path, double *v, int64_t n);
/* Fluid output: the six datasets of fluid<insert>.hdf (density, x flux,
   y flux, z flux, rhs, potential) written as consecutive PETSc binary Vecs
   to fluid<insert>.bin (HDF5 is not available to this build). */
int ecs_write_fluid(const char *path, const double *moments, const double *rhs,
                    const double *phi, int64_t ncell);

#ifdef __cplusplus
}
#endif
#endif /* ECS_HOST_H */
