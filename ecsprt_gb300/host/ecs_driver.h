/*
 * Helpers shared by the re-hosted programs (pic, solver): the options file
 * and command line (src/common.c:16-22), --version (src/common.c:26-31),
 * --log-level (src/common.c:33-50) and the options that select the GPU
 * path.  Not part of the library's ABI.
 */
#ifndef ECS_DRIVER_H
#define ECS_DRIVER_H

#include <stdint.h>

#include "ecs_host.h"

/* Options file argv[1] when that names an existing file, else ./petsc.ini
   when it exists; the remaining command-line tokens override it. */
int ecs_drv_load_options(int argc, char **argv, EcsOptions *o);
/* --version: print the reference's banner for `name`; returns 1 if printed. */
int ecs_drv_version(const EcsOptions *o, const char *name);
/* --log-level (default 1): 0 silent, >= 1 status lines, >= 2 details. */
void ecs_drv_log_level(const EcsOptions *o);
void ecs_drv_status(const char *fmt, ...);
void ecs_drv_detail(const char *fmt, ...);
/* Print the message and return the process status for an ECS_ERR_* code. */
int ecs_drv_fail(int code, const char *msg);

typedef struct EcsDrvExtra {
  int precision;      /* --precision fp64|mixed (default mixed) */
  int sort_every;     /* --sort-every (default 2) */
  uint64_t seed;      /* --seed (default 20261203) */
  double rtol;        /* -ksp_rtol (PETSc's default 1e-5) */
  int32_t max_it;     /* -ksp_max_it (PETSc's default 10000) */
} EcsDrvExtra;
void ecs_drv_extra(const EcsOptions *o, EcsDrvExtra *x);

#endif /* ECS_DRIVER_H */
