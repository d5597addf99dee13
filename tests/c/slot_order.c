/*
 * The reference's time loop (src/pic.c:244-258) through the operator slots
 * it binds (src/setup.c:23-114): UpdateVelocities (push, then collide when
 * mn > 0), UpdatePositions (move + BC), collect, ComputePotential (RHS,
 * LHS, KSPSolve), on one context; the fused ecs_step on another context
 * from the same initial ions.  Both must give the same moments, potential
 * and ions bit for bit.
 *
 *   slot_order fp64|mixed NSTEPS
 *
 * Exit status 0 when every step matched, 1 on a mismatch, 2 on an error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ecs_compat.h"
#include "ecs_host.h"

#define CHECK(x)                                                                  \
  do {                                                                            \
    int rc_ = (x);                                                                \
    if (rc_) {                                                                    \
      fprintf(stderr, "%s:%d %s -> %d (%s)\n", __FILE__, __LINE__, #x, rc_,        \
              ecs_last_error(NULL));                                              \
      return 2;                                                                   \
    }                                                                             \
  } while (0)

/* the ions of a context in the order of their identities */
static int ions_by_id(EcsCtx *c, int64_t np, double *pos, double *vel) {
  double *p = malloc(sizeof(double) * 3 * np), *v = malloc(sizeof(double) * 3 * np);
  int32_t *id = malloc(sizeof(int32_t) * np);
  int rc = ecs_particles_download(c, p, v);
  if (!rc) rc = ecs_particles_ids(c, id);
  for (int64_t i = 0; !rc && i < np; i++)
    for (int d = 0; d < 3; d++) {
      pos[3 * (int64_t)id[i] + d] = p[3 * i + d];
      vel[3 * (int64_t)id[i] + d] = v[3 * i + d];
    }
  free(p); free(v); free(id);
  return rc;
}

static int differ(const char *what, int step, const double *a, const double *b, int64_t n) {
  int64_t bad = 0, first = -1;
  for (int64_t i = 0; i < n; i++)
    if (memcmp(&a[i], &b[i], sizeof(double)) != 0) {
      if (first < 0) first = i;
      bad++;
    }
  if (bad) printf("step %d: %s differs in %lld of %lld values (first %lld: %.17g vs %.17g)\n", step, what,
                  (long long)bad, (long long)n, (long long)first, a[first], b[first]);
  return bad != 0;
}

int main(int argc, char **argv) {
  const int prec = argc > 1 && strcmp(argv[1], "fp64") == 0 ? ECS_PREC_FP64 : ECS_PREC_MIXED;
  const int nsteps = argc > 2 ? atoi(argv[2]) : 4;
  EcsOptions *o = ecs_options_create();
  ecs_options_parse(o, "-Nx 16 -Ny 16 -Nz 16 -dx 1 -dy 1 -dz 1 -qi 1 -mi 1 -B0 0.1 -viT 1 -vi0x 0.5 "
                       "-nui 0.5 -nue 8.79e9 -Te 11604.5 -E0 0 -Np -16");
  EcsParams p;
  char err[256];
  CHECK(ecs_params_from_options(o, &p, err, sizeof err));
  const int64_t np = 16 * 16 * 16 * 16, n = 16 * 16 * 16;
  const double dt = 0.1, rtol = 1e-8;
  const int max_it = 200;
  EcsCtx *a = NULL, *b = NULL;
  CHECK(ecs_ctx_create(&p, prec, np, NULL, &a));
  CHECK(ecs_ctx_create(&p, prec, np, NULL, &b));
  CHECK(ecs_particles_init(a, ECS_INIT_SOBOL, np, 7, NULL));
  CHECK(ecs_particles_init(b, ECS_INIT_SOBOL, np, 7, NULL));

  EcsOperators ops;
  CHECK(EcsGpuBindOperatorsFor(&ops, &p));
  EcsGpuContext ga, gb;
  memset(&ga, 0, sizeof ga);
  ga.ctx = a; ga.params = p; ga.rtol = rtol; ga.max_it = max_it;
  gb = ga;
  gb.ctx = b;
  /* initial moments and potential (src/pic.c:212-217), both contexts */
  CHECK(ops.collect(&ga));
  CHECK(EcsGpuComputePotential(&ops, &ga));
  CHECK(ops.collect(&gb));
  CHECK(EcsGpuComputePotential(&ops, &gb));

  double *ma = malloc(sizeof(double) * 4 * n), *mb = malloc(sizeof(double) * 4 * n);
  double *fa = malloc(sizeof(double) * n), *fb = malloc(sizeof(double) * n);
  double *pa = malloc(sizeof(double) * 3 * np), *pb = malloc(sizeof(double) * 3 * np);
  double *va = malloc(sizeof(double) * 3 * np), *vb = malloc(sizeof(double) * 3 * np);
  int bad = 0;
  long long collisions = 0;
  for (int it = 0; it < nsteps; it++) {
    CHECK(EcsGpuUpdateVelocities(&ops, p.ndim, dt, &ga));
    CHECK(EcsGpuUpdatePositions(&ops, p.ndim, dt, &ga));
    CHECK(ops.collect(&ga));
    CHECK(EcsGpuComputePotential(&ops, &ga));
    EcsStepStats st;
    CHECK(ecs_step(b, dt, rtol, max_it, &st));
    collisions += st.collisions;
    CHECK(ecs_moments_download(a, ma));
    CHECK(ecs_moments_download(b, mb));
    CHECK(ecs_phi_download(a, fa));
    CHECK(ecs_phi_download(b, fb));
    CHECK(ions_by_id(a, np, pa, va));
    CHECK(ions_by_id(b, np, pb, vb));
    bad |= differ("moments", it, ma, mb, 4 * n);
    bad |= differ("potential", it, fa, fb, n);
    bad |= differ("positions", it, pa, pb, 3 * np);
    bad |= differ("velocities", it, va, vb, 3 * np);
    printf("step %d: solve %d iterations (slots) / %d (step), relres %.3e\n", it, ga.last_solve.iterations,
           st.solve.iterations, st.solve.relres);
  }
  printf("%s: %d steps, %lld collisions, %s\n", prec == ECS_PREC_FP64 ? "fp64" : "mixed", nsteps, collisions,
         bad ? "MISMATCH" : "bit-identical");
  ecs_ctx_destroy(a);
  ecs_ctx_destroy(b);
  ecs_options_destroy(o);
  return bad ? 1 : 0;
}
