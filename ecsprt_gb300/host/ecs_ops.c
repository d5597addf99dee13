/*
 * The reference's operator slots bound to libecsgpu (include/ecs_compat.h).
 *
 * SetUpContext (src/setup.c:106-114) binds BorisMoverBz3D, ScatterElastic,
 * Apply3DBC, Collect3DFluidMoments, ComputeFullLHS3D and ComputeFullRHS3D;
 * EcsGpuBindOperators binds their GPU counterparts into the same slots.  The
 * stage wrappers keep UpdateVelocities' rule that collisions run only when the
 * neutral mass is positive (src/velocities.c:384).
 */
#include <stddef.h>

#include "ecs_compat.h"

static EcsGpuContext *gctx(void *opts) { return (EcsGpuContext *)opts; }

PetscErrorCode EcsGpuPushBz3D(PetscReal dt, void *opts) { return ecs_push(gctx(opts)->ctx, dt); }

PetscErrorCode EcsGpuScatterElastic(PetscInt ndim, PetscReal dt, void *opts) {
  if (ndim != 3) return ECS_ERR_UNSUPPORTED;
  return ecs_collide(gctx(opts)->ctx, dt);
}

/* Periodic wrap of src/boundaries.c:19-31 applied to host arrays, or (NULL
   arrays) to the device-resident ions, whose boundary is applied by the
   position advance itself. */
PetscErrorCode EcsGpuApply3DBC(PetscInt np, PetscReal *pos, PetscReal *vel, void *opts) {
  EcsGpuContext *g = gctx(opts);
  if (!pos) return ECS_OK;
  const EcsParams *p = &g->params;
  const double r0[3] = {p->x0, p->y0, p->z0}, r1[3] = {p->x1, p->y1, p->z1};
  const double L[3] = {p->Lx, p->Ly, p->Lz};
  for (PetscInt ip = 0; ip < np; ip++)
    for (int d = 0; d < 3; d++) {
      double r = pos[ip * 3 + d];
      if (p->bc[d] == ECS_BC_PERIODIC) {
        if (r < r0[d]) r += L[d];
        if (r >= r1[d]) r -= L[d];
      } else if (p->bc[d] == ECS_BC_INJECT_REFLECT) {
        if (r < r0[d]) { r = 2.0 * r0[d] - r; if (vel) vel[ip * 3 + d] = -vel[ip * 3 + d]; }
        if (r >= r1[d]) { r = 2.0 * r1[d] - r; if (vel) vel[ip * 3 + d] = -vel[ip * 3 + d]; }
      }
      pos[ip * 3 + d] = r;
    }
  return ECS_OK;
}

PetscErrorCode EcsGpuCollect3D(void *opts) { return ecs_collect(gctx(opts)->ctx); }

PetscErrorCode EcsGpuFullLHS3D(KSP ksp, Mat J, Mat A, void *opts) {
  (void)ksp; (void)J; (void)A;
  return ecs_lhs(gctx(opts)->ctx);
}

PetscErrorCode EcsGpuFullRHS3D(KSP ksp, Vec b, void *opts) {
  (void)ksp; (void)b;
  return ecs_rhs(gctx(opts)->ctx);
}

void EcsGpuBindOperators(EcsOperators *ops) {
  ops->applyBC = EcsGpuApply3DBC;
  ops->collect = EcsGpuCollect3D;
  ops->push = EcsGpuPushBz3D;
  ops->collide = EcsGpuScatterElastic;
  ops->lhs = EcsGpuFullLHS3D;
  ops->rhs = EcsGpuFullRHS3D;
}

PetscErrorCode EcsGpuUpdateVelocities(const EcsOperators *ops, PetscInt ndim, PetscReal dt,
                                      EcsGpuContext *g) {
  PetscErrorCode rc = ops->push(dt, g);
  if (rc) return rc;
  if (g->params.mn > 0.0) rc = ops->collide(ndim, dt, g);
  return rc;
}

PetscErrorCode EcsGpuUpdatePositions(const EcsOperators *ops, PetscInt ndim, PetscReal dt,
                                     EcsGpuContext *g) {
  (void)ndim;
  PetscErrorCode rc = ecs_move(g->ctx, dt);
  if (rc) return rc;
  return ops->applyBC(0, NULL, NULL, g);
}

PetscErrorCode EcsGpuComputePotential(const EcsOperators *ops, EcsGpuContext *g) {
  PetscErrorCode rc = ops->rhs(NULL, NULL, g);
  if (rc) return rc;
  rc = ops->lhs(NULL, NULL, NULL, g);
  if (rc) return rc;
  return ecs_solve(g->ctx, g->rtol > 0 ? g->rtol : 1e-8, g->max_it > 0 ? g->max_it : 200, 0, &g->last_solve);
}
