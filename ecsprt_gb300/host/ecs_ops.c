/*
 * The reference's operator slots bound to libecsgpu (include/ecs_compat.h).
 *
 * SetUpContext (src/setup.c:23-114) binds the LHS and RHS by -lhs / -rhs and
 * ndim, and the particle operators by ndim (BorisMoverBz3D/2D, ScatterElastic,
 * Apply3DBC/2DBC, Collect3DFluidMoments/2D).  EcsGpuBindOperatorsFor fills
 * the same slots with the GPU counterparts by the same rules;
 * EcsGpuBindOperators is the default 3-D full binding.  The GPU LHS and RHS
 * read the operator type from the context's parameters, so every LHS slot
 * calls ecs_lhs and every RHS slot ecs_rhs.  The stage wrappers keep
 * UpdateVelocities' rule that collisions run only when the neutral mass is
 * positive (src/velocities.c:384).
 */
#include <stddef.h>

#include "ecs_compat.h"

static EcsGpuContext *gctx(void *opts) { return (EcsGpuContext *)opts; }

PetscErrorCode EcsGpuPushBz3D(PetscReal dt, void *opts) { return ecs_push(gctx(opts)->ctx, dt); }
PetscErrorCode EcsGpuPushBz2D(PetscReal dt, void *opts) { return ecs_push(gctx(opts)->ctx, dt); }

/* 2-D collisions are undefined in the reference (ScatterElastic reads the
   unset z component of the relative velocity, src/collisions.c:104). */
PetscErrorCode EcsGpuScatterElastic(PetscInt ndim, PetscReal dt, void *opts) {
  if (ndim != 3) return ECS_ERR_UNSUPPORTED;
  return ecs_collide(gctx(opts)->ctx, dt);
}

/* Periodic wrap of src/boundaries.c:19-31 (reflection on z, as the device
   move) applied to host arrays of nd components an ion, or (NULL arrays) to
   the device-resident ions, whose boundary is applied by the position
   advance itself. */
static PetscErrorCode apply_bc(int nd, PetscInt np, PetscReal *pos, PetscReal *vel, void *opts) {
  EcsGpuContext *g = gctx(opts);
  if (!pos) return ECS_OK;
  const EcsParams *p = &g->params;
  const double r0[3] = {p->x0, p->y0, p->z0}, r1[3] = {p->x1, p->y1, p->z1};
  const double L[3] = {p->Lx, p->Ly, p->Lz};
  for (PetscInt ip = 0; ip < np; ip++)
    for (int d = 0; d < nd; d++) {
      double r = pos[ip * nd + d];
      if (p->bc[d] == ECS_BC_PERIODIC) {
        if (r < r0[d]) r += L[d];
        if (r >= r1[d]) r -= L[d];
      } else if (p->bc[d] == ECS_BC_INJECT_REFLECT) {
        if (r < r0[d]) { r = 2.0 * r0[d] - r; if (vel) vel[ip * nd + d] = -vel[ip * nd + d]; }
        if (r >= r1[d]) { r = 2.0 * r1[d] - r; if (vel) vel[ip * nd + d] = -vel[ip * nd + d]; }
      }
      pos[ip * nd + d] = r;
    }
  return ECS_OK;
}
PetscErrorCode EcsGpuApply3DBC(PetscInt np, PetscReal *pos, PetscReal *vel, void *opts) {
  return apply_bc(3, np, pos, vel, opts);
}
PetscErrorCode EcsGpuApply2DBC(PetscInt np, PetscReal *pos, PetscReal *vel, void *opts) {
  return apply_bc(2, np, pos, vel, opts);
}

PetscErrorCode EcsGpuCollect3D(void *opts) { return ecs_collect(gctx(opts)->ctx); }
PetscErrorCode EcsGpuCollect2D(void *opts) { return ecs_collect(gctx(opts)->ctx); }

PetscErrorCode EcsGpuFullLHS3D(KSP ksp, Mat J, Mat A, void *opts) {
  (void)ksp; (void)J; (void)A;
  return ecs_lhs(gctx(opts)->ctx);
}

PetscErrorCode EcsGpuFullRHS3D(KSP ksp, Vec b, void *opts) {
  (void)ksp; (void)b;
  return ecs_rhs(gctx(opts)->ctx);
}

/* The other operators of src/lhs.c:11-335 and src/rhs.c:6-258 (the context's
   lhs_type / rhs_type / ndim select the arithmetic on the device). */
PetscErrorCode EcsGpuIdentityLHS(KSP ksp, Mat J, Mat A, void *opts) { return EcsGpuFullLHS3D(ksp, J, A, opts); }
PetscErrorCode EcsGpuLaplacianLHS2D(KSP ksp, Mat J, Mat A, void *opts) { return EcsGpuFullLHS3D(ksp, J, A, opts); }
PetscErrorCode EcsGpuLaplacianLHS3D(KSP ksp, Mat J, Mat A, void *opts) { return EcsGpuFullLHS3D(ksp, J, A, opts); }
PetscErrorCode EcsGpuFullLHS2D(KSP ksp, Mat J, Mat A, void *opts) { return EcsGpuFullLHS3D(ksp, J, A, opts); }
PetscErrorCode EcsGpuConstantRHS(KSP ksp, Vec b, void *opts) { return EcsGpuFullRHS3D(ksp, b, opts); }
PetscErrorCode EcsGpuSinusoidalRHS2D(KSP ksp, Vec b, void *opts) { return EcsGpuFullRHS3D(ksp, b, opts); }
PetscErrorCode EcsGpuSinusoidalRHS3D(KSP ksp, Vec b, void *opts) { return EcsGpuFullRHS3D(ksp, b, opts); }
PetscErrorCode EcsGpuFullRHS2D(KSP ksp, Vec b, void *opts) { return EcsGpuFullRHS3D(ksp, b, opts); }

void EcsGpuBindOperators(EcsOperators *ops) {
  ops->applyBC = EcsGpuApply3DBC;
  ops->collect = EcsGpuCollect3D;
  ops->push = EcsGpuPushBz3D;
  ops->collide = EcsGpuScatterElastic;
  ops->lhs = EcsGpuFullLHS3D;
  ops->rhs = EcsGpuFullRHS3D;
}

int EcsGpuBindOperatorsFor(EcsOperators *ops, const EcsParams *p) {
  if (!ops || !p || (p->ndim != 2 && p->ndim != 3)) return ECS_ERR_INVALID;
  const int three = p->ndim == 3;
  switch (p->lhs_type) {  /* src/setup.c:27-57 */
    case ECS_LHS_IDENTITY: ops->lhs = EcsGpuIdentityLHS; break;
    case ECS_LHS_LAPLACIAN: ops->lhs = three ? EcsGpuLaplacianLHS3D : EcsGpuLaplacianLHS2D; break;
    case ECS_LHS_FULL: ops->lhs = three ? EcsGpuFullLHS3D : EcsGpuFullLHS2D; break;
    default: return ECS_ERR_INVALID;
  }
  switch (p->rhs_type) {  /* src/setup.c:60-88 */
    case ECS_RHS_CONSTANT: ops->rhs = EcsGpuConstantRHS; break;
    case ECS_RHS_SINUSOIDAL: ops->rhs = three ? EcsGpuSinusoidalRHS3D : EcsGpuSinusoidalRHS2D; break;
    case ECS_RHS_FULL: ops->rhs = three ? EcsGpuFullRHS3D : EcsGpuFullRHS2D; break;
    default: return ECS_ERR_INVALID;
  }
  /* src/setup.c:91-105 */
  ops->applyBC = three ? EcsGpuApply3DBC : EcsGpuApply2DBC;
  ops->collect = three ? EcsGpuCollect3D : EcsGpuCollect2D;
  ops->push = three ? EcsGpuPushBz3D : EcsGpuPushBz2D;
  ops->collide = EcsGpuScatterElastic;
  return ECS_OK;
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
