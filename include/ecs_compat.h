/*
 * ecs_compat.h -- the reference's operator function-pointer interface over
 * plain C types, with GPU implementations to bind into the same slots.
 *
 * Reference interface kept (paths relative to the reference project):
 *   typedefs LHSFunc, RHSFunc, BCFunc, CollectFunc, CollideFunc, PushFunc
 *     src/global.h:27-32
 *   slots ions.{push,collide,applyBC,collect}, potential.{lhs,rhs}
 *     src/ecsprt.h:89-92,100-101, bound in SetUpContext src/setup.c:23-114
 *   stage wrappers UpdateVelocities src/velocities.c:375,
 *     UpdatePositions src/positions.c:436, ComputePotential src/potential.c:6
 *
 * Without PETSc the scalar types become plain C types and KSP/Mat/Vec become
 * opaque handles.  Every function takes `void *opts` exactly as the
 * reference's operators do; here opts is an EcsGpuContext*, which owns the
 * device state (ecsgpu.h) of one simulation.  Return value: 0 on success,
 * otherwise a negative ECS_ERR_* status (the reference's PetscErrorCode
 * convention: non-zero is failure).
 */
#ifndef ECS_COMPAT_H
#define ECS_COMPAT_H

#include <stdint.h>

#include "ecsgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifndef PETSC_SUCCESS
typedef int PetscErrorCode;
typedef int32_t PetscInt;
typedef double PetscReal;
typedef struct EcsKspHandle *KSP;
typedef struct EcsMatHandle *Mat;
typedef struct EcsVecHandle *Vec;
#endif

/* src/global.h:28-33 */
typedef PetscErrorCode (*LHSFunc)(KSP ksp, Mat J, Mat A, void *opts);
typedef PetscErrorCode (*RHSFunc)(KSP ksp, Vec b, void *opts);
typedef PetscErrorCode (*BCFunc)(PetscInt np, PetscReal *pos, PetscReal *vel, void *opts);
typedef PetscErrorCode (*CollectFunc)(void *opts);
typedef PetscErrorCode (*CollideFunc)(PetscInt ndim, PetscReal dt, void *opts);
typedef PetscErrorCode (*PushFunc)(PetscReal dt, void *opts);

/* The operator slots of Species/Linear (src/ecsprt.h:89-92,100-101). */
typedef struct EcsOperators {
  BCFunc applyBC;
  CollectFunc collect;
  PushFunc push;
  CollideFunc collide;
  LHSFunc lhs;
  RHSFunc rhs;
} EcsOperators;

/* What `opts` points to for the GPU operators. */
typedef struct EcsGpuContext {
  EcsCtx *ctx;           /* device state */
  EcsParams params;      /* derived parameters */
  double rtol;           /* potential solve tolerance (default 1e-8) */
  int32_t max_it;        /* solve iteration cap (default 200) */
  EcsSolveStats last_solve;
} EcsGpuContext;

/* GPU implementations for the slots (same signatures as the reference's
   BorisMoverBz3D, ScatterElastic, Apply3DBC, Collect3DFluidMoments,
   ComputeFullLHS3D, ComputeFullRHS3D). */
PetscErrorCode EcsGpuPushBz3D(PetscReal dt, void *opts);
PetscErrorCode EcsGpuScatterElastic(PetscInt ndim, PetscReal dt, void *opts);
/* pos/vel NULL: apply to the device-resident ions (the GPU analogue of
   ApplyBCAndMigrate); host arrays: applied to those np ions in place. */
PetscErrorCode EcsGpuApply3DBC(PetscInt np, PetscReal *pos, PetscReal *vel, void *opts);
PetscErrorCode EcsGpuCollect3D(void *opts);
PetscErrorCode EcsGpuFullLHS3D(KSP ksp, Mat J, Mat A, void *opts);
PetscErrorCode EcsGpuFullRHS3D(KSP ksp, Vec b, void *opts);
/* 2-D (src/velocities.c:186, src/boundaries.c:35, src/moments.c:5,
   src/lhs.c:194, src/rhs.c:151) and the other operator options
   (src/lhs.c:11-191, src/rhs.c:6-148). */
PetscErrorCode EcsGpuPushBz2D(PetscReal dt, void *opts);
PetscErrorCode EcsGpuApply2DBC(PetscInt np, PetscReal *pos, PetscReal *vel, void *opts);
PetscErrorCode EcsGpuCollect2D(void *opts);
PetscErrorCode EcsGpuFullLHS2D(KSP ksp, Mat J, Mat A, void *opts);
PetscErrorCode EcsGpuFullRHS2D(KSP ksp, Vec b, void *opts);
PetscErrorCode EcsGpuIdentityLHS(KSP ksp, Mat J, Mat A, void *opts);
PetscErrorCode EcsGpuLaplacianLHS2D(KSP ksp, Mat J, Mat A, void *opts);
PetscErrorCode EcsGpuLaplacianLHS3D(KSP ksp, Mat J, Mat A, void *opts);
PetscErrorCode EcsGpuConstantRHS(KSP ksp, Vec b, void *opts);
PetscErrorCode EcsGpuSinusoidalRHS2D(KSP ksp, Vec b, void *opts);
PetscErrorCode EcsGpuSinusoidalRHS3D(KSP ksp, Vec b, void *opts);

/* SetUpContext analogue: fill the slots with the GPU operators (3-D, full). */
void EcsGpuBindOperators(EcsOperators *ops);
/* The same by the parameters' ndim, lhs_type and rhs_type, as SetUpContext's
   switches (src/setup.c:23-105); ECS_ERR_INVALID for unknown types. */
int EcsGpuBindOperatorsFor(EcsOperators *ops, const EcsParams *p);

/* Stage wrappers with the reference's semantics. */
PetscErrorCode EcsGpuUpdateVelocities(const EcsOperators *ops, PetscInt ndim, PetscReal dt,
                                      EcsGpuContext *g);
PetscErrorCode EcsGpuUpdatePositions(const EcsOperators *ops, PetscInt ndim, PetscReal dt,
                                     EcsGpuContext *g);
PetscErrorCode EcsGpuComputePotential(const EcsOperators *ops, EcsGpuContext *g);

#ifdef __cplusplus
}
#endif
#endif /* ECS_COMPAT_H */
