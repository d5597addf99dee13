/*
 * ecsgpu.h -- C ABI of libecsgpu, the GB300 (sm_103a) implementation of the
 * ECSPRT per-timestep hot path.
 *
 * Plain C types only: pointers, sizes, doubles.  Every entry point returns an
 * int status (ECS_OK = 0, negative on error, see ecs_status_string).  A
 * context owns all device state of one simulation or solver instance and
 * runs on one CUDA stream; calls on one context must come from one host
 * thread at a time.  Different contexts are independent.
 *
 * Reference interface replaced (paths relative to the reference project):
 *   PushFunc    BorisMoverBz3D          src/velocities.c:281   -> ecs_push
 *   CollideFunc ScatterElastic          src/collisions.c:9     -> ecs_collide
 *   (positions) UpdatePositions         src/positions.c:436    -> ecs_move
 *   BCFunc      Apply3DBC/ApplyBCAndMigrate src/boundaries.c:45,57 -> ecs_move
 *   CollectFunc Collect3DFluidMoments   src/moments.c:108      -> ecs_collect
 *   RHSFunc     ComputeFullRHS3D        src/rhs.c:259          -> ecs_rhs
 *   LHSFunc     ComputeFullLHS3D        src/lhs.c:337          -> ecs_lhs
 *   ComputePotential (KSPSolve)         src/potential.c:6      -> ecs_solve
 *   one time step of the loop           src/pic.c:238-269      -> ecs_step
 * The function-pointer typedefs themselves are kept in ecs_compat.h.
 */
#ifndef ECSGPU_H
#define ECSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define ECS_OK 0
#define ECS_ERR_INVALID (-1)       /* bad argument or size */
#define ECS_ERR_NOMEM (-2)         /* device or host allocation failed */
#define ECS_ERR_NOT_CONVERGED (-3) /* Krylov solve hit max_it above rtol */
#define ECS_ERR_NONFINITE (-4)     /* NaN/Inf in a velocity, moment or potential */
#define ECS_ERR_TIMEOUT (-5)       /* a bounded device wait gave up */
#define ECS_ERR_CUDA (-6)          /* CUDA runtime error (message in ecs_last_error) */
#define ECS_ERR_COLLISION (-7)     /* >= 10 collisions refused in one call (reference aborts) */
#define ECS_ERR_RANGE (-8)         /* particle outside the domain, or deposit range exceeded */
#define ECS_ERR_STATE (-9)         /* call out of order (e.g. solve before lhs) */
#define ECS_ERR_UNSUPPORTED (-10)  /* option the GPU path does not implement */

/* ---- enumerations (values match the reference's enums) ------------------ */
/* BCType, src/ecsprt.h:26-30.  BC_INJECT_REFLECT is honoured on z only, as
   specular reflection with Dirichlet-0 ghost nodes (no reference behaviour). */
enum { ECS_BC_PERIODIC = 0, ECS_BC_INJECT_REFLECT = 1, ECS_BC_INJECT_ADVECT = 2 };
/* LHSType / RHSType, src/global.h:8-22. */
enum { ECS_LHS_IDENTITY = 0, ECS_LHS_LAPLACIAN = 1, ECS_LHS_FULL = 2 };
enum { ECS_RHS_CONSTANT = 0, ECS_RHS_SINUSOIDAL = 1, ECS_RHS_FULL = 2 };
/* Arithmetic of the particle phase and of the inner solve. */
enum {
  ECS_PREC_FP64 = 0,  /* plain: FP64 SoA particles, FP64 multigrid + FGMRES */
  ECS_PREC_MIXED = 1  /* cell-sorted SoA (int32 cell, FP32 offset/velocity),
                         FP32 multigrid-FGMRES inside FP64 iterative refinement */
};

/* Physical and grid parameters after the reference's derivations
   (ProcessOptions src/parameters.c:25, SetUpContext src/setup.c:13,
   NormalizeGrid src/setup.c:296).  ecs_host.h fills it from options. */
typedef struct EcsParams {
  int32_t ndim, Nx, Ny, Nz;
  int32_t bc[3];
  int32_t lhs_type, rhs_type;
  double dx, dy, dz;
  double x0, y0, z0, x1, y1, z1;
  double Lx, Ly, Lz;
  double qi, mi, B0, E0, n0;
  double nui;                        /* ion-neutral collision frequency */
  double viT, viTx, viTy, viTz;      /* ion thermal speed: magnitude, components */
  double vi0x, vi0y, vi0z, vi0;      /* ion drift */
  double Ti;
  double qe, me, nue, Te;
  double veTx, veTy, veTz, veT;
  double ve0x, ve0y, ve0z, ve0;      /* electron drift */
  double Omega_e, kappa_e, Omega_i, kappa_i;
  double gammaT;
  double mn, Tn, vnT;                /* neutral mass (0 disables collisions), temperature, thermal speed */
  double vn0x, vn0y, vn0z, vn0;
  double scale;                      /* potential.scale = 1/(1+kappa_e^2) */
  double cth, cG;                    /* RHS coefficients gammaT*KB*Te/Q and (1+kappa^2)*me*nue/Q */
} EcsParams;

typedef struct EcsCtx EcsCtx;

typedef struct EcsSolveStats {
  int32_t iterations;     /* inner Krylov iterations, all refinement sweeps */
  int32_t refinements;    /* FP64 outer corrections (1 for ECS_PREC_FP64) */
  double relres;          /* final ||b - A phi||_2 / ||b||_2, measured in FP64 */
  double seconds;         /* wall time of the solve on the context stream */
} EcsSolveStats;

typedef struct EcsStepStats {
  int64_t collisions;     /* accepted collisions this step */
  int64_t refused;        /* collisions refused (final speed > 10 viT) */
  int32_t sorted;         /* 1 if the particles were cell-sorted this step */
  EcsSolveStats solve;
  double particle_seconds;/* device time of the fused particle kernel (CUDA events) */
  double sort_seconds;    /* device time of the cell sort (0 if none) */
} EcsStepStats;

/* ---- library ------------------------------------------------------------ */
const char *ecs_version(void);
const char *ecs_status_string(int status);
/* Message of the last error on this context (or of the last failed create
   when ctx is NULL). */
const char *ecs_last_error(const EcsCtx *ctx);

/* ---- context lifecycle -------------------------------------------------- */
/* np_capacity bounds the ion count; stream is a cudaStream_t (NULL: the
   context creates its own non-blocking stream).  ndim = 2 (-ndim 2:
   BorisMoverBz2D, Collect2DFluidMoments, ComputeFullLHS2D/RHS2D) takes
   Nz = 1 and no collisions (the reference's ScatterElastic reads an unset
   z component in 2-D): ECS_ERR_UNSUPPORTED when mn > 0. */
int ecs_ctx_create(const EcsParams *params, int precision, int64_t np_capacity,
                   void *stream, EcsCtx **out);
int ecs_ctx_destroy(EcsCtx *ctx);
int ecs_ctx_sync(EcsCtx *ctx);
/* Device bytes held by a context of these sizes (for admission control). */
int64_t ecs_ctx_device_bytes(const EcsParams *params, int precision, int64_t np_capacity);
/* Cell-sort cadence of the mixed path (default 2; 0 disables sorting). */
int ecs_set_sort_every(EcsCtx *ctx, int every);
/* Seed of the counter-based collision RNG (default 20261203). */
int ecs_set_seed(EcsCtx *ctx, uint64_t seed);
/* ecs_step starts each solve from the previous potential instead of zero
   (default 0, the reference's zero guess, src/potential.c:20-29). */
int ecs_set_warm_start(EcsCtx *ctx, int warm);
/* Run each FGMRES cycle of the solve as one CUDA graph (default 1), or let
   the host launch its Arnoldi steps one by one (0).  Both give identical
   results.  No counterpart in the reference (PETSc's KSP runs on the host). */
int ecs_set_solver_graphs(EcsCtx *ctx, int on);

/* ---- particles (host arrays in the reference's DMSwarm layout) ---------- */
/* pos/vel are AoS FP64: pos[ip*ndim+d], vel[ip*ndim+d] (src/velocities.c:342-356;
   ndim = 2 for -ndim 2, src/velocities.c:254-266). */
int ecs_particles_upload(EcsCtx *ctx, const double *pos, const double *vel, int64_t np);
/* The mixed path keeps its ions counting-sorted by cell, so a download
   returns them in the device's order, not the order of the upload (as
   DMSwarmMigrate reorders a swarm across ranks, src/boundaries.c:92). */
int ecs_particles_download(EcsCtx *ctx, double *pos, double *vel);
int64_t ecs_particles_count(const EcsCtx *ctx);
/* ids[i] = the identity of the i-th ion of a download: its index in the
   arrays of the last ecs_particles_upload (or in ecs_particles_init).  The
   FP64 path never reorders, so there ids[i] = i.  No counterpart in the
   reference (a single-rank DMSwarm keeps its order). */
int ecs_particles_ids(EcsCtx *ctx, int32_t *ids);

/* ---- initial ions generated on the device -------------------------------- */
/* Position distributions: the PDistType values of src/positions.c:8-10 that
   the reference implements, plus Fourier-mode densities. */
enum {
  ECS_INIT_SOBOL = 0,      /* SobolDistribution src/positions.c:139-233: the same
                              positions, bit for bit (np < 2^30) */
  ECS_INIT_RANDOM = 2,     /* "normal", src/positions.c:42-137: uniform s*L (ran3 there,
                              a counter-based generator here: same distribution) */
  ECS_INIT_SINUSOIDAL = 4, /* Rejection + SinusoidalDistribution src/positions.c:236-388:
                              density 1 + 0.25 sin(2 pi x/Lx), same acceptance test */
  ECS_INIT_MODES = 16      /* density 1 + sum_m a_m cos(2 pi k_m.(x/L) + phase_m) by
                              rejection (no reference counterpart; sum |a_m| < 1) */
};
typedef struct EcsDensityModes {
  int32_t nmodes;       /* at most 16 */
  int32_t k[16][3];     /* integer wavevectors, cycles per box length */
  double amplitude[16];
  double phase[16];
} EcsDensityModes;
/* np ions (np <= np_capacity): positions from `dist` (modes only for
   ECS_INIT_MODES), velocities vT_d * N(0,1) + v0_d as NormalVelocities
   (src/velocities.c:14-47; gasdev there, Box-Muller on Philox4x32-10 keyed
   by `seed` here).  Replaces the host generation and broadcast of
   InitializePositions / InitializeVelocities (src/positions.c:390-431). */
int ecs_particles_init(EcsCtx *ctx, int dist, int64_t np, uint64_t seed, const EcsDensityModes *modes);

/* ---- grid fields (host arrays, [Nz][Ny][Nx], x fastest) ----------------- */
int ecs_phi_upload(EcsCtx *ctx, const double *phi);
int ecs_phi_download(EcsCtx *ctx, double *phi);
/* Moments as FluidNode{n,Gx,Gy,Gz} per node (src/ecsprt.h:194-199). */
int ecs_moments_upload(EcsCtx *ctx, const double *moments);
int ecs_moments_download(EcsCtx *ctx, double *moments);
int ecs_rhs_download(EcsCtx *ctx, double *b);

/* ---- operators (one kernel phase each, on the context stream) ----------- */
int ecs_push(EcsCtx *ctx, double dt);            /* BorisMoverBz3D */
int ecs_collide(EcsCtx *ctx, double dt);         /* ScatterElastic (if mn > 0) */
int ecs_move(EcsCtx *ctx, double dt);            /* UpdatePositions + Apply3DBC */
int ecs_collect(EcsCtx *ctx);                    /* Collect3DFluidMoments */
int ecs_rhs(EcsCtx *ctx);                        /* ComputeFullRHS3D (+ mean removal) */
int ecs_lhs(EcsCtx *ctx);                        /* ComputeFullLHS3D (matrix-free set-up) */
/* ComputePotential: solve A(n) phi = b to ||b-A phi||/||b|| <= rtol (FP64
   measured).  The initial guess is phi = 0 as in the reference
   (src/potential.c:20-29) unless warm_start != 0. */
int ecs_solve(EcsCtx *ctx, double rtol, int max_it, int warm_start, EcsSolveStats *stats);
/* y = A x with the current operator, host FP64 arrays (test hook). */
int ecs_lhs_apply_host(EcsCtx *ctx, const double *x, double *y);

/* RHS for callers that cannot allocate device memory (no counterpart in the
   reference; it computes what ecs_rhs computes for the same parameters:
   -rhs full in 3-D or 2-D, -rhs sinusoidal, -rhs constant).  For code that
   owns all of its device memory in its own pool and may not call cudaMalloc
   inside its step loop, or cannot accept the device synchronisation an
   allocation may cause: no allocation of any kind is made.  d_moments
   (device, FluidNode {n,Gx,Gy,Gz} per node, [Nz][Ny][Nx][4]; unused, and
   may be NULL, unless -rhs full) and d_rhs (device, [Nz][Ny][Nx]) belong to
   the caller; the work is queued on `stream` (a cudaStream_t, NULL for the
   default stream).  The parameters are checked as ecs_ctx_create checks
   them.  Its reduction scratch is a fixed __device__ array of 32 KiB + 8 B
   held by every device that loads the library, so grids of more than
   8,388,608 nodes (256 x 256 x 128) are rejected with ECS_ERR_INVALID.  The
   first call on a device looks up the array's device address
   (cudaGetSymbolAddress) and keeps it for the life of the process; make
   that first call before any stream capture, and do not call it on a device
   after cudaDeviceReset.  Every call shares the one scratch array: calls
   that overlap on the GPU (unordered streams) race.  Errors are reported by
   ecs_last_error(NULL). */
int ecs_rhs_noalloc(const EcsParams *params, const double *d_moments, double *d_rhs, void *stream);

/* One time step of src/pic.c:244-258: push, collide (if mn > 0), move + BC,
   collect, rhs, lhs, solve.  In the mixed path push..collect run as one fused
   kernel over the cell-sorted particles. */
int ecs_step(EcsCtx *ctx, double dt, double rtol, int max_it, EcsStepStats *stats);

/* The same step through host buffers, for callers that keep the particles in
   host memory (the reference's DMSwarm arrays): pos/vel (AoS FP64) are copied
   in, stepped, and copied back, and the step's moments (FluidNode layout) and
   potential are copied out (either may be NULL). */
int ecs_step_host(EcsCtx *ctx, double *pos, double *vel, int64_t np, double dt, double rtol,
                  int max_it, double *moments_out, double *phi_out, EcsStepStats *stats);

/* Kernel launches issued by this context since creation (all libecsgpu
   kernels; used to report launch counts). */
int64_t ecs_launch_count(const EcsCtx *ctx);

/* Fixed-point shifts of the deposition for these parameters: density
   contributions are rounded to multiples of 2^-shift_density and flux
   contributions to multiples of 2^-shift_flux.  The flux shift is
   S_f - e_v, with S_f = 48 (FP64) or 22 (mixed) and 2^e_v the velocity bound
   (16 (viT + vi0) rounded up to a power of two); |v| above 2^e_v makes a
   deposit report ECS_ERR_RANGE. */
int ecs_fix_shifts(const EcsParams *params, int precision, int32_t *shift_density, int32_t *shift_flux);

#ifdef __cplusplus
}
#endif
#endif /* ECSGPU_H */
