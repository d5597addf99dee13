// Internal declarations shared by the libecsgpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <utility>
#include <string>
#include <vector>

#include "ecsgpu.h"

#define ECS_FULL_MASK 0xffffffffu

// Fixed-point scales of the deposit accumulators: contributions are rounded
// to integer multiples of 2^-S and summed exactly in int64, which makes the
// moments independent of the order in which particles are processed.  The
// density uses S = ECS_FIX_SHIFT_*; the flux uses S_f - e_v, where 2^e_v
// bounds |v| (ecs_fix_shifts), so every flux contribution is at most 2^S_f in
// magnitude: S_f = S on the FP64 path, ECS_FIX_SHIFT_MIXED_FLUX on the mixed
// path (one int32 word a flux contribution in the tile window).
#define ECS_FIX_SHIFT_FP64 48
#define ECS_FIX_SHIFT_MIXED 38
#define ECS_FIX_SHIFT_MIXED_FLUX 22

// Cell tiles of the mixed path (the deposit accumulates a tile in shared
// memory).
#define ECS_TILE_X 4
#define ECS_TILE_Y 4
#define ECS_TILE_Z 2
#define ECS_TILE_CELLS (ECS_TILE_X * ECS_TILE_Y * ECS_TILE_Z)

// Device status word bits (EcsDevStatus::flags).
#define ECS_FLAG_NONFINITE 1u
#define ECS_FLAG_RANGE 2u
#define ECS_FLAG_COLLISION 4u

struct EcsDevStatus {
  unsigned long long collisions;   // accepted collisions
  unsigned long long refused;      // refused collisions (final speed > 10 viT)
  unsigned long long acc_fix;      // fixed-point sum (2^-24 units) of acceptance probabilities
  unsigned long long acc_count;    // number of acceptance samples in acc_fix
  unsigned int flags;              // ECS_FLAG_*
  unsigned int pad;
};

// Multigrid level (one precision).
template <typename T>
struct MgLevel {
  int nx, ny, nz;
  size_t n;
  double hx, hy, hz;
  T *dens = nullptr;   // density defining the operator on this level
  T *x = nullptr;      // iterate (correction) on this level
  T *b = nullptr;      // right-hand side on this level
  T *r = nullptr;      // residual / scratch
  T *t = nullptr;      // smoother scratch
  // z-line factorisation of the (lower, diag, upper) z-tridiagonal part,
  // cyclic closure by Sherman-Morrison (periodic z) or plain (reflecting z).
  T *zl_a = nullptr, *zl_cp = nullptr, *zl_minv = nullptr, *zl_q = nullptr;
  T *zl_fb = nullptr, *zl_bb = nullptr;     // in-segment products of the recurrences
  T *zl_a0g = nullptr, *zl_qden = nullptr;  // per-column Sherman-Morrison scalars
};

template <typename T>
struct Multigrid {
  std::vector<MgLevel<T>> lv;
  bool built = false;
  // explicit inverse of the coarsest operator (transposed), when it is small
  T *cinv = nullptr;
  T *cwork = nullptr;  // Gauss-Jordan work matrix [n][2n]
};

// Instantiated graph of a whole potential solve (refinement sweeps, each an
// FGMRES cycle), built for one (rtol, max_it, warm start).
struct SolverGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double rtol = 0.0;
  int max_it = 0, warm = -1;
  int setup = -1;  // 1: the graph starts with the RHS and the operator set-up
  // kernels of: the set-up prefix, the head (up to the first check), one
  // sweep outside its Arnoldi steps, one Arnoldi step
  int64_t k_pre = 0, k_head = 0, k_sweep = 0, k_step = 0;
};

// Instantiated graph of one stand-alone solve request (src/solver.c:107-170):
// density in, fluxes = flux_scale * density, RHS, operator set-up, the solve,
// potential and solve status out.  The two copy nodes are re-pointed at the
// request's own buffers when those are pinned, else at the staging buffers.
struct RequestGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t in_node = nullptr, out_node = nullptr;
  double rtol = 0.0;
  int max_it = 0;
  double flux_scale[3] = {0.0, 0.0, 0.0};
  int64_t k_pre = 0;                          // kernels before the solve nodes
  double *h_in = nullptr, *h_out = nullptr;   // pinned staging, ncell doubles each
  const double *src = nullptr;                // the launched request's buffers
  double *dst = nullptr;
  bool staged_out = false;
};

struct EcsCtx {
  EcsParams p;
  int prec = ECS_PREC_FP64;
  int64_t cap = 0, np = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int device = 0;
  int nsm = 0;
  size_t ncell = 0;    // Nx*Ny*Nz
  size_t next = 0;     // (Nx+1)*(Ny+1)*(Nz+1) extended nodes

  // FP64 plain particles: absolute positions and velocities, SoA.
  double *px = nullptr, *py = nullptr, *pz = nullptr;
  double *vx = nullptr, *vy = nullptr, *vz = nullptr;

  // Mixed particles: one 32-byte record per ion (a DRAM sector), two float4:
  //   (int32 cell bits, FP32 in-cell offsets ox, oy, oz), (FP32 vx, vy, vz, int32 identity),
  // double-buffered for the counting sort.
  float4 *ions[2] = {nullptr, nullptr};
  int cur = 0;
  // The sort key orders the ions by tiles of ECS_TILE_X x ECS_TILE_Y x
  // ECS_TILE_Z cells (tile-major, x fastest), then by cell within the tile.
  int ntile[3] = {0, 0, 0};        // tiles per axis
  size_t nkeys = 0;                // ntiles * cells per tile
  int32_t *sort_count = nullptr;   // [nkeys]
  int32_t *sort_offset = nullptr;  // [nkeys+1]: ions of key q at [offset[q], offset[q+1])
  int32_t *scan_blocks = nullptr;  // block sums of the scan
  bool tiles_valid = false;        // the buffer is ordered by the keys of sort_offset
  // Index sort: the counting sort writes the permutation only, and the next
  // particle pass reads ions[cur][perm[i]] and writes ions[1 - cur][i].
  int32_t *sort_keys = nullptr;    // [cap] key of each ion's cell, by buffer position (counting passes)
  int32_t *perm = nullptr;         // [cap] buffer position of the i-th ion in key order
  bool perm_pending = false;       // ions[cur] is in key order only through perm
  int sort_every = 2;
  int steps_since_sort = 0;

  // Grid fields.
  double *phi = nullptr;            // potential [ncell]
  double4_32a *eext64 = nullptr;        // difference numerators on extended nodes
  float4 *eext32 = nullptr;
  long long *acc = nullptr;         // fixed-point moments [4][ncell]
  double *mom = nullptr;            // FP64 moments SoA [4][ncell]
  double *rhs = nullptr;            // [ncell]
  double *red = nullptr;            // reduction scratch (FP64)
  int nred = 0;

  // Solver state.
  Multigrid<double> mg64;
  Multigrid<float> mg32;
  int krylov_m = 30;
  double *kv64 = nullptr;           // FP64 Krylov basis V [(m+1)*ncell]
  double *kz64 = nullptr;           // FP64 preconditioned basis Z [m*ncell]
  float *kv32 = nullptr;            // FP32 Krylov basis for the inner solve
  float *kz32 = nullptr;
  double *w64 = nullptr;            // FP64 work vectors
  double *r64 = nullptr;
  double *coef64 = nullptr;         // the FP64 operator's 11 row coefficients a cell (SoA), for the refinement residuals
  double *dots = nullptr;           // device scalars (norms, means) [m+2]
  double *h_dots = nullptr;         // pinned host copy
  void *kdev = nullptr;             // device FGMRES control block
  void *kdev_host = nullptr;        // pinned copy read back after a cycle
  void *kctl_host = nullptr;        // pinned staging of the cycle's tolerance and step limit
  SolverGraph sgraph;               // the whole solve as one CUDA graph
  RequestGraph rgraph;              // a stand-alone solve request as one CUDA graph
  int use_graphs = 1;               // 0: the host drives the refinement and the Arnoldi steps
  void *rdev = nullptr;             // device state of the refinement loop
  void *rdev_host = nullptr;        // pinned copy
  cudaStream_t capst[3] = {nullptr, nullptr, nullptr};  // capture streams (graph nesting levels)
  // side streams and events of the field set-up (multigrid levels, FP64 row
  // coefficients, right-hand side), which forks off the context's stream and
  // joins it again
  cudaStream_t sst[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t sev[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t ev_solve[2] = {nullptr, nullptr};
  bool lhs_ready = false;
  bool moments_ready = false;
  bool eext_ready = false;          // difference numerators valid for the current phi
  int warm_start = 0;               // ecs_step starts the solve from the previous phi

  // Collision state.
  uint64_t seed = 20261203ull;
  int64_t step_index = 0;
  double attempt_rate = -1.0;       // attempts per ion per call (< 0: not yet estimated)
  EcsDevStatus *dstat = nullptr;
  EcsDevStatus *hstat = nullptr;    // pinned
  // A step's counters are copied to hstat behind its particle pass (event
  // ev_stat) and read while the field phase runs; the collision-rate update
  // of a fused pass waits for that read (coll_pending, with the pass's dt).
  cudaEvent_t ev_stat = nullptr;
  bool stat_queued = false;         // the copy behind ev_stat is the current pass's
  bool coll_pending = false;
  double coll_dt = 0.0;
  cudaEvent_t ev_mom = nullptr;     // moments converted for the host (ecs_step_host)

  int shift_n = 48, shift_f = 48;   // deposit fixed-point shifts (density, flux)
  int64_t launches = 0;
  std::string err;
  // events around the particle kernel [0,1] and the sort [2,3] of a step
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  bool ev_particle = false, ev_sort = false;

  // Host transfers of the ions: two device staging buffers, conversion
  // kernels on xs[0], copies on xs[1] (created on first use).
  cudaStream_t xs[2] = {nullptr, nullptr};
  cudaEvent_t xev_copy[2] = {nullptr, nullptr}, xev_kern[2] = {nullptr, nullptr};
  cudaEvent_t xev_ready = nullptr;  // the ions are ready for a download
  double *stage[2] = {nullptr, nullptr};
  int64_t stage_n = 0;              // ions per staging buffer
  // Host hand-off of ecs_step_host: the ions' download runs beside the next
  // chunk's upload, through its own staging buffers and events.
  static constexpr int kStageDn = 3;
  double *stage_dn[kStageDn] = {nullptr, nullptr, nullptr};
  cudaStream_t xs_conv = nullptr;   // conversions of the download
  cudaStream_t xs_up = nullptr;     // conversions of the upload
  cudaEvent_t xev_tiled[kStageDn] = {nullptr, nullptr, nullptr};
  cudaEvent_t xev_dn_conv[kStageDn] = {nullptr, nullptr, nullptr}, xev_dn_copy[kStageDn] = {nullptr, nullptr, nullptr};
  std::vector<cudaEvent_t> xev_upc;  // upload chunk k converted (one event a chunk)
  uint64_t pgen = 0;                // bumped by every change of the device ions
  uint64_t host_gen = ~0ull;        // pgen when ecs_step_host last returned the ions to the host
  bool bounds_valid = false;        // tile_bounds holds the current sort's tile offsets
  // Page-locked host tables, filled through a device buffer of the same
  // layout (both allocated once, on first use):
  int32_t *tile_bounds = nullptr;   // first ion of every tile, and np (ntiles + 1)
  int32_t *tile_srcmax = nullptr;   // largest source position a tile's ions are gathered from (pending sort)
  int32_t *tile_tables_dev = nullptr;
};

// ---- error helpers -------------------------------------------------------
int ecs_fail(EcsCtx *ctx, int code, const char *fmt, ...);
// The parameter checks of ecs_ctx_create (ECS_OK or the failing status).
int ecs_validate_params(const EcsParams *p);
// Ions per staging chunk of the host transfers (two chunks are held): an
// eighth of the capacity, between 2^16 and 2^22 ions.
inline int64_t ecs_stage_ions(int64_t cap) {
  int64_t n = cap / 8;
  if (n < ((int64_t)1 << 16)) n = (int64_t)1 << 16;
  if (n > ((int64_t)1 << 22)) n = (int64_t)1 << 22;
  return cap < n ? (cap > 0 ? cap : 1) : n;
}
// Doubles per array region of a staging buffer of n ions (3 doubles an ion,
// plus room for the rounding of ecs_step_host's copies to 256-byte host
// boundaries); a buffer holds a position region and a velocity region.
inline int64_t ecs_stage_stride(int64_t n) { return 3 * n + 64; }

int ecs_cuda_check(EcsCtx *ctx, cudaError_t e, const char *what);
#define ECS_CUDA(ctx, call)                                        \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) return ecs_cuda_check((ctx), e_, #call); \
  } while (0)
#define ECS_LAUNCHED(ctx)                                                   \
  do {                                                                      \
    (ctx)->launches++;                                                      \
    cudaError_t e_ = cudaGetLastError();                                    \
    if (e_ != cudaSuccess) return ecs_cuda_check((ctx), e_, "kernel launch"); \
  } while (0)

static inline unsigned int ecs_div_up(size_t a, size_t b) { return (unsigned int)((a + b - 1) / b); }

// Programmatic dependent launch: a kernel launched by ecs_launch_pdl may be
// scheduled while the kernel before it on the stream (or before it in a
// captured graph) is still finishing, and waits in ecs_pdl_wait until that
// kernel has completed and its writes are visible.  Every kernel launched
// this way calls ecs_pdl_wait before touching global memory, and then lets
// its own successor be scheduled (ecs_pdl_trigger); for a kernel launched
// the ordinary way both are no-ops.
__device__ __forceinline__ void ecs_pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void ecs_pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
#define ECS_PDL_ENTRY() \
  do {                  \
    ecs_pdl_wait();     \
    ecs_pdl_trigger();  \
  } while (0)

template <typename... KArgs, typename... Args>
inline cudaError_t ecs_launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                  Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// ---- counter-based RNG: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) --
struct EcsU4 {
  uint32_t x, y, z, w;
};
__device__ __forceinline__ EcsU4 ecs_philox(EcsU4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    EcsU4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}
// Uniform in (0,1): 24 random bits, offset by half a step.
__device__ __forceinline__ float ecs_u01f(uint32_t u) { return ((u >> 8) + 0.5f) * (1.0f / 16777216.0f); }
__device__ __forceinline__ double ecs_u01d(uint32_t a, uint32_t b) {
  uint64_t v = ((uint64_t)(a >> 6) << 26) | (uint64_t)(b >> 6);  // 52 bits
  return ((double)v + 0.5) * (1.0 / 4503599627370496.0);
}
// 32-bit mixing (splitmix-style finaliser) for hashing particle state.
__device__ __forceinline__ uint32_t ecs_mix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x7feb352du;
  h ^= h >> 15;
  h *= 0x846ca68bu;
  h ^= h >> 16;
  return h;
}

// ---- kernels launched from several translation units --------------------
// (defined in ecs_grid.cu and ecs_solver.cu)
int ecs_grid_eext(EcsCtx *ctx);          // difference numerators from phi
int ecs_grid_moments(EcsCtx *ctx);       // fixed-point -> FP64 moments
int ecs_grid_rhs(EcsCtx *ctx);           // RHS (+ mean removal) from moments
int ecs_grid_clear_acc(EcsCtx *ctx);
int ecs_solver_alloc(EcsCtx *ctx);       // reductions, Krylov bases, control block
int ecs_solver_setup(EcsCtx *ctx);       // multigrid hierarchy from the density
// setup = 1: compute the RHS and set up the operator first (the step's field
// phase), in the same graph launch as the solve.
// `between` (optional) runs on the host once the solve is enqueued and
// before the host waits for it; its status is returned if nonzero.
typedef int (*EcsHostHook)(EcsCtx *ctx, void *arg);
int ecs_solver_run(EcsCtx *ctx, double rtol, int max_it, int warm, EcsSolveStats *st, int setup = 0,
                   EcsHostHook between = nullptr, void *arg = nullptr);
int ecs_operator_apply64(EcsCtx *ctx, const double *x, double *y);
int ecs_solver_free(EcsCtx *ctx);
// Stand-alone solve request: launch (asynchronous, on ctx->stream) and, once
// the stream's work is complete, finish (potential to the caller, stats).
int ecs_request_launch(EcsCtx *ctx, const double *density, double *phi, const double flux_scale[3], double rtol,
                       int max_it);
int ecs_request_finish(EcsCtx *ctx, EcsSolveStats *st);
// (defined in ecs_particles.cu)
int ecs_particles_alloc(EcsCtx *ctx);
int ecs_particles_free(EcsCtx *ctx);
int ecs_part_upload(EcsCtx *ctx, const double *pos, const double *vel, int64_t np);
int ecs_part_init(EcsCtx *ctx, int dist, int64_t np, uint64_t seed, const EcsDensityModes *modes);
int ecs_part_download(EcsCtx *ctx, double *pos, double *vel);
int ecs_part_ids(EcsCtx *ctx, int32_t *ids);
// The particle pass of ecs_step_host when the host arrays hold the ions as
// the previous ecs_step_host call returned them: upload, pass and download
// pipelined by ranges of tiles.  ECS_ERR_STATE (nothing done) otherwise.
int ecs_part_host_pass(EcsCtx *ctx, double *pos, double *vel, int64_t np, double dt, int *sorted);
// Enqueue the download after ctx->stream's current work; ecs_part_xfer_wait
// waits for it.
int ecs_part_download_async(EcsCtx *ctx, double *pos, double *vel);
int ecs_part_xfer_wait(EcsCtx *ctx);
int ecs_part_push(EcsCtx *ctx, double dt);
int ecs_part_collide(EcsCtx *ctx, double dt);
int ecs_part_move(EcsCtx *ctx, double dt);
int ecs_part_collect(EcsCtx *ctx);
int ecs_part_fused(EcsCtx *ctx, double dt, int do_collide, int *sorted);
// Copy of the step's device counters to the host, behind the work enqueued
// so far; ecs_part_status_finish waits for it, applies the pending
// collision-rate update and returns the first error the counters show.
int ecs_part_status_async(EcsCtx *ctx);
int ecs_part_status_finish(EcsCtx *ctx);
// Applies a pending collision-rate update (reading the counters first if
// their copy was not queued); called before the counters are cleared.
int ecs_part_settle(EcsCtx *ctx);
int ecs_part_sort(EcsCtx *ctx);
int ecs_part_estimate_rate(EcsCtx *ctx, double dt);
extern "C" int ecs_fix_shifts(const EcsParams *p, int precision, int32_t *shift_density, int32_t *shift_flux);
