// C ABI of libecsgpu (declared in include/ecsgpu.h).
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <new>

#include "ecs_internal.cuh"

static thread_local std::string g_create_err;

int ecs_fail(EcsCtx *ctx, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  else g_create_err = buf;
  return code;
}

int ecs_cuda_check(EcsCtx *ctx, cudaError_t e, const char *what) {
  return ecs_fail(ctx, e == cudaErrorMemoryAllocation ? ECS_ERR_NOMEM : ECS_ERR_CUDA, "%s: %s", what,
                  cudaGetErrorString(e));
}

namespace {

__global__ void k_moments_aos(size_t n, const double *__restrict__ mom, double *__restrict__ out) {
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    for (int d = 0; d < 4; d++) out[4 * c + d] = mom[(size_t)d * n + c];
}
__global__ void k_moments_soa(size_t n, const double *__restrict__ in, double *__restrict__ mom) {
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    for (int d = 0; d < 4; d++) mom[(size_t)d * n + c] = in[4 * c + d];
}

unsigned int blocks(const EcsCtx *ctx, size_t n) {
  size_t want = (n + 255) / 256, cap = (size_t)ctx->nsm * 8;
  return (unsigned int)(want < 1 ? 1 : (want > cap ? cap : want));
}

int validate(const EcsParams *p) {
  if (!p) return ecs_fail(nullptr, ECS_ERR_INVALID, "params is NULL");
  if (p->ndim != 3 && p->ndim != 2) return ecs_fail(nullptr, ECS_ERR_UNSUPPORTED, "ndim %d", p->ndim);
  const bool flat = p->ndim == 2;
  if (p->Nx < 4 || p->Ny < 4 || p->Nx > 1024 || p->Ny > 1024 || (flat ? p->Nz != 1 : (p->Nz < 4 || p->Nz > 1024)))
    return ecs_fail(nullptr, ECS_ERR_INVALID, "grid %dx%dx%d outside 4..1024 per axis (Nz = 1 for ndim 2)", p->Nx,
                    p->Ny, p->Nz);
  if (!(p->dx > 0 && p->dy > 0 && (flat || p->dz > 0))) return ecs_fail(nullptr, ECS_ERR_INVALID, "non-positive cell width");
  // ScatterElastic reads the relative velocity's z component (src/collisions.c:104),
  // which a 2-D run never sets (src/collisions.c:78-83): undefined in the reference.
  if (flat && p->mn > 0.0)
    return ecs_fail(nullptr, ECS_ERR_UNSUPPORTED, "2-D collisions are undefined in the reference; use -mn 0 with -ndim 2");
  if (!(p->mi > 0)) return ecs_fail(nullptr, ECS_ERR_INVALID, "non-positive ion mass");
  for (int d = 0; d < (flat ? 2 : 3); d++) {
    if (p->bc[d] == ECS_BC_INJECT_ADVECT) return ecs_fail(nullptr, ECS_ERR_UNSUPPORTED, "inject-advect boundaries are not implemented");
    if (p->bc[d] == ECS_BC_INJECT_REFLECT && d != 2) return ecs_fail(nullptr, ECS_ERR_UNSUPPORTED, "reflecting boundaries are supported on z only");
  }
  if (p->lhs_type < ECS_LHS_IDENTITY || p->lhs_type > ECS_LHS_FULL || p->rhs_type < ECS_RHS_CONSTANT ||
      p->rhs_type > ECS_RHS_FULL)
    return ecs_fail(nullptr, ECS_ERR_INVALID, "unknown -lhs %d / -rhs %d", p->lhs_type, p->rhs_type);
  return ECS_OK;
}

int ensure_eext(EcsCtx *ctx, bool &ready) {
  if (ready) return ECS_OK;
  int rc = ecs_grid_eext(ctx);
  if (rc) return rc;
  ready = true;
  return ECS_OK;
}

int read_status(EcsCtx *ctx) {
  ECS_CUDA(ctx, cudaMemcpyAsync(ctx->hstat, ctx->dstat, sizeof(EcsDevStatus), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  unsigned int f = ctx->hstat->flags;
  if (f & ECS_FLAG_NONFINITE) return ecs_fail(ctx, ECS_ERR_NONFINITE, "non-finite particle velocity");
  if (f & ECS_FLAG_RANGE) return ecs_fail(ctx, ECS_ERR_RANGE, "particle outside the domain or deposit range exceeded");
  return ECS_OK;
}

}  // namespace

// The parameter checks of ecs_ctx_create, shared with ecs_rhs_noalloc.
int ecs_validate_params(const EcsParams *p) { return validate(p); }

extern "C" {

const char *ecs_version(void) { return "ecsprt-gb300 0.1.0 (sm_103a)"; }

const char *ecs_status_string(int s) {
  switch (s) {
    case ECS_OK: return "ok";
    case ECS_ERR_INVALID: return "invalid argument";
    case ECS_ERR_NOMEM: return "out of memory";
    case ECS_ERR_NOT_CONVERGED: return "solve did not converge";
    case ECS_ERR_NONFINITE: return "non-finite value";
    case ECS_ERR_TIMEOUT: return "device wait timed out";
    case ECS_ERR_CUDA: return "CUDA error";
    case ECS_ERR_COLLISION: return "too many refused collisions";
    case ECS_ERR_RANGE: return "out of range";
    case ECS_ERR_STATE: return "call out of order";
    case ECS_ERR_UNSUPPORTED: return "unsupported option";
    default: return "unknown status";
  }
}

const char *ecs_last_error(const EcsCtx *ctx) { return ctx ? ctx->err.c_str() : g_create_err.c_str(); }

int64_t ecs_ctx_device_bytes(const EcsParams *p, int precision, int64_t cap) {
  if (!p) return -1;
  const int64_t n = (int64_t)p->Nx * p->Ny * p->Nz;
  const int64_t ne = (int64_t)(p->Nx + 1) * (p->Ny + 1) * (p->Nz + 1);
  const int64_t m = 30;  // Krylov basis vectors (FGMRES restart)
  const int64_t t = precision == ECS_PREC_FP64 ? 8 : 4;  // solver arithmetic
  int64_t b = 0;
  b += n * 8 * (1 + 4 + 1) + n * 8 * 4;  // phi, moments, rhs; fixed-point accumulators
  b += n * 8 * 2 + (m + 2) * 1024 * 8;   // FP64 residual and correction, reductions
  if (p->lhs_type != ECS_LHS_IDENTITY) b += n * 8 * 11;  // FP64 row coefficients of the residuals
  // multigrid: 11 cell arrays and 2 plane arrays a level, levels summing to
  // at most 8/7 of the finest; the coarsest level's inverse (<= 128 cells)
  b += (n * 11 + n / 4) * t * 8 / 7 + 128 * 128 * 3 * t;
  if (precision == ECS_PREC_FP64) {
    b += (2 * m + 1) * n * 8;  // Krylov bases V, Z
    b += cap * 48 + ne * 32;   // ions (6 FP64), E numerators
  } else {
    b += (2 * m + 3) * n * 4;  // Krylov bases V, Z, two FP32 work vectors
    b += cap * 72 + ne * 16;   // ions (two 32-byte record buffers, sort keys, permutation), E numerators
    const int64_t keys = (int64_t)((p->Nx + ECS_TILE_X - 1) / ECS_TILE_X) * ((p->Ny + ECS_TILE_Y - 1) / ECS_TILE_Y) *
                         ((p->Nz + ECS_TILE_Z - 1) / ECS_TILE_Z) * ECS_TILE_CELLS;
    b += keys * 4 * 2 + keys / 1024 * 4;  // sort counts and offsets
  }
  if (cap > 0) b += (2 + EcsCtx::kStageDn) * 2 * ecs_stage_stride(ecs_stage_ions(cap)) * 8;  // host-transfer staging
  // allocation rounding (about 40 allocations) and instantiated CUDA graphs
  b += (int64_t)8 << 20;
  return b;
}

int ecs_ctx_create(const EcsParams *params, int precision, int64_t np_capacity, void *stream, EcsCtx **out) {
  if (!out) return ecs_fail(nullptr, ECS_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int rc = validate(params);
  if (rc) return rc;
  if (precision != ECS_PREC_FP64 && precision != ECS_PREC_MIXED) return ecs_fail(nullptr, ECS_ERR_INVALID, "unknown precision %d", precision);
  if (np_capacity < 0 || np_capacity > (int64_t)2147483647) return ecs_fail(nullptr, ECS_ERR_INVALID, "np_capacity out of range");
  EcsCtx *ctx = new (std::nothrow) EcsCtx();
  if (!ctx) return ecs_fail(nullptr, ECS_ERR_NOMEM, "host allocation failed");
  ctx->p = *params;
  if (params->ndim == 2) {
    // 2-D runs on a one-cell-deep grid with the ions at z = 0: a unit z cell,
    // periodic, so that every z term is exactly zero rather than 0/0 (the
    // reference's 2-D context has dz = Lz = 0).
    ctx->p.dz = 1.0; ctx->p.Lz = 1.0; ctx->p.z0 = 0.0; ctx->p.z1 = 1.0;
    ctx->p.bc[2] = ECS_BC_PERIODIC;
  }
  ctx->prec = precision;
  ctx->cap = np_capacity;
  ctx->ncell = (size_t)params->Nx * params->Ny * params->Nz;
  ctx->next = (size_t)(params->Nx + 1) * (params->Ny + 1) * (params->Nz + 1);
  ecs_fix_shifts(params, precision, &ctx->shift_n, &ctx->shift_f);
  cudaError_t ce = cudaGetDevice(&ctx->device);
  if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, ctx->device);
  if (ce != cudaSuccess) {
    ecs_fail(nullptr, ECS_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(ce));
    delete ctx;
    return ECS_ERR_CUDA;
  }
  if (stream) {
    ctx->stream = (cudaStream_t)stream;
  } else {
    ce = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    ctx->own_stream = true;
  }
#define CREATE_ALLOC(ptr, bytes)                                                   \
  do {                                                                            \
    cudaError_t a_ = cudaMalloc((void **)&(ptr), (bytes));                        \
    if (a_ != cudaSuccess) {                                                      \
      ecs_fail(nullptr, ECS_ERR_NOMEM, "cudaMalloc %zu bytes: %s", (size_t)(bytes), \
               cudaGetErrorString(a_));                                           \
      ecs_ctx_destroy(ctx);                                                       \
      return ECS_ERR_NOMEM;                                                       \
    }                                                                             \
  } while (0)
  CREATE_ALLOC(ctx->phi, ctx->ncell * sizeof(double));
  CREATE_ALLOC(ctx->acc, ctx->ncell * 4 * sizeof(long long));
  CREATE_ALLOC(ctx->mom, ctx->ncell * 4 * sizeof(double));
  CREATE_ALLOC(ctx->rhs, ctx->ncell * sizeof(double));
  CREATE_ALLOC(ctx->dstat, sizeof(EcsDevStatus));
  if (precision == ECS_PREC_FP64) CREATE_ALLOC(ctx->eext64, ctx->next * sizeof(double4_32a));
  else CREATE_ALLOC(ctx->eext32, ctx->next * sizeof(float4));
#undef CREATE_ALLOC
  if (cudaMallocHost((void **)&ctx->hstat, sizeof(EcsDevStatus)) != cudaSuccess) {
    ecs_fail(nullptr, ECS_ERR_NOMEM, "pinned allocation failed");
    ecs_ctx_destroy(ctx);
    return ECS_ERR_NOMEM;
  }
  for (int q = 0; q < 4; q++) cudaEventCreate(&ctx->ev[q]);
  cudaMemsetAsync(ctx->phi, 0, ctx->ncell * sizeof(double), ctx->stream);
  cudaMemsetAsync(ctx->mom, 0, ctx->ncell * 4 * sizeof(double), ctx->stream);
  cudaMemsetAsync(ctx->dstat, 0, sizeof(EcsDevStatus), ctx->stream);
  rc = ecs_particles_alloc(ctx);
  if (rc) {
    g_create_err = ctx->err;
    ecs_ctx_destroy(ctx);
    return rc;
  }
  ce = cudaStreamSynchronize(ctx->stream);
  if (ce != cudaSuccess) {
    ecs_fail(nullptr, ECS_ERR_CUDA, "stream sync: %s", cudaGetErrorString(ce));
    ecs_ctx_destroy(ctx);
    return ECS_ERR_CUDA;
  }
  *out = ctx;
  return ECS_OK;
}

int ecs_ctx_destroy(EcsCtx *ctx) {
  if (!ctx) return ECS_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ecs_particles_free(ctx);
  ecs_solver_free(ctx);
  void *ptrs[] = {ctx->phi, ctx->acc, ctx->mom, ctx->rhs, ctx->dstat, ctx->eext64, ctx->eext32};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  if (ctx->hstat) cudaFreeHost(ctx->hstat);
  for (int q = 0; q < 4; q++)
    if (ctx->ev[q]) cudaEventDestroy(ctx->ev[q]);
  if (ctx->ev_stat) cudaEventDestroy(ctx->ev_stat);
  if (ctx->ev_mom) cudaEventDestroy(ctx->ev_mom);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return ECS_OK;
}

int ecs_ctx_sync(EcsCtx *ctx) {
  if (!ctx) return ECS_ERR_INVALID;
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return ECS_OK;
}

int ecs_set_sort_every(EcsCtx *ctx, int every) {
  if (!ctx || every < 0) return ECS_ERR_INVALID;
  ctx->sort_every = every;
  return ECS_OK;
}

int ecs_set_seed(EcsCtx *ctx, uint64_t seed) {
  if (!ctx) return ECS_ERR_INVALID;
  ctx->seed = seed;
  return ECS_OK;
}

int ecs_set_warm_start(EcsCtx *ctx, int warm) {
  if (!ctx) return ECS_ERR_INVALID;
  ctx->warm_start = warm ? 1 : 0;
  return ECS_OK;
}

int ecs_set_solver_graphs(EcsCtx *ctx, int on) {
  if (!ctx) return ECS_ERR_INVALID;
  ctx->use_graphs = on ? 1 : 0;
  return ECS_OK;
}

int ecs_particles_upload(EcsCtx *ctx, const double *pos, const double *vel, int64_t np) {
  if (!ctx || (np > 0 && (!pos || !vel))) return ECS_ERR_INVALID;
  int rc = ecs_part_upload(ctx, pos, vel, np);
  if (rc) return rc;
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return ECS_OK;
}

int ecs_particles_download(EcsCtx *ctx, double *pos, double *vel) {
  if (!ctx) return ECS_ERR_INVALID;
  return ecs_part_download(ctx, pos, vel);
}

int64_t ecs_particles_count(const EcsCtx *ctx) { return ctx ? ctx->np : -1; }

int ecs_particles_ids(EcsCtx *ctx, int32_t *ids) {
  if (!ctx || (ctx->np > 0 && !ids)) return ECS_ERR_INVALID;
  return ecs_part_ids(ctx, ids);
}

int ecs_particles_init(EcsCtx *ctx, int dist, int64_t np, uint64_t seed, const EcsDensityModes *modes) {
  if (!ctx) return ECS_ERR_INVALID;
  return ecs_part_init(ctx, dist, np, seed, modes);
}

int ecs_phi_upload(EcsCtx *ctx, const double *phi) {
  if (!ctx || !phi) return ECS_ERR_INVALID;
  ECS_CUDA(ctx, cudaMemcpyAsync(ctx->phi, phi, ctx->ncell * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->eext_ready = false;
  return ECS_OK;
}

int ecs_phi_download(EcsCtx *ctx, double *phi) {
  if (!ctx || !phi) return ECS_ERR_INVALID;
  ECS_CUDA(ctx, cudaMemcpyAsync(phi, ctx->phi, ctx->ncell * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return ECS_OK;
}

int ecs_moments_upload(EcsCtx *ctx, const double *m) {
  if (!ctx || !m) return ECS_ERR_INVALID;
  double *stage = nullptr;
  ECS_CUDA(ctx, cudaMallocAsync((void **)&stage, ctx->ncell * 4 * sizeof(double), ctx->stream));
  ECS_CUDA(ctx, cudaMemcpyAsync(stage, m, ctx->ncell * 4 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  k_moments_soa<<<blocks(ctx, ctx->ncell), 256, 0, ctx->stream>>>(ctx->ncell, stage, ctx->mom);
  ECS_LAUNCHED(ctx);
  ECS_CUDA(ctx, cudaFreeAsync(stage, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->moments_ready = true;
  ctx->lhs_ready = false;
  return ECS_OK;
}

static int moments_to_host(EcsCtx *ctx, double *m) {
  double *stage = nullptr;
  ECS_CUDA(ctx, cudaMallocAsync((void **)&stage, ctx->ncell * 4 * sizeof(double), ctx->stream));
  k_moments_aos<<<blocks(ctx, ctx->ncell), 256, 0, ctx->stream>>>(ctx->ncell, ctx->mom, stage);
  ECS_LAUNCHED(ctx);
  ECS_CUDA(ctx, cudaMemcpyAsync(m, stage, ctx->ncell * 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaFreeAsync(stage, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return ECS_OK;
}

// The same without waiting, for ecs_step_host after its pipelined pass: the
// conversion into the free upload staging buffer on the context's stream,
// the copy behind the ions' download (xs[0], waited for with them).  *sent
// stays false when the staging buffer is too small (then use the above).
static int moments_to_host_async(EcsCtx *ctx, double *m, bool *sent) {
  *sent = false;
  const size_t bytes = ctx->ncell * 4 * sizeof(double);
  if (!ctx->stage[0] || !ctx->xs[0] || bytes > (size_t)ecs_stage_stride(ctx->stage_n) * 2 * sizeof(double))
    return ECS_OK;
  if (!ctx->ev_mom) ECS_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_mom, cudaEventDisableTiming));
  k_moments_aos<<<blocks(ctx, ctx->ncell), 256, 0, ctx->stream>>>(ctx->ncell, ctx->mom, ctx->stage[0]);
  ECS_LAUNCHED(ctx);
  ECS_CUDA(ctx, cudaEventRecord(ctx->ev_mom, ctx->stream));
  ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->xs[0], ctx->ev_mom, 0));
  ECS_CUDA(ctx, cudaMemcpyAsync(m, ctx->stage[0], bytes, cudaMemcpyDeviceToHost, ctx->xs[0]));
  *sent = true;
  return ECS_OK;
}

int ecs_moments_download(EcsCtx *ctx, double *m) {
  if (!ctx || !m) return ECS_ERR_INVALID;
  return moments_to_host(ctx, m);
}

int ecs_rhs_download(EcsCtx *ctx, double *b) {
  if (!ctx || !b) return ECS_ERR_INVALID;
  ECS_CUDA(ctx, cudaMemcpyAsync(b, ctx->rhs, ctx->ncell * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return ECS_OK;
}

int ecs_push(EcsCtx *ctx, double dt) {
  if (!ctx) return ECS_ERR_INVALID;
  int rc = ensure_eext(ctx, ctx->eext_ready);
  if (rc) return rc;
  ECS_CUDA(ctx, cudaMemsetAsync(ctx->dstat, 0, sizeof(EcsDevStatus), ctx->stream));
  if ((rc = ecs_part_push(ctx, dt))) return rc;
  return read_status(ctx);
}

int ecs_collide(EcsCtx *ctx, double dt) {
  if (!ctx) return ECS_ERR_INVALID;
  return ecs_part_collide(ctx, dt);
}

int ecs_move(EcsCtx *ctx, double dt) {
  if (!ctx) return ECS_ERR_INVALID;
  ECS_CUDA(ctx, cudaMemsetAsync(ctx->dstat, 0, sizeof(EcsDevStatus), ctx->stream));
  int rc = ecs_part_move(ctx, dt);  // sorts the ions by cell when due
  if (rc) return rc;
  return read_status(ctx);
}

int ecs_collect(EcsCtx *ctx) {
  if (!ctx) return ECS_ERR_INVALID;
  ECS_CUDA(ctx, cudaMemsetAsync(ctx->dstat, 0, sizeof(EcsDevStatus), ctx->stream));
  int rc = ecs_part_collect(ctx);
  if (rc) return rc;
  if ((rc = ecs_grid_moments(ctx))) return rc;
  ctx->lhs_ready = false;
  return read_status(ctx);
}

int ecs_rhs(EcsCtx *ctx) {
  if (!ctx) return ECS_ERR_INVALID;
  if (!ctx->moments_ready) return ecs_fail(ctx, ECS_ERR_STATE, "rhs called before collect");
  int rc = ecs_grid_rhs(ctx);
  if (rc) return rc;
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return ECS_OK;
}

int ecs_lhs(EcsCtx *ctx) {
  if (!ctx) return ECS_ERR_INVALID;
  if (!ctx->moments_ready) return ecs_fail(ctx, ECS_ERR_STATE, "lhs called before collect");
  int rc = ecs_solver_setup(ctx);
  if (rc) return rc;
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return ECS_OK;
}

int ecs_solve(EcsCtx *ctx, double rtol, int max_it, int warm_start, EcsSolveStats *stats) {
  if (!ctx || !(rtol > 0) || max_it < 1) return ECS_ERR_INVALID;
  int rc = ecs_solver_run(ctx, rtol, max_it, warm_start, stats);
  ctx->eext_ready = false;
  return rc;
}

int ecs_lhs_apply_host(EcsCtx *ctx, const double *x, double *y) {
  if (!ctx || !x || !y) return ECS_ERR_INVALID;
  if (!ctx->moments_ready) return ecs_fail(ctx, ECS_ERR_STATE, "lhs apply before moments");
  double *dx = nullptr, *dy = nullptr;
  ECS_CUDA(ctx, cudaMallocAsync((void **)&dx, ctx->ncell * sizeof(double), ctx->stream));
  ECS_CUDA(ctx, cudaMallocAsync((void **)&dy, ctx->ncell * sizeof(double), ctx->stream));
  ECS_CUDA(ctx, cudaMemcpyAsync(dx, x, ctx->ncell * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  int rc = ecs_operator_apply64(ctx, dx, dy);
  if (rc) return rc;
  ECS_CUDA(ctx, cudaMemcpyAsync(y, dy, ctx->ncell * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaFreeAsync(dx, ctx->stream));
  ECS_CUDA(ctx, cudaFreeAsync(dy, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return ECS_OK;
}

// Particle phase of a step (src/pic.c:244-252): push, collide, move + BC,
// deposit, the cell sort when due, and the FP64 moments; the copy of the
// pass's counters to the host is queued behind them (read by status_hook).
static int step_particles(EcsCtx *ctx, double dt, int *sorted) {
  int rc = ecs_part_settle(ctx);
  if (rc) return rc;
  if ((rc = ensure_eext(ctx, ctx->eext_ready))) return rc;
  *sorted = 0;
  ctx->ev_particle = ctx->ev_sort = false;
  ECS_CUDA(ctx, cudaMemsetAsync(ctx->dstat, 0, sizeof(EcsDevStatus), ctx->stream));
  if ((rc = ecs_part_fused(ctx, dt, 1, sorted))) return rc;
  if ((rc = ecs_grid_moments(ctx))) return rc;
  return ecs_part_status_async(ctx);
}

// Runs while the field phase is on the device: the particle pass's counters
// (collision-rate update, refusals, range and finiteness flags).
struct StepStatus {
  EcsDevStatus coll;
};
static int status_hook(EcsCtx *ctx, void *arg) {
  StepStatus *ss = (StepStatus *)arg;
  const int rc = ecs_part_status_finish(ctx);
  ss->coll = *ctx->hstat;
  if (ctx->p.mn <= 0.0) memset(&ss->coll, 0, sizeof ss->coll);
  return rc;
}

// Field phase (src/pic.c:253-258): RHS, operator, potential solve.
// The RHS, the operator set-up and the solve are one graph launch; the
// particle status is read while it runs.
static int step_field(EcsCtx *ctx, double rtol, int max_it, EcsSolveStats *st, StepStatus *ss) {
  memset(st, 0, sizeof *st);
  int rc = ecs_solver_run(ctx, rtol, max_it, ctx->warm_start, st, 1, status_hook, ss);
  ctx->eext_ready = false;
  return rc;
}

static void step_stats(EcsCtx *ctx, const EcsDevStatus &coll, int sorted, const EcsSolveStats &st,
                       EcsStepStats *stats) {
  if (!stats) return;
  stats->collisions = (int64_t)coll.collisions;
  stats->refused = (int64_t)coll.refused;
  stats->sorted = sorted;
  stats->solve = st;
  float ms = 0.f;
  cudaStreamSynchronize(ctx->stream);
  stats->particle_seconds = (ctx->ev_particle && cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]) == cudaSuccess) ? ms * 1e-3 : 0.0;
  ms = 0.f;
  stats->sort_seconds = (ctx->ev_sort && cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]) == cudaSuccess) ? ms * 1e-3 : 0.0;
}

int ecs_step(EcsCtx *ctx, double dt, double rtol, int max_it, EcsStepStats *stats) {
  if (!ctx || !(rtol > 0) || max_it < 1) return ECS_ERR_INVALID;
  int sorted = 0;
  int rc = step_particles(ctx, dt, &sorted);
  if (rc) return rc;
  EcsSolveStats st;
  StepStatus ss = {};
  rc = step_field(ctx, rtol, max_it, &st, &ss);
  step_stats(ctx, ss.coll, sorted, st, stats);
  return rc;
}

// The ions come from and go back to the host arrays.  When the arrays hold
// the ions as the previous call returned them, the upload, the particle pass
// and the download are pipelined by ranges of tiles (ecs_part_host_pass);
// otherwise the ions are uploaded and sorted first.  Either way the ions'
// download overlaps the potential solve.
int ecs_step_host(EcsCtx *ctx, double *pos, double *vel, int64_t np, double dt, double rtol, int max_it,
                  double *moments_out, double *phi_out, EcsStepStats *stats) {
  if (!ctx || !pos || !vel || !(rtol > 0) || max_it < 1) return ECS_ERR_INVALID;
  int sorted = 0;
  int rc = ecs_part_settle(ctx);
  if (rc) return rc;
  if ((rc = ensure_eext(ctx, ctx->eext_ready))) return rc;
  ctx->ev_particle = ctx->ev_sort = false;
  ECS_CUDA(ctx, cudaMemsetAsync(ctx->dstat, 0, sizeof(EcsDevStatus), ctx->stream));
  rc = ecs_part_host_pass(ctx, pos, vel, np, dt, &sorted);
  bool moments_sent = false;
  if (rc == ECS_ERR_STATE) {  // no hand-off from a previous call: upload (and sort) first
    if ((rc = ecs_part_upload(ctx, pos, vel, np))) return rc;
    if ((rc = step_particles(ctx, dt, &sorted))) return rc;
    if ((rc = ecs_part_download_async(ctx, pos, vel))) return rc;
  } else {
    if (rc) return rc;
    if ((rc = ecs_grid_moments(ctx))) return rc;
    if ((rc = ecs_part_status_async(ctx))) return rc;
    // the moments go out behind the ions' download while the solve runs
    if (moments_out && (rc = moments_to_host_async(ctx, moments_out, &moments_sent))) return rc;
  }
  EcsSolveStats st;
  StepStatus ss = {};
  const int rc_field = step_field(ctx, rtol, max_it, &st, &ss);
  if ((rc = ecs_part_xfer_wait(ctx))) return rc;
  ctx->host_gen = ctx->pgen;  // the host arrays now hold the device's ions, in the buffer's next order
  if (rc_field) return rc_field;
  step_stats(ctx, ss.coll, sorted, st, stats);
  if (moments_out && !moments_sent && (rc = moments_to_host(ctx, moments_out))) return rc;
  if (phi_out) {
    ECS_CUDA(ctx, cudaMemcpyAsync(phi_out, ctx->phi, ctx->ncell * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return ECS_OK;
}

int64_t ecs_launch_count(const EcsCtx *ctx) { return ctx ? ctx->launches : -1; }

// Velocity bound 2^e_v: sixteen times the thermal speed plus drift,
// rounded up to a power of two; the flux quantum is 2^-(S - e_v).
int ecs_fix_shifts(const EcsParams *p, int precision, int32_t *shift_density, int32_t *shift_flux) {
  if (!p || !shift_density || !shift_flux) return ECS_ERR_INVALID;
  int S = precision == ECS_PREC_FP64 ? ECS_FIX_SHIFT_FP64 : ECS_FIX_SHIFT_MIXED;
  int Sf = precision == ECS_PREC_FP64 ? ECS_FIX_SHIFT_FP64 : ECS_FIX_SHIFT_MIXED_FLUX;
  double vmax = 16.0 * (p->viT + p->vi0);
  int ev = vmax > 0.0 ? (int)ceil(log2(vmax)) : 0;
  if (ev < -8) ev = -8;
  if (ev > 40) ev = 40;
  *shift_density = S;
  *shift_flux = Sf - ev;
  return ECS_OK;
}

}  // extern "C"
