// Grid phase of the ECSPRT hot path on sm_103a (everything but the solver):
//   difference numerators of phi on the extended node grid (input to push)
//   fixed-point -> FP64 moments                       src/moments.c:208-211
//   RHS of the quasineutral potential equation         src/rhs.c:259-373
// All kernels are 3-D launches over (x, y) tiles and z (no index division);
// the RHS mean is a fixed-order reduction, so results repeat run to run.
#include <math.h>

#include <algorithm>

#include "ecs_stencil.cuh"

namespace {

// ---- difference numerators on the extended (N+1)^3 node grid -------------
// src/vector-math.c:619-712: central difference at every node index < N, the
// backward formula at index N (reached only as the high corner of the last
// cell).  FP64, separately rounded.
__device__ __forceinline__ double dnum(const double *F, const GridG &g, int axis, int k, int j, int i) {
  int N = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
  int h = axis == 0 ? i : (axis == 1 ? j : k);
  auto at = [&](int o) -> rd {
    return rd{axis == 0 ? gval(F, g, k, j, i + o) : (axis == 1 ? gval(F, g, k, j + o, i) : gval(F, g, k + o, j, i))};
  };
  if (h < N) return (at(1) - at(-1)).v;
  return ((rd{3.0} * at(0) - rd{4.0} * at(-1)) + rd{1.0} * at(-2)).v;
}

__global__ void k_eext(GridG g, const double *__restrict__ phi, double4_32a *__restrict__ e64,
                       float4 *__restrict__ e32) {
  const int sx = g.nx + 1, sy = g.ny + 1;
  int i, j, k;
  if (!at3(sx, sy, i, j, k)) return;
  const unsigned e = ((unsigned)k * sy + j) * sx + i;
  double dx = dnum(phi, g, 0, k, j, i), dy = dnum(phi, g, 1, k, j, i), dz = dnum(phi, g, 2, k, j, i);
  if (e64) e64[e] = make_double4_32a(dx, dy, dz, 0.0);
  if (e32) e32[e] = make_float4((float)dx, (float)dy, (float)dz, 0.0f);
}

// ---- moments -----------------------------------------------------------------
__global__ void k_moments(size_t n, const long long *__restrict__ acc, double *__restrict__ mom,
                          double iscale_n, double iscale_f, EcsDevStatus *st) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < 4 * n; e += (size_t)gridDim.x * blockDim.x) {
    long long a = acc[e];
    if (a > (1ll << 62) || a < -(1ll << 62)) atomicOr(&st->flags, ECS_FLAG_RANGE);
    mom[e] = __ll2double_rn(a) * (e < n ? iscale_n : iscale_f);
  }
}

// ---- RHS: src/rhs.c:321-354 --------------------------------------------------
struct RhsK {
  double kappa, hx, hy, hz, hxx, hyy, hzz, E0, cth, cG, scale;
};

// Fixed-order sum of `local` over the block into partial[block].
__device__ __forceinline__ void block_partial(double local, double *sh, double *__restrict__ partial) {
  for (int s = 16; s >= 1; s >>= 1) local += __shfl_xor_sync(ECS_FULL_MASK, local, s);
  const int t = thread_lin();
  if ((t & 31) == 0) sh[t >> 5] = local;
  __syncthreads();
  if (t == 0) {
    double u = 0.0;
    for (int w = 0; w < kTx * kTy / 32; w++) u += sh[w];
    partial[block_lin()] = u;
  }
}

// b at every cell; each block writes the sum of its cells to partial[block]
// (z loop with stride gridDim.z, so the block count stays bounded).
__global__ void k_rhs(GridG g, RhsK r, const double *__restrict__ mom, double *__restrict__ b,
                      double *__restrict__ partial) {
  __shared__ double sh[kTx * kTy / 32];
  double local = 0.0;
  const double *n = mom, *Gx = mom + g.n, *Gy = mom + 2 * g.n, *Gz = mom + 3 * g.n;
  int i, j, k0;
  if (at3(g.nx, g.ny, i, j, k0)) {
    for (int k = k0; k < g.nz; k += gridDim.z) {
      const Nbr q = nbr_of(g, i, j, k);  // the neighbours' offsets (gval's wrap and ghosts)
      rd nijk{n[q.c]};
      rd npjk{nval(n, q, q.xp, q.vxp)}, nmjk{nval(n, q, q.xm, q.vxm)};
      rd nipk{nval(n, q, q.yp, q.vyp)}, nimk{nval(n, q, q.ym, q.vym)};
      rd nijp{nval(n, q, q.zp, q.vzp)}, nijm{nval(n, q, q.zm, q.vzm)};
      rd two{2.0}, one{1.0}, kap{r.kappa};
      rd dndx = rd{r.hx} * (npjk - nmjk);
      rd dndy = rd{r.hy} * (nipk - nimk);
      rd d2ndxx = rd{r.hxx} * ((npjk - two * nijk) + nmjk);
      rd d2ndyy = rd{r.hyy} * ((nipk - two * nijk) + nimk);
      rd d2ndzz = rd{r.hzz} * ((nijp - two * nijk) + nijm);
      rd dGxdx = rd{r.hx} * (rd{nval(Gx, q, q.xp, q.vxp)} - rd{nval(Gx, q, q.xm, q.vxm)});
      rd dGydy = rd{r.hy} * (rd{nval(Gy, q, q.yp, q.vyp)} - rd{nval(Gy, q, q.ym, q.vym)});
      rd dGzdz = rd{r.hz} * (rd{nval(Gz, q, q.zp, q.vzp)} - rd{nval(Gz, q, q.zm, q.vzm)});
      rd Eterm = (dndy - kap * dndx) * rd{r.E0};
      rd Pterm = rd{r.cth} * ((d2ndxx + d2ndyy) + (one + kap * kap) * d2ndzz);
      rd Gterm = rd{r.cG} * ((dGxdx + dGydy) + dGzdz);
      double v = (rd{r.scale} * ((Eterm + Pterm) + Gterm)).v;
      b[q.c] = v;
      local += v;
    }
  }
  block_partial(local, sh, partial);
}

// -rhs sinusoidal (ComputeSinusoidalRHS3D, src/rhs.c:82-148): b = n0 cos(2 pi
// x) cos(2 pi y) cos(2 pi z) scale at the cell centres x = (i + 1/2) dx (in
// the grid's own units, as the reference), block partials for the mean that
// MatNullSpaceRemove takes out (src/rhs.c:138-141).
__global__ void k_rhs_sin(GridG g, int ndim, double dx, double dy, double dz, double n0, double scale,
                          double *__restrict__ b, double *__restrict__ partial) {
  __shared__ double sh[kTx * kTy / 32];
  double local = 0.0;
  int i, j, k0;
  if (at3(g.nx, g.ny, i, j, k0)) {
    const double twopi = 2 * M_PI;
    const double cx = cos(__dmul_rn(twopi, __dmul_rn(__dadd_rn((double)i, 0.5), dx)));
    const double cy = cos(__dmul_rn(twopi, __dmul_rn(__dadd_rn((double)j, 0.5), dy)));
    for (int k = k0; k < g.nz; k += gridDim.z) {
      // 2-D (ComputeSinusoidalRHS2D src/rhs.c:26-79): n0 Cx Cy scale
      const double cxy = __dmul_rn(cx, cy);
      const double val =
          ndim == 2 ? cxy : __dmul_rn(cxy, cos(__dmul_rn(twopi, __dmul_rn(__dadd_rn((double)k, 0.5), dz))));
      const double v = __dmul_rn(__dmul_rn(n0, val), scale);
      b[lin3(g, i, j, k)] = v;
      local += v;
    }
  }
  block_partial(local, sh, partial);
}

// -rhs constant (ComputeConstantRHS, src/rhs.c:6-23): b = n0 * scale, no
// projection.
__global__ void k_fill(size_t n, double v, double *__restrict__ b) {
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) b[c] = v;
}

// out[0] = (sum of partial[0..nb)) / div, one block, fixed order.
__global__ void __launch_bounds__(1024) k_sum_final(int nb, const double *__restrict__ partial, double div,
                                                    double *__restrict__ out) {
  __shared__ double sh[32];
  double t = 0.0;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) t += partial[q];
  for (int s = 16; s >= 1; s >>= 1) t += __shfl_xor_sync(ECS_FULL_MASK, t, s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) u += sh[q];
    out[0] = u / div;
  }
}

// v -= mean (src/rhs.c:363-366)
__global__ void k_sub_value(size_t n, double *__restrict__ v, const double *__restrict__ mean) {
  const double m = *mean;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    v[c] -= m;
}

unsigned int blocks1d(const EcsCtx *ctx, size_t n) {
  size_t want = (n + 255) / 256;
  size_t cap = (size_t)ctx->nsm * 8;
  if (want > cap) want = cap;
  return (unsigned int)(want ? want : 1);
}

}  // namespace

// ============================================================================
// entry points used by ecs_api.cu
// ============================================================================
int ecs_grid_eext(EcsCtx *ctx) {
  GridG g = make_grid(ctx->p, ctx->p.Nx, ctx->p.Ny, ctx->p.Nz);
  k_eext<<<blocks3(g.nx + 1, g.ny + 1, g.nz + 1), threads3(), 0, ctx->stream>>>(
      g, ctx->phi, ctx->prec == ECS_PREC_FP64 ? ctx->eext64 : nullptr,
      ctx->prec == ECS_PREC_MIXED ? ctx->eext32 : nullptr);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

int ecs_grid_clear_acc(EcsCtx *ctx) {
  ECS_CUDA(ctx, cudaMemsetAsync(ctx->acc, 0, ctx->ncell * 4 * sizeof(long long), ctx->stream));
  return ECS_OK;
}

int ecs_grid_moments(EcsCtx *ctx) {
  k_moments<<<blocks1d(ctx, ctx->ncell * 4), 256, 0, ctx->stream>>>(ctx->ncell, ctx->acc, ctx->mom,
                                                                   ldexp(1.0, -ctx->shift_n),
                                                                   ldexp(1.0, -ctx->shift_f), ctx->dstat);
  ECS_LAUNCHED(ctx);
  ctx->moments_ready = true;
  return ECS_OK;
}

int ecs_grid_rhs(EcsCtx *ctx) {
  int rc = ecs_solver_alloc(ctx);
  if (rc) return rc;
  const EcsParams &p = ctx->p;
  if (p.rhs_type == ECS_RHS_CONSTANT) {
    k_fill<<<blocks1d(ctx, ctx->ncell), 256, 0, ctx->stream>>>(ctx->ncell, p.n0 * p.scale, ctx->rhs);
    ECS_LAUNCHED(ctx);
    return ECS_OK;
  }
  GridG g = make_grid(p, p.Nx, p.Ny, p.Nz);
  dim3 grid = blocks3(g);
  const unsigned plane_blocks = grid.x * grid.y;
  grid.z = std::max(1u, std::min(grid.z, (unsigned)ctx->nred / plane_blocks));
  const int nb = (int)(grid.x * grid.y * grid.z);
  if (p.rhs_type == ECS_RHS_SINUSOIDAL) {
    k_rhs_sin<<<grid, threads3(), 0, ctx->stream>>>(g, p.ndim, p.dx, p.dy, p.dz, p.n0, p.scale, ctx->rhs, ctx->red);
  } else {
    RhsK r;
    r.kappa = p.kappa_e;
    r.hx = 1.0 / (2.0 * p.dx); r.hy = 1.0 / (2.0 * p.dy); r.hz = 1.0 / (2.0 * p.dz);
    r.hxx = 1.0 / (p.dx * p.dx); r.hyy = 1.0 / (p.dy * p.dy); r.hzz = 1.0 / (p.dz * p.dz);
    r.E0 = p.E0; r.cth = p.cth; r.cG = p.cG; r.scale = p.scale;
    k_rhs<<<grid, threads3(), 0, ctx->stream>>>(g, r, ctx->mom, ctx->rhs, ctx->red);
  }
  ECS_LAUNCHED(ctx);
  k_sum_final<<<1, 1024, 0, ctx->stream>>>(nb, ctx->red, (double)ctx->ncell, ctx->dots);
  ECS_LAUNCHED(ctx);
  k_sub_value<<<blocks1d(ctx, ctx->ncell), 256, 0, ctx->stream>>>(ctx->ncell, ctx->rhs, ctx->dots);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}
