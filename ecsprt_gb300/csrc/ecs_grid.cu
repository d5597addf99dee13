// Grid phase of the ECSPRT hot path on sm_103a:
//   difference numerators of phi on the extended node grid (input to push)
//   fixed-point -> FP64 moments                       src/moments.c:208-211
//   RHS of the quasineutral potential equation         src/rhs.c:259-373
//   matrix-free 11-point operator                       src/lhs.c:337-505
//   potential solve                                     src/potential.c:6-15
//
// Solver: FGMRES(m) preconditioned by one geometric-multigrid V(1,1) cycle
// (full coarsening, full-weighting restriction, trilinear prolongation,
// coarse operators rediscretised from the full-weighted density, damped
// z-line Jacobi smoothing: the z couplings carry (1+kappa^2) and dominate).
//   ECS_PREC_FP64:  FGMRES and multigrid in FP64 to the requested rtol.
//   ECS_PREC_MIXED: FP64 iterative refinement; each correction is an FP32
//     FGMRES/multigrid solve; residuals, dot products, the update of phi and
//     the mean projection are FP64.
// All reductions use fixed block partials summed in a fixed order, so every
// result is reproducible run to run.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>

#include <algorithm>

#include "ecs_internal.cuh"

namespace {

struct rd {
  double v;
};
__device__ __forceinline__ rd operator+(rd a, rd b) { return {__dadd_rn(a.v, b.v)}; }
__device__ __forceinline__ rd operator-(rd a, rd b) { return {__dsub_rn(a.v, b.v)}; }
__device__ __forceinline__ rd operator*(rd a, rd b) { return {__dmul_rn(a.v, b.v)}; }

struct GridG {
  int nx, ny, nz;
  int bc[3];  // 0 periodic, else ghosted (value 0 outside)
  size_t n;
};

template <typename T>
__device__ __forceinline__ T gval(const T *__restrict__ F, const GridG &g, int k, int j, int i) {
  if (i < 0 || i >= g.nx) { if (g.bc[0]) return T(0); i = i < 0 ? i + g.nx : i - g.nx; }
  if (j < 0 || j >= g.ny) { if (g.bc[1]) return T(0); j = j < 0 ? j + g.ny : j - g.ny; }
  if (k < 0 || k >= g.nz) { if (g.bc[2]) return T(0); k = k < 0 ? k + g.nz : k - g.nz; }
  return F[((size_t)k * g.ny + j) * g.nx + i];
}

__device__ __forceinline__ void cell_ijk(size_t c, const GridG &g, int &i, int &j, int &k) {
  i = (int)(c % g.nx);
  size_t r = c / g.nx;
  j = (int)(r % g.ny);
  k = (int)(r / g.ny);
}

// ---- difference numerators on the extended (N+1)^3 node grid -------------
// src/vector-math.c:619-712: central difference at every node index < N, the
// backward formula at index N (reached only as the high corner of the last
// cell).  FP64, separately rounded.
__device__ __forceinline__ double dnum(const double *F, const GridG &g, int axis, int k, int j,
                                       int i) {
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
  const size_t sx = (size_t)g.nx + 1, sy = (size_t)g.ny + 1;
  const size_t ne = sx * sy * ((size_t)g.nz + 1);
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(e % sx), j = (int)((e / sx) % sy), k = (int)(e / (sx * sy));
    double dx = dnum(phi, g, 0, k, j, i), dy = dnum(phi, g, 1, k, j, i), dz = dnum(phi, g, 2, k, j, i);
    if (e64) e64[e] = make_double4_32a(dx, dy, dz, 0.0);
    if (e32) e32[e] = make_float4((float)dx, (float)dy, (float)dz, 0.0f);
  }
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
__global__ void k_rhs(GridG g, RhsK r, const double *__restrict__ mom, double *__restrict__ b,
                      double *__restrict__ partial) {
  __shared__ double sh[32];
  double local = 0.0;
  const double *n = mom, *Gx = mom + g.n, *Gy = mom + 2 * g.n, *Gz = mom + 3 * g.n;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(c, g, i, j, k);
    rd nijk{gval(n, g, k, j, i)};
    rd npjk{gval(n, g, k, j, i + 1)}, nmjk{gval(n, g, k, j, i - 1)};
    rd nipk{gval(n, g, k, j + 1, i)}, nimk{gval(n, g, k, j - 1, i)};
    rd nijp{gval(n, g, k + 1, j, i)}, nijm{gval(n, g, k - 1, j, i)};
    rd two{2.0}, one{1.0}, kap{r.kappa};
    rd dndx = rd{r.hx} * (npjk - nmjk);
    rd dndy = rd{r.hy} * (nipk - nimk);
    rd d2ndxx = rd{r.hxx} * ((npjk - two * nijk) + nmjk);
    rd d2ndyy = rd{r.hyy} * ((nipk - two * nijk) + nimk);
    rd d2ndzz = rd{r.hzz} * ((nijp - two * nijk) + nijm);
    rd dGxdx = rd{r.hx} * (rd{gval(Gx, g, k, j, i + 1)} - rd{gval(Gx, g, k, j, i - 1)});
    rd dGydy = rd{r.hy} * (rd{gval(Gy, g, k, j + 1, i)} - rd{gval(Gy, g, k, j - 1, i)});
    rd dGzdz = rd{r.hz} * (rd{gval(Gz, g, k + 1, j, i)} - rd{gval(Gz, g, k - 1, j, i)});
    rd Eterm = (dndy - kap * dndx) * rd{r.E0};
    rd Pterm = rd{r.cth} * ((d2ndxx + d2ndyy) + (one + kap * kap) * d2ndzz);
    rd Gterm = rd{r.cG} * ((dGxdx + dGydy) + dGzdz);
    double v = (rd{r.scale} * ((Eterm + Pterm) + Gterm)).v;
    b[c] = v;
    local += v;
  }
  // fixed-order block sum
  for (int s = 16; s >= 1; s >>= 1) local += __shfl_xor_sync(ECS_FULL_MASK, local, s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    partial[blockIdx.x] = t;
  }
}

// sum of nb partials in order, then v -= sum/n (src/rhs.c:363-366)
__global__ void k_sub_mean(size_t n, double *__restrict__ v, const double *__restrict__ partial, int nb) {
  __shared__ double mean;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < nb; q++) t += partial[q];
    mean = t / (double)n;
  }
  __syncthreads();
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    v[c] -= mean;
}

// ---- operator (src/lhs.c:366-423), templated on the arithmetic type --------
struct OpK {
  GridG g;
  double sxx, syy, szz, sod;
};

// 11 coefficients of row (k,j,i) in the reference's order:
// x+, x-, y+, y-, z+, z-, (x+,y+), (x+,y-), (x-,y+), (x-,y-), centre.
template <typename T>
__device__ __forceinline__ void row11(const T *__restrict__ n, const OpK &o, int i, int j, int k, T v[11]) {
  const GridG &g = o.g;
  T nijk = gval(n, g, k, j, i);
  T nmjk = gval(n, g, k, j, i - 1), npjk = gval(n, g, k, j, i + 1);
  T nimk = gval(n, g, k, j - 1, i), nipk = gval(n, g, k, j + 1, i);
  T nijm = gval(n, g, k - 1, j, i), nijp = gval(n, g, k + 1, j, i);
  T sxx = T(o.sxx), syy = T(o.syy), szz = T(o.szz), sod = T(o.sod);
  v[6] = sod * (nipk - npjk);
  v[7] = sod * (npjk - nimk);
  v[8] = sod * (nmjk - nipk);
  v[9] = sod * (nimk - nmjk);
  v[0] = sxx * (npjk + nijk) + sod * (nipk - nimk);
  v[1] = sxx * (nijk + nmjk) - sod * (nipk - nimk);
  v[2] = syy * (nipk + nijk) - sod * (npjk - nmjk);
  v[3] = syy * (nijk + nimk) + sod * (npjk - nmjk);
  v[4] = szz * (nijp + nijk);
  v[5] = szz * (nijk + nijm);
  v[10] = -(sxx * (npjk + T(2) * nijk + nmjk) + syy * (nipk + T(2) * nijk + nimk) +
            szz * (nijp + T(2) * nijk + nijm));
}

__constant__ int c_off[11][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
                                 {1, 1, 0}, {1, -1, 0}, {-1, 1, 0}, {-1, -1, 0}, {0, 0, 0}};

// y = A x   (mode 0)     or     y = b - A x   (mode 1)
template <typename T>
__global__ void k_apply(OpK o, const T *__restrict__ n, const T *__restrict__ x,
                        const T *__restrict__ b, T *__restrict__ y, int mode) {
  const GridG &g = o.g;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(c, g, i, j, k);
    T v[11];
    row11(n, o, i, j, k, v);
    T s = T(0);
#pragma unroll
    for (int e = 0; e < 11; e++) s += v[e] * gval(x, g, k + c_off[e][2], j + c_off[e][1], i + c_off[e][0]);
    y[c] = mode ? b[c] - s : s;
  }
}

// Mixed-precision residual: r64 = b64 - A64(n64) x64.
__global__ void k_residual64(OpK o, const double *__restrict__ n, const double *__restrict__ x,
                             const double *__restrict__ b, double *__restrict__ r) {
  const GridG &g = o.g;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(c, g, i, j, k);
    double v[11];
    row11(n, o, i, j, k, v);
    double s = 0.0;
#pragma unroll
    for (int e = 0; e < 11; e++) s += v[e] * gval(x, g, k + c_off[e][2], j + c_off[e][1], i + c_off[e][0]);
    r[c] = b[c] - s;
  }
}


// ---- z-line smoother --------------------------------------------------------------
// Column (i,j) carries the z-tridiagonal part of the rows: lo = z- entry,
// diag = centre, up = z+ entry.  A periodic z closes the cycle, solved with
// Sherman-Morrison around the Thomas factorisation of the modified matrix;
// reflecting z drops the out-of-range couplings (Dirichlet-0 ghosts).
template <typename T>
struct ZlP {
  T *a, *cp, *minv, *q, *dp;  // per cell
  T *a0g, *qden;              // per column
};

template <typename T>
__global__ void k_zline_setup(OpK o, const T *__restrict__ n, ZlP<T> z) {
  const GridG &g = o.g;
  const int ncol = g.nx * g.ny;
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const int i = col % g.nx, j = col / g.nx;
  const size_t plane = (size_t)g.nx * g.ny;
  const bool cyc = g.bc[2] == 0;
  const int N = g.nz;
  T v[11];
  row11(n, o, i, j, 0, v);
  const T lo0 = cyc ? v[5] : T(0), d0 = v[10];
  const T gamma = -d0;
  T cp_prev = T(0), dq_prev = T(0);
  // forward: factor T' and forward-substitute u = (gamma, 0, .., up_{N-1})
  for (int k = 0; k < N; k++) {
    row11(n, o, i, j, k, v);
    T a = (k == 0) ? T(0) : v[5];
    T up = (k == N - 1) ? T(0) : v[4];
    T bb = v[10];
    if (cyc && k == 0) bb = d0 - gamma;
    if (cyc && k == N - 1) bb = v[10] - v[4] * lo0 / gamma;
    T m = bb - a * cp_prev;
    T minv = T(1) / m;
    T cp = up * minv;
    T u = cyc ? ((k == 0) ? gamma : ((k == N - 1) ? v[4] : T(0))) : T(0);
    T dq = (u - a * dq_prev) * minv;
    size_t c = (size_t)k * plane + col;
    z.a[c] = a;
    z.cp[c] = cp;
    z.minv[c] = minv;
    z.q[c] = dq;
    cp_prev = cp;
    dq_prev = dq;
  }
  // backward substitution for q
  T qn = z.q[(size_t)(N - 1) * plane + col];
  for (int k = N - 2; k >= 0; k--) {
    size_t c = (size_t)k * plane + col;
    qn = z.q[c] - z.cp[c] * qn;
    z.q[c] = qn;
  }
  if (cyc) {
    T a0g = lo0 / gamma;
    T q0 = z.q[col], qN = z.q[(size_t)(N - 1) * plane + col];
    z.a0g[col] = a0g;
    z.qden[col] = T(1) / (T(1) + q0 + a0g * qN);
  } else {
    z.a0g[col] = T(0);
    z.qden[col] = T(0);
  }
}

// Right-hand side of the z-line systems: r = b - A_xy xo, where A_xy holds
// the 8 in-plane entries of each row (x+-, y+-, the four xy corners).
template <typename T>
__global__ void k_zline_rhs(OpK o, const T *__restrict__ n, const T *__restrict__ b,
                            const T *__restrict__ xo, T *__restrict__ r) {
  const GridG &g = o.g;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_ijk(c, g, i, j, k);
    T v[11];
    row11(n, o, i, j, k, v);
    T s = b[c];
#pragma unroll
    for (int e = 0; e < 10; e++) {
      if (e == 4 || e == 5) continue;
      s -= v[e] * gval(xo, g, k, j + c_off[e][1], i + c_off[e][0]);
    }
    r[c] = s;
  }
}

constexpr int kZChunk = 8;

// Thomas solve of one column with the precomputed factors (a, cp, minv) and
// the Sherman-Morrison closure (q, a0g, qden), then damping against xo
// (nullptr: zero).  Loads of chunk c+1 are issued before chunk c is used.
template <typename T>
__device__ __forceinline__ void zline_column(const GridG &g, const ZlP<T> &z, const T *__restrict__ r,
                                             const T *__restrict__ xo, T *__restrict__ xn, T omega, int col) {
  const size_t plane = (size_t)g.nx * g.ny;
  const int N = g.nz;
  T ra[kZChunk], aa[kZChunk], ma[kZChunk];
  T rb[kZChunk], ab[kZChunk], mb[kZChunk];
#pragma unroll
  for (int q = 0; q < kZChunk; q++) {
    size_t c = (size_t)q * plane + col;
    bool in = q < N;
    ra[q] = in ? r[c] : T(0);
    aa[q] = in ? z.a[c] : T(0);
    ma[q] = in ? z.minv[c] : T(0);
  }
  T dp = T(0);
  for (int k0 = 0; k0 < N; k0 += kZChunk) {
#pragma unroll
    for (int q = 0; q < kZChunk; q++) {  // prefetch next chunk
      int k = k0 + kZChunk + q;
      size_t c = (size_t)k * plane + col;
      bool in = k < N;
      rb[q] = in ? r[c] : T(0);
      ab[q] = in ? z.a[c] : T(0);
      mb[q] = in ? z.minv[c] : T(0);
    }
#pragma unroll
    for (int q = 0; q < kZChunk; q++) {
      int k = k0 + q;
      if (k < N) {
        dp = (ra[q] - aa[q] * dp) * ma[q];
        z.dp[(size_t)k * plane + col] = dp;
      }
    }
#pragma unroll
    for (int q = 0; q < kZChunk; q++) {
      ra[q] = rb[q];
      aa[q] = ab[q];
      ma[q] = mb[q];
    }
  }
  // backward substitution, chunks from the top
  T y = T(0);
  const T yN = z.dp[(size_t)(N - 1) * plane + col];
  const int last0 = ((N - 1) / kZChunk) * kZChunk;
  T da[kZChunk], ca[kZChunk], db[kZChunk], cb[kZChunk];
#pragma unroll
  for (int q = 0; q < kZChunk; q++) {
    int k = last0 + q;
    size_t c = (size_t)k * plane + col;
    bool in = k < N;
    da[q] = in ? z.dp[c] : T(0);
    ca[q] = in ? z.cp[c] : T(0);
  }
  for (int k0 = last0; k0 >= 0; k0 -= kZChunk) {
#pragma unroll
    for (int q = 0; q < kZChunk; q++) {
      int k = k0 - kZChunk + q;
      size_t c = (size_t)(k < 0 ? 0 : k) * plane + col;
      bool in = k >= 0;
      db[q] = in ? z.dp[c] : T(0);
      cb[q] = in ? z.cp[c] : T(0);
    }
#pragma unroll
    for (int q = kZChunk - 1; q >= 0; q--) {
      int k = k0 + q;
      if (k < N) {
        y = (k == N - 1) ? da[q] : da[q] - ca[q] * y;
        z.dp[(size_t)k * plane + col] = y;
      }
    }
#pragma unroll
    for (int q = 0; q < kZChunk; q++) {
      da[q] = db[q];
      ca[q] = cb[q];
    }
  }
  const T s = (y + z.a0g[col] * yN) * z.qden[col];
  for (int k0 = 0; k0 < N; k0 += kZChunk) {
    T yv[kZChunk], qv[kZChunk], ov[kZChunk];
#pragma unroll
    for (int q = 0; q < kZChunk; q++) {
      int k = k0 + q;
      size_t c = (size_t)k * plane + col;
      bool in = k < N;
      yv[q] = in ? z.dp[c] : T(0);
      qv[q] = in ? z.q[c] : T(0);
      ov[q] = (in && xo) ? xo[c] : T(0);
    }
#pragma unroll
    for (int q = 0; q < kZChunk; q++) {
      int k = k0 + q;
      if (k < N) xn[(size_t)k * plane + col] = ov[q] + omega * ((yv[q] - s * qv[q]) - ov[q]);
    }
  }
}

template <typename T>
__global__ void k_zline_solve(GridG g, ZlP<T> z, const T *__restrict__ r, const T *__restrict__ xo,
                              T *__restrict__ xn, T omega) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= g.nx * g.ny) return;
  zline_column<T>(g, z, r, xo, xn, omega, col);
}

// All sweeps of a small level in one block: each sweep forms r in `rbuf`,
// solves every column, and alternates between x and t; the result ends in x.
template <typename T>
__global__ void k_zline_block(OpK o, const T *__restrict__ n, ZlP<T> z, const T *__restrict__ b,
                              T *__restrict__ x, T *__restrict__ t, T *__restrict__ rbuf, int nsweeps,
                              T omega) {
  const GridG &g = o.g;
  const int ncol = g.nx * g.ny;
  T *cur = x, *nxt = t;
  for (int sw = 0; sw < nsweeps; sw++) {
    const T *xo = sw == 0 ? nullptr : cur;
    if (xo) {
      for (size_t c = threadIdx.x; c < g.n; c += blockDim.x) {
        int i, j, k;
        cell_ijk(c, g, i, j, k);
        T v[11];
        row11(n, o, i, j, k, v);
        T s = b[c];
#pragma unroll
        for (int e = 0; e < 10; e++) {
          if (e == 4 || e == 5) continue;
          s -= v[e] * gval(xo, g, k, j + c_off[e][1], i + c_off[e][0]);
        }
        rbuf[c] = s;
      }
      __syncthreads();
    }
    for (int col = threadIdx.x; col < ncol; col += blockDim.x)
      zline_column<T>(g, z, xo ? rbuf : b, xo, nxt, omega, col);
    __syncthreads();
    T *tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  if (cur != x) {
    for (size_t c = threadIdx.x; c < g.n; c += blockDim.x) x[c] = cur[c];
  }
}

// ---- inter-grid transfer ---------------------------------------------------------
// Full weighting (1/4,1/2,1/4 per axis) from fine (2I+a) to coarse I.
template <typename T>
__device__ __forceinline__ T restrict_at(const GridG &gf, const GridG &gc, const T *__restrict__ f, size_t e) {
  int I, J, K;
  cell_ijk(e, gc, I, J, K);
  T s = T(0);
#pragma unroll
  for (int dk = -1; dk <= 1; dk++) {
    T wk = dk == 0 ? T(0.5) : T(0.25);
#pragma unroll
    for (int dj = -1; dj <= 1; dj++) {
      T wj = dj == 0 ? T(0.5) : T(0.25);
#pragma unroll
      for (int di = -1; di <= 1; di++) {
        T wi = di == 0 ? T(0.5) : T(0.25);
        s += wk * wj * wi * gval(f, gf, 2 * K + dk, 2 * J + dj, 2 * I + di);
      }
    }
  }
  return s;
}
template <typename T>
__global__ void k_restrict(GridG gf, GridG gc, const T *__restrict__ f, T *__restrict__ c) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < gc.n; e += (size_t)gridDim.x * blockDim.x)
    c[e] = restrict_at(gf, gc, f, e);
}

// Trilinear prolongation value at fine cell e.
template <typename T>
__device__ __forceinline__ T prolong_at(const GridG &gf, const GridG &gc, const T *__restrict__ c, size_t e) {
  int i, j, k;
  cell_ijk(e, gf, i, j, k);
  int i0 = i >> 1, j0 = j >> 1, k0 = k >> 1;
  int ni = (i & 1) ? 2 : 1, nj = (j & 1) ? 2 : 1, nk = (k & 1) ? 2 : 1;
  T wi = ni == 2 ? T(0.5) : T(1), wj = nj == 2 ? T(0.5) : T(1), wk = nk == 2 ? T(0.5) : T(1);
  T s = T(0);
  for (int a = 0; a < nk; a++)
    for (int bq = 0; bq < nj; bq++)
      for (int q = 0; q < ni; q++) s += gval(c, gc, k0 + a, j0 + bq, i0 + q);
  return wi * wj * wk * s;
}
// f += P c.
template <typename T>
__global__ void k_prolong_add(GridG gf, GridG gc, const T *__restrict__ c, T *__restrict__ f) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < gf.n; e += (size_t)gridDim.x * blockDim.x)
    f[e] += prolong_at(gf, gc, c, e);
}

// ---- whole V-cycle of the small levels in one thread block -------------------
template <typename T>
struct SmallLevel {
  OpK o;
  T *dens, *x, *b, *r, *t;
  ZlP<T> z;
};
constexpr int kMaxSmall = 8;
template <typename T>
struct SmallCycle {
  int nl;
  SmallLevel<T> lv[kMaxSmall];
};

template <typename T>
__device__ void blk_sweep(const SmallLevel<T> &L, const T *b, const T *xo, T *xn, T omega) {
  const GridG &g = L.o.g;
  if (xo) {
    for (size_t c = threadIdx.x; c < g.n; c += blockDim.x) {
      int i, j, k;
      cell_ijk(c, g, i, j, k);
      T v[11];
      row11(L.dens, L.o, i, j, k, v);
      T s = b[c];
#pragma unroll
      for (int e = 0; e < 10; e++) {
        if (e == 4 || e == 5) continue;
        s -= v[e] * gval(xo, g, k, j + c_off[e][1], i + c_off[e][0]);
      }
      L.r[c] = s;
    }
    __syncthreads();
  }
  for (int col = threadIdx.x; col < g.nx * g.ny; col += blockDim.x)
    zline_column<T>(g, L.z, xo ? L.r : b, xo, xn, omega, col);
  __syncthreads();
}

// x_out = M(l0) b_in: V(1,1) over levels l0..l0+nl-1, all in this block.
template <typename T>
__global__ void __launch_bounds__(512) k_vcycle_small(SmallCycle<T> sc, const T *__restrict__ b_in,
                                                      T *__restrict__ x_out, int coarse_sweeps, T omega) {
  const int nl = sc.nl;
  // down
  for (int l = 0; l < nl - 1; l++) {
    const SmallLevel<T> &L = sc.lv[l];
    const T *b = l == 0 ? b_in : L.b;
    blk_sweep(L, b, (const T *)nullptr, L.t, omega);
    const GridG &g = L.o.g;
    for (size_t c = threadIdx.x; c < g.n; c += blockDim.x) {
      int i, j, k;
      cell_ijk(c, g, i, j, k);
      T v[11];
      row11(L.dens, L.o, i, j, k, v);
      T s = T(0);
#pragma unroll
      for (int e = 0; e < 11; e++) s += v[e] * gval(L.t, g, k + c_off[e][2], j + c_off[e][1], i + c_off[e][0]);
      L.r[c] = b[c] - s;
    }
    __syncthreads();
    const SmallLevel<T> &C = sc.lv[l + 1];
    for (size_t c = threadIdx.x; c < C.o.g.n; c += blockDim.x) C.b[c] = restrict_at(g, C.o.g, L.r, c);
    __syncthreads();
  }
  // coarsest: damped z-line Jacobi sweeps, result in its x (or x_out if nl == 1)
  {
    const SmallLevel<T> &L = sc.lv[nl - 1];
    const T *b = nl == 1 ? b_in : L.b;
    T *dst = nl == 1 ? x_out : L.x;
    T *cur = dst, *nxt = L.t;
    for (int sw = 0; sw < coarse_sweeps; sw++) {
      blk_sweep(L, b, sw == 0 ? (const T *)nullptr : cur, nxt, omega);
      T *tmp = cur;
      cur = nxt;
      nxt = tmp;
    }
    if (cur != dst) {
      for (size_t c = threadIdx.x; c < L.o.g.n; c += blockDim.x) dst[c] = cur[c];
      __syncthreads();
    }
  }
  // up
  for (int l = nl - 2; l >= 0; l--) {
    const SmallLevel<T> &L = sc.lv[l], &C = sc.lv[l + 1];
    const GridG &g = L.o.g;
    for (size_t c = threadIdx.x; c < g.n; c += blockDim.x) L.t[c] += prolong_at(g, C.o.g, C.x, c);
    __syncthreads();
    const T *b = l == 0 ? b_in : L.b;
    blk_sweep(L, b, L.t, l == 0 ? x_out : L.x, omega);
  }
}

// ---- vectors and reductions ------------------------------------------------------
template <typename T>
__global__ void k_fill(size_t n, T *v, T a) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) v[e] = a;
}
template <typename TS, typename TD>
__global__ void k_scale_copy(size_t n, const TS *__restrict__ s, TD *__restrict__ d, double a) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    d[e] = (TD)(a * (double)s[e]);
}
// x64 += a * e (e in T)
template <typename T>
__global__ void k_axpy64(size_t n, double a, const T *__restrict__ e, double *__restrict__ x) {
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    x[q] += a * (double)e[q];
}

// partial[v*nb + block] = sum_k V_v[k] * w[k] for v < nv; slot nv holds w.w.
// Products and sums over runs of 8 consecutive elements are formed in the
// vectors' own precision T; the runs are accumulated in FP64.
template <typename T>
__global__ void k_mdot_partial(size_t n, int nv, const T *__restrict__ V, size_t ld, const T *__restrict__ w,
                               int with_ww, double *__restrict__ partial) {
  extern __shared__ double shm[];  // [nwarps][nv+1]
  const int nwarp = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nslot = nv + (with_ww ? 1 : 0);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (int v0 = 0; v0 < nslot; v0 += 8) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    while (e < n) {
      T run[8] = {T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0)};
#pragma unroll 1
      for (int r = 0; r < 8 && e < n; r++, e += stride) {
        const T we = w[e];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int v = v0 + q;
          if (v < nv) run[q] += V[(size_t)v * ld + e] * we;
          else if (v == nv && with_ww) run[q] += we * we;
        }
      }
#pragma unroll
      for (int q = 0; q < 8; q++) acc[q] += (double)run[q];
    }
#pragma unroll
    for (int q = 0; q < 8; q++) {
      double a = acc[q];
      for (int s = 16; s >= 1; s >>= 1) a += __shfl_xor_sync(ECS_FULL_MASK, a, s);
      if (lane == 0 && v0 + q < nslot) shm[warp * nslot + v0 + q] = a;
    }
  }
  __syncthreads();
  for (int v = threadIdx.x; v < nslot; v += blockDim.x) {
    double t = 0.0;
    for (int q = 0; q < nwarp; q++) t += shm[q * nslot + v];
    partial[(size_t)v * gridDim.x + blockIdx.x] = t;
  }
}
__global__ void k_mdot_final(int nslot, int nb, const double *__restrict__ partial, double *__restrict__ out) {
  __shared__ double sh[32];
  const int v = blockIdx.x;
  double t = 0.0;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) t += partial[(size_t)v * nb + q];
  for (int s = 16; s >= 1; s >>= 1) t += __shfl_xor_sync(ECS_FULL_MASK, t, s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) u += sh[q];
    out[v] = u;
  }
  (void)nslot;
}

// w -= sum_v h[v] V_v   (h in device memory)
template <typename T>
__global__ void k_maxpy(size_t n, int nv, const double *__restrict__ h, const T *__restrict__ V, size_t ld,
                        T *__restrict__ w) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    T s = w[e];
    for (int v = 0; v < nv; v++) s -= (T)h[v] * V[(size_t)v * ld + e];
    w[e] = s;
  }
}
// x += sum_v y[v] Z_v
template <typename T>
__global__ void k_combine(size_t n, int nv, const double *__restrict__ y, const T *__restrict__ Z, size_t ld,
                          T *__restrict__ x) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    T s = x[e];
    for (int v = 0; v < nv; v++) s += (T)y[v] * Z[(size_t)v * ld + e];
    x[e] = s;
  }
}
// v -= mean(v) using a precomputed sum
template <typename T>
__global__ void k_shift(size_t n, T *__restrict__ v, const double *__restrict__ sum, double inv_n) {
  const double m = sum[0] * inv_n;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    v[e] = (T)((double)v[e] - m);
}
template <typename T>
__global__ void k_sum_partial(size_t n, const T *__restrict__ v, double *__restrict__ partial) {
  __shared__ double sh[32];
  double t = 0.0;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) t += (double)v[e];
  for (int s = 16; s >= 1; s >>= 1) t += __shfl_xor_sync(ECS_FULL_MASK, t, s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) u += sh[q];
    partial[blockIdx.x] = u;
  }
}

constexpr int kB = 256;

unsigned int blocks_for(const EcsCtx *ctx, size_t n) {
  size_t want = (n + kB - 1) / kB;
  size_t cap = (size_t)ctx->nsm * 8;
  if (want > cap) want = cap;
  return (unsigned int)(want ? want : 1);
}

GridG grid_of(const EcsCtx *ctx, int nx, int ny, int nz) {
  GridG g;
  g.nx = nx; g.ny = ny; g.nz = nz;
  for (int d = 0; d < 3; d++) g.bc[d] = ctx->p.bc[d] == ECS_BC_PERIODIC ? 0 : 1;
  g.n = (size_t)nx * ny * nz;
  return g;
}

// Operator scale factors for spacing (hx, hy, hz), src/lhs.c:366-375.
OpK op_of(const EcsCtx *ctx, int nx, int ny, int nz, double hx, double hy, double hz) {
  OpK o;
  o.g = grid_of(ctx, nx, ny, nz);
  double kappa = ctx->p.kappa_e, scale = ctx->p.scale;
  double hxx = 1.0 / (2.0 * hx * hx), hyy = 1.0 / (2.0 * hy * hy), hzz = 1.0 / (2.0 * hz * hz);
  double hod = 1.0 / (8.0 * hy * hx);
  o.sxx = scale * hxx;
  o.syy = scale * hyy;
  o.szz = scale * (1 + kappa * kappa) * hzz;
  o.sod = scale * kappa * hod;
  return o;
}

bool fully_periodic(const EcsCtx *ctx) {
  return ctx->p.bc[0] == ECS_BC_PERIODIC && ctx->p.bc[1] == ECS_BC_PERIODIC && ctx->p.bc[2] == ECS_BC_PERIODIC;
}

// ---- multigrid ------------------------------------------------------------------------
template <typename T>
Multigrid<T> &mg_of(EcsCtx *ctx);
template <>
Multigrid<double> &mg_of<double>(EcsCtx *ctx) { return ctx->mg64; }
template <>
Multigrid<float> &mg_of<float>(EcsCtx *ctx) { return ctx->mg32; }

template <typename T>
int mg_alloc(EcsCtx *ctx) {
  Multigrid<T> &mg = mg_of<T>(ctx);
  if (mg.built) return ECS_OK;
  int nx = ctx->p.Nx, ny = ctx->p.Ny, nz = ctx->p.Nz;
  double hx = ctx->p.dx, hy = ctx->p.dy, hz = ctx->p.dz;
  for (;;) {
    MgLevel<T> L;
    L.nx = nx; L.ny = ny; L.nz = nz;
    L.n = (size_t)nx * ny * nz;
    L.hx = hx; L.hy = hy; L.hz = hz;
    T **arr[] = {&L.dens, &L.x, &L.b, &L.r, &L.t, &L.zl_a, &L.zl_cp, &L.zl_minv, &L.zl_q, &L.zl_dp};
    for (auto a : arr) ECS_CUDA(ctx, cudaMalloc((void **)a, L.n * sizeof(T)));
    ECS_CUDA(ctx, cudaMalloc((void **)&L.zl_a0g, (size_t)nx * ny * sizeof(T)));
    ECS_CUDA(ctx, cudaMalloc((void **)&L.zl_qden, (size_t)nx * ny * sizeof(T)));
    mg.lv.push_back(L);
    bool even = (nx % 2 == 0) && (ny % 2 == 0) && (nz % 2 == 0);
    if (!even || std::min(nx, std::min(ny, nz)) < 8 || mg.lv.size() >= 12) break;
    nx /= 2; ny /= 2; nz /= 2;
    hx *= 2; hy *= 2; hz *= 2;
  }
  mg.built = true;
  return ECS_OK;
}


template <typename T>
ZlP<T> zl_of(MgLevel<T> &L) {
  ZlP<T> z;
  z.a = L.zl_a; z.cp = L.zl_cp; z.minv = L.zl_minv; z.q = L.zl_q; z.dp = L.zl_dp;
  z.a0g = L.zl_a0g; z.qden = L.zl_qden;
  return z;
}
template <typename T>
OpK op_level(const EcsCtx *ctx, const MgLevel<T> &L) {
  return op_of(ctx, L.nx, L.ny, L.nz, L.hx, L.hy, L.hz);
}

constexpr int kColBlock = 128;
constexpr int kCoarseSweeps = 21;
template <typename T>
constexpr T kOmega() { return T(0.8); }

// Level densities (level 0 from the deposited density, coarser ones by full
// weighting) and the z-line factorisation of every level.
template <typename T>
int mg_setup(EcsCtx *ctx) {
  int rc = mg_alloc<T>(ctx);
  if (rc) return rc;
  Multigrid<T> &mg = mg_of<T>(ctx);
  MgLevel<T> &L0 = mg.lv[0];
  k_scale_copy<double, T><<<blocks_for(ctx, L0.n), kB, 0, ctx->stream>>>(L0.n, ctx->mom, L0.dens, 1.0);
  ECS_LAUNCHED(ctx);
  for (size_t l = 1; l < mg.lv.size(); l++) {
    MgLevel<T> &F = mg.lv[l - 1], &C = mg.lv[l];
    k_restrict<T><<<blocks_for(ctx, C.n), kB, 0, ctx->stream>>>(grid_of(ctx, F.nx, F.ny, F.nz),
                                                              grid_of(ctx, C.nx, C.ny, C.nz), F.dens, C.dens);
    ECS_LAUNCHED(ctx);
  }
  for (auto &L : mg.lv) {
    int ncol = L.nx * L.ny;
    k_zline_setup<T><<<ecs_div_up(ncol, kColBlock), kColBlock, 0, ctx->stream>>>(op_level(ctx, L), L.dens, zl_of(L));
    ECS_LAUNCHED(ctx);
  }
  return ECS_OK;
}

template <typename T>
int sweep(EcsCtx *ctx, MgLevel<T> &L, const T *b, const T *xo, T *xn) {
  const OpK o = op_level(ctx, L);
  const T *r = b;
  if (xo) {
    k_zline_rhs<T><<<blocks_for(ctx, L.n), kB, 0, ctx->stream>>>(o, L.dens, b, xo, L.r);
    ECS_LAUNCHED(ctx);
    r = L.r;
  }
  int ncol = L.nx * L.ny;
  k_zline_solve<T><<<ecs_div_up(ncol, kColBlock), kColBlock, 0, ctx->stream>>>(o.g, zl_of(L), r, xo, xn, kOmega<T>());
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

constexpr size_t kSmallCells = 4096;

// One V(1,1) cycle on level l: xout = M(l) b, zero initial guess.  Levels of
// at most kSmallCells cells run as one single-block kernel.
template <typename T>
int vcycle(EcsCtx *ctx, size_t l, const T *b, T *xout) {
  Multigrid<T> &mg = mg_of<T>(ctx);
  MgLevel<T> &L = mg.lv[l];
  int rc;
  if (L.n <= kSmallCells && mg.lv.size() - l <= (size_t)kMaxSmall) {
    SmallCycle<T> sc;
    sc.nl = (int)(mg.lv.size() - l);
    for (int q = 0; q < sc.nl; q++) {
      MgLevel<T> &M = mg.lv[l + q];
      sc.lv[q].o = op_level(ctx, M);
      sc.lv[q].dens = M.dens; sc.lv[q].x = M.x; sc.lv[q].b = M.b; sc.lv[q].r = M.r; sc.lv[q].t = M.t;
      sc.lv[q].z = zl_of(M);
    }
    k_vcycle_small<T><<<1, 512, 0, ctx->stream>>>(sc, b, xout, kCoarseSweeps, kOmega<T>());
    ECS_LAUNCHED(ctx);
    return ECS_OK;
  }
  if (l + 1 == mg.lv.size()) {
    if ((rc = sweep<T>(ctx, L, b, nullptr, xout))) return rc;
    for (int s = 0; s < (kCoarseSweeps - 1) / 2; s++) {
      if ((rc = sweep<T>(ctx, L, b, xout, L.t))) return rc;
      if ((rc = sweep<T>(ctx, L, b, L.t, xout))) return rc;
    }
    return ECS_OK;
  }
  MgLevel<T> &C = mg.lv[l + 1];
  if ((rc = sweep<T>(ctx, L, b, nullptr, L.t))) return rc;
  k_apply<T><<<blocks_for(ctx, L.n), kB, 0, ctx->stream>>>(op_level(ctx, L), L.dens, L.t, b, L.r, 1);
  ECS_LAUNCHED(ctx);
  k_restrict<T><<<blocks_for(ctx, C.n), kB, 0, ctx->stream>>>(grid_of(ctx, L.nx, L.ny, L.nz),
                                                            grid_of(ctx, C.nx, C.ny, C.nz), L.r, C.b);
  ECS_LAUNCHED(ctx);
  if ((rc = vcycle<T>(ctx, l + 1, C.b, C.x))) return rc;
  k_prolong_add<T><<<blocks_for(ctx, L.n), kB, 0, ctx->stream>>>(grid_of(ctx, L.nx, L.ny, L.nz),
                                                               grid_of(ctx, C.nx, C.ny, C.nz), C.x, L.t);
  ECS_LAUNCHED(ctx);
  return sweep<T>(ctx, L, b, L.t, xout);
}

// Dot products of w with V_0..V_{nv-1} (and w.w), FP64 accumulation, copied
// to the host (ctx->h_dots).
template <typename T>
int mdot(EcsCtx *ctx, const T *V, int nv, const T *w, int with_ww) {
  size_t n = ctx->ncell;
  unsigned int nb = std::min(blocks_for(ctx, n), 1024u);
  int nslot = nv + (with_ww ? 1 : 0);
  size_t shm = (size_t)(kB / 32) * nslot * sizeof(double);
  k_mdot_partial<T><<<nb, kB, shm, ctx->stream>>>(n, nv, V, n, w, with_ww, ctx->red);
  ECS_LAUNCHED(ctx);
  k_mdot_final<<<nslot, 256, 0, ctx->stream>>>(nslot, (int)nb, ctx->red, ctx->dots);
  ECS_LAUNCHED(ctx);
  ECS_CUDA(ctx, cudaMemcpyAsync(ctx->h_dots, ctx->dots, nslot * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return ECS_OK;
}

template <typename T>
int project_mean(EcsCtx *ctx, T *v) {
  if (!fully_periodic(ctx)) return ECS_OK;
  size_t n = ctx->ncell;
  unsigned int nb = std::min(blocks_for(ctx, n), 1024u);
  k_sum_partial<T><<<nb, kB, 0, ctx->stream>>>(n, v, ctx->red);
  ECS_LAUNCHED(ctx);
  k_mdot_final<<<1, 256, 0, ctx->stream>>>(1, (int)nb, ctx->red, ctx->dots);
  ECS_LAUNCHED(ctx);
  k_shift<T><<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(n, v, ctx->dots, 1.0 / (double)n);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

template <typename T>
T *basis_v(EcsCtx *ctx);
template <>
double *basis_v<double>(EcsCtx *ctx) { return ctx->kv64; }
template <>
float *basis_v<float>(EcsCtx *ctx) { return ctx->kv32; }
template <typename T>
T *basis_z(EcsCtx *ctx);
template <>
double *basis_z<double>(EcsCtx *ctx) { return ctx->kz64; }
template <>
float *basis_z<float>(EcsCtx *ctx) { return ctx->kz32; }

// FGMRES(m) for A x = b in precision T, x from zero, one cycle of at most
// min(m, maxit) iterations; stops when the estimated residual falls below
// tol*||b||.  Returns the estimate in *est and the iteration count in *its.
template <typename T>
int fgmres(EcsCtx *ctx, const T *b, T *x, double tol, int maxit, int *its, double *est) {
  const size_t n = ctx->ncell;
  const int m = std::min(ctx->krylov_m, std::max(maxit, 1));
  Multigrid<T> &mg = mg_of<T>(ctx);
  MgLevel<T> &L0 = mg.lv[0];
  const OpK o0 = op_level(ctx, L0);
  T *V = basis_v<T>(ctx), *Z = basis_z<T>(ctx);
  int rc;
  *its = 0;
  k_fill<T><<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(n, x, T(0));
  ECS_LAUNCHED(ctx);
  if ((rc = mdot<T>(ctx, b, 1, b, 0))) return rc;
  const double beta = sqrt(ctx->h_dots[0]);
  if (!(beta > 0.0)) {
    *est = 0.0;
    return ECS_OK;
  }
  k_scale_copy<T, T><<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(n, b, V, 1.0 / beta);
  ECS_LAUNCHED(ctx);
  std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0), h1(m + 1), h2(m + 2);
  g[0] = beta;
  int j = 0;
  double res = beta;
  for (; j < m; j++) {
    T *vj = V + (size_t)j * n, *zj = Z + (size_t)j * n, *w = V + (size_t)(j + 1) * n;
    if ((rc = vcycle<T>(ctx, 0, vj, zj))) return rc;
    if ((rc = project_mean<T>(ctx, zj))) return rc;
    k_apply<T><<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(o0, L0.dens, zj, nullptr, w, 0);
    ECS_LAUNCHED(ctx);
    // classical Gram-Schmidt, two passes
    if ((rc = mdot<T>(ctx, V, j + 1, w, 0))) return rc;
    for (int q = 0; q <= j; q++) h1[q] = ctx->h_dots[q];
    ECS_CUDA(ctx, cudaMemcpyAsync(ctx->dots, h1.data(), (j + 1) * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    k_maxpy<T><<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(n, j + 1, ctx->dots, V, n, w);
    ECS_LAUNCHED(ctx);
    if ((rc = mdot<T>(ctx, V, j + 1, w, 1))) return rc;
    double ss = 0.0;
    for (int q = 0; q <= j; q++) {
      h2[q] = ctx->h_dots[q];
      ss += h2[q] * h2[q];
    }
    double ww = ctx->h_dots[j + 1];
    ECS_CUDA(ctx, cudaMemcpyAsync(ctx->dots, h2.data(), (j + 1) * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    k_maxpy<T><<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(n, j + 1, ctx->dots, V, n, w);
    ECS_LAUNCHED(ctx);
    double hn = sqrt(std::max(ww - ss, 0.0));
    for (int q = 0; q <= j; q++) H[(size_t)q * m + j] = h1[q] + h2[q];
    H[(size_t)(j + 1) * m + j] = hn;
    if (hn > 0) {
      k_scale_copy<T, T><<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(n, w, w, 1.0 / hn);
      ECS_LAUNCHED(ctx);
    }
    for (int q = 0; q < j; q++) {
      double a = H[(size_t)q * m + j], c = H[(size_t)(q + 1) * m + j];
      H[(size_t)q * m + j] = cs[q] * a + sn[q] * c;
      H[(size_t)(q + 1) * m + j] = -sn[q] * a + cs[q] * c;
    }
    double a = H[(size_t)j * m + j], c = H[(size_t)(j + 1) * m + j];
    double r = sqrt(a * a + c * c);
    cs[j] = r > 0 ? a / r : 1.0;
    sn[j] = r > 0 ? c / r : 0.0;
    H[(size_t)j * m + j] = r;
    H[(size_t)(j + 1) * m + j] = 0.0;
    g[j + 1] = -sn[j] * g[j];
    g[j] = cs[j] * g[j];
    res = fabs(g[j + 1]);
    if (res <= tol * beta || hn == 0.0 || j + 1 >= maxit) {
      j++;
      break;
    }
  }
  std::vector<double> y(j, 0.0);
  for (int q = j - 1; q >= 0; q--) {
    double s = g[q];
    for (int r2 = q + 1; r2 < j; r2++) s -= H[(size_t)q * m + r2] * y[r2];
    y[q] = s / H[(size_t)q * m + q];
  }
  ECS_CUDA(ctx, cudaMemcpyAsync(ctx->dots, y.data(), j * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  k_combine<T><<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(n, j, ctx->dots, Z, n, x);
  ECS_LAUNCHED(ctx);
  *its = j;
  *est = res / beta;
  return ECS_OK;
}

// ||v||_2 of an FP64 vector
int norm64(EcsCtx *ctx, const double *v, double *out) {
  int rc = mdot<double>(ctx, v, 1, v, 0);
  if (rc) return rc;
  *out = sqrt(ctx->h_dots[0]);
  return ECS_OK;
}

int alloc_krylov(EcsCtx *ctx) {
  size_t n = ctx->ncell;
  int m = ctx->krylov_m;
  if (!ctx->red) {
    ctx->nred = (m + 2) * 1024;
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->red, (size_t)ctx->nred * sizeof(double)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->dots, (size_t)(m + 2) * sizeof(double)));
    ECS_CUDA(ctx, cudaMallocHost((void **)&ctx->h_dots, (size_t)(m + 2) * sizeof(double)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->r64, n * sizeof(double)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->w64, n * sizeof(double)));
  }
  if (ctx->prec == ECS_PREC_FP64 && !ctx->kv64) {
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->kv64, (size_t)(m + 1) * n * sizeof(double)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->kz64, (size_t)m * n * sizeof(double)));
  }
  if (ctx->prec == ECS_PREC_MIXED && !ctx->kv32) {
    // V, Z and two extra FP32 vectors (normalised residual, correction)
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->kv32, (size_t)(m + 1) * n * sizeof(float)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->kz32, (size_t)(m + 2) * n * sizeof(float)));
  }
  return ECS_OK;
}

}  // namespace

// ============================================================================
// entry points used by ecs_api.cu
// ============================================================================
int ecs_grid_eext(EcsCtx *ctx) {
  GridG g = grid_of(ctx, ctx->p.Nx, ctx->p.Ny, ctx->p.Nz);
  k_eext<<<blocks_for(ctx, ctx->next), kB, 0, ctx->stream>>>(g, ctx->phi, ctx->prec == ECS_PREC_FP64 ? ctx->eext64 : nullptr,
                                                           ctx->prec == ECS_PREC_MIXED ? ctx->eext32 : nullptr);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

int ecs_grid_clear_acc(EcsCtx *ctx) {
  ECS_CUDA(ctx, cudaMemsetAsync(ctx->acc, 0, ctx->ncell * 4 * sizeof(long long), ctx->stream));
  return ECS_OK;
}

int ecs_grid_moments(EcsCtx *ctx) {
  k_moments<<<blocks_for(ctx, ctx->ncell * 4), kB, 0, ctx->stream>>>(ctx->ncell, ctx->acc, ctx->mom,
                                                                    ldexp(1.0, -ctx->shift_n),
                                                                    ldexp(1.0, -ctx->shift_f), ctx->dstat);
  ECS_LAUNCHED(ctx);
  ctx->moments_ready = true;
  return ECS_OK;
}

int ecs_grid_rhs(EcsCtx *ctx) {
  int rc = alloc_krylov(ctx);
  if (rc) return rc;
  const EcsParams &p = ctx->p;
  GridG g = grid_of(ctx, p.Nx, p.Ny, p.Nz);
  RhsK r;
  r.kappa = p.kappa_e;
  r.hx = 1.0 / (2.0 * p.dx); r.hy = 1.0 / (2.0 * p.dy); r.hz = 1.0 / (2.0 * p.dz);
  r.hxx = 1.0 / (p.dx * p.dx); r.hyy = 1.0 / (p.dy * p.dy); r.hzz = 1.0 / (p.dz * p.dz);
  r.E0 = p.E0; r.cth = p.cth; r.cG = p.cG; r.scale = p.scale;
  unsigned int nb = std::min(blocks_for(ctx, ctx->ncell), 1024u);
  k_rhs<<<nb, kB, 0, ctx->stream>>>(g, r, ctx->mom, ctx->rhs, ctx->red);
  ECS_LAUNCHED(ctx);
  k_sub_mean<<<blocks_for(ctx, ctx->ncell), kB, 0, ctx->stream>>>(ctx->ncell, ctx->rhs, ctx->red, (int)nb);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

int ecs_solver_setup(EcsCtx *ctx) {
  int rc = alloc_krylov(ctx);
  if (rc) return rc;
  rc = ctx->prec == ECS_PREC_FP64 ? mg_setup<double>(ctx) : mg_setup<float>(ctx);
  if (rc) return rc;
  ctx->lhs_ready = true;
  return ECS_OK;
}

int ecs_solver_run(EcsCtx *ctx, double rtol, int max_it, int warm, EcsSolveStats *st) {
  if (!ctx->lhs_ready) return ecs_fail(ctx, ECS_ERR_STATE, "solve called before lhs");
  const size_t n = ctx->ncell;
  const EcsParams &p = ctx->p;
  const OpK o64 = op_of(ctx, p.Nx, p.Ny, p.Nz, p.dx, p.dy, p.dz);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, ctx->stream);
  int rc;
  if (!warm) ECS_CUDA(ctx, cudaMemsetAsync(ctx->phi, 0, n * sizeof(double), ctx->stream));
  double bnorm;
  if ((rc = norm64(ctx, ctx->rhs, &bnorm))) return rc;
  int its = 0, sweeps = 0;
  double rel = 0.0;
  if (bnorm > 0.0) {
    for (;;) {
      k_residual64<<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(o64, ctx->mom, ctx->phi, ctx->rhs, ctx->r64);
      ECS_LAUNCHED(ctx);
      double rn;
      if ((rc = norm64(ctx, ctx->r64, &rn))) return rc;
      rel = rn / bnorm;
      if (!isfinite(rel)) return ecs_fail(ctx, ECS_ERR_NONFINITE, "non-finite residual in solve");
      if (rel <= rtol || its >= max_it) break;
      int k = 0;
      double est = 0.0;
      double tol_cycle = std::max(0.5 * rtol / rel, 1e-14);
      if (ctx->prec == ECS_PREC_FP64) {
        if ((rc = fgmres<double>(ctx, ctx->r64, ctx->w64, tol_cycle, max_it - its, &k, &est))) return rc;
        k_axpy64<double><<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(n, 1.0, ctx->w64, ctx->phi);
      } else {
        float *r32 = ctx->kz32 + (size_t)ctx->krylov_m * n, *e32 = r32 + n;
        k_scale_copy<double, float><<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(n, ctx->r64, r32, 1.0 / rn);
        ECS_LAUNCHED(ctx);
        double tol32 = std::max(tol_cycle, 2e-6);
        if ((rc = fgmres<float>(ctx, r32, e32, tol32, max_it - its, &k, &est))) return rc;
        k_axpy64<float><<<blocks_for(ctx, n), kB, 0, ctx->stream>>>(n, rn, e32, ctx->phi);
      }
      ECS_LAUNCHED(ctx);
      if ((rc = project_mean<double>(ctx, ctx->phi))) return rc;
      its += k;
      sweeps++;
      if (k == 0) break;
    }
  }
  cudaEventRecord(e1, ctx->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) {
    st->iterations = its;
    st->refinements = sweeps;
    st->relres = rel;
    st->seconds = ms * 1e-3;
  }
  if (bnorm > 0.0 && rel > rtol) return ecs_fail(ctx, ECS_ERR_NOT_CONVERGED, "solve stopped at relres %.3e > %.3e after %d iterations", rel, rtol, its);
  return ECS_OK;
}

int ecs_operator_apply64(EcsCtx *ctx, const double *x, double *y) {
  const EcsParams &p = ctx->p;
  const OpK o64 = op_of(ctx, p.Nx, p.Ny, p.Nz, p.dx, p.dy, p.dz);
  k_apply<double><<<blocks_for(ctx, ctx->ncell), kB, 0, ctx->stream>>>(o64, ctx->mom, x, nullptr, y, 0);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

template <typename T>
static void free_mg(Multigrid<T> &mg) {
  for (auto &L : mg.lv) {
    T *arr[] = {L.dens, L.x, L.b, L.r, L.t, L.zl_a, L.zl_cp, L.zl_minv, L.zl_q, L.zl_dp, L.zl_a0g, L.zl_qden};
    for (T *a : arr)
      if (a) cudaFree(a);
  }
  mg.lv.clear();
  mg.built = false;
}

int ecs_solver_free(EcsCtx *ctx) {
  free_mg(ctx->mg64);
  free_mg(ctx->mg32);
  void *ptrs[] = {ctx->kv64, ctx->kz64, ctx->kv32, ctx->kz32, ctx->w64, ctx->r64, ctx->dots, ctx->red};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  if (ctx->h_dots) cudaFreeHost(ctx->h_dots);
  return ECS_OK;
}
