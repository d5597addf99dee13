// Potential solve of the ECSPRT hot path on sm_103a: the matrix-free
// 11-point operator of src/lhs.c:337-505 and the KSP solve of
// src/potential.c:6-15.
//
// FGMRES(m) preconditioned by one geometric-multigrid V(1,1) cycle (full
// coarsening, full-weighting restriction, trilinear prolongation, coarse
// operators rediscretised from the full-weighted density, damped z-line
// Jacobi smoothing: the z couplings carry (1+kappa^2) and dominate).
//   ECS_PREC_FP64:  FGMRES and multigrid in FP64 to the requested rtol.
//   ECS_PREC_MIXED: FP64 iterative refinement; each correction is an FP32
//     FGMRES/multigrid solve; residuals, their norms, the update of phi and
//     the mean projection are FP64.
//
// One FGMRES cycle runs entirely on the device: the Gram-Schmidt
// coefficients, the Hessenberg matrix, the Givens rotations and the
// convergence test live in a device control block (KrylovDev), and the
// kernels that need the Arnoldi index read it from there.  The cycle is a
// CUDA graph whose Arnoldi step is the body of a conditional WHILE node; the
// step's last small kernel clears the condition once the residual estimate
// meets the tolerance, so the host waits once per cycle.  Without graphs the
// host launches the same kernels step by step and reads the stop flag after
// each step.
//
// All reductions use fixed block partials summed in a fixed order, so every
// result is reproducible run to run.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "ecs_stencil.cuh"

namespace {

constexpr int kKrylovMax = 30;            // restart length m (upper bound)
constexpr int kSlots = kKrylovMax + 2;    // dot-product slots per pass
constexpr int kDotBlocks = 1024;          // block partials per dot pass
constexpr int kB = 256;

// Device control block of one FGMRES cycle.
struct KrylovDev {
  // set by the host before a cycle
  double tol_rel;  // stop when the estimate <= tol_rel * beta
  int maxit;       // Arnoldi steps allowed in this cycle (<= kKrylovMax)
  int pad0;
  // cycle state
  int j;           // current Arnoldi index
  int jprev;       // index of the step that just finished
  int done;        // 1: converged, broke down or out of steps
  int nits;        // Arnoldi steps taken
  double beta, res, inv_scale, mean;
  double h1[kSlots], h2[kSlots];
  double H[(kKrylovMax + 1) * kKrylovMax];
  double cs[kKrylovMax], sn[kKrylovMax], g[kKrylovMax + 1], y[kKrylovMax];
  // completion tickets of the grid-wide reductions (0 between launches)
  unsigned int ticket[8];
};

// ---- operator ------------------------------------------------------------------
// y = A x   (mode 0)     or     y = b - A x   (mode 1)
template <typename T>
__global__ void k_apply(OpK o, const T *__restrict__ n, const T *__restrict__ x, const T *__restrict__ b,
                        T *__restrict__ y, int mode) {
  ECS_PDL_ENTRY();
  int i, j, k;
  if (!at3(o.g.nx, o.g.ny, i, j, k)) return;
  const Nbr q = nbr_of(o.g, i, j, k);
  T v[11], xe[11];
  row11_n(n, o, q, v);
  row_x(x, q, xe);
  T s = T(0);
#pragma unroll
  for (int e = 0; e < 11; e++) s += v[e] * xe[e];
  y[q.c] = mode ? b[q.c] - s : s;
}

// ---- z-line smoother --------------------------------------------------------------
// Column (i,j) carries the z-tridiagonal part of the rows: lo = z- entry,
// diag = centre, up = z+ entry.  A periodic z closes the cycle, solved with
// Sherman-Morrison around the Thomas factorisation of the modified matrix;
// reflecting z drops the out-of-range couplings (Dirichlet-0 ghosts).
// The solve runs in segments of S cells along z, one thread per segment; the
// forward recurrence d_k = (r_k - a_k d_{k-1}) / m_k and the backward one
// y_k = d_k - cp_k y_{k+1} are affine in the value carried in, so each
// segment solves from zero and the carried values are stitched afterwards
// with the in-segment products fb_k = prod(-a_i/m_i) and bb_k = prod(-cp_i).
template <typename T>
struct ZlP {
  T *a, *cp, *minv, *q, *fb, *bb;  // per cell
  T *a0g, *qden;                   // per column
};
// At most 16 segments a column (block of 32 x 16 threads); segments of 8,
// 16, 32 or 64 cells, the shortest that fits.
constexpr int kMaxSeg = 16;
template <typename T>
static inline int seg_len(int N) {
  for (int S = 8; S < 64; S *= 2)
    if (N <= S * kMaxSeg) return S;
  return 64;
}

// The z entries of every row (lower, upper, diagonal), one thread per cell:
// the parallel half of the z-line set-up.
template <typename T>
__global__ void k_zline_rows(OpK o, const T *__restrict__ n, T *__restrict__ lo, T *__restrict__ up,
                             T *__restrict__ dg) {
  ECS_PDL_ENTRY();
  int i, j, k;
  if (!at3(o.g.nx, o.g.ny, i, j, k)) return;
  const Nbr q = nbr_of(o.g, i, j, k);
  T v[11];
  row11_n(n, o, q, v);
  const unsigned c = q.c;
  lo[c] = v[5];
  up[c] = v[4];
  dg[c] = v[10];
}

// Factorisation of every column's z tridiagonal (one thread a column) from
// the rows of k_zline_rows.
template <typename T>
__global__ void k_zline_setup(GridG g, const T *__restrict__ lo, const T *__restrict__ up,
                              const T *__restrict__ dg, ZlP<T> z, int S) {
  ECS_PDL_ENTRY();
  const int ncol = g.nx * g.ny;
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const size_t plane = (size_t)g.nx * g.ny;
  // a one-cell column (2-D) has no z coupling: the plain solve, no periodic closure
  const bool cyc = g.bc[2] == 0 && g.nz > 1;
  const int N = g.nz;
  const T lo0 = cyc ? __ldg(&lo[col]) : T(0), d0 = __ldg(&dg[col]);
  const T gamma = -d0;
  T cp_prev = T(0), dq_prev = T(0), fprod = T(1);
  // forward: factor T' and forward-substitute u = (gamma, 0, .., up_{N-1});
  // the rows are read kBatch at a time, all loads first, so the recurrence
  // waits on one memory latency a batch rather than one a cell
  constexpr int kBatch = 8;
  for (int k0 = 0; k0 < N; k0 += kBatch) {
    T lv[kBatch], uv[kBatch], dv[kBatch];
#pragma unroll
    for (int e = 0; e < kBatch; e++) {
      const size_t c = (size_t)min(k0 + e, N - 1) * plane + col;
      lv[e] = __ldg(&lo[c]);
      uv[e] = __ldg(&up[c]);
      dv[e] = __ldg(&dg[c]);
    }
#pragma unroll
    for (int e = 0; e < kBatch; e++) {
      const int k = k0 + e;
      if (k >= N) break;
      const size_t c = (size_t)k * plane + col;
      const T lk = lv[e], uk = uv[e], dk = dv[e];
      T a = (k == 0) ? T(0) : lk;
      T upk = (k == N - 1) ? T(0) : uk;
      T bb = dk;
      if (cyc && k == 0) bb = d0 - gamma;
      if (cyc && k == N - 1) bb = dk - uk * lo0 / gamma;
      T m = bb - a * cp_prev;
      T minv = T(1) / m;
      T cp = upk * minv;
      T u = cyc ? ((k == 0) ? gamma : ((k == N - 1) ? uk : T(0))) : T(0);
      T dq = (u - a * dq_prev) * minv;
      z.a[c] = a;
      z.cp[c] = cp;
      z.minv[c] = minv;
      z.q[c] = dq;
      if (k % S == 0) fprod = T(1);
      fprod *= -(a * minv);
      z.fb[c] = fprod;
      cp_prev = cp;
      dq_prev = dq;
    }
  }
  // backward substitution for q, in-segment products of -cp (this thread's
  // own values from above, read back a batch at a time)
  T qn = z.q[(size_t)(N - 1) * plane + col];
  T bprod = -z.cp[(size_t)(N - 1) * plane + col];
  z.bb[(size_t)(N - 1) * plane + col] = bprod;
  for (int k0 = N - 2; k0 >= 0; k0 -= kBatch) {
    T qv[kBatch], cv[kBatch];
#pragma unroll
    for (int e = 0; e < kBatch; e++) {
      const size_t c = (size_t)max(k0 - e, 0) * plane + col;
      qv[e] = z.q[c];
      cv[e] = z.cp[c];
    }
#pragma unroll
    for (int e = 0; e < kBatch; e++) {
      const int k = k0 - e;
      if (k < 0) break;
      const size_t c = (size_t)k * plane + col;
      qn = qv[e] - cv[e] * qn;
      z.q[c] = qn;
      if ((k + 1) % S == 0) bprod = T(1);
      bprod *= -cv[e];
      z.bb[c] = bprod;
    }
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

// Right-hand side of the z-line systems: r = b - A_xy xo.
template <typename T>
__global__ void k_zline_rhs(OpK o, const T *__restrict__ n, const T *__restrict__ b, const T *__restrict__ xo,
                            T *__restrict__ r) {
  ECS_PDL_ENTRY();
  int i, j, k;
  if (!at3(o.g.nx, o.g.ny, i, j, k)) return;
  const Nbr q = nbr_of(o.g, i, j, k);
  T v[11], xe[11];
  row11_n(n, o, q, v);
  row_x(xo, q, xe);
  T s = b[q.c];
#pragma unroll
  for (int e = 0; e < 10; e++) {
    if (e == 4 || e == 5) continue;
    s -= v[e] * xe[e];
  }
  r[q.c] = s;
}

// Damped z-line Jacobi update: T' y = r by segments, Sherman-Morrison
// closure of the periodic cycle, xn = xo + omega (y - s q - xo) (xo nullptr:
// zero).  Block = 32 columns (consecutive x at one y) x P segments of S
// cells; each phase loads its segment's operands at once so that one memory
// latency covers the whole segment.
template <typename T, int S>
__global__ void __launch_bounds__(32 * kMaxSeg) k_zline_seg(GridG g, ZlP<T> z, const T *__restrict__ r,
                                                            const T *__restrict__ xo, T *__restrict__ xn,
                                                            T omega) {
  ECS_PDL_ENTRY();
  __shared__ T sA[kMaxSeg][33], sB[kMaxSeg][33], sIn[kMaxSeg][33];
  __shared__ T sLast[32], sS[32];
  const int tx = threadIdx.x, p = threadIdx.y, P = blockDim.y;
  const int i = blockIdx.x * 32 + tx, j = blockIdx.y;
  const bool act = i < g.nx;
  const size_t plane = (size_t)g.nx * g.ny;
  const int col = j * g.nx + i;
  const int N = g.nz, k0 = p * S, k1 = min(N, k0 + S);
  const size_t c0 = (size_t)k0 * plane + col;
  auto in = [&](int q) { return act && k0 + q < k1; };
  T loc[S];
  // forward, from zero at the segment start
  {
    T rv[S], av[S], mv[S];
#pragma unroll
    for (int q = 0; q < S; q++) {
      const size_t c = c0 + (size_t)q * plane;
      rv[q] = in(q) ? r[c] : T(0);
      av[q] = in(q) ? z.a[c] : T(0);
      mv[q] = in(q) ? z.minv[c] : T(0);
    }
    T d = T(0);
#pragma unroll
    for (int q = 0; q < S; q++) {
      if (in(q)) d = (rv[q] - av[q] * d) * mv[q];
      loc[q] = d;
    }
    sA[p][tx] = d;
    sB[p][tx] = act ? z.fb[(size_t)(k1 - 1) * plane + col] : T(0);
  }
  __syncthreads();
  if (p == 0) {
    T din = T(0);
    for (int pp = 0; pp < P; pp++) {
      sIn[pp][tx] = din;
      din = sA[pp][tx] + sB[pp][tx] * din;
    }
  }
  __syncthreads();
  // carried value in, then backward from zero at the segment end
  {
    const T din = sIn[p][tx];
    T fv[S], cv[S];
#pragma unroll
    for (int q = 0; q < S; q++) {
      const size_t c = c0 + (size_t)q * plane;
      fv[q] = in(q) ? z.fb[c] : T(0);
      cv[q] = in(q) ? z.cp[c] : T(0);
    }
    T y = T(0);
#pragma unroll
    for (int q = S - 1; q >= 0; q--) {
      if (in(q)) y = (loc[q] + fv[q] * din) - cv[q] * y;
      loc[q] = y;
    }
    // sA, sB are free again: the forward scan finished before the last barrier
    sA[p][tx] = y;
    sB[p][tx] = act ? z.bb[c0] : T(0);
    if (p == P - 1) {  // y_{N-1}: nothing is carried into the last segment
#pragma unroll
      for (int q = 0; q < S; q++)
        if (k0 + q == N - 1) sLast[tx] = loc[q];
    }
  }
  __syncthreads();
  if (p == 0) {
    T yin = T(0);
    for (int pp = P - 1; pp >= 0; pp--) {
      sIn[pp][tx] = yin;
      yin = sA[pp][tx] + sB[pp][tx] * yin;
    }
    sS[tx] = act ? (yin + z.a0g[col] * sLast[tx]) * z.qden[col] : T(0);  // yin = y_0
  }
  __syncthreads();
  {
    const T yin = sIn[p][tx], s = sS[tx];
    T bv[S], qv[S], ov[S];
#pragma unroll
    for (int q = 0; q < S; q++) {
      const size_t c = c0 + (size_t)q * plane;
      bv[q] = in(q) ? z.bb[c] : T(0);
      qv[q] = in(q) ? z.q[c] : T(0);
      ov[q] = (in(q) && xo) ? xo[c] : T(0);
    }
#pragma unroll
    for (int q = 0; q < S; q++) {
      if (in(q)) {
        const T yk = loc[q] + bv[q] * yin;
        xn[c0 + (size_t)q * plane] = ov[q] + omega * ((yk - s * qv[q]) - ov[q]);
      }
    }
  }
}

// ---- inter-grid transfer ---------------------------------------------------------
// A level of more than one plane whose coarser level has as many planes is
// coarsened in x and y only (reflecting z, see mg_alloc): its transfers act
// within each plane.
__device__ __forceinline__ bool semi_z(const GridG &gf, const GridG &gc) { return gf.nz == gc.nz && gf.nz > 1; }

// Full weighting (1/4,1/2,1/4 per coarsened axis) from fine (2I+a) to coarse
// I: the 27 (9 when z is not coarsened) fine cells through the neighbour
// offsets of the fine cell (2I, 2J, 2K) (or (2I, 2J, K)).
template <typename T>
__global__ void k_restrict(GridG gf, GridG gc, const T *__restrict__ f, T *__restrict__ c) {
  ECS_PDL_ENTRY();
  int I, J, K;
  if (!at3(gc.nx, gc.ny, I, J, K)) return;
  const bool semi = semi_z(gf, gc);
  const Nbr q = nbr_of(gf, 2 * I, 2 * J, semi ? K : 2 * K);
  const int oz[3] = {q.zm, 0, q.zp}, oy[3] = {q.ym, 0, q.yp}, ox[3] = {q.xm, 0, q.xp};
  const bool vz[3] = {q.vzm, true, q.vzp}, vy[3] = {q.vym, true, q.vyp}, vx[3] = {q.vxm, true, q.vxp};
  T s = T(0);
#pragma unroll
  for (int dk = 0; dk < 3; dk++) {
    if (semi && dk != 1) continue;
    const T wk = semi ? T(1) : (dk == 1 ? T(0.5) : T(0.25));
#pragma unroll
    for (int dj = 0; dj < 3; dj++) {
      const T wj = dj == 1 ? T(0.5) : T(0.25);
#pragma unroll
      for (int di = 0; di < 3; di++) {
        const T wi = di == 1 ? T(0.5) : T(0.25);
        s += wk * wj * wi * nval(f, q, oz[dk] + oy[dj] + ox[di], vz[dk] && vy[dj] && vx[di]);
      }
    }
  }
  c[lin3(gc, I, J, K)] = s;
}

// The same full-weighting sum with the loops kept rolled (less code, for the
// single-block cycle); the terms are added in the same order as k_restrict.
template <typename T>
__device__ __forceinline__ T restrict_at_rolled(const GridG &gf, const GridG &gc, const T *__restrict__ f, int I,
                                                int J, int K) {
  const bool semi = semi_z(gf, gc);
  const int zl = semi ? 0 : -1, zc = semi ? K : 2 * K;
  T s = T(0);
#pragma unroll 1
  for (int dk = zl; dk <= -zl; dk++) {
    const T wk = semi ? T(1) : (dk == 0 ? T(0.5) : T(0.25));
#pragma unroll 1
    for (int dj = -1; dj <= 1; dj++) {
      const T wj = dj == 0 ? T(0.5) : T(0.25);
#pragma unroll 1
      for (int di = -1; di <= 1; di++) {
        const T wi = di == 0 ? T(0.5) : T(0.25);
        s += wk * wj * wi * gval(f, gf, zc + dk, 2 * J + dj, 2 * I + di);
      }
    }
  }
  return s;
}

// Trilinear prolongation value at fine cell (i,j,k).
template <typename T>
__device__ __forceinline__ T prolong_at(const GridG &gf, const GridG &gc, const T *__restrict__ c, int i, int j,
                                        int k) {
  const bool semi = semi_z(gf, gc);
  int i0 = i >> 1, j0 = j >> 1, k0 = semi ? k : k >> 1;
  int ni = (i & 1) ? 2 : 1, nj = (j & 1) ? 2 : 1, nk = (!semi && (k & 1)) ? 2 : 1;
  T wi = ni == 2 ? T(0.5) : T(1), wj = nj == 2 ? T(0.5) : T(1), wk = nk == 2 ? T(0.5) : T(1);
  T s = T(0);
  for (int a = 0; a < nk; a++)
    for (int bq = 0; bq < nj; bq++)
      for (int q = 0; q < ni; q++) s += gval(c, gc, k0 + a, j0 + bq, i0 + q);
  return wi * wj * wk * s;
}
// f += P c.
// The kernel's form: the coarse cells through the neighbour offsets of the
// coarse cell (i/2, j/2, k/2); a term of the second cell along an axis is
// added only for an odd index, in the order of prolong_at.
template <typename T>
__global__ void k_prolong_add(GridG gf, GridG gc, const T *__restrict__ c, T *__restrict__ f) {
  ECS_PDL_ENTRY();
  int i, j, k;
  if (!at3(gf.nx, gf.ny, i, j, k)) return;
  const bool semi = semi_z(gf, gc);
  const Nbr q = nbr_of(gc, i >> 1, j >> 1, semi ? k : k >> 1);
  const bool ti = i & 1, tj = j & 1, tk = !semi && (k & 1);
  const T wi = ti ? T(0.5) : T(1), wj = tj ? T(0.5) : T(1), wk = tk ? T(0.5) : T(1);
  T s = T(0);
#pragma unroll
  for (int a = 0; a < 2; a++) {
    if (a == 1 && !tk) break;
    const int oz = a ? q.zp : 0;
    const bool vz = a ? q.vzp : true;
#pragma unroll
    for (int bq = 0; bq < 2; bq++) {
      if (bq == 1 && !tj) break;
      const int oy = bq ? q.yp : 0;
      const bool vy = bq ? q.vyp : true;
#pragma unroll
      for (int e = 0; e < 2; e++) {
        if (e == 1 && !ti) break;
        s += nval(c, q, oz + oy + (e ? q.xp : 0), vz && vy && (e ? q.vxp : true));
      }
    }
  }
  f[lin3(gf, i, j, k)] += wi * wj * wk * s;
}

// ---- whole V-cycle of the small levels in one thread block -------------------
// The iterate, right-hand side, residual and scratch vectors of every small
// level live in shared memory (s* are element offsets into it); the density
// and the z-line factors are read-only and come through the L1 cache.
template <typename T>
struct SmallLevel {
  OpK o;
  const T *dens;   // in global memory, staged at sd
  ZlP<T> z;        // in global memory, staged at sa, sc, sm, sq (cells) and s0, sqd (columns)
  int sx, sb, sr, st;
  int sd, sa, sc, sm, sq, s0, sqd;
};
constexpr int kMaxSmall = 8;
template <typename T>
struct SmallCycle {
  int nl;
  const T *cinv;  // transposed inverse of the coarsest operator, or nullptr; staged at scinv
  int scinv;
  SmallLevel<T> lv[kMaxSmall];
};
constexpr int kSmallThreads = 1024;

// Thomas solve of one column with all vectors in shared memory: rin (right-
// hand side) may be the same array as dp (the substitution scratch).
// One column's z-line solve with the factors staged in shared memory.
template <typename T>
__device__ __forceinline__ void zline_col_s(const GridG &g, const ZlP<T> &z, const T *rin, T *dp,
                                            const T *xo, T *xn, T omega, int col) {
  const int plane = g.nx * g.ny, N = g.nz;
  T d = T(0);
  for (int k = 0; k < N; k++) {
    const int c = k * plane + col;
    d = (rin[c] - z.a[c] * d) * z.minv[c];
    dp[c] = d;
  }
  const T yN = d;
  T y = d;
  for (int k = N - 2; k >= 0; k--) {
    const int c = k * plane + col;
    y = dp[c] - z.cp[c] * y;
    dp[c] = y;
  }
  const T s = (y + z.a0g[col] * yN) * z.qden[col];
  for (int k = 0; k < N; k++) {
    const int c = k * plane + col;
    const T ov = xo ? xo[c] : T(0);
    xn[c] = ov + omega * ((dp[c] - s * z.q[c]) - ov);
  }
}

// A small level's density and z-line factors as staged in shared memory.
template <typename T>
struct SmallView {
  const T *dens;
  ZlP<T> z;
};
template <typename T>
__device__ __forceinline__ SmallView<T> staged(const SmallLevel<T> &L, T *sm) {
  SmallView<T> v;
  v.dens = sm + L.sd;
  v.z = L.z;
  v.z.a = sm + L.sa; v.z.cp = sm + L.sc; v.z.minv = sm + L.sm; v.z.q = sm + L.sq;
  v.z.a0g = sm + L.s0; v.z.qden = sm + L.sqd;
  return v;
}

// One damped z-line Jacobi sweep of level L from xo (nullptr: zero) into xn.
// The single-block cycle runs its code once per launch, so its time goes to
// instruction fetch as much as to arithmetic: the sweep, called three times,
// is kept out of line (one copy of its code).
template <typename T>
__device__ __noinline__ void blk_sweep(const SmallLevel<T> &L, T *sm, const T *b, const T *xo, T *xn, T omega) {
  const GridG &g = L.o.g;
  const SmallView<T> v = staged(L, sm);
  T *r = sm + L.sr;
  const T *rin = b;
  if (xo) {
    for (unsigned c = threadIdx.x; c < g.n; c += blockDim.x) {
      int i, j, k;
      cell_ijk(c, g, i, j, k);
      r[c] = zline_rhs_at(v.dens, b, xo, L.o, i, j, k, c);
    }
    __syncthreads();
    rin = r;
  }
  for (int col = threadIdx.x; col < g.nx * g.ny; col += blockDim.x) zline_col_s<T>(g, v.z, rin, r, xo, xn, omega, col);
  __syncthreads();
}

// x_out = M(l0) b_in: V(1,1) over levels l0..l0+nl-1, all in this block.
template <typename T>
__global__ void __launch_bounds__(kSmallThreads) k_vcycle_small(SmallCycle<T> sc, const T *__restrict__ b_in,
                                                                T *__restrict__ x_out, int coarse_sweeps, T omega) {
  ECS_PDL_ENTRY();
  extern __shared__ unsigned char small_smem[];
  T *sm = reinterpret_cast<T *>(small_smem);
  const int nl = sc.nl;
  // stage the levels' densities and z-line factors, the coarse inverse and
  // the right-hand side: every later load is a shared-memory load
  for (int l = 0; l < nl; l++) {
    const SmallLevel<T> &L = sc.lv[l];
    const unsigned n = (unsigned)L.o.g.n, ncol = (unsigned)(L.o.g.nx * L.o.g.ny);
    for (unsigned c = threadIdx.x; c < n; c += blockDim.x) {
      sm[L.sd + c] = __ldg(&L.dens[c]);
      sm[L.sa + c] = __ldg(&L.z.a[c]);
      sm[L.sc + c] = __ldg(&L.z.cp[c]);
      sm[L.sm + c] = __ldg(&L.z.minv[c]);
      sm[L.sq + c] = __ldg(&L.z.q[c]);
    }
    for (unsigned c = threadIdx.x; c < ncol; c += blockDim.x) {
      sm[L.s0 + c] = __ldg(&L.z.a0g[c]);
      sm[L.sqd + c] = __ldg(&L.z.qden[c]);
    }
  }
  if (sc.cinv) {
    const unsigned nn = (unsigned)(sc.lv[nl - 1].o.g.n * sc.lv[nl - 1].o.g.n);
    for (unsigned e = threadIdx.x; e < nn; e += blockDim.x) sm[sc.scinv + e] = __ldg(&sc.cinv[e]);
  }
  {
    const SmallLevel<T> &L = sc.lv[0];
    for (unsigned c = threadIdx.x; c < L.o.g.n; c += blockDim.x) sm[L.sb + c] = b_in[c];
    __syncthreads();
  }
  // down
  for (int l = 0; l < nl - 1; l++) {
    const SmallLevel<T> &L = sc.lv[l];
    const GridG &g = L.o.g;
    T *b = sm + L.sb, *t = sm + L.st, *r = sm + L.sr;
    blk_sweep(L, sm, b, (const T *)nullptr, t, omega);
    const T *dl = sm + L.sd;
    for (unsigned c = threadIdx.x; c < g.n; c += blockDim.x) {
      int i, j, k;
      cell_ijk(c, g, i, j, k);
      r[c] = b[c] - apply_row(dl, (const T *)t, L.o, i, j, k);
    }
    __syncthreads();
    const SmallLevel<T> &C = sc.lv[l + 1];
    T *cb = sm + C.sb;
    for (unsigned c = threadIdx.x; c < C.o.g.n; c += blockDim.x) {
      int I, J, K;
      cell_ijk(c, C.o.g, I, J, K);
      cb[c] = restrict_at_rolled(g, C.o.g, (const T *)r, I, J, K);
    }
    __syncthreads();
  }
  // coarsest: direct solve with the precomputed inverse, else damped z-line
  // Jacobi sweeps; the result in its x
  if (sc.cinv) {  // x = inv b: each row's sum split over the 32 lanes of a warp
    const SmallLevel<T> &L = sc.lv[nl - 1];
    const int n = (int)L.o.g.n;
    const T *b = sm + L.sb;
    const T *ci = sm + sc.scinv;
    const int lane = threadIdx.x & 31;
    for (int r = threadIdx.x >> 5; r < n; r += blockDim.x >> 5) {
      T acc = T(0);
      for (int k = lane; k < n; k += 32) acc += ci[k * n + r] * b[k];
      for (int s2 = 16; s2 >= 1; s2 >>= 1) acc += __shfl_xor_sync(ECS_FULL_MASK, acc, s2);
      if (lane == 0) sm[L.sx + r] = acc;
    }
    __syncthreads();
  } else {
    const SmallLevel<T> &L = sc.lv[nl - 1];
    const T *b = sm + L.sb;
    T *cur = sm + L.sx, *nxt = sm + L.st;
    for (int sw = 0; sw < coarse_sweeps; sw++) {
      blk_sweep(L, sm, b, sw == 0 ? (const T *)nullptr : cur, nxt, omega);
      T *tmp = cur;
      cur = nxt;
      nxt = tmp;
    }
    if (cur != sm + L.sx) {
      for (unsigned c = threadIdx.x; c < L.o.g.n; c += blockDim.x) sm[L.sx + c] = cur[c];
      __syncthreads();
    }
  }
  // up
  for (int l = nl - 2; l >= 0; l--) {
    const SmallLevel<T> &L = sc.lv[l], &C = sc.lv[l + 1];
    const GridG &g = L.o.g;
    T *t = sm + L.st;
    const T *cx = sm + C.sx;
    for (unsigned c = threadIdx.x; c < g.n; c += blockDim.x) {
      int i, j, k;
      cell_ijk(c, g, i, j, k);
      t[c] += prolong_at(g, C.o.g, cx, i, j, k);
    }
    __syncthreads();
    blk_sweep(L, sm, sm + L.sb, t, sm + L.sx, omega);
  }
  {
    const SmallLevel<T> &L = sc.lv[0];
    for (unsigned c = threadIdx.x; c < L.o.g.n; c += blockDim.x) x_out[c] = sm[L.sx + c];
  }
}

// ---- direct solve of the coarsest level -----------------------------------------
constexpr int kDirectMax = 128;           // largest coarsest level solved directly
constexpr size_t kInverseSmem = 160 * 1024;  // shared memory of its Gauss-Jordan work matrix
// One block of 32 warps (fewer warps make a pivot step slower: the row
// updates dominate, not the barriers).
constexpr int kInvThreads = 1024;

// invT = (A + sigma 1 1^T)^-1, transposed (invT[k n + r] = inv[r][k]), by
// Gauss-Jordan elimination with partial pivoting on M = [A | I] (n x 2n, in
// global memory), one block.  sigma = mean |A_rr| / n removes the constant
// null space of a fully periodic operator (regularize = 1); without it the
// operator is regular.  Pivot ties go to the lowest row, so the result is
// reproducible.
template <typename T>
__global__ void __launch_bounds__(kInvThreads) k_coarse_inverse(OpK o, const T *__restrict__ dens, int regularize,
                                                         T *__restrict__ Mg, T *__restrict__ invT) {
  ECS_PDL_ENTRY();
  extern __shared__ unsigned char inv_smem[];
  T *M = Mg ? Mg : reinterpret_cast<T *>(inv_smem);  // work matrix in shared memory when it fits
  __shared__ T fac[kDirectMax];
  __shared__ T wv[32];
  __shared__ int piv;
  __shared__ T sigma;
  const GridG &g = o.g;
  const int n = (int)g.n, w = 2 * n, tid = threadIdx.x, bs = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  for (int e = tid; e < n * w; e += bs) M[e] = T(0);
  __syncthreads();
  for (int r = tid; r < n; r += bs) {
    int i, j, k;
    cell_ijk((unsigned)r, g, i, j, k);
    T v[11];
    row11(dens, o, i, j, k, v);
    for (int e = 0; e < 11; e++) {
      int ii = i + off_i(e), jj = j + off_j(e), kk = k + off_k(e);
      bool out = false;
      if (ii < 0 || ii >= g.nx) { if (g.bc[0]) out = true; else ii = ii < 0 ? ii + g.nx : ii - g.nx; }
      if (jj < 0 || jj >= g.ny) { if (g.bc[1]) out = true; else jj = jj < 0 ? jj + g.ny : jj - g.ny; }
      if (kk < 0 || kk >= g.nz) { if (g.bc[2]) out = true; else kk = kk < 0 ? kk + g.nz : kk - g.nz; }
      if (!out) M[(size_t)r * w + ((kk * g.ny + jj) * g.nx + ii)] += v[e];
    }
    M[(size_t)r * w + n + r] = T(1);
  }
  __syncthreads();
  if (regularize) {
    T t = T(0);
    for (int r = tid; r < n; r += bs) t += fabs(M[(size_t)r * w + r]);
    for (int s = 16; s >= 1; s >>= 1) t += __shfl_xor_sync(ECS_FULL_MASK, t, s);
    if (lane == 0) wv[warp] = t;
    __syncthreads();
    if (tid == 0) {
      T u = T(0);
      for (int q = 0; q < (bs >> 5); q++) u += wv[q];
      sigma = u / (T(n) * T(n));
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += bs) M[(size_t)(e / n) * w + (e % n)] += sigma;
    __syncthreads();
  }
  // elimination: rows by warp, columns by lane
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int c = 0; c < n; c++) {
    // pivot: largest |M[r][c]|, r >= c, lowest row on ties (warp 0)
    if (ty == 0) {
      T best = T(-1);
      int bi = n;
      for (int r = c + tx; r < n; r += 32) {
        const T a = fabs(M[(size_t)r * w + c]);
        if (a > best) { best = a; bi = r; }
      }
      for (int s = 16; s >= 1; s >>= 1) {
        const T ob = __shfl_xor_sync(ECS_FULL_MASK, best, s);
        const int oi = __shfl_xor_sync(ECS_FULL_MASK, bi, s);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (tx == 0) {
        piv = bi < n ? bi : c;
        const T pv = M[(size_t)piv * w + c];
        sigma = pv != T(0) ? T(1) / pv : T(0);  // reused as 1 / pivot
      }
    }
    __syncthreads();
    const int pr = piv;
    if (pr != c)
      for (int e = threadIdx.x; e < w; e += blockDim.x) {
        const T t = M[(size_t)c * w + e];
        M[(size_t)c * w + e] = M[(size_t)pr * w + e];
        M[(size_t)pr * w + e] = t;
      }
    __syncthreads();
    const T ip = sigma;
    for (int e = threadIdx.x; e < w; e += blockDim.x) M[(size_t)c * w + e] *= ip;
    for (int r = threadIdx.x; r < n; r += blockDim.x) fac[r] = r == c ? T(0) : M[(size_t)r * w + c];
    __syncthreads();
    for (int r = ty; r < n; r += bs >> 5) {
      const T f = fac[r];
      if (f != T(0))
        for (int q = tx; q < w; q += 32) M[(size_t)r * w + q] -= f * M[(size_t)c * w + q];
    }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += bs) {
    const int r = e / n, k = e - r * n;
    invT[(size_t)k * n + r] = M[(size_t)r * w + n + k];
  }
}

// The same inverse for n <= kRegInvMax with the work matrix in registers:
// row r of M = [A | I] belongs to the tpr threads tid / tpr == r, thread jr
// holding columns jr + tpr u.  Pivoting is implicit: the pivot of column c
// is the largest |M[r][c]| among rows not yet used (lowest row on ties),
// and the row used at step c ends up holding row c of the inverse.  Each
// step needs two barriers: column c and the scaled pivot row pass through
// shared memory (double-buffered by the parity of c).
constexpr int kRegInvMax = 64;
constexpr int kRegCols = 2 * kRegInvMax * kRegInvMax / kInvThreads;  // 8 columns a thread
template <typename T>
__global__ void __launch_bounds__(kInvThreads) k_coarse_inverse_reg(OpK o, const T *__restrict__ dens,
                                                                    int regularize, T *__restrict__ invT) {
  ECS_PDL_ENTRY();
  __shared__ T colbuf[2][kRegInvMax];
  __shared__ T prow[2][2 * kRegInvMax];
  __shared__ int rowpos[kRegInvMax];
  __shared__ T wsum[32];
  __shared__ T sigma;
  const GridG &g = o.g;
  const int n = (int)g.n, w = 2 * n, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tpr = n <= 32 ? 32 : 16;  // threads a row
  const int r = tid / tpr, jr = tid % tpr;
  const bool live = r < n;
  // Every access to M below has a compile-time index (u), so M stays in
  // registers.
  T M[kRegCols];
#pragma unroll
  for (int u = 0; u < kRegCols; u++) M[u] = T(0);
  if (live) {  // row r: the operator's entries in the reference's order, then the identity
    int i, j, k;
    cell_ijk((unsigned)r, g, i, j, k);
    T v[11];
    int tc[11];
    row11(dens, o, i, j, k, v);
#pragma unroll
    for (int e = 0; e < 11; e++) {
      int ii = i + off_i(e), jj = j + off_j(e), kk = k + off_k(e);
      bool out = false;
      if (ii < 0 || ii >= g.nx) { if (g.bc[0]) out = true; else ii = ii < 0 ? ii + g.nx : ii - g.nx; }
      if (jj < 0 || jj >= g.ny) { if (g.bc[1]) out = true; else jj = jj < 0 ? jj + g.ny : jj - g.ny; }
      if (kk < 0 || kk >= g.nz) { if (g.bc[2]) out = true; else kk = kk < 0 ? kk + g.nz : kk - g.nz; }
      tc[e] = out ? -1 : (kk * g.ny + jj) * g.nx + ii;
    }
#pragma unroll
    for (int u = 0; u < kRegCols; u++) {
      const int q = jr + tpr * u;
#pragma unroll
      for (int e = 0; e < 11; e++)
        if (tc[e] == q) M[u] += v[e];
      if (q == n + r) M[u] = T(1);
    }
  }
  if (regularize) {  // sigma = sum |A_rr| / n^2 over the diagonal, added to every entry of A
#pragma unroll
    for (int u = 0; u < kRegCols; u++)
      if (live && jr + tpr * u == r) colbuf[0][r] = fabs(M[u]);
    __syncthreads();
    T t = tid < n ? colbuf[0][tid] : T(0);
    for (int s2 = 16; s2 >= 1; s2 >>= 1) t += __shfl_xor_sync(ECS_FULL_MASK, t, s2);
    if (lane == 0) wsum[warp] = t;
    __syncthreads();
    if (tid == 0) {
      T u2 = T(0);
      for (int q = 0; q < (kInvThreads >> 5); q++) u2 += wsum[q];
      sigma = u2 / (T(n) * T(n));
    }
    __syncthreads();
    const T sg = sigma;
#pragma unroll
    for (int u = 0; u < kRegCols; u++)
      if (live && jr + tpr * u < n) M[u] += sg;
  }
  __syncthreads();  // colbuf[0] is free again
  if (live && jr == 0) colbuf[0][r] = M[0];  // column 0
  unsigned long long used = 0ull;
  // step c = j0 + tpr u0: column c is column u0 of the threads jr == j0
#pragma unroll
  for (int u0 = 0; u0 < kRegCols; u0++) {
    for (int j0 = 0; j0 < tpr; j0++) {
      const int c = j0 + tpr * u0;
      if (c >= n) break;
      const int b = c & 1;
      __syncthreads();  // column c complete
      T best = T(-1);
      int bi = n;
      for (int rr = lane; rr < n; rr += 32) {
        if ((used >> rr) & 1ull) continue;
        const T a = fabs(colbuf[b][rr]);
        if (a > best) { best = a; bi = rr; }
      }
      for (int s2 = 16; s2 >= 1; s2 >>= 1) {
        const T ob = __shfl_xor_sync(ECS_FULL_MASK, best, s2);
        const int oi = __shfl_xor_sync(ECS_FULL_MASK, bi, s2);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      const int pr = bi < n ? bi : __ffsll((long long)~used) - 1;
      used |= 1ull << pr;
      const T pv = colbuf[b][pr];
      const T ip = pv != T(0) ? T(1) / pv : T(0);
      if (tid == 0) rowpos[pr] = c;
      if (r == pr) {
#pragma unroll
        for (int u = 0; u < kRegCols; u++) {
          const int q = jr + tpr * u;
          if (q < w) {
            M[u] *= ip;
            prow[b][q] = M[u];
          }
        }
      }
      __syncthreads();  // scaled pivot row complete
      if (live && r != pr) {
        const T f = colbuf[b][r];
        if (f != T(0)) {
#pragma unroll
          for (int u = 0; u < kRegCols; u++) {
            const int q = jr + tpr * u;
            if (q < w) M[u] -= f * prow[b][q];
          }
        }
      }
      // column c + 1 for the next step: column u0 of j0 + 1, or column
      // u0 + 1 of thread 0 of the row
      if (live && c + 1 < n) {
        if (j0 + 1 < tpr) {
          if (jr == j0 + 1) colbuf[b ^ 1][r] = M[u0];
        } else if (u0 + 1 < kRegCols) {
          if (jr == 0) colbuf[b ^ 1][r] = M[u0 + 1 < kRegCols ? u0 + 1 : u0];
        }
      }
    }
  }
  __syncthreads();
  if (live) {
    const int row = rowpos[r];
#pragma unroll
    for (int u = 0; u < kRegCols; u++) {
      const int q = jr + tpr * u;
      if (q >= n && q < w) invT[(size_t)(q - n) * n + row] = M[u];
    }
  }
}

// ---- vectors ----------------------------------------------------------------------
// Sums of one thread use compensated (Kahan) summation in FP32; a warp adds
// its 32 lanes in T (fixed tree); from there on (warps of a block, blocks)
// the sums are FP64 in a fixed order.  FP32 sums thus need no FP64
// instruction per element, which matters on sm_103 where FP64 issues on a
// narrow pipe.  An FP64 thread sum (a dozen terms or so) is plain, one
// multiply-add a term for the norms: compensation would add four FP64
// operations a term for digits beyond what a norm or a mean needs.
template <typename T>
struct KSum {
  T s, c;
  __device__ __forceinline__ KSum() : s(T(0)), c(T(0)) {}
  __device__ __forceinline__ void add(T x) {
    const T y = x - c;
    const T t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ T value() const { return s - c; }
};
template <>
struct KSum<double> {
  double s;
  __device__ __forceinline__ KSum() : s(0.0) {}
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double value() const { return s; }
};
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int s = 16; s >= 1; s >>= 1) v += __shfl_xor_sync(ECS_FULL_MASK, v, s);
  return v;
}

// W consecutive elements of a vector.  W = kPack<T> (4 floats, 2 doubles)
// moves them with one 16-byte access: the caller guarantees the alignment
// (a basis vector of n cells starts on a 16-byte boundary when n % 4 == 0);
// W = 1 is the plain form.
template <typename T>
constexpr int kPack = 16 / (int)sizeof(T);
template <typename T, int W>
struct Pack {
  T v[W];
};
template <typename T, int W>
__device__ __forceinline__ Pack<T, W> ld_pack(const T *__restrict__ p) {
  Pack<T, W> r;
  if constexpr (W == 4 && sizeof(T) == 4) {
    const float4 f = *reinterpret_cast<const float4 *>(p);
    r.v[0] = f.x; r.v[1] = f.y; r.v[2] = f.z; r.v[3] = f.w;
  } else if constexpr (W == 2 && sizeof(T) == 8) {
    const double2 a = *reinterpret_cast<const double2 *>(p);
    r.v[0] = a.x; r.v[1] = a.y;
  } else {
#pragma unroll
    for (int i = 0; i < W; i++) r.v[i] = p[i];
  }
  return r;
}
template <typename T, int W>
__device__ __forceinline__ void st_pack(T *__restrict__ p, const Pack<T, W> &r) {
  if constexpr (W == 4 && sizeof(T) == 4) {
    *reinterpret_cast<float4 *>(p) = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
  } else if constexpr (W == 2 && sizeof(T) == 8) {
    *reinterpret_cast<double2 *>(p) = make_double2(r.v[0], r.v[1]);
  } else {
#pragma unroll
    for (int i = 0; i < W; i++) p[i] = r.v[i];
  }
}

// Completion ticket of a grid-wide reduction: true in the block that
// finishes last, to which every block's partials (written before the call)
// are then visible; it reads them through L2 (__ldcg).  That block puts the
// counter back to 0 for the next launch.  No block waits on another.
__device__ __forceinline__ bool last_block(unsigned int *ticket) {
  __shared__ int last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int t = atomicAdd(ticket, 1u);
    last = t == gridDim.x - 1;
    if (last) {
      *ticket = 0u;
      __threadfence();
    }
  }
  __syncthreads();
  return last != 0;
}

// partial[blockIdx.x] = the block's sum of the threads' values (Kahan runs
// in T, warps in T, the block's warps in FP64).
template <typename T>
__device__ __forceinline__ void block_partial(const KSum<T> &acc, double *__restrict__ partial) {
  __shared__ double sh[32];
  const T t = warp_sum(acc.value());
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) u += sh[q];
    partial[blockIdx.x] = u;
  }
}

// Sum of partial[0..nb) in a fixed order, valid in thread 0 (the last block).
__device__ __forceinline__ double partials_total(const double *partial, int nb) {
  __shared__ double sh[32];
  double t = 0.0;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) t += __ldcg(partial + q);
  t = warp_sum(t);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  double u = 0.0;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) u += sh[q];
  return u;
}

// out[q] = sum over blocks of slot q's partials (partial[q * nb + b]), one
// warp a slot, for slots 0..ns.
__device__ __forceinline__ void slot_totals(const double *partial, int ns, int nb, double *out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int q = warp; q < ns; q += (int)(blockDim.x >> 5)) {
    double t = 0.0;
    for (int b = lane; b < nb; b += 32) t += __ldcg(partial + (size_t)q * nb + b);
    t = warp_sum(t);
    if (lane == 0) out[q] = t;
  }
}

// x64 += a * e (e in T)
template <typename T>
__global__ void k_axpy64(size_t n, double a, const T *__restrict__ e, double *__restrict__ x) {
  ECS_PDL_ENTRY();
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    x[q] += a * (double)e[q];
}
// d = s * scale[0] in the precision of d (the FP64 residual, normalised, to T)
template <typename T>
__global__ void k_scale_to(size_t n, const double *__restrict__ s, const double *__restrict__ scale, T *__restrict__ d) {
  ECS_PDL_ENTRY();
  const T a = (T)scale[0];
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    d[q] = (T)s[q] * a;
}
// v -= value[0]
template <typename T>
__global__ void k_sub_value(size_t n, T *__restrict__ v, const double *__restrict__ value) {
  ECS_PDL_ENTRY();
  const double m = value[0];
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    v[e] = (T)((double)v[e] - m);
}

// ---- FGMRES on the device -----------------------------------------------------------
// Dot products are formed 8 slots at a time, then a fixed-order block
// reduction; slot q of block b goes to partial[q * gridDim.x + b].
constexpr int kChunk = 8;
template <typename T>
__device__ __forceinline__ void block_chunk(const KSum<T> (&acc)[kChunk], int v0, int nslot,
                                            double *__restrict__ partial) {
  __shared__ double sh[kB / 32][kChunk];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < kChunk; q++) {
    const T a = warp_sum(acc[q].value());
    if (lane == 0) sh[warp][q] = (double)a;
  }
  __syncthreads();
  if (threadIdx.x < kChunk && v0 + (int)threadIdx.x < nslot) {
    double t = 0.0;
    for (int w = 0; w < kB / 32; w++) t += sh[w][threadIdx.x];
    partial[(size_t)(v0 + threadIdx.x) * gridDim.x + blockIdx.x] = t;
  }
  __syncthreads();
}

// Pass 1 of classical Gram-Schmidt: dots of V_0..V_j with w = V_{j+1}.
// Block partials, then the last block forms h1[q] (one warp a slot).  Packs
// of W cells; one resident wave of blocks (4 an SM), so that every thread
// has its loads of several packs in flight.
template <typename T, int W>
__global__ void __launch_bounds__(kB, 4) k_dots1(size_t n, const T *__restrict__ V, KrylovDev *__restrict__ kd,
                                                 double *__restrict__ partial) {
  ECS_PDL_ENTRY();
  const int nv = kd->j + 1;
  const T *w = V + (size_t)nv * n;
  const size_t nw = n / W, stride = (size_t)gridDim.x * blockDim.x;
  for (int v0 = 0; v0 < nv; v0 += kChunk) {
    KSum<T> acc[kChunk];
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < nw; e += stride) {
      const Pack<T, W> we = ld_pack<T, W>(w + e * W);
#pragma unroll
      for (int q = 0; q < kChunk; q++)
        if (v0 + q < nv) {
          const Pack<T, W> vq = ld_pack<T, W>(V + (size_t)(v0 + q) * n + e * W);
#pragma unroll
          for (int i = 0; i < W; i++) acc[q].add(vq.v[i] * we.v[i]);
        }
    }
    block_chunk(acc, v0, nv, partial);
  }
  if (!last_block(&kd->ticket[0])) return;
  slot_totals(partial, nv, (int)gridDim.x, kd->h1);
}

// Arnoldi bookkeeping of step j, in the last block of the pass-2 launch:
// reduce the pass-2 partials into h2 and w.w, form column j of the
// Hessenberg matrix, apply the previous Givens rotations and a new one,
// update the residual estimate and decide whether the cycle stops.
__device__ __forceinline__ void arnoldi_update(KrylovDev *kd, int nb, const double *partial,
                                               cudaGraphConditionalHandle cond, int use_graph) {
  __shared__ double red[kSlots];
  if (kd->done) {  // stopped before this step (b = 0): keep the state
    if (threadIdx.x == 0 && use_graph) cudaGraphSetConditional(cond, 0u);
    return;
  }
  const int j = kd->j, nv = j + 1;
  slot_totals(partial, nv + 1, nb, red);
  __syncthreads();
  if (threadIdx.x != 0) return;
  const int m = kKrylovMax;
  double ss = 0.0;
  for (int q = 0; q <= j; q++) {
    kd->h2[q] = red[q];
    ss += red[q] * red[q];
  }
  const double ww = red[nv];
  const double hn = sqrt(fmax(ww - ss, 0.0));
  double *H = kd->H;
  for (int q = 0; q <= j; q++) H[q * m + j] = kd->h1[q] + kd->h2[q];
  H[(j + 1) * m + j] = hn;
  for (int q = 0; q < j; q++) {
    const double a = H[q * m + j], c = H[(q + 1) * m + j];
    H[q * m + j] = kd->cs[q] * a + kd->sn[q] * c;
    H[(q + 1) * m + j] = -kd->sn[q] * a + kd->cs[q] * c;
  }
  const double a = H[j * m + j], c = H[(j + 1) * m + j];
  const double r = sqrt(a * a + c * c);
  kd->cs[j] = r > 0 ? a / r : 1.0;
  kd->sn[j] = r > 0 ? c / r : 0.0;
  H[j * m + j] = r;
  H[(j + 1) * m + j] = 0.0;
  kd->g[j + 1] = -kd->sn[j] * kd->g[j];
  kd->g[j] = kd->cs[j] * kd->g[j];
  const double res = fabs(kd->g[j + 1]);
  kd->res = res;
  kd->nits = j + 1;
  kd->inv_scale = hn > 0 ? 1.0 / hn : 0.0;
  kd->jprev = j;
  const int done = (res <= kd->tol_rel * kd->beta) || hn == 0.0 || (j + 1 >= kd->maxit) ||
                   (j + 1 >= kKrylovMax) || !isfinite(res);
  kd->done = done;
  if (!done) kd->j = j + 1;
  if (use_graph) cudaGraphSetConditional(cond, done ? 0u : 1u);
}

// w = V_{j+1} - sum_q h1[q] V_q (stored, in the first slot chunk), then
// pass 2: partial dots of V_0..V_j with the new w (slots 0..j) and of w with
// itself (slot j+1); the last block runs the Arnoldi bookkeeping.
template <typename T, int W>
__global__ void __launch_bounds__(kB, 4) k_orth1_dots2(size_t n, T *__restrict__ V, KrylovDev *__restrict__ kd,
                                                       double *__restrict__ partial, cudaGraphConditionalHandle cond,
                                                       int use_graph) {
  ECS_PDL_ENTRY();
  __shared__ T h[kSlots];
  const int nv = kd->j + 1, nslot = nv + 1;
  if (threadIdx.x < kSlots) h[threadIdx.x] = (int)threadIdx.x < nv ? (T)kd->h1[threadIdx.x] : T(0);
  __syncthreads();
  T *w = V + (size_t)nv * n;
  const size_t nw = n / W, stride = (size_t)gridDim.x * blockDim.x;
  for (int v0 = 0; v0 < nslot; v0 += kChunk) {
    KSum<T> acc[kChunk];
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < nw; e += stride) {
      Pack<T, W> s = ld_pack<T, W>(w + e * W);
      if (v0 == 0) {
        for (int q = 0; q < nv; q++) {
          const Pack<T, W> vq = ld_pack<T, W>(V + (size_t)q * n + e * W);
          const T hq = h[q];
#pragma unroll
          for (int i = 0; i < W; i++) s.v[i] -= hq * vq.v[i];
        }
        st_pack<T, W>(w + e * W, s);
      }
#pragma unroll
      for (int q = 0; q < kChunk; q++) {
        const int v = v0 + q;
        if (v < nv) {
          const Pack<T, W> vq = ld_pack<T, W>(V + (size_t)v * n + e * W);
#pragma unroll
          for (int i = 0; i < W; i++) acc[q].add(vq.v[i] * s.v[i]);
        } else if (v == nv) {
#pragma unroll
          for (int i = 0; i < W; i++) acc[q].add(s.v[i] * s.v[i]);
        }
      }
    }
    block_chunk(acc, v0, nslot, partial);
  }
  if (!last_block(&kd->ticket[1])) return;
  arnoldi_update(kd, (int)gridDim.x, partial, cond, use_graph);
}

// V_{j+1} = (w - sum_q h2[q] V_q) / h_{j+1,j}, also copied to the
// preconditioner input vin (j = the step that just finished).
template <typename T, int W>
__global__ void k_orth2_scale(size_t n, T *__restrict__ V, const KrylovDev *__restrict__ kd, T *__restrict__ vin) {
  ECS_PDL_ENTRY();
  __shared__ T h[kSlots + 1];
  const int j = kd->jprev, nv = j + 1;
  if (threadIdx.x < kSlots) h[threadIdx.x] = (int)threadIdx.x < nv ? (T)kd->h2[threadIdx.x] : T(0);
  if (threadIdx.x == kSlots) h[kSlots] = (T)kd->inv_scale;
  __syncthreads();
  T *w = V + (size_t)(j + 1) * n;
  const T sc = h[kSlots];
  const size_t nw = n / W;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < nw; e += (size_t)gridDim.x * blockDim.x) {
    Pack<T, W> s = ld_pack<T, W>(w + e * W);
    for (int q = 0; q < nv; q++) {
      const Pack<T, W> vq = ld_pack<T, W>(V + (size_t)q * n + e * W);
      const T hq = h[q];
#pragma unroll
      for (int i = 0; i < W; i++) s.v[i] -= hq * vq.v[i];
    }
#pragma unroll
    for (int i = 0; i < W; i++) s.v[i] *= sc;
    st_pack<T, W>(w + e * W, s);
    st_pack<T, W>(vin + e * W, s);
  }
}

// Z_j = x - mean (mean = nullptr: x) and V_{j+1} = A Z_j.  Z_j is formed
// at every stencil point on the fly, with the rounding of the stored value;
// a mean is removed only on fully periodic grids, which have no ghosts.
template <typename T>
__global__ void k_apply_dyn(OpK o, const T *__restrict__ n, const T *__restrict__ x, const double *__restrict__ mean,
                            T *__restrict__ Z, T *__restrict__ V, const KrylovDev *__restrict__ kd) {
  ECS_PDL_ENTRY();
  int i, j, k;
  if (!at3(o.g.nx, o.g.ny, i, j, k)) return;
  const int jj = kd->j;
  const T m = mean ? (T)mean[0] : T(0);
  const Nbr q = nbr_of(o.g, i, j, k);
  const unsigned c = q.c;
  T v[11], xe[11];
  row11_n(n, o, q, v);
  row_x(x, q, xe);
  T s = T(0);
#pragma unroll
  for (int e = 0; e < 11; e++) s += v[e] * (xe[e] - m);
  Z[(size_t)jj * o.g.n + c] = x[c] - m;
  V[(size_t)(jj + 1) * o.g.n + c] = s;
}

// Grid-wide sums of a vector in packs of W, finished by the last block:
//   kRedMean  out[0] = sum(v) / div
//   kRedNorm  out[0] = ||v||, out[1] = 1 / ||v|| (0 for v = 0)
//   kRedBeta  start of an FGMRES cycle: beta = ||v|| into the control block;
//             in a graph it also (re)arms the Arnoldi loop's condition,
//             which keeps its last value between cycles of one launch.
enum { kRedMean = 0, kRedNorm = 1, kRedBeta = 2 };
template <typename T, int W, int M>
__global__ void __launch_bounds__(kB) k_reduce(size_t nw, const T *__restrict__ v, double *__restrict__ partial,
                                               double div, double *out, KrylovDev *kd,
                                               cudaGraphConditionalHandle cond, int use_graph) {
  ECS_PDL_ENTRY();
  KSum<T> acc;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < nw; e += (size_t)gridDim.x * blockDim.x) {
    const Pack<T, W> p = ld_pack<T, W>(v + e * W);
#pragma unroll
    for (int i = 0; i < W; i++) acc.add(M == kRedMean ? p.v[i] : p.v[i] * p.v[i]);
  }
  block_partial(acc, partial);
  if (!last_block(&kd->ticket[2 + M])) return;
  const double u = partials_total(partial, (int)gridDim.x);
  if (threadIdx.x != 0) return;
  if (M == kRedMean) {
    out[0] = u / div;
  } else if (M == kRedNorm) {
    out[0] = sqrt(u);
    out[1] = u > 0.0 ? 1.0 / sqrt(u) : 0.0;
  } else {
    const double beta = sqrt(u);
    kd->beta = beta;
    kd->res = beta;
    kd->j = 0;
    kd->jprev = 0;
    kd->nits = 0;
    kd->done = !(beta > 0.0) || kd->maxit < 1;
    kd->inv_scale = beta > 0.0 ? 1.0 / beta : 0.0;
    for (int q = 0; q <= kKrylovMax; q++) kd->g[q] = 0.0;
    kd->g[0] = beta;
    if (use_graph) cudaGraphSetConditional(cond, kd->done ? 0u : 1u);
  }
}

// V_0 = b / beta, vin = V_0, x = 0
template <typename T>
__global__ void k_cycle_start(size_t n, const T *__restrict__ b, T *__restrict__ V, T *__restrict__ vin,
                              T *__restrict__ x, const KrylovDev *__restrict__ kd) {
  ECS_PDL_ENTRY();
  const T sc = (T)kd->inv_scale;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const T v = b[e] * sc;
    V[e] = v;
    vin[e] = v;
    x[e] = T(0);
  }
}

// y = H^-1 g (upper triangular, nits x nits)
__global__ void k_cycle_solve(KrylovDev *kd) {
  ECS_PDL_ENTRY();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int m = kKrylovMax, nj = kd->nits;
  for (int q = nj - 1; q >= 0; q--) {
    double s = kd->g[q];
    for (int r2 = q + 1; r2 < nj; r2++) s -= kd->H[q * m + r2] * kd->y[r2];
    kd->y[q] = s / kd->H[q * m + q];
  }
}

// x += sum_q y[q] Z_q
template <typename T>
__global__ void k_cycle_combine(size_t n, const T *__restrict__ Z, const KrylovDev *__restrict__ kd, T *__restrict__ x) {
  ECS_PDL_ENTRY();
  __shared__ T y[kKrylovMax];
  const int nj = kd->nits;
  if (threadIdx.x < kKrylovMax) y[threadIdx.x] = (int)threadIdx.x < nj ? (T)kd->y[threadIdx.x] : T(0);
  __syncthreads();
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    T s = x[e];
    for (int q = 0; q < nj; q++) s += y[q] * Z[(size_t)q * n + e];
    x[e] = s;
  }
}

// ---- host side -----------------------------------------------------------------------
unsigned int blocks_for(const EcsCtx *ctx, size_t n) {
  size_t want = (n + kB - 1) / kB;
  size_t cap = (size_t)ctx->nsm * 8;
  if (want > cap) want = cap;
  return (unsigned int)(want ? want : 1);
}
// Grid of a reduction over `units` packs: at most one resident wave (4
// blocks of kB threads an SM), so that no block starts after another's end.
unsigned int dot_blocks(const EcsCtx *ctx, size_t units) {
  size_t want = (units + kB - 1) / kB;
  want = std::min(want, std::min((size_t)ctx->nsm * 4, (size_t)kDotBlocks));
  return (unsigned int)(want ? want : 1);
}
// Vectors go in packs of 4 cells (16-byte accesses) when every basis vector
// starts on a 16-byte boundary, i.e. when the cell count is a multiple of 4.
inline bool packed4(size_t n) { return (n & 3) == 0; }

// A grid-wide sum of v (kRed* mode M) on the context's stream.
template <typename T, int M>
int launch_reduce(EcsCtx *ctx, size_t n, const T *v, double div, double *out, cudaGraphConditionalHandle cond,
                  int use_graph) {
  KrylovDev *kd = (KrylovDev *)ctx->kdev;
  constexpr int W = kPack<T>;
  if (packed4(n))
    ecs_launch_pdl(k_reduce<T, W, M>, dot_blocks(ctx, n / W), kB, 0, ctx->stream, n / W, v, ctx->red, div, out, kd, cond, use_graph);
  else
    ecs_launch_pdl(k_reduce<T, 1, M>, dot_blocks(ctx, n), kB, 0, ctx->stream, n, v, ctx->red, div, out, kd, cond, use_graph);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

bool fully_periodic(const EcsCtx *ctx) {
  return ctx->p.bc[0] == ECS_BC_PERIODIC && ctx->p.bc[1] == ECS_BC_PERIODIC && ctx->p.bc[2] == ECS_BC_PERIODIC;
}

// The density the operator is built from (-lhs laplacian ignores it: see
// make_op).
const double *op_density(const EcsCtx *ctx) { return ctx->mom; }
bool identity_lhs(const EcsCtx *ctx) { return ctx->p.lhs_type == ECS_LHS_IDENTITY; }

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
    T **arr[] = {&L.dens, &L.x, &L.b, &L.r, &L.t, &L.zl_a, &L.zl_cp, &L.zl_minv, &L.zl_q, &L.zl_fb, &L.zl_bb};
    for (auto a : arr) ECS_CUDA(ctx, cudaMalloc((void **)a, L.n * sizeof(T)));
    ECS_CUDA(ctx, cudaMalloc((void **)&L.zl_a0g, (size_t)nx * ny * sizeof(T)));
    ECS_CUDA(ctx, cudaMalloc((void **)&L.zl_qden, (size_t)nx * ny * sizeof(T)));
    mg.lv.push_back(L);
    // A 2-D grid (nz = 1) coarsens in x and y only.  So does a grid with a
    // reflecting z: its ghost planes one spacing outside the walls do not
    // nest under z coarsening, and the z-line smoother resolves z on every
    // level, so the levels keep all planes down to one column (x y = 1 x 1,
    // whose Nz cells the coarsest inverse solves directly).
    const bool flat = nz == 1;
    const bool semi = !flat && ctx->p.bc[2] != ECS_BC_PERIODIC;
    if (semi) {
      if (nx % 2 || ny % 2 || mg.lv.size() >= 12) break;
    } else {
      bool even = (nx % 2 == 0) && (ny % 2 == 0) && (flat || nz % 2 == 0);
      if (!even || std::min(nx, std::min(ny, flat ? nx : nz)) < 8 || mg.lv.size() >= 12) break;
    }
    nx /= 2; ny /= 2;
    hx *= 2; hy *= 2;
    if (!flat && !semi) {
      nz /= 2;
      hz *= 2;
    }
  }
  const size_t nc = mg.lv.back().n;
  if (nc <= (size_t)kDirectMax) {
    ECS_CUDA(ctx, cudaMalloc((void **)&mg.cinv, nc * nc * sizeof(T)));
    ECS_CUDA(ctx, cudaMalloc((void **)&mg.cwork, nc * 2 * nc * sizeof(T)));
  }
  mg.built = true;
  return ECS_OK;
}

template <typename T>
ZlP<T> zl_of(MgLevel<T> &L) {
  ZlP<T> z;
  z.a = L.zl_a; z.cp = L.zl_cp; z.minv = L.zl_minv; z.q = L.zl_q; z.fb = L.zl_fb; z.bb = L.zl_bb;
  z.a0g = L.zl_a0g; z.qden = L.zl_qden;
  return z;
}
template <typename T>
OpK op_level(const EcsCtx *ctx, const MgLevel<T> &L) {
  return make_op(ctx->p, L.nx, L.ny, L.nz, L.hx, L.hy, L.hz);
}
GridG grid_level(const EcsCtx *ctx, int nx, int ny, int nz) { return make_grid(ctx->p, nx, ny, nz); }

constexpr int kColBlock = 32;  // one warp a block: the columns spread over the SMs
constexpr int kCoarseSweeps = 21;
template <typename T>
constexpr T kOmega() { return T(0.8); }

// Level densities (level 0 from the deposited density, coarser ones by full
// weighting) and the z-line factorisation of every level.
template <typename T>
__global__ void k_density_in(size_t n, const double *__restrict__ mom, T *__restrict__ d) {
  ECS_PDL_ENTRY();
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    d[e] = (T)mom[e];
}

int ensure_setup_streams(EcsCtx *ctx) {
  for (auto &c : ctx->sst)
    if (!c) ECS_CUDA(ctx, cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking));
  for (auto &e : ctx->sev)
    if (!e) ECS_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return ECS_OK;
}

// z-line rows and factors of level L on stream s.
template <typename T>
int zline_factor(EcsCtx *ctx, MgLevel<T> &L, cudaStream_t s) {
  const int ncol = L.nx * L.ny;
  const OpK o = op_level(ctx, L);
  ecs_launch_pdl(k_zline_rows<T>, blocks3(o.g), threads3(), 0, s, o, L.dens, L.x, L.b, L.r);  // x, b, r are free here
  ECS_LAUNCHED(ctx);
  ecs_launch_pdl(k_zline_setup<T>, ecs_div_up(ncol, kColBlock), kColBlock, 0, s, o.g, L.x, L.b, L.r, zl_of(L), seg_len<T>(L.nz));
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

// The 11 FP64 row coefficients of every cell, coef[e * n + c] (e in the
// order of off_i/off_j/off_k), computed once per operator set-up: FP64
// arithmetic runs at a small fraction of the FP32 rate on this GPU, and the
// coefficients take about three quarters of a residual's FP64 operations.
__global__ void k_coef64(OpK o, const double *__restrict__ n, double *__restrict__ coef) {
  ECS_PDL_ENTRY();
  int i, j, k;
  if (!at3(o.g.nx, o.g.ny, i, j, k)) return;
  const Nbr q = nbr_of(o.g, i, j, k);
  double v[11];
  row11_n(n, o, q, v);
#pragma unroll
  for (int e = 0; e < 11; e++) coef[(size_t)e * o.g.n + q.c] = v[e];
}

// Operator set-up of the multigrid levels: level densities, z-line factors,
// coarsest inverse, and the FP64 row coefficients of the refinement
// residuals.  The pieces are latency-bound small launches with few
// dependencies (and one FP64-bound kernel), so they run on four streams
// (also inside a graph capture, where the fork and join become graph edges):
//   context stream: fine density, fine z-line factors
//   sst[0]:         restriction chain of the densities, then the coarse inverse
//   sst[1]:         z-line factors of the coarse levels (after the chain)
//   sst[2]:         FP64 row coefficients
// and the context stream waits for the side streams at the end.
template <typename T>
int mg_setup(EcsCtx *ctx) {
  int rc = mg_alloc<T>(ctx);
  if (rc) return rc;
  if ((rc = ensure_setup_streams(ctx))) return rc;
  Multigrid<T> &mg = mg_of<T>(ctx);
  cudaStream_t s0 = ctx->stream, sa = ctx->sst[0], sb = ctx->sst[1], sc = ctx->sst[2];
  MgLevel<T> &L0 = mg.lv[0];
  ECS_CUDA(ctx, cudaEventRecord(ctx->sev[4], s0));
  ECS_CUDA(ctx, cudaStreamWaitEvent(sc, ctx->sev[4], 0));
  {
    const EcsParams &p = ctx->p;
    const OpK o64 = make_op(p, p.Nx, p.Ny, p.Nz, p.dx, p.dy, p.dz);
    ecs_launch_pdl(k_coef64, blocks3(o64.g), threads3(), 0, sc, o64, op_density(ctx), ctx->coef64);
    ECS_LAUNCHED(ctx);
  }
  ECS_CUDA(ctx, cudaEventRecord(ctx->sev[5], sc));
  ecs_launch_pdl(k_density_in<T>, blocks_for(ctx, L0.n), kB, 0, s0, L0.n, op_density(ctx), L0.dens);
  ECS_LAUNCHED(ctx);
  ECS_CUDA(ctx, cudaEventRecord(ctx->sev[0], s0));
  ECS_CUDA(ctx, cudaStreamWaitEvent(sa, ctx->sev[0], 0));
  for (size_t l = 1; l < mg.lv.size(); l++) {
    MgLevel<T> &F = mg.lv[l - 1], &C = mg.lv[l];
    ecs_launch_pdl(k_restrict<T>, blocks3(C.nx, C.ny, C.nz), threads3(), 0, sa, 
        grid_level(ctx, F.nx, F.ny, F.nz), grid_level(ctx, C.nx, C.ny, C.nz), F.dens, C.dens);
    ECS_LAUNCHED(ctx);
  }
  ECS_CUDA(ctx, cudaEventRecord(ctx->sev[1], sa));
  ECS_CUDA(ctx, cudaStreamWaitEvent(sb, ctx->sev[1], 0));
  for (size_t l = 1; l < mg.lv.size(); l++)
    if ((rc = zline_factor<T>(ctx, mg.lv[l], sb))) return rc;
  ECS_CUDA(ctx, cudaEventRecord(ctx->sev[2], sb));
  if (mg.cinv) {
    MgLevel<T> &C = mg.lv.back();
    const size_t bytes = C.n * 2 * C.n * sizeof(T);
    const bool in_smem = bytes <= kInverseSmem;
    static std::atomic<bool> attr_set[2];  // zero-initialised: false
    if (!attr_set[sizeof(T) == 8]) {
      ECS_CUDA(ctx, cudaFuncSetAttribute(k_coarse_inverse<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInverseSmem));
      attr_set[sizeof(T) == 8] = true;
    }
    if (C.n <= (size_t)kRegInvMax)
      ecs_launch_pdl(k_coarse_inverse_reg<T>, 1, kInvThreads, 0, sa, op_level(ctx, C), C.dens, fully_periodic(ctx) ? 1 : 0,
                                                          mg.cinv);
    else
      ecs_launch_pdl(k_coarse_inverse<T>, 1, kInvThreads, in_smem ? bytes : 0, sa, 
          op_level(ctx, C), C.dens, fully_periodic(ctx) ? 1 : 0, in_smem ? nullptr : mg.cwork, mg.cinv);
    ECS_LAUNCHED(ctx);
  }
  ECS_CUDA(ctx, cudaEventRecord(ctx->sev[3], sa));
  if ((rc = zline_factor<T>(ctx, L0, s0))) return rc;
  ECS_CUDA(ctx, cudaStreamWaitEvent(s0, ctx->sev[2], 0));
  ECS_CUDA(ctx, cudaStreamWaitEvent(s0, ctx->sev[3], 0));
  ECS_CUDA(ctx, cudaStreamWaitEvent(s0, ctx->sev[5], 0));
  return ECS_OK;
}

template <typename T>
int sweep(EcsCtx *ctx, MgLevel<T> &L, const T *b, const T *xo, T *xn) {
  const OpK o = op_level(ctx, L);
  const T *r = b;
  if (xo) {
    ecs_launch_pdl(k_zline_rhs<T>, blocks3(o.g), threads3(), 0, ctx->stream, o, L.dens, b, xo, L.r);
    ECS_LAUNCHED(ctx);
    r = L.r;
  }
  const int S = seg_len<T>(L.nz);
  const dim3 grid((unsigned)((L.nx + 31) / 32), (unsigned)L.ny);
  const dim3 block(32, (unsigned)((L.nz + S - 1) / S));
  if (S == 8)
    ecs_launch_pdl(k_zline_seg<T, 8>, grid, block, 0, ctx->stream, o.g, zl_of(L), r, xo, xn, kOmega<T>());
  else if (S == 16)
    ecs_launch_pdl(k_zline_seg<T, 16>, grid, block, 0, ctx->stream, o.g, zl_of(L), r, xo, xn, kOmega<T>());
  else if (S == 32)
    ecs_launch_pdl(k_zline_seg<T, 32>, grid, block, 0, ctx->stream, o.g, zl_of(L), r, xo, xn, kOmega<T>());
  else
    ecs_launch_pdl(k_zline_seg<T, 64>, grid, block, 0, ctx->stream, o.g, zl_of(L), r, xo, xn, kOmega<T>());
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

constexpr size_t kSmallCells = 512;
constexpr size_t kSmallSmem = 200 * 1024;  // shared memory of the single-block cycle

// Shared memory of a single-block cycle over levels l..: per level 4
// vectors, the staged density and 4 z-line factor arrays, 2 column arrays;
// the coarse inverse.
template <typename T>
size_t small_bytes(const Multigrid<T> &mg, size_t l) {
  size_t words = 0;
  for (size_t q = l; q < mg.lv.size(); q++) words += mg.lv[q].n * 9 + (size_t)mg.lv[q].nx * mg.lv[q].ny * 2;
  if (mg.cinv) words += mg.lv.back().n * mg.lv.back().n;
  return words * sizeof(T);
}

// One V(1,1) cycle on level l: xout = M(l) b, zero initial guess.  Levels of
// at most kSmallCells cells run as one single-block kernel.
template <typename T>
int vcycle(EcsCtx *ctx, size_t l, const T *b, T *xout) {
  Multigrid<T> &mg = mg_of<T>(ctx);
  MgLevel<T> &L = mg.lv[l];
  int rc;
  if (L.n <= kSmallCells && mg.lv.size() - l <= (size_t)kMaxSmall && small_bytes(mg, l) <= kSmallSmem) {
    SmallCycle<T> sc;
    sc.nl = (int)(mg.lv.size() - l);
    sc.cinv = mg.cinv;
    int off = 0;
    for (int q = 0; q < sc.nl; q++) {
      MgLevel<T> &M = mg.lv[l + q];
      SmallLevel<T> &S = sc.lv[q];
      S.o = op_level(ctx, M);
      S.dens = M.dens;
      S.z = zl_of(M);
      const int nq = (int)M.n, nc = M.nx * M.ny;
      S.sx = off; S.sb = off + nq; S.sr = off + 2 * nq; S.st = off + 3 * nq;
      S.sd = off + 4 * nq; S.sa = off + 5 * nq; S.sc = off + 6 * nq; S.sm = off + 7 * nq; S.sq = off + 8 * nq;
      S.s0 = off + 9 * nq; S.sqd = off + 9 * nq + nc;
      off += 9 * nq + 2 * nc;
    }
    sc.scinv = off;
    if (sc.cinv) off += (int)(mg.lv.back().n * mg.lv.back().n);
    const size_t bytes = (size_t)off * sizeof(T);
    static std::atomic<bool> attr_set[2];  // zero-initialised: false
    if (!attr_set[sizeof(T) == 8]) {
      ECS_CUDA(ctx, cudaFuncSetAttribute(k_vcycle_small<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallSmem));
      attr_set[sizeof(T) == 8] = true;
    }
    ecs_launch_pdl(k_vcycle_small<T>, 1, kSmallThreads, bytes, ctx->stream, sc, b, xout, kCoarseSweeps, kOmega<T>());
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
  const OpK o = op_level(ctx, L);
  if ((rc = sweep<T>(ctx, L, b, nullptr, L.t))) return rc;
  ecs_launch_pdl(k_apply<T>, blocks3(o.g), threads3(), 0, ctx->stream, o, L.dens, L.t, b, L.r, 1);
  ECS_LAUNCHED(ctx);
  const GridG gc = grid_level(ctx, C.nx, C.ny, C.nz);
  ecs_launch_pdl(k_restrict<T>, blocks3(gc), threads3(), 0, ctx->stream, o.g, gc, L.r, C.b);
  ECS_LAUNCHED(ctx);
  if ((rc = vcycle<T>(ctx, l + 1, C.b, C.x))) return rc;
  ecs_launch_pdl(k_prolong_add<T>, blocks3(o.g), threads3(), 0, ctx->stream, o.g, gc, C.x, L.t);
  ECS_LAUNCHED(ctx);
  return sweep<T>(ctx, L, b, L.t, xout);
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
// right-hand side and correction of the FGMRES cycle in precision T
template <typename T>
T *cycle_b(EcsCtx *ctx);
template <>
double *cycle_b<double>(EcsCtx *ctx) { return ctx->r64; }
template <>
float *cycle_b<float>(EcsCtx *ctx) { return ctx->kz32 + (size_t)ctx->krylov_m * ctx->ncell; }
template <typename T>
T *cycle_x(EcsCtx *ctx);
template <>
double *cycle_x<double>(EcsCtx *ctx) { return ctx->w64; }
template <>
float *cycle_x<float>(EcsCtx *ctx) { return ctx->kz32 + (size_t)(ctx->krylov_m + 1) * ctx->ncell; }

// Kernels before the Arnoldi loop: ||b||, V_0, x = 0.
template <typename T>
int cycle_pre(EcsCtx *ctx, cudaGraphConditionalHandle cond, int use_graph) {
  const size_t n = ctx->ncell;
  KrylovDev *kd = (KrylovDev *)ctx->kdev;
  Multigrid<T> &mg = mg_of<T>(ctx);
  const T *b = cycle_b<T>(ctx);
  int rc = launch_reduce<T, kRedBeta>(ctx, n, b, 1.0, nullptr, cond, use_graph);
  if (rc) return rc;
  ecs_launch_pdl(k_cycle_start<T>, blocks_for(ctx, n), kB, 0, ctx->stream, n, b, basis_v<T>(ctx), mg.lv[0].b, cycle_x<T>(ctx), kd);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

// One Arnoldi step j (j read from the control block).
template <typename T>
int cycle_step(EcsCtx *ctx, cudaGraphConditionalHandle cond, int use_graph) {
  const size_t n = ctx->ncell;
  KrylovDev *kd = (KrylovDev *)ctx->kdev;
  Multigrid<T> &mg = mg_of<T>(ctx);
  MgLevel<T> &L0 = mg.lv[0];
  const OpK o0 = op_level(ctx, L0);
  T *V = basis_v<T>(ctx), *Z = basis_z<T>(ctx);
  int rc;
  // z = M v_j  (vin = L0.b holds v_j, the V-cycle writes L0.x)
  if ((rc = vcycle<T>(ctx, 0, L0.b, L0.x))) return rc;
  const double *mean = nullptr;
  if (fully_periodic(ctx)) {  // the operator's null space: project out the mean
    if ((rc = launch_reduce<T, kRedMean>(ctx, n, L0.x, (double)n, &kd->mean, cond, use_graph))) return rc;
    mean = &kd->mean;
  }
  ecs_launch_pdl(k_apply_dyn<T>, blocks3(o0.g), threads3(), 0, ctx->stream, o0, L0.dens, L0.x, mean, Z, V, kd);
  ECS_LAUNCHED(ctx);
  // classical Gram-Schmidt, two passes (the second ends with the Arnoldi
  // bookkeeping)
  constexpr int W = kPack<T>;
  if (packed4(n)) {
    const unsigned nb = dot_blocks(ctx, n / W);
    ecs_launch_pdl(k_dots1<T, W>, nb, kB, 0, ctx->stream, n, V, kd, ctx->red);
    ECS_LAUNCHED(ctx);
    ecs_launch_pdl(k_orth1_dots2<T, W>, nb, kB, 0, ctx->stream, n, V, kd, ctx->red, cond, use_graph);
    ECS_LAUNCHED(ctx);
  } else {
    const unsigned nb = dot_blocks(ctx, n);
    ecs_launch_pdl(k_dots1<T, 1>, nb, kB, 0, ctx->stream, n, V, kd, ctx->red);
    ECS_LAUNCHED(ctx);
    ecs_launch_pdl(k_orth1_dots2<T, 1>, nb, kB, 0, ctx->stream, n, V, kd, ctx->red, cond, use_graph);
    ECS_LAUNCHED(ctx);
  }
  if (packed4(n))
    ecs_launch_pdl(k_orth2_scale<T, W>, blocks_for(ctx, n / W), kB, 0, ctx->stream, n, V, kd, L0.b);
  else
    ecs_launch_pdl(k_orth2_scale<T, 1>, blocks_for(ctx, n), kB, 0, ctx->stream, n, V, kd, L0.b);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

// Kernels after the loop: x = sum_q y_q Z_q.
template <typename T>
int cycle_post(EcsCtx *ctx) {
  const size_t n = ctx->ncell;
  KrylovDev *kd = (KrylovDev *)ctx->kdev;
  ecs_launch_pdl(k_cycle_solve, 1, 32, 0, ctx->stream, kd);
  ECS_LAUNCHED(ctx);
  ecs_launch_pdl(k_cycle_combine<T>, blocks_for(ctx, n), kB, 0, ctx->stream, n, basis_z<T>(ctx), kd, cycle_x<T>(ctx));
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

// One FGMRES cycle on (cycle_b, cycle_x) with tolerance tol (relative to
// ||b||) and at most maxit steps, launched from the host step by step (the
// host reads the stop flag after each step); the control block ends up in
// ctx->kdev_host.
template <typename T>
int fgmres_cycle(EcsCtx *ctx, double tol, int maxit) {
  KrylovDev *kd = (KrylovDev *)ctx->kdev;
  KrylovDev *ctl = (KrylovDev *)ctx->kctl_host;
  ctl->tol_rel = tol;
  ctl->maxit = std::min(std::min(ctx->krylov_m, kKrylovMax), std::max(maxit, 1));
  ECS_CUDA(ctx, cudaMemcpyAsync(kd, ctl, offsetof(KrylovDev, j), cudaMemcpyHostToDevice, ctx->stream));
  int rc;
  cudaGraphConditionalHandle none = 0;
  if ((rc = cycle_pre<T>(ctx, none, 0))) return rc;
  KrylovDev *hk = (KrylovDev *)ctx->kdev_host;
  for (int s = 0; s < kKrylovMax; s++) {
    ECS_CUDA(ctx, cudaMemcpyAsync(&hk->done, &kd->done, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (hk->done) break;
    if ((rc = cycle_step<T>(ctx, none, 0))) return rc;
  }
  return cycle_post<T>(ctx);
}

// ||v||_2 of an FP64 vector into out2[0], its inverse into out2[1], on the device.
int norm64_dev(EcsCtx *ctx, const double *v, double *out2) {
  return launch_reduce<double, kRedNorm>(ctx, ctx->ncell, v, 1.0, out2, 0, 0);
}

template <typename T>
int project_mean(EcsCtx *ctx, T *v) {
  if (!fully_periodic(ctx)) return ECS_OK;
  size_t n = ctx->ncell;
  int rc = launch_reduce<T, kRedMean>(ctx, n, v, (double)n, ctx->dots + 2, 0, 0);
  if (rc) return rc;
  ecs_launch_pdl(k_sub_value<T>, blocks_for(ctx, n), kB, 0, ctx->stream, n, v, ctx->dots + 2);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

// ---- the whole solve on the device ------------------------------------------
// Device state of the iterative-refinement loop.
struct RefineDev {
  double bnorm, rel;
  int its, sweeps;
  int done;  // converged, out of iterations, stalled or non-finite
  int nonfinite;
};

__global__ void k_solve_init(RefineDev *rd, const double *__restrict__ dots) {
  ECS_PDL_ENTRY();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  rd->bnorm = dots[0];
  rd->rel = 0.0;
  rd->its = 0;
  rd->sweeps = 0;
  rd->done = !(dots[0] > 0.0);
  rd->nonfinite = 0;
}

// Refinement sweeps in one solve: each sweep runs at least one FGMRES step
// (or ends the solve), so max_it bounds them; this caps the loop regardless.
constexpr int kMaxSweeps = 64;

// Relative residual of the current sweep (norm in dots[0]); decides whether
// another correction follows (condition `cond` of the sweep loop) and sets
// the FGMRES tolerance and step limit of that correction.
__global__ void k_refine_check(RefineDev *rd, KrylovDev *kd, const double *__restrict__ dots, double rtol,
                               int max_it, double tol_floor, cudaGraphConditionalHandle cond) {
  ECS_PDL_ENTRY();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (rd->bnorm > 0.0) {
    const double rel = dots[0] / rd->bnorm;
    rd->rel = rel;
    if (!isfinite(rel)) rd->nonfinite = 1;
  }
  const bool stop = rd->done || rd->nonfinite || rd->rel <= rtol || rd->its >= max_it || rd->sweeps >= kMaxSweeps;
  if (stop) {
    rd->done = 1;
  } else {
    const double tol = fmax(fmax(0.5 * rtol / rd->rel, 1e-14), tol_floor);
    kd->tol_rel = tol;
    kd->maxit = min(kKrylovMax, max(max_it - rd->its, 1));
  }
  cudaGraphSetConditional(cond, stop ? 0u : 1u);
}

__global__ void k_refine_update(RefineDev *rd, const KrylovDev *__restrict__ kd) {
  ECS_PDL_ENTRY();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  rd->its += kd->nits;
  rd->sweeps += 1;
  if (kd->nits == 0) rd->done = 1;
}

// x64 += scale[0] * e (scale nullptr: 1)
template <typename T>
__global__ void k_axpy64_dev(size_t n, const double *__restrict__ scale, const T *__restrict__ e, double *__restrict__ x) {
  ECS_PDL_ENTRY();
  const double a = scale ? scale[0] : 1.0;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    x[q] += a * (double)e[q];
}

// Mixed-precision residual: r64 = b64 - A64(n64) x64.
// r = b - A x in FP64 from the stored coefficients (the same products and
// sum as computing them in place).
__global__ void k_residual64(OpK o, const double *__restrict__ coef, const double *__restrict__ x,
                             const double *__restrict__ b, double *__restrict__ r) {
  ECS_PDL_ENTRY();
  int i, j, k;
  if (!at3(o.g.nx, o.g.ny, i, j, k)) return;
  const Nbr q = nbr_of(o.g, i, j, k);
  double xe[11];
  row_x(x, q, xe);
  double s = 0.0;
#pragma unroll
  for (int e = 0; e < 11; e++) s += __ldg(&coef[(size_t)e * o.g.n + q.c]) * xe[e];
  r[q.c] = b[q.c] - s;
}

template <typename T>
void free_mg(Multigrid<T> &mg) {
  for (auto &L : mg.lv) {
    T *arr[] = {L.dens, L.x, L.b, L.r, L.t, L.zl_a, L.zl_cp, L.zl_minv, L.zl_q, L.zl_fb, L.zl_bb, L.zl_a0g, L.zl_qden};
    for (T *a : arr)
      if (a) cudaFree(a);
  }
  mg.lv.clear();
  if (mg.cinv) cudaFree(mg.cinv);
  if (mg.cwork) cudaFree(mg.cwork);
  mg.cinv = mg.cwork = nullptr;
  mg.built = false;
}

void free_graph(SolverGraph &sg) {
  if (sg.exec) cudaGraphExecDestroy(sg.exec);
  if (sg.graph) cudaGraphDestroy(sg.graph);
  sg = SolverGraph();
}

// ---- graph construction ----------------------------------------------------------
// Conditional node appended to the graph being captured on stream s (after
// its current dependencies); the node's body graph is returned, to be
// captured on another stream.
int capture_conditional(EcsCtx *ctx, cudaStream_t s, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                        cudaGraph_t *body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  const cudaGraphEdgeData *edges = nullptr;
  size_t nd = 0;
  ECS_CUDA(ctx, cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, &edges, &nd));
  // zero-initialised storage (the parameter union has no default constructor)
  alignas(cudaGraphNodeParams) unsigned char cp_store[sizeof(cudaGraphNodeParams)];
  memset(cp_store, 0, sizeof cp_store);
  cudaGraphNodeParams *cp = reinterpret_cast<cudaGraphNodeParams *>(cp_store);
  cp->type = cudaGraphNodeTypeConditional;
  cp->conditional.handle = h;
  cp->conditional.type = type;
  cp->conditional.size = 1;
  cudaGraphNode_t node;
  ECS_CUDA(ctx, cudaGraphAddNode(&node, g, deps, edges, nd, cp));
  ECS_CUDA(ctx, cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  *body = cp->conditional.phGraph_out[0];
  return ECS_OK;
}
// The graph being captured on stream s.
int capture_graph(EcsCtx *ctx, cudaStream_t s, cudaGraph_t *g) {
  cudaStreamCaptureStatus cs;
  ECS_CUDA(ctx, cudaStreamGetCaptureInfo(s, &cs, nullptr, g, nullptr, nullptr, nullptr));
  return ECS_OK;
}

template <typename T>
int refine_decide(EcsCtx *ctx, double rtol, int max_it, cudaGraphConditionalHandle h) {
  const double tol_floor = sizeof(T) == 4 ? 2e-6 : 0.0;
  ecs_launch_pdl(k_refine_check, 1, 32, 0, ctx->stream, (RefineDev *)ctx->rdev, (KrylovDev *)ctx->kdev, ctx->dots, rtol, max_it,
                                            tol_floor, h);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

// Residual of the current phi, its norm and the check that sets the sweep
// loop's condition h (on ctx->stream).
template <typename T>
int refine_check(EcsCtx *ctx, double rtol, int max_it, cudaGraphConditionalHandle h) {
  const EcsParams &p = ctx->p;
  const OpK o64 = make_op(p, p.Nx, p.Ny, p.Nz, p.dx, p.dy, p.dz);
  ecs_launch_pdl(k_residual64, blocks3(o64.g), threads3(), 0, ctx->stream, o64, (const double *)ctx->coef64, ctx->phi, ctx->rhs, ctx->r64);
  ECS_LAUNCHED(ctx);
  int rc = norm64_dev(ctx, ctx->r64, ctx->dots);
  if (rc) return rc;
  return refine_decide<T>(ctx, rtol, max_it, h);
}

// The correction of one sweep: the FGMRES cycle (the Arnoldi loop as a WHILE
// node captured on capture stream `lvl`), phi update, mean projection.
template <typename T>
int refine_correct(EcsCtx *ctx, int lvl) {
  const size_t n = ctx->ncell;
  int rc;
  if (sizeof(T) == 4) {  // the normalised FP64 residual to FP32
    ecs_launch_pdl(k_scale_to<float>, blocks_for(ctx, n), kB, 0, ctx->stream, n, ctx->r64, ctx->dots + 1, (float *)cycle_b<T>(ctx));
    ECS_LAUNCHED(ctx);
  }
  cudaGraph_t g = nullptr, body = nullptr;
  if ((rc = capture_graph(ctx, ctx->stream, &g))) return rc;
  cudaGraphConditionalHandle hw;
  ECS_CUDA(ctx, cudaGraphConditionalHandleCreate(&hw, g, 0, 0));
  if ((rc = cycle_pre<T>(ctx, hw, 1))) return rc;
  if ((rc = capture_conditional(ctx, ctx->stream, hw, cudaGraphCondTypeWhile, &body))) return rc;
  cudaStream_t outer = ctx->stream;
  ctx->stream = ctx->capst[lvl];
  ECS_CUDA(ctx, cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  const int64_t l0 = ctx->launches;
  rc = cycle_step<T>(ctx, hw, 1);
  ctx->sgraph.k_step = ctx->launches - l0;
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &body);
  ctx->stream = outer;
  if (rc) return rc;
  ECS_CUDA(ctx, ce);
  if ((rc = cycle_post<T>(ctx))) return rc;
  ecs_launch_pdl(k_axpy64_dev<T>, blocks_for(ctx, n), kB, 0, ctx->stream, n, sizeof(T) == 4 ? ctx->dots : nullptr,
                                                             cycle_x<T>(ctx), ctx->phi);
  ECS_LAUNCHED(ctx);
  if ((rc = project_mean<double>(ctx, ctx->phi))) return rc;
  ecs_launch_pdl(k_refine_update, 1, 32, 0, ctx->stream, (RefineDev *)ctx->rdev, (const KrylovDev *)ctx->kdev);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

// The nodes of one solve, appended to the graph being captured on
// ctx->stream:
//   [phi = 0, r = b | r = b - A phi]  ||r||  init  check
//   WHILE( scale  cycle(WHILE Arnoldi)  phi += e  update  residual  norm  check )
// The checks set the sweep loop's condition; everything stays on the device.
// The kernel counts of the head, a sweep and an Arnoldi step go to sgraph.
template <typename T>
int capture_solve(EcsCtx *ctx, double rtol, int max_it, int warm) {
  SolverGraph &sg = ctx->sgraph;
  const size_t n = ctx->ncell;
  const int64_t launches0 = ctx->launches;
  int rc;
  cudaError_t ce;
  cudaGraph_t top = nullptr;
  if ((rc = capture_graph(ctx, ctx->stream, &top))) return rc;
  if ((rc = norm64_dev(ctx, ctx->rhs, ctx->dots))) return rc;  // ||b||
  ecs_launch_pdl(k_solve_init, 1, 32, 0, ctx->stream, (RefineDev *)ctx->rdev, ctx->dots);
  ECS_LAUNCHED(ctx);
  if (identity_lhs(ctx)) {  // -lhs identity (ComputeIdentityLHS, src/lhs.c:11-23): phi = b exactly
    ECS_CUDA(ctx, cudaMemcpyAsync(ctx->phi, ctx->rhs, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    sg.k_head = ctx->launches - launches0;
    sg.k_sweep = sg.k_step = 0;
    return ECS_OK;
  }
  cudaGraphConditionalHandle hs;
  ECS_CUDA(ctx, cudaGraphConditionalHandleCreate(&hs, top, 0, cudaGraphCondAssignDefault));
  if (!warm) {  // phi = 0: the residual is b and its norm is known
    ECS_CUDA(ctx, cudaMemsetAsync(ctx->phi, 0, n * sizeof(double), ctx->stream));
    ECS_CUDA(ctx, cudaMemcpyAsync(ctx->r64, ctx->rhs, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    rc = refine_decide<T>(ctx, rtol, max_it, hs);
  } else {
    rc = refine_check<T>(ctx, rtol, max_it, hs);
  }
  if (rc) return rc;
  sg.k_head = ctx->launches - launches0;
  cudaGraph_t body = nullptr;
  if ((rc = capture_conditional(ctx, ctx->stream, hs, cudaGraphCondTypeWhile, &body))) return rc;
  cudaStream_t outer = ctx->stream;
  ctx->stream = ctx->capst[1];
  ce = cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) {
    ctx->stream = outer;
    return ecs_cuda_check(ctx, ce, "sweep capture");
  }
  const int64_t l1 = ctx->launches;
  rc = refine_correct<T>(ctx, 2);
  if (!rc) rc = refine_check<T>(ctx, rtol, max_it, hs);
  sg.k_sweep = ctx->launches - l1 - sg.k_step;
  ce = cudaStreamEndCapture(ctx->stream, &body);
  ctx->stream = outer;
  if (rc) return rc;
  ECS_CUDA(ctx, ce);
  return ECS_OK;
}

int ensure_capture_streams(EcsCtx *ctx) {
  for (auto &c : ctx->capst)
    if (!c) ECS_CUDA(ctx, cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking));
  return ECS_OK;
}

// The right-hand side (FP64-bound) on sst[3] beside the operator set-up
// (latency-bound) on the context's stream and sst[0..2]; both need only the
// moments, and the context's stream waits for both.
template <typename T>
int rhs_beside_setup(EcsCtx *ctx) {
  int rc = ensure_setup_streams(ctx);
  if (rc) return rc;
  if (identity_lhs(ctx)) return ecs_grid_rhs(ctx);
  cudaStream_t s0 = ctx->stream;
  ECS_CUDA(ctx, cudaEventRecord(ctx->sev[6], s0));
  ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->sst[3], ctx->sev[6], 0));
  ctx->stream = ctx->sst[3];
  rc = ecs_grid_rhs(ctx);
  ctx->stream = s0;
  if (rc) return rc;
  ECS_CUDA(ctx, cudaEventRecord(ctx->sev[7], ctx->sst[3]));
  if ((rc = mg_setup<T>(ctx))) return rc;
  ECS_CUDA(ctx, cudaStreamWaitEvent(s0, ctx->sev[7], 0));
  return ECS_OK;
}

// One solve as one graph (see capture_solve), built for (rtol, max_it, warm).
template <typename T>
int build_solve_graph(EcsCtx *ctx, double rtol, int max_it, int warm, int setup) {
  SolverGraph &sg = ctx->sgraph;
  if (sg.exec && sg.rtol == rtol && sg.max_it == max_it && sg.warm == warm && sg.setup == setup) return ECS_OK;
  free_graph(sg);
  int rc = ensure_capture_streams(ctx);
  if (rc) return rc;
  if (setup) {  // allocations happen before the capture
    if ((rc = ecs_solver_alloc(ctx))) return rc;
    if (!identity_lhs(ctx) && (rc = mg_alloc<T>(ctx))) return rc;
    if ((rc = ensure_setup_streams(ctx))) return rc;
  }
  const int64_t launches0 = ctx->launches;
  cudaStream_t user = ctx->stream;
  ctx->stream = ctx->capst[0];
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) {
    ctx->stream = user;
    return ecs_cuda_check(ctx, ce, "solve graph capture");
  }
  rc = ECS_OK;
  sg.k_pre = 0;
  if (setup) {
    rc = rhs_beside_setup<T>(ctx);
    sg.k_pre = ctx->launches - launches0;
  }
  if (!rc) rc = capture_solve<T>(ctx, rtol, max_it, warm);
  ce = cudaStreamEndCapture(ctx->stream, &g);
  ctx->stream = user;
  ctx->launches = launches0;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  ECS_CUDA(ctx, ce);
  sg.graph = g;
  ECS_CUDA(ctx, cudaGraphInstantiate(&sg.exec, g, 0));
  sg.rtol = rtol;
  sg.max_it = max_it;
  sg.warm = warm;
  sg.setup = setup;
  return ECS_OK;
}

// Launch the solve graph (asynchronous).
int solve_graph_launch(EcsCtx *ctx, double rtol, int max_it, int warm, int setup) {
  int rc = ctx->prec == ECS_PREC_FP64 ? build_solve_graph<double>(ctx, rtol, max_it, warm, setup)
                                      : build_solve_graph<float>(ctx, rtol, max_it, warm, setup);
  if (rc) return rc;
  ECS_CUDA(ctx, cudaGraphLaunch(ctx->sgraph.exec, ctx->stream));
  return ECS_OK;
}

// ---- stand-alone solve request ----------------------------------------------
// Fluxes of a loaded density (src/file-io.c:51-59: VecAXPY into a zeroed
// vector, so G_d = 0 + flux_scale_d * n), into the SoA moment planes 1..3.
__global__ void k_density_flux(size_t n, double f0, double f1, double f2, double *__restrict__ mom) {
  ECS_PDL_ENTRY();
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const double d = mom[c];
    mom[n + c] = __dadd_rn(0.0, __dmul_rn(f0, d));
    mom[2 * n + c] = __dadd_rn(0.0, __dmul_rn(f1, d));
    mom[3 * n + c] = __dadd_rn(0.0, __dmul_rn(f2, d));
  }
}

// The node that the last call captured on stream s.
int last_captured(EcsCtx *ctx, cudaStream_t s, cudaGraphNode_t *node) {
  cudaStreamCaptureStatus cs;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  ECS_CUDA(ctx, cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &deps, nullptr, &nd));
  if (nd != 1) return ecs_fail(ctx, ECS_ERR_CUDA, "capture: expected one tail node, found %zu", nd);
  *node = deps[0];
  return ECS_OK;
}

void free_request_graph(RequestGraph &rg) {
  if (rg.exec) cudaGraphExecDestroy(rg.exec);
  if (rg.graph) cudaGraphDestroy(rg.graph);
  rg.exec = nullptr;
  rg.graph = nullptr;
  rg.in_node = rg.out_node = nullptr;
}

// density -> moments -> RHS -> operator set-up -> solve -> phi, as one graph.
template <typename T>
int build_request_graph(EcsCtx *ctx, const double fs[3], double rtol, int max_it) {
  RequestGraph &rg = ctx->rgraph;
  if (rg.exec && rg.rtol == rtol && rg.max_it == max_it && rg.flux_scale[0] == fs[0] && rg.flux_scale[1] == fs[1] &&
      rg.flux_scale[2] == fs[2])
    return ECS_OK;
  free_request_graph(rg);
  const size_t n = ctx->ncell, bytes = n * sizeof(double);
  if (!rg.h_in) {
    ECS_CUDA(ctx, cudaMallocHost((void **)&rg.h_in, bytes));
    ECS_CUDA(ctx, cudaMallocHost((void **)&rg.h_out, bytes));
  }
  int rc;
  // allocations and one-time attributes outside the capture
  if ((rc = ecs_solver_alloc(ctx))) return rc;
  if (!identity_lhs(ctx) && (rc = mg_alloc<T>(ctx))) return rc;
  if ((rc = ensure_capture_streams(ctx))) return rc;
  if ((rc = ensure_setup_streams(ctx))) return rc;  // the set-up forks onto them inside the capture
  const int64_t launches0 = ctx->launches;
  cudaStream_t user = ctx->stream;
  ctx->stream = ctx->capst[0];
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) {
    ctx->stream = user;
    return ecs_cuda_check(ctx, ce, "request graph capture");
  }
  do {
    if ((ce = cudaMemcpyAsync(ctx->mom, rg.h_in, bytes, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess) {
      rc = ecs_cuda_check(ctx, ce, "density copy");
      break;
    }
    if ((rc = last_captured(ctx, ctx->stream, &rg.in_node))) break;
    ecs_launch_pdl(k_density_flux, blocks_for(ctx, n), kB, 0, ctx->stream, n, fs[0], fs[1], fs[2], ctx->mom);
    if ((ce = cudaGetLastError()) != cudaSuccess) {
      rc = ecs_cuda_check(ctx, ce, "kernel launch");
      break;
    }
    ctx->launches++;
    if ((rc = rhs_beside_setup<T>(ctx))) break;
    rg.k_pre = ctx->launches - launches0;
    if ((rc = capture_solve<T>(ctx, rtol, max_it, 0))) break;
    if ((ce = cudaMemcpyAsync(rg.h_out, ctx->phi, bytes, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess) {
      rc = ecs_cuda_check(ctx, ce, "potential copy");
      break;
    }
    if ((rc = last_captured(ctx, ctx->stream, &rg.out_node))) break;
    if ((ce = cudaMemcpyAsync(ctx->rdev_host, ctx->rdev, sizeof(RefineDev), cudaMemcpyDeviceToHost, ctx->stream)) !=
        cudaSuccess) {
      rc = ecs_cuda_check(ctx, ce, "status copy");
      break;
    }
  } while (0);
  ce = cudaStreamEndCapture(ctx->stream, &g);
  ctx->stream = user;
  ctx->launches = launches0;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    rg.in_node = rg.out_node = nullptr;
    return rc;
  }
  ECS_CUDA(ctx, ce);
  rg.graph = g;
  ECS_CUDA(ctx, cudaGraphInstantiate(&rg.exec, g, 0));
  rg.rtol = rtol;
  rg.max_it = max_it;
  for (int d = 0; d < 3; d++) rg.flux_scale[d] = fs[d];
  return ECS_OK;
}

// Page-locked (or registered) host memory: the copy engines read and write it
// directly.
bool host_pinned(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

}  // namespace

// ============================================================================
// entry points used by ecs_api.cu and ecs_grid.cu
// ============================================================================
int ecs_solver_alloc(EcsCtx *ctx) {
  size_t n = ctx->ncell;
  int m = ctx->krylov_m;
  if (!ctx->red) {
    ctx->nred = kSlots * 4096;
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->red, (size_t)ctx->nred * sizeof(double)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->dots, (size_t)(m + 2) * sizeof(double)));
    ECS_CUDA(ctx, cudaMallocHost((void **)&ctx->h_dots, (size_t)(m + 2) * sizeof(double)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->r64, n * sizeof(double)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->w64, n * sizeof(double)));
    ECS_CUDA(ctx, cudaMalloc(&ctx->kdev, sizeof(KrylovDev)));
    ECS_CUDA(ctx, cudaMemset(ctx->kdev, 0, sizeof(KrylovDev)));
    ECS_CUDA(ctx, cudaMallocHost(&ctx->kdev_host, sizeof(KrylovDev)));
    ECS_CUDA(ctx, cudaMallocHost(&ctx->kctl_host, sizeof(KrylovDev)));
    memset(ctx->kdev_host, 0, sizeof(KrylovDev));
    memset(ctx->kctl_host, 0, sizeof(KrylovDev));
    if (!identity_lhs(ctx)) ECS_CUDA(ctx, cudaMalloc((void **)&ctx->coef64, 11 * n * sizeof(double)));
    ECS_CUDA(ctx, cudaMalloc(&ctx->rdev, sizeof(RefineDev)));
    ECS_CUDA(ctx, cudaMemset(ctx->rdev, 0, sizeof(RefineDev)));
    ECS_CUDA(ctx, cudaMallocHost(&ctx->rdev_host, sizeof(RefineDev)));
    memset(ctx->rdev_host, 0, sizeof(RefineDev));
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

int ecs_solver_setup(EcsCtx *ctx) {
  int rc = ecs_solver_alloc(ctx);
  if (rc) return rc;
  if (!identity_lhs(ctx)) rc = ctx->prec == ECS_PREC_FP64 ? mg_setup<double>(ctx) : mg_setup<float>(ctx);
  if (rc) return rc;
  ctx->lhs_ready = true;
  return ECS_OK;
}

// Iterative refinement around FGMRES cycles.  Per refinement the host waits
// once, for the FP64 residual norm and the finished cycle's control block.
int ecs_solver_run(EcsCtx *ctx, double rtol, int max_it, int warm, EcsSolveStats *st, int setup,
                   EcsHostHook between, void *arg) {
  const bool graphs = ctx->use_graphs || identity_lhs(ctx);
  if (between && !graphs) {  // the host-driven loop waits on the device from its start
    const int rc_h = between(ctx, arg);
    if (rc_h) return rc_h;
    between = nullptr;
  }
  if (setup && !graphs) {  // the host-driven loop: RHS and set-up launched one by one
    int rc0 = ecs_grid_rhs(ctx);
    if (!rc0) rc0 = ecs_solver_setup(ctx);
    if (rc0) return rc0;
    setup = 0;
  }
  if (setup) ctx->lhs_ready = true;  // the graph sets the operator up before it solves
  if (!ctx->lhs_ready) return ecs_fail(ctx, ECS_ERR_STATE, "solve called before lhs");
  const size_t n = ctx->ncell;
  const EcsParams &p = ctx->p;
  const OpK o64 = make_op(p, p.Nx, p.Ny, p.Nz, p.dx, p.dy, p.dz);
  KrylovDev *hk = (KrylovDev *)ctx->kdev_host;
  if (!ctx->ev_solve[0]) {
    ECS_CUDA(ctx, cudaEventCreate(&ctx->ev_solve[0]));
    ECS_CUDA(ctx, cudaEventCreate(&ctx->ev_solve[1]));
  }
  ECS_CUDA(ctx, cudaEventRecord(ctx->ev_solve[0], ctx->stream));
  int rc;
  if (graphs) {  // the whole solve as one graph launch, one wait
    if ((rc = solve_graph_launch(ctx, rtol, max_it, warm, setup))) return rc;
    RefineDev *hr = (RefineDev *)ctx->rdev_host;
    ECS_CUDA(ctx, cudaMemcpyAsync(hr, ctx->rdev, sizeof(RefineDev), cudaMemcpyDeviceToHost, ctx->stream));
    ECS_CUDA(ctx, cudaEventRecord(ctx->ev_solve[1], ctx->stream));
    const int rc_h = between ? between(ctx, arg) : ECS_OK;
    ECS_CUDA(ctx, cudaEventSynchronize(ctx->ev_solve[1]));
    if (rc_h) return rc_h;
    const SolverGraph &sg = ctx->sgraph;
    ctx->launches += sg.k_pre + sg.k_head + hr->sweeps * sg.k_sweep + (int64_t)hr->its * sg.k_step;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev_solve[0], ctx->ev_solve[1]);
    if (st) {
      st->iterations = hr->its;
      st->refinements = hr->sweeps;
      st->relres = hr->rel;
      st->seconds = ms * 1e-3;
    }
    if (hr->nonfinite) return ecs_fail(ctx, ECS_ERR_NONFINITE, "non-finite residual in solve");
    if (hr->bnorm > 0.0 && hr->rel > rtol)
      return ecs_fail(ctx, ECS_ERR_NOT_CONVERGED, "solve stopped at relres %.3e > %.3e after %d iterations", hr->rel,
                      rtol, hr->its);
    return ECS_OK;
  }
  if (!warm) ECS_CUDA(ctx, cudaMemsetAsync(ctx->phi, 0, n * sizeof(double), ctx->stream));
  // ||b|| -> dots[0], 1/||b|| -> dots[1]
  if ((rc = norm64_dev(ctx, ctx->rhs, ctx->dots))) return rc;
  ECS_CUDA(ctx, cudaMemcpyAsync(ctx->h_dots, ctx->dots, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const double bnorm = ctx->h_dots[0];
  int its = 0, sweeps = 0;
  double rel = 0.0;
  bool cycle_pending = false;
  bool zero_guess = !warm;
  if (bnorm > 0.0) {
    for (;;) {
      if (zero_guess) {  // phi = 0: the residual is b, its norm (dots[0..1]) is known
        ECS_CUDA(ctx, cudaMemcpyAsync(ctx->r64, ctx->rhs, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        zero_guess = false;
      } else {
        ecs_launch_pdl(k_residual64, blocks3(o64.g), threads3(), 0, ctx->stream, o64, (const double *)ctx->coef64, ctx->phi, ctx->rhs, ctx->r64);
        ECS_LAUNCHED(ctx);
        if ((rc = norm64_dev(ctx, ctx->r64, ctx->dots))) return rc;
        ECS_CUDA(ctx, cudaMemcpyAsync(ctx->h_dots, ctx->dots, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        if (cycle_pending)
          ECS_CUDA(ctx, cudaMemcpyAsync(hk, ctx->kdev, sizeof(KrylovDev), cudaMemcpyDeviceToHost, ctx->stream));
        ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      }
      if (cycle_pending) {
        its += hk->nits;
        sweeps++;
        cycle_pending = false;
        if (hk->nits == 0) {
          rel = ctx->h_dots[0] / bnorm;
          break;
        }
      }
      const double rn = ctx->h_dots[0];
      rel = rn / bnorm;
      if (!isfinite(rel)) return ecs_fail(ctx, ECS_ERR_NONFINITE, "non-finite residual in solve");
      if (rel <= rtol || its >= max_it) break;
      const double tol_cycle = std::max(0.5 * rtol / rel, 1e-14);
      if (ctx->prec == ECS_PREC_FP64) {
        // the cycle solves A e = r64 directly (beta = ||r64||)
        if ((rc = fgmres_cycle<double>(ctx, tol_cycle, max_it - its))) return rc;
        ecs_launch_pdl(k_axpy64<double>, blocks_for(ctx, n), kB, 0, ctx->stream, n, 1.0, ctx->w64, ctx->phi);
      } else {
        float *r32 = cycle_b<float>(ctx), *e32 = cycle_x<float>(ctx);
        ecs_launch_pdl(k_scale_to<float>, blocks_for(ctx, n), kB, 0, ctx->stream, n, ctx->r64, ctx->dots + 1, r32);
        ECS_LAUNCHED(ctx);
        if ((rc = fgmres_cycle<float>(ctx, std::max(tol_cycle, 2e-6), max_it - its))) return rc;
        ecs_launch_pdl(k_axpy64<float>, blocks_for(ctx, n), kB, 0, ctx->stream, n, rn, e32, ctx->phi);
      }
      ECS_LAUNCHED(ctx);
      if ((rc = project_mean<double>(ctx, ctx->phi))) return rc;
      cycle_pending = true;
    }
  }
  ECS_CUDA(ctx, cudaEventRecord(ctx->ev_solve[1], ctx->stream));
  ECS_CUDA(ctx, cudaEventSynchronize(ctx->ev_solve[1]));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev_solve[0], ctx->ev_solve[1]);
  if (st) {
    st->iterations = its;
    st->refinements = sweeps;
    st->relres = rel;
    st->seconds = ms * 1e-3;
  }
  if (bnorm > 0.0 && rel > rtol)
    return ecs_fail(ctx, ECS_ERR_NOT_CONVERGED, "solve stopped at relres %.3e > %.3e after %d iterations", rel, rtol, its);
  return ECS_OK;
}

int ecs_operator_apply64(EcsCtx *ctx, const double *x, double *y) {
  const EcsParams &p = ctx->p;
  const OpK o64 = make_op(p, p.Nx, p.Ny, p.Nz, p.dx, p.dy, p.dz);
  if (identity_lhs(ctx)) {
    ECS_CUDA(ctx, cudaMemcpyAsync(y, x, ctx->ncell * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    return ECS_OK;
  }
  ecs_launch_pdl(k_apply<double>, blocks3(o64.g), threads3(), 0, ctx->stream, o64, op_density(ctx), x, nullptr, y, 0);
  ECS_LAUNCHED(ctx);
  return ECS_OK;
}

int ecs_solver_free(EcsCtx *ctx) {
  free_graph(ctx->sgraph);
  free_request_graph(ctx->rgraph);
  if (ctx->rgraph.h_in) cudaFreeHost(ctx->rgraph.h_in);
  if (ctx->rgraph.h_out) cudaFreeHost(ctx->rgraph.h_out);
  for (auto &c : ctx->capst)
    if (c) cudaStreamDestroy(c);
  for (auto &c : ctx->sst)
    if (c) cudaStreamDestroy(c);
  for (auto &e : ctx->sev)
    if (e) cudaEventDestroy(e);
  free_mg(ctx->mg64);
  free_mg(ctx->mg32);
  void *ptrs[] = {ctx->kv64, ctx->kz64, ctx->kv32, ctx->kz32, ctx->w64, ctx->r64, ctx->coef64, ctx->dots, ctx->red,
                  ctx->kdev, ctx->rdev};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  if (ctx->h_dots) cudaFreeHost(ctx->h_dots);
  if (ctx->kdev_host) cudaFreeHost(ctx->kdev_host);
  if (ctx->kctl_host) cudaFreeHost(ctx->kctl_host);
  if (ctx->rdev_host) cudaFreeHost(ctx->rdev_host);
  for (auto &e : ctx->ev_solve)
    if (e) cudaEventDestroy(e);
  return ECS_OK;
}

// ---- stand-alone solve requests ---------------------------------------------
int ecs_request_launch(EcsCtx *ctx, const double *density, double *phi, const double flux_scale[3], double rtol,
                       int max_it) {
  int rc = ctx->prec == ECS_PREC_FP64 ? build_request_graph<double>(ctx, flux_scale, rtol, max_it)
                                      : build_request_graph<float>(ctx, flux_scale, rtol, max_it);
  if (rc) return rc;
  RequestGraph &rg = ctx->rgraph;
  const size_t bytes = ctx->ncell * sizeof(double);
  const double *src = density;
  if (!host_pinned(density)) {
    memcpy(rg.h_in, density, bytes);
    src = rg.h_in;
  }
  rg.staged_out = !host_pinned(phi);
  rg.dst = phi;
  double *dst = rg.staged_out ? rg.h_out : phi;
  ECS_CUDA(ctx, cudaGraphExecMemcpyNodeSetParams1D(rg.exec, rg.in_node, ctx->mom, src, bytes, cudaMemcpyHostToDevice));
  ECS_CUDA(ctx, cudaGraphExecMemcpyNodeSetParams1D(rg.exec, rg.out_node, dst, ctx->phi, bytes, cudaMemcpyDeviceToHost));
  if (!ctx->ev_solve[0]) {
    ECS_CUDA(ctx, cudaEventCreate(&ctx->ev_solve[0]));
    ECS_CUDA(ctx, cudaEventCreate(&ctx->ev_solve[1]));
  }
  ECS_CUDA(ctx, cudaEventRecord(ctx->ev_solve[0], ctx->stream));
  ECS_CUDA(ctx, cudaGraphLaunch(rg.exec, ctx->stream));
  ECS_CUDA(ctx, cudaEventRecord(ctx->ev_solve[1], ctx->stream));
  ctx->moments_ready = true;
  ctx->lhs_ready = true;
  ctx->eext_ready = false;
  return ECS_OK;
}

int ecs_request_finish(EcsCtx *ctx, EcsSolveStats *st) {
  RequestGraph &rg = ctx->rgraph;
  const RefineDev *hr = (const RefineDev *)ctx->rdev_host;
  if (rg.staged_out) memcpy(rg.dst, rg.h_out, ctx->ncell * sizeof(double));
  const SolverGraph &sg = ctx->sgraph;
  ctx->launches += rg.k_pre + sg.k_head + hr->sweeps * sg.k_sweep + (int64_t)hr->its * sg.k_step;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev_solve[0], ctx->ev_solve[1]);
  if (st) {
    st->iterations = hr->its;
    st->refinements = hr->sweeps;
    st->relres = hr->rel;
    st->seconds = ms * 1e-3;
  }
  if (hr->nonfinite) return ecs_fail(ctx, ECS_ERR_NONFINITE, "non-finite residual in solve");
  if (hr->bnorm > 0.0 && hr->rel > rg.rtol)
    return ecs_fail(ctx, ECS_ERR_NOT_CONVERGED, "solve stopped at relres %.3e > %.3e after %d iterations", hr->rel,
                    rg.rtol, hr->its);
  return ECS_OK;
}
