// Structured-grid helpers shared by the grid and solver translation units:
// grid shape, ghost-aware loads, 3-D launch indexing (no integer division)
// and the 11-coefficient operator row of src/lhs.c:366-423.
#pragma once

#include "ecs_internal.cuh"

// FP64 arithmetic with every operation separately rounded (no contraction),
// for kernels that must match the reference's FP64 results operand for
// operand.
struct rd {
  double v;
};
__device__ __forceinline__ rd operator+(rd a, rd b) { return {__dadd_rn(a.v, b.v)}; }
__device__ __forceinline__ rd operator-(rd a, rd b) { return {__dsub_rn(a.v, b.v)}; }
__device__ __forceinline__ rd operator*(rd a, rd b) { return {__dmul_rn(a.v, b.v)}; }

struct GridG {
  int nx, ny, nz;
  int bc[3];  // 0 periodic, else ghosted (value 0 outside)
  size_t n;   // nx*ny*nz (at most 2^30)
};

// Value at (k,j,i) with the reference's ghost semantics: periodic wrap, or 0
// outside a ghosted (non-periodic) dimension.  Offsets are at most one grid
// length.
template <typename T>
__device__ __forceinline__ T gval(const T *__restrict__ F, const GridG &g, int k, int j, int i) {
  if (i < 0 || i >= g.nx) { if (g.bc[0]) return T(0); i = i < 0 ? i + g.nx : i - g.nx; }
  if (j < 0 || j >= g.ny) { if (g.bc[1]) return T(0); j = j < 0 ? j + g.ny : j - g.ny; }
  if (k < 0 || k >= g.nz) { if (g.bc[2]) return T(0); k = k < 0 ? k + g.nz : k - g.nz; }
  return F[((unsigned)k * g.ny + j) * g.nx + i];
}

// ---- 3-D launches: one thread per cell, (x, y) tiles of kTx x kTy, z from
// blockIdx.z.  No division anywhere in the index arithmetic.
constexpr int kTx = 32, kTy = 8;
static inline dim3 threads3() { return dim3(kTx, kTy, 1); }
static inline dim3 blocks3(int nx, int ny, int nz) {
  return dim3((unsigned)((nx + kTx - 1) / kTx), (unsigned)((ny + kTy - 1) / kTy), (unsigned)nz);
}
static inline dim3 blocks3(const GridG &g) { return blocks3(g.nx, g.ny, g.nz); }
__device__ __forceinline__ bool at3(int nx, int ny, int &i, int &j, int &k) {
  i = blockIdx.x * kTx + threadIdx.x;
  j = blockIdx.y * kTy + threadIdx.y;
  k = blockIdx.z;
  return i < nx && j < ny;
}
__device__ __forceinline__ unsigned lin3(const GridG &g, int i, int j, int k) {
  return ((unsigned)k * g.ny + j) * g.nx + i;
}
// Linear block index and thread index of a 3-D launch (for block partials).
__device__ __forceinline__ unsigned block_lin() {
  return (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
}
__device__ __forceinline__ int thread_lin() { return threadIdx.y * blockDim.x + threadIdx.x; }

// (i, j, k) of linear cell c, 32-bit (single-block loops over small levels).
__device__ __forceinline__ void cell_ijk(unsigned c, const GridG &g, int &i, int &j, int &k) {
  i = (int)(c % (unsigned)g.nx);
  unsigned r = c / (unsigned)g.nx;
  j = (int)(r % (unsigned)g.ny);
  k = (int)(r / (unsigned)g.ny);
}

// ---- operator (src/lhs.c:366-423), templated on the arithmetic type --------
struct OpK {
  GridG g;
  double sxx, syy, szz, sod;
  float fxx, fyy, fzz, fod;  // the same scales rounded to FP32 (FP32 rows)
  int unit;                  // density 1 at every stencil point, ghosts included (-lhs laplacian)
};
__device__ __forceinline__ void op_scales(const OpK &o, double &a, double &b, double &c, double &d) {
  a = o.sxx; b = o.syy; c = o.szz; d = o.sod;
}
__device__ __forceinline__ void op_scales(const OpK &o, float &a, float &b, float &c, float &d) {
  a = o.fxx; b = o.fyy; c = o.fzz; d = o.fod;
}

// Stencil offsets (di, dj, dk) of the 11 row entries, in the reference's
// order: x+, x-, y+, y-, z+, z-, (x+,y+), (x+,y-), (x-,y+), (x-,y-), centre.
__device__ __forceinline__ int off_i(int e) { return (e == 0 || e == 6 || e == 7) ? 1 : ((e == 1 || e == 8 || e == 9) ? -1 : 0); }
__device__ __forceinline__ int off_j(int e) { return (e == 2 || e == 6 || e == 8) ? 1 : ((e == 3 || e == 7 || e == 9) ? -1 : 0); }
__device__ __forceinline__ int off_k(int e) { return e == 4 ? 1 : (e == 5 ? -1 : 0); }

// 11 coefficients of a row in the order above, from the density at the
// centre and its six face neighbours.
template <typename T>
__device__ __forceinline__ void row11_vals(const OpK &o, T nijk, T nmjk, T npjk, T nimk, T nipk, T nijm, T nijp,
                                           T v[11]) {
  if (o.unit) nijk = nmjk = npjk = nimk = nipk = nijm = nijp = T(1);
  T sxx, syy, szz, sod;
  op_scales(o, sxx, syy, szz, sod);
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

// 11 coefficients of row (k,j,i) in the order above.
template <typename T>
__device__ __forceinline__ void row11(const T *__restrict__ n, const OpK &o, int i, int j, int k, T v[11]) {
  const GridG &g = o.g;
  row11_vals(o, gval(n, g, k, j, i), gval(n, g, k, j, i - 1), gval(n, g, k, j, i + 1), gval(n, g, k, j - 1, i),
             gval(n, g, k, j + 1, i), gval(n, g, k - 1, j, i), gval(n, g, k + 1, j, i), v);
}

// The neighbours of cell (i,j,k) as offsets from its linear index, with the
// ghost semantics of gval: a periodic axis wraps, a ghosted one reads 0 past
// its edge (valid flag false).  Computed once per cell, so that the row's 18
// loads need no wrap logic of their own.
struct Nbr {
  unsigned c;                   // linear index of the cell
  int xm, xp, ym, yp, zm, zp;   // offsets of the six face neighbours
  bool vxm, vxp, vym, vyp, vzm, vzp;
};
__device__ __forceinline__ Nbr nbr_of(const GridG &g, int i, int j, int k) {
  Nbr q;
  const int sy = g.nx, sz = g.nx * g.ny;
  q.c = ((unsigned)k * g.ny + j) * g.nx + i;
  q.xm = i > 0 ? -1 : g.nx - 1;
  q.xp = i < g.nx - 1 ? 1 : 1 - g.nx;
  q.ym = j > 0 ? -sy : (g.ny - 1) * sy;
  q.yp = j < g.ny - 1 ? sy : (1 - g.ny) * sy;
  q.zm = k > 0 ? -sz : (g.nz - 1) * sz;
  q.zp = k < g.nz - 1 ? sz : (1 - g.nz) * sz;
  q.vxm = i > 0 || !g.bc[0];
  q.vxp = i < g.nx - 1 || !g.bc[0];
  q.vym = j > 0 || !g.bc[1];
  q.vyp = j < g.ny - 1 || !g.bc[1];
  q.vzm = k > 0 || !g.bc[2];
  q.vzp = k < g.nz - 1 || !g.bc[2];
  return q;
}
template <typename T>
__device__ __forceinline__ T nval(const T *__restrict__ F, const Nbr &q, int off, bool valid) {
  return valid ? F[(unsigned)((int)q.c + off)] : T(0);
}
// The 11 coefficients of the row (the same operands as row11).
template <typename T>
__device__ __forceinline__ void row11_n(const T *__restrict__ n, const OpK &o, const Nbr &q, T v[11]) {
  row11_vals(o, n[q.c], nval(n, q, q.xm, q.vxm), nval(n, q, q.xp, q.vxp), nval(n, q, q.ym, q.vym),
             nval(n, q, q.yp, q.vyp), nval(n, q, q.zm, q.vzm), nval(n, q, q.zp, q.vzp), v);
}
// x at the row's 11 entries, in the order of off_i/off_j/off_k.
template <typename T>
__device__ __forceinline__ void row_x(const T *__restrict__ x, const Nbr &q, T xe[11]) {
  xe[0] = nval(x, q, q.xp, q.vxp);
  xe[1] = nval(x, q, q.xm, q.vxm);
  xe[2] = nval(x, q, q.yp, q.vyp);
  xe[3] = nval(x, q, q.ym, q.vym);
  xe[4] = nval(x, q, q.zp, q.vzp);
  xe[5] = nval(x, q, q.zm, q.vzm);
  xe[6] = nval(x, q, q.xp + q.yp, q.vxp && q.vyp);
  xe[7] = nval(x, q, q.xp + q.ym, q.vxp && q.vym);
  xe[8] = nval(x, q, q.xm + q.yp, q.vxm && q.vyp);
  xe[9] = nval(x, q, q.xm + q.ym, q.vxm && q.vym);
  xe[10] = x[q.c];
}

// (A x)(k,j,i)
template <typename T>
__device__ __forceinline__ T apply_row(const T *__restrict__ n, const T *__restrict__ x, const OpK &o, int i,
                                       int j, int k) {
  T v[11];
  row11(n, o, i, j, k, v);
  T s = T(0);
#pragma unroll
  for (int e = 0; e < 11; e++) s += v[e] * gval(x, o.g, k + off_k(e), j + off_j(e), i + off_i(e));
  return s;
}

// b - A_xy x at (k,j,i), A_xy = the 8 in-plane entries of the row.
template <typename T>
__device__ __forceinline__ T zline_rhs_at(const T *__restrict__ n, const T *__restrict__ b,
                                          const T *__restrict__ x, const OpK &o, int i, int j, int k,
                                          unsigned c) {
  T v[11];
  row11(n, o, i, j, k, v);
  T s = b[c];
#pragma unroll
  for (int e = 0; e < 10; e++) {
    if (e == 4 || e == 5) continue;
    s -= v[e] * gval(x, o.g, k, j + off_j(e), i + off_i(e));
  }
  return s;
}

// Operator scale factors for spacing (hx, hy, hz), src/lhs.c:366-375.  The
// constant-coefficient Laplacian of -lhs laplacian (ComputeLaplacianLHS3D,
// src/lhs.c:101-191: 1/h^2 off the diagonal, minus their sum on it, the same
// in boundary rows whose out-of-range columns are dropped) is this operator
// with kappa = 0, scale = 1 and the density 1 everywhere, ghost points
// included (`unit`): 2 * (1/(2 h^2)) equals 1/h^2 exactly.
static inline OpK make_op(const EcsParams &p, int nx, int ny, int nz, double hx, double hy, double hz) {
  OpK o;
  o.g.nx = nx; o.g.ny = ny; o.g.nz = nz;
  for (int d = 0; d < 3; d++) o.g.bc[d] = p.bc[d] == ECS_BC_PERIODIC ? 0 : 1;
  o.g.n = (size_t)nx * ny * nz;
  const bool lap = p.lhs_type == ECS_LHS_LAPLACIAN;
  double kappa = lap ? 0.0 : p.kappa_e, scale = lap ? 1.0 : p.scale;
  double hxx = 1.0 / (2.0 * hx * hx), hyy = 1.0 / (2.0 * hy * hy), hzz = 1.0 / (2.0 * hz * hz);
  double hod = 1.0 / (8.0 * hy * hx);
  o.sxx = scale * hxx;
  o.syy = scale * hyy;
  // 2-D (ComputeFullLHS2D src/lhs.c:194-335, ComputeLaplacianLHS2D
  // src/lhs.c:26-97): the same in-plane entries, no z coupling
  o.szz = p.ndim == 2 ? 0.0 : scale * (1 + kappa * kappa) * hzz;
  o.sod = scale * kappa * hod;
  o.fxx = (float)o.sxx; o.fyy = (float)o.syy; o.fzz = (float)o.szz; o.fod = (float)o.sod;
  o.unit = lap ? 1 : 0;
  return o;
}
static inline GridG make_grid(const EcsParams &p, int nx, int ny, int nz) {
  return make_op(p, nx, ny, nz, 1.0, 1.0, 1.0).g;
}
