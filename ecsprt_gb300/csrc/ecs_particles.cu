// Particle phase of the ECSPRT hot path on sm_103a.
//
//   push     BorisMoverBz3D + DifferenceVector3D   src/velocities.c:281-371,
//                                                  src/vector-math.c:596-722
//   collide  ScatterElastic                        src/collisions.c:9-167
//   move     UpdatePositions + ApplyBC             src/positions.c:436-472,
//                                                  src/boundaries.c:6-34
//   collect  Collect3DFluidMoments                 src/moments.c:108-226
//
// Two data layouts:
//   FP64 plain: absolute positions and velocities, FP64 SoA, reference
//     arithmetic operand for operand (separately rounded, no FMA), so push and
//     move agree bit for bit with the reference.
//   Mixed: packed int32 cell (i | j<<10 | k<<20) + FP32 in-cell offset in
//     [0,1) + FP32 velocity in one 32-byte record per ion (a DRAM sector, so
//     the sort's scattered writes never leave a sector half written),
//     counting-sorted by cell every few steps; the cells are counted by the
//     particle pass that precedes the sort.
//
// Deposition: every contribution is rounded to an integer multiple of 2^-S and
// added into int64 accumulators, so moments do not depend on the order of
// particles or atomics (bit-reproducible run to run).  A warp transposes its
// 32 x 32 contributions through shared memory and sums them per cell group, so
// cell-sorted particles issue about one atomic per node and field per warp.
//
// Collisions: the reference picks Nc random ions with replacement and accepts
// each attempt with the product of two uniforms below |vr|^2/vrm^2
// (PetscSqr(ran3()) expands to two draws).  Here every ion draws a Poisson
// number of attempts with mean rate = Nc / (np * <P_accept>), so the expected
// number of accepted collisions is Nc and each ion is chosen with probability
// proportional to its acceptance, as in the reference.  <P_accept> is
// measured (fixed-point, order independent) on every pass and used on the
// next one.  Random numbers come from Philox4x32-10 keyed by a hash of the
// particle's own state and the step index, so results do not depend on the
// particle order in memory.
#include <math.h>

#include <algorithm>

#include "ecs_internal.cuh"

namespace {

// ---- exact FP64 arithmetic: every operation separately rounded ------------
struct rd {
  double v;
};
__device__ __forceinline__ rd operator+(rd a, rd b) { return {__dadd_rn(a.v, b.v)}; }
__device__ __forceinline__ rd operator-(rd a, rd b) { return {__dsub_rn(a.v, b.v)}; }
__device__ __forceinline__ rd operator*(rd a, rd b) { return {__dmul_rn(a.v, b.v)}; }
__device__ __forceinline__ rd operator/(rd a, rd b) { return {__ddiv_rn(a.v, b.v)}; }

constexpr int kBlock = 256;

struct TileG {
  int ntx, nty, ntz;  // tiles per axis
};

// ---- deposit fixed point ---------------------------------------------------
// FP64: rint(v 2^S) by the FP64 conversion.
struct FixScale64 {
  double s;
  __device__ __forceinline__ long long put(double v) const { return __double2ll_rn(v * s); }
  // flux contribution v w
  __device__ __forceinline__ long long putvw(double v, double w) const { return put(v * w); }
};

// FP32: the same integer, rint(v 2^S) with |v 2^S| <= 2^38 (S = 38 on the
// mixed path), from FP32 adds and multiply-adds only (on sm_103 a
// float-to-int64 conversion issues on the narrow FP64 pipe).  With the split
// bit B = kFixSplit and H = rint(v 2^(S-B)), |H| <= 2^19:
//   v 2^S = H 2^B + r,  |r| <= 2^(B-1), r exact in FP32,
//   rint(v 2^S) = H 2^B + rint(r)   (2^B H is even, so ties round alike).
// Both integers come from adding the bias 1.5 * 2^23: for |t| <= 2^22,
// fl(t + bias) lies in [2^23, 2^24], where the spacing of floats is 1, so
// the addition rounds t to the nearest integer (ties to even; the bias is
// even) and the bit pattern of the sum is bits(bias) + rint(t).  H and
// rint(r) are each summed in int32: over at most kWindowMax contributions
// they cannot overflow.  This is the density's representation.
constexpr float kFixBias = 12582912.0f;  // 1.5 * 2^23
constexpr unsigned kFixBiasBits = 0x4B400000u;
constexpr int kFixSplit = 19;
struct FixScale32 {
  float s, s_hi, s_back;  // 2^S, 2^(S-B), -2^(B-S)
  // unbiased (H, rint(r))
  __device__ __forceinline__ void split(float v, int &hi, int &lo) const {
    const float h = __fmaf_rn(v, s_hi, kFixBias);
    const float r = __fmaf_rn(__fsub_rn(h, kFixBias), s_back, v);
    const float l = __fmaf_rn(r, s, kFixBias);
    hi = (int)(__float_as_uint(h) - kFixBiasBits);
    lo = (int)(__float_as_uint(l) - kFixBiasBits);
  }
  // biased words packed in one 64-bit entry (low word H, high word rint(r))
  __device__ __forceinline__ long long put(float v) const {
    const float h = __fmaf_rn(v, s_hi, kFixBias);
    const float r = __fmaf_rn(__fsub_rn(h, kFixBias), s_back, v);
    const float l = __fmaf_rn(r, s, kFixBias);
    return (long long)(((unsigned long long)__float_as_uint(l) << 32) | __float_as_uint(h));
  }
};
__device__ __forceinline__ long long fix_join(int hi, int lo) { return (long long)hi * (1ll << kFixSplit) + lo; }
// sums of n biased entries: remove n * bits(bias) from each word (wrap-around
// int32 arithmetic), then recombine in int64
__device__ __forceinline__ long long fix_unbias(unsigned hi_sum, unsigned lo_sum, int n) {
  return fix_join((int)(hi_sum - (unsigned)n * kFixBiasBits), (int)(lo_sum - (unsigned)n * kFixBiasBits));
}

// The flux in one word: rint(v 2^S) with |v 2^S| <= 2^22 (S = 22 - e_v on
// the mixed path, 2^e_v bounding |v|), from one FP32 multiply-add of the
// same bias (the fused product v 2^S is exact, then rounded once; the bias
// trick needs |t| <= 2^22).  The tile kernel's window sums these words in
// int32 only for ions whose velocity components are within 2^(e_v - 3)
// (words <= 2^19: kWindowMax x 2^19 < 2^31); faster ions add theirs to the
// int64 accumulators directly.
// A flux contribution v w is rounded once: with vs = v 2^S (exact), the
// fused multiply-add vs w + bias rounds the exact product to an integer.
struct FixWord32 {
  float s;  // 2^S
  // the biased word bits(bias) + rint(vs w)
  __device__ __forceinline__ unsigned biased(float vs, float w) const {
    return __float_as_uint(__fmaf_rn(vs, w, kFixBias));
  }
  __device__ __forceinline__ int word(float vs, float w) const { return (int)(biased(vs, w) - kFixBiasBits); }
  // the biased word in a 64-bit tile entry
  __device__ __forceinline__ long long putvw(float v, float w) const { return (long long)biased(v * s, w); }
};

// Exact sum of the tile entries q in `m` (bit mask of lanes).
__device__ __forceinline__ long long group_sum(const long long *row, unsigned m, const FixScale64 &) {
  long long sum = 0;
  while (m) {
    const int q = __ffs(m) - 1;
    m &= m - 1;
    sum += row[q];
  }
  return sum;
}
__device__ __forceinline__ long long group_sum(const long long *row, unsigned m, const FixScale32 &) {
  const int n = __popc(m);
  unsigned hs = 0, ls = 0;
  while (m) {
    const int q = __ffs(m) - 1;
    m &= m - 1;
    const unsigned long long e = (unsigned long long)row[q];
    hs += (unsigned)e;
    ls += (unsigned)(e >> 32);
  }
  return fix_unbias(hs, ls, n);
}
__device__ __forceinline__ long long group_sum(const long long *row, unsigned m, const FixWord32 &) {
  const int n = __popc(m);
  unsigned sum = 0;
  while (m) {
    const int q = __ffs(m) - 1;
    m &= m - 1;
    sum += (unsigned)row[q];
  }
  return (long long)(int)(sum - (unsigned)n * kFixBiasBits);
}
__device__ __forceinline__ long long full_sum(const long long *row, const FixScale64 &) {
  long long sum = 0;
#pragma unroll
  for (int q = 0; q < 32; q++) sum += row[q];
  return sum;
}
__device__ __forceinline__ long long full_sum(const long long *row, const FixScale32 &) {
  unsigned hs = 0, ls = 0;
#pragma unroll
  for (int q = 0; q < 32; q++) {
    const unsigned long long e = (unsigned long long)row[q];
    hs += (unsigned)e;
    ls += (unsigned)(e >> 32);
  }
  return fix_unbias(hs, ls, 32);
}
__device__ __forceinline__ long long full_sum(const long long *row, const FixWord32 &) {
  unsigned sum = 0;
#pragma unroll
  for (int q = 0; q < 32; q++) sum += (unsigned)row[q];
  return (long long)(int)(sum - 32u * kFixBiasBits);
}


struct PartK {
  int ndim;  // 2: ions in the z = 0 plane of a one-cell-deep grid (-ndim 2)
  int Nx, Ny, Nz;
  int bc[3];
  size_t ncell;
  double dx, dy, dz;
  double lo[3], hi[3], L[3];  // grid bounds (x0, x1, Lx per axis)
  // Boris constants, src/velocities.c:307-320
  double t, s, esc[3];
  float tf, sf, escf[3];
  double dt;
  float dtc[3];  // dt / cell width, FP32 (mixed move)
  // collisions, src/collisions.c:18-63
  int collide;
  double rate, vrm2, viT, vnT, vn0[3], mi, mn, M;
  // the same in FP32 (mixed path): attempt rate, 1/vrm^2, neutral thermal
  // speed and drift, mi/M, mn/M, 10 viT
  float ratef, ivrm2f, vnTf, vn0f[3], wif, wnf, vlimf;
  float p0f;          // exp(-rate)
  uint32_t stepmix;   // step and seed mixed for the attempt uniform
  uint32_t key0, key1, step;
  // fixed-point scales of the deposit: density 2^Sn, flux 2^Sf (Sf = Sn - e_v
  // for the velocity bound 2^e_v), and the bound itself
  double fixn64, fixf64;
  FixScale32 fixn32;  // density: two words
  FixWord32 fixf32;   // flux: one word
  double vmax;
  float vmaxf;
  float vwinf;  // vmax / 8: velocity components of ions deposited through the tile window
  TileG tg;
};

// ---- deposit ---------------------------------------------------------------
// Linear node index of corner b (xb = b&1, yb = b>>1&1, zb = b>>2) of cell
// (i,j,k), or -1 when it falls outside a non-periodic dimension.
__device__ __forceinline__ long long corner_node(const PartK &k, int i, int j, int kk, int b) {
  int ii = i + (b & 1), jj = j + ((b >> 1) & 1), zz = kk + (b >> 2);
  if (ii >= k.Nx) { if (k.bc[0]) return -1; ii -= k.Nx; }
  if (jj >= k.Ny) { if (k.bc[1]) return -1; jj -= k.Ny; }
  if (zz >= k.Nz) { if (k.bc[2]) return -1; zz -= k.Nz; }
  return ((long long)zz * k.Ny + jj) * k.Nx + ii;
}

// Deposit one particle's CIC contributions (src/moments.c:162-205): weights
// w_b = wz*wy*wx over the 8 corners (the reference's product order),
// density += w_b, flux_d += v_d*w_b, each rounded to an integer multiple of
// the field's fixed-point quantum.
//
// Warp aggregation: every lane writes its 32 values (slot = b + 8*field) to
// the warp's shared-memory tile, transposed so that lane l then reads slot l
// of all 32 lanes.  Lanes are grouped by cell (__match_any_sync); for each
// group lane l adds slot l over the group's lanes (exact int64) and issues
// one atomic for that node and field.  Any mix of cells in a warp is handled;
// cell-sorted ions give few groups and so few atomics.  `tile` is this warp's
// 32 x 33 int64 scratch (padded against bank conflicts).  All lanes of the
// warp must call this together.
constexpr int kTileStride = 33;

template <typename T, typename FixN, typename FixF>
__device__ __forceinline__ void deposit_warp(long long *__restrict__ acc, long long *tile, const PartK &k,
                                             bool active, int i, int j, int kk, T wxh, T wyh,
                                             T wzh, T v0, T v1, T v2, const FixN &fn, const FixF &ff) {
  const int lane = threadIdx.x & 31;
  const T wxl = T(1) - wxh, wyl = T(1) - wyh, wzl = T(1) - wzh;
  // inactive lanes contribute the zero entry (bias included for FP32)
  const long long zero_n = fn.put(T(0)), zero_f = ff.putvw(T(0), T(0));
#pragma unroll
  for (int b = 0; b < 8; b++) {
    const T wz = (b & 4) ? wzh : wzl, wy = (b & 2) ? wyh : wyl, wx = (b & 1) ? wxh : wxl;
    const T w = wz * wy * wx;
    tile[(b + 0) * kTileStride + lane] = active ? fn.put(w) : zero_n;
    tile[(b + 8) * kTileStride + lane] = active ? ff.putvw(v0, w) : zero_f;
    tile[(b + 16) * kTileStride + lane] = active ? ff.putvw(v1, w) : zero_f;
    tile[(b + 24) * kTileStride + lane] = active ? ff.putvw(v2, w) : zero_f;
  }
  const int key = active ? (i | (j << 10) | (kk << 20)) : -1;
  const unsigned peers = __match_any_sync(ECS_FULL_MASK, key);
  __syncwarp();
  const long long *row = tile + lane * kTileStride;
  unsigned rem = __ballot_sync(ECS_FULL_MASK, active);
  if (rem == ECS_FULL_MASK && peers == ECS_FULL_MASK) {
    // the whole warp deposits into one cell: plain 32-term sums
    const long long sum = lane < 8 ? full_sum(row, fn) : full_sum(row, ff);
    const long long node = corner_node(k, i, j, kk, lane & 7);
    if (node >= 0 && sum != 0)
      atomicAdd((unsigned long long *)&acc[(size_t)(lane >> 3) * k.ncell + node], (unsigned long long)sum);
    rem = 0;
  }
  while (rem) {
    const int lead = __ffs(rem) - 1;
    const unsigned grp = __shfl_sync(ECS_FULL_MASK, peers, lead);
    const int gi = __shfl_sync(ECS_FULL_MASK, i, lead);
    const int gj = __shfl_sync(ECS_FULL_MASK, j, lead);
    const int gk = __shfl_sync(ECS_FULL_MASK, kk, lead);
    rem &= ~grp;
    const long long sum = lane < 8 ? group_sum(row, grp, fn) : group_sum(row, grp, ff);
    const long long node = corner_node(k, gi, gj, gk, lane & 7);
    if (node >= 0 && sum != 0)
      atomicAdd((unsigned long long *)&acc[(size_t)(lane >> 3) * k.ncell + node], (unsigned long long)sum);
  }
  __syncwarp();
}

// ---- collisions --------------------------------------------------------------
__device__ __forceinline__ void state_hash(const uint32_t *w, int n, uint32_t &h0, uint32_t &h1) {
  // two multiply-xor chains over the state words, finalised by mixing
  uint32_t a = 0x811C9DC5u, b = 0x27D4EB2Fu;
  for (int q = 0; q < n; q++) {
    a = (a ^ w[q]) * 0x01000193u;
    b = b * 0x9E3779B1u + w[q];
  }
  h0 = ecs_mix32(a);
  h1 = ecs_mix32(b ^ h0);
}

template <typename T>
struct RMath;
template <>
struct RMath<float> {
  static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
  static __device__ __forceinline__ float log_(float x) { return logf(x); }
  static __device__ __forceinline__ void sincospi_(float x, float *s, float *c) { sincospif(x, s, c); }
  static __device__ __forceinline__ float u01(uint32_t a, uint32_t) { return ecs_u01f(a); }
};
template <>
struct RMath<double> {
  static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
  static __device__ __forceinline__ double log_(double x) { return log(x); }
  static __device__ __forceinline__ void sincospi_(double x, double *s, double *c) { sincospi(x, s, c); }
  static __device__ __forceinline__ double u01(uint32_t a, uint32_t b) { return ecs_u01d(a, b); }
};

// Acceptance probability of one attempt: P(U1*U2 < a) = a(1 - ln a), a < 1.
template <typename T>
__device__ __forceinline__ T accept_prob(T a) {
  if (a >= T(1)) return T(1);
  if (a <= T(0)) return T(0);
  return a * (T(1) - RMath<T>::log_(a));
}

// Acceptance-probability sample of one ion against one neutral drawn from
// its own stream (used only to seed the attempt rate before the first pass).
template <typename T>
__device__ float accept_sample(const PartK &k, uint32_t h0, uint32_t h1, T vx, T vy, T vz) {
  typedef RMath<T> M;
  EcsU4 e = ecs_philox({h0, h1, 0xFFFFFFFEu, k.step}, k.key0, k.key1);
  T r1 = M::sqrt_(T(-2) * M::log_(M::u01(e.x, e.x)));
  T r2 = M::sqrt_(T(-2) * M::log_(M::u01(e.z, e.z)));
  T s1, c1, s2, c2;
  M::sincospi_(T(2) * M::u01(e.y, e.y), &s1, &c1);
  M::sincospi_(T(2) * M::u01(e.w, e.w), &s2, &c2);
  T wx = vx - (r1 * c1 * T(k.vnT) + T(k.vn0[0]));
  T wy = vy - (r1 * s1 * T(k.vnT) + T(k.vn0[1]));
  T wz = vz - (r2 * c2 * T(k.vnT) + T(k.vn0[2]));
  return (float)accept_prob<T>((wx * wx + wy * wy + wz * wz) / T(k.vrm2));
}

// Collision constants in the arithmetic type of the pass.
template <typename T>
struct CollK;
template <>
struct CollK<float> {
  float rate, ivrm2, vnT, vn0[3], wi, wn, vlim;
  __device__ __forceinline__ explicit CollK(const PartK &k)
      : rate(k.ratef), ivrm2(k.ivrm2f), vnT(k.vnTf), vn0{k.vn0f[0], k.vn0f[1], k.vn0f[2]}, wi(k.wif),
        wn(k.wnf), vlim(k.vlimf) {}
};
template <>
struct CollK<double> {
  double rate, vrm2, vnT, vn0[3], mi, mn, M, viT;
  __device__ __forceinline__ explicit CollK(const PartK &k)
      : rate(k.rate), vrm2(k.vrm2), vnT(k.vnT), vn0{k.vn0[0], k.vn0[1], k.vn0[2]}, mi(k.mi), mn(k.mn), M(k.M),
        viT(k.viT) {}
};
// acceptance test U1 U2 < |vr|^2 / vrm^2, centre-of-mass velocity, refusal
__device__ __forceinline__ bool coll_accept(const CollK<float> &c, float u, float vrr2) { return u < vrr2 * c.ivrm2; }
__device__ __forceinline__ bool coll_accept(const CollK<double> &c, double u, double vrr2) { return u < vrr2 / c.vrm2; }
__device__ __forceinline__ float coll_vc(const CollK<float> &c, float vi, float vn) { return vi * c.wi + vn * c.wn; }
__device__ __forceinline__ double coll_vc(const CollK<double> &c, double vi, double vn) { return (vi * c.mi + vn * c.mn) / c.M; }
__device__ __forceinline__ bool coll_refuse(const CollK<float> &c, float vf2) { return sqrtf(vf2) > c.vlim; }
__device__ __forceinline__ bool coll_refuse(const CollK<double> &c, double vf2) { return sqrt(vf2) / c.viT > 10.0; }

// Gate uniform of one ion in one pass: a uniform from the hash `a` (the
// FP64 path: its state hash; the mixed path: its identity) mixed with the
// step and seed.  The ion makes at least one collision attempt when
// u > exp(-rate) (gate_open), the common case being none.
__device__ __forceinline__ float gate_uniform(const PartK &k, uint32_t a) {
  return ecs_u01f(ecs_mix32(a ^ k.stepmix));
}
__device__ __forceinline__ bool gate_open(const PartK &k, float u) { return u > k.p0f; }

// Counter words of the mixed path's collision streams: the ion's identity
// and a tag (the FP64 path keys by its 64-bit state hash instead).
constexpr uint32_t kIdTag = 0x49444B59u;

// One ion's collisions in one pass (src/collisions.c:70-157) once its gate is
// open: a Poisson number of attempts (rate k.rate) by inversion of the gate
// uniform u; each attempt draws a Maxwellian neutral from Philox keyed by
// (c0, c1, attempt, step), accepts with U1*U2 < |vr|^2/vrm^2, and scatters
// isotropically in the centre-of-mass frame.
template <typename T>
__device__ void collide_attempts(const PartK &k, uint32_t h0, uint32_t h1, float u, T &vx, T &vy, T &vz,
                                 unsigned int &nacc, unsigned int &nref) {
  typedef RMath<T> M;
  const CollK<T> ck(k);
  float p = k.p0f, cdf = p;
  const float rate = k.ratef;
  int natt = 0;
  while (u > cdf && natt < 16) {
    natt++;
    p *= rate / (float)natt;
    cdf += p;
  }
  for (int a = 0; a < natt; a++) {
    // neutral velocity: three normal deviates by Box-Muller
    EcsU4 q1 = ecs_philox({h0, h1, 2u * a, k.step}, k.key0, k.key1);
    EcsU4 q2 = ecs_philox({h0, h1, 2u * a + 1u, k.step}, k.key0, k.key1);
    T ra, rb, sa, ca, sb, cb;
    if (sizeof(T) == 4) {
      ra = M::sqrt_(T(-2) * M::log_(M::u01(q1.x, q1.x)));
      rb = M::sqrt_(T(-2) * M::log_(M::u01(q1.z, q1.z)));
      M::sincospi_(T(2) * M::u01(q1.y, q1.y), &sa, &ca);
      M::sincospi_(T(2) * M::u01(q1.w, q1.w), &sb, &cb);
    } else {
      EcsU4 q3 = ecs_philox({h0, h1, 0x40000000u + a, k.step}, k.key0, k.key1);
      ra = M::sqrt_(T(-2) * M::log_(M::u01(q1.x, q1.y)));
      rb = M::sqrt_(T(-2) * M::log_(M::u01(q3.x, q3.y)));
      M::sincospi_(T(2) * M::u01(q1.z, q1.w), &sa, &ca);
      M::sincospi_(T(2) * M::u01(q3.z, q3.w), &sb, &cb);
    }
    T vn[3] = {ra * ca * ck.vnT + ck.vn0[0], ra * sa * ck.vnT + ck.vn0[1], rb * cb * ck.vnT + ck.vn0[2]};
    T vi[3] = {vx, vy, vz};
    T vr[3] = {vi[0] - vn[0], vi[1] - vn[1], vi[2] - vn[2]};
    T vrr2 = vr[0] * vr[0] + vr[1] * vr[1] + vr[2] * vr[2];
    T U1 = M::u01(q2.x, q2.x), U2 = M::u01(q2.y, q2.y);
    if (!coll_accept(ck, U1 * U2, vrr2)) continue;
    T vrr = M::sqrt_(vrr2);
    T vc[3], tmp = T(0);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      vc[d] = coll_vc(ck, vi[d], vn[d]);
      tmp += (vi[d] - vc[d]) * (vi[d] - vc[d]);
    }
    T vcr = M::sqrt_(tmp);
    T u0z = T(2) * M::u01(q2.z, q2.z) - T(1);
    T uperp = M::sqrt_(T(1) - u0z * u0z);
    T sphi, cphi;
    M::sincospi_(T(2) * M::u01(q2.w, q2.w), &sphi, &cphi);
    T u0x = uperp * cphi, u0y = uperp * sphi;
    // frame of the incident relative velocity; when it lies along z (where
    // the reference divides 0 by 0) any azimuth is valid for an isotropic
    // scattering vector, so phi = 0 is used
    T costht = vr[2] / vrr;
    T s2 = T(1) - costht * costht;
    T sintht = s2 > T(0) ? M::sqrt_(s2) : T(0);
    T cosphi = T(1), sinphi = T(0);
    if (sintht > T(0)) {
      cosphi = vr[0] / (vrr * sintht);
      sinphi = vr[1] / (vrr * sintht);
    }
    T u1x = u0z * sintht + u0x * costht;
    T u1y = u0y;
    T u1z = u0z * costht - u0x * sintht;
    T u2[3] = {u1x * cosphi - u1y * sinphi, u1x * sinphi + u1y * cosphi, u1z};
    T vf[3], vf2 = T(0);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      vf[d] = vc[d] + vcr * u2[d];
      vf2 += vf[d] * vf[d];
    }
    if (coll_refuse(ck, vf2)) {
      nref++;
    } else {
      vx = vf[0];
      vy = vf[1];
      vz = vf[2];
      nacc++;
    }
  }
}

template <typename T>
__device__ __forceinline__ void collide_ion(const PartK &k, uint32_t h0, uint32_t h1, uint32_t a, T &vx, T &vy,
                                            T &vz, unsigned int &nacc, unsigned int &nref) {
  const float u = gate_uniform(k, a);
  if (gate_open(k, u)) collide_attempts<T>(k, h0, h1, u, vx, vy, vz, nacc, nref);
}

// Warp-aggregated status counters.
__device__ __forceinline__ void flush_counts(EcsDevStatus *st, unsigned int nacc, unsigned int nref) {
  unsigned int a = __reduce_add_sync(ECS_FULL_MASK, nacc);
  unsigned int r = __reduce_add_sync(ECS_FULL_MASK, nref);
  if ((threadIdx.x & 31) == 0) {
    if (a) atomicAdd(&st->collisions, (unsigned long long)a);
    if (r) atomicAdd(&st->refused, (unsigned long long)r);
  }
}
__device__ __forceinline__ void flush_samples(EcsDevStatus *st, float sample, bool has) {
  unsigned int f = __reduce_add_sync(ECS_FULL_MASK, has ? (unsigned int)__float2uint_rn(sample * 16777216.0f) : 0u);
  unsigned int n = __popc(__ballot_sync(ECS_FULL_MASK, has));
  if ((threadIdx.x & 31) == 0 && n) {
    atomicAdd(&st->acc_fix, (unsigned long long)f);
    atomicAdd(&st->acc_count, (unsigned long long)n);
  }
}

// ==========================================================================
// FP64 plain path
// ==========================================================================

// Difference numerators at the 8 corners, interpolated with the reference's
// weight order (src/vector-math.c:645-651): along y with wyh, across the z
// pair with wxh, across the x pair with wzh.  In 2-D the four corners of the
// z = 0 plane, along y with wyh, across x with wxh.
__device__ __forceinline__ void gather64(const double4_32a *__restrict__ E, const PartK &k, int i,
                                         int j, int kk, rd wx, rd wy, rd wz, rd f[3]) {
  const size_t sx = (size_t)k.Nx + 1, sxy = sx * ((size_t)k.Ny + 1);
  const size_t base = (size_t)kk * sxy + (size_t)j * sx + i;
  double4_32a D[8];
  D[0] = E[base];
  D[1] = E[base + 1];
  D[2] = E[base + sx];
  D[3] = E[base + sx + 1];
  D[4] = E[base + sxy];
  D[5] = E[base + sxy + 1];
  D[6] = E[base + sxy + sx];
  D[7] = E[base + sxy + sx + 1];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    rd v[8];
#pragma unroll
    for (int b = 0; b < 8; b++) v[b] = {c == 0 ? D[b].x : (c == 1 ? D[b].y : D[b].z)};
    // a[zb][xb] = D(zb,0,xb) + wy*(D(zb,1,xb) - D(zb,0,xb)); index b = zb*4+yb*2+xb
    rd a00 = v[0] + wy * (v[2] - v[0]);
    rd a01 = v[1] + wy * (v[3] - v[1]);
    rd a10 = v[4] + wy * (v[6] - v[4]);
    rd a11 = v[5] + wy * (v[7] - v[5]);
    if (k.ndim == 2) {  // DifferenceVector2D src/vector-math.c:576-591: bilinear, no swap
      f[c] = c == 2 ? rd{0.0} : a00 + wx * (a01 - a00);
      continue;
    }
    rd c0 = a00 + wx * (a10 - a00);
    rd c1 = a01 + wx * (a11 - a01);
    f[c] = c0 + wz * (c1 - c0);
  }
}

// Fractional grid coordinate and cell index along one axis; positions at
// exactly the upper bound (possible only when r + L rounds to L in the
// reference's single wrap) are folded onto the lower bound.
__device__ __forceinline__ bool cell_coord(double pos, double d, int N, rd &x, int &ix) {
  x = rd{pos} / rd{d};
  ix = (int)x.v;
  if (ix >= N) {
    x = x - rd{(double)N};
    ix -= N;
  }
  return ix >= 0 && ix < N && x.v >= 0.0;
}

__device__ __forceinline__ void push64(const PartK &k, const double4_32a *__restrict__ E, double px,
                                       double py, double pz, double &vx, double &vy, double &vz,
                                       bool &ok) {
  rd x, y, z;
  int i, j, kk;
  ok = cell_coord(px, k.dx, k.Nx, x, i) & cell_coord(py, k.dy, k.Ny, y, j) &
       cell_coord(pz, k.dz, k.Nz, z, kk);
  if (!ok) return;
  rd f[3];
  gather64(E, k, i, j, kk, x - rd{(double)i}, y - rd{(double)j}, z - rd{(double)kk}, f);
  rd vxm = rd{vx} + rd{k.esc[0]} * f[0];
  rd vym = rd{vy} + rd{k.esc[1]} * f[1];
  rd vzm = rd{vz} + rd{k.esc[2]} * f[2];
  rd vxt = vxm + vym * rd{k.t};
  rd vyp = vym - vxt * rd{k.s};
  rd vxp = vxt + vyp * rd{k.t};
  vx = vxp.v;
  vy = vyp.v;
  vz = vzm.v;
}

// src/positions.c:455-459 then src/boundaries.c:19-31 (one periodic wrap);
// reflecting axes reflect specularly.
__device__ __forceinline__ void move64(const PartK &k, double &p, double &v, int d) {
  rd r = rd{p} + rd{v} * rd{k.dt};
  if (k.bc[d] == ECS_BC_PERIODIC) {
    if (r.v < k.lo[d]) r = r + rd{k.L[d]};
    if (r.v >= k.hi[d]) r = r - rd{k.L[d]};
  } else {
    if (r.v < k.lo[d]) { r = rd{2.0 * k.lo[d]} - r; v = -v; }
    if (r.v >= k.hi[d]) { r = rd{2.0 * k.hi[d]} - r; v = -v; }
  }
  p = r.v;
}

__device__ __forceinline__ void deposit64(long long *acc, long long *tile, const PartK &k, bool active, double px,
                                          double py, double pz, double vx, double vy, double vz) {
  rd x{0}, y{0}, z{0};
  int i = 0, j = 0, kk = 0;
  bool ok = active;
  if (active)
    ok = cell_coord(px, k.dx, k.Nx, x, i) & cell_coord(py, k.dy, k.Ny, y, j) &
         cell_coord(pz, k.dz, k.Nz, z, kk);
  double wx = ok ? (x - rd{(double)i}).v : 0.0;
  double wy = ok ? (y - rd{(double)j}).v : 0.0;
  double wz = ok ? (z - rd{(double)kk}).v : 0.0;
  deposit_warp<double>(acc, tile, k, ok, i, j, kk, wx, wy, wz, vx, vy, vz, FixScale64{k.fixn64},
                       FixScale64{k.fixf64});
}

__device__ __forceinline__ void hash64(double px, double py, double pz, double vx, double vy,
                                       double vz, uint32_t &h0, uint32_t &h1) {
  uint32_t w[12];
  double s[6] = {px, py, pz, vx, vy, vz};
#pragma unroll
  for (int q = 0; q < 6; q++) {
    unsigned long long b = __double_as_longlong(s[q]);
    w[2 * q] = (uint32_t)b;
    w[2 * q + 1] = (uint32_t)(b >> 32);
  }
  state_hash(w, 12, h0, h1);
}

// mode bits: 1 push, 2 collide, 4 move, 8 deposit
__global__ void __launch_bounds__(kBlock) k_particles64(PartK k, int mode, int64_t np,
                                                        double *__restrict__ px,
                                                        double *__restrict__ py,
                                                        double *__restrict__ pz,
                                                        double *__restrict__ vxa,
                                                        double *__restrict__ vya,
                                                        double *__restrict__ vza,
                                                        const double4_32a *__restrict__ E,
                                                        long long *__restrict__ acc,
                                                        EcsDevStatus *st) {
  extern __shared__ long long shm_tiles[];
  long long *tile = shm_tiles + (threadIdx.x >> 5) * 32 * kTileStride;
  const int64_t lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < np;
       base += stride) {
    const int64_t ip = base + lane;
    const bool active = ip < np;
    double x = 0, y = 0, z = 0, vx = 0, vy = 0, vz = 0;
    if (active) {
      x = px[ip]; y = py[ip]; z = pz[ip];
      vx = vxa[ip]; vy = vya[ip]; vz = vza[ip];
    }
    bool ok = true;
    if ((mode & 1) && active) {
      push64(k, E, x, y, z, vx, vy, vz, ok);
      if (!ok) atomicOr(&st->flags, ECS_FLAG_RANGE);
    }
    unsigned int nacc = 0, nref = 0;
    if ((mode & 2) && k.collide) {
      if (active) {
        uint32_t h0, h1;
        hash64(x, y, z, vx, vy, vz, h0, h1);
        collide_ion<double>(k, h0, h1, h1, vx, vy, vz, nacc, nref);
      }
      flush_counts(st, nacc, nref);
    }
    if ((mode & 4) && active) {
      move64(k, x, vx, 0);
      move64(k, y, vy, 1);
      move64(k, z, vz, 2);
    }
    if (active && !(isfinite(vx) && isfinite(vy) && isfinite(vz))) atomicOr(&st->flags, ECS_FLAG_NONFINITE);
    if (mode & 8) {
      if (active && !(fabs(vx) <= k.vmax && fabs(vy) <= k.vmax && fabs(vz) <= k.vmax))
        atomicOr(&st->flags, ECS_FLAG_RANGE);
      deposit64(acc, tile, k, active, x, y, z, vx, vy, vz);
    }
    if (active) {
      if (mode & 4) { px[ip] = x; py[ip] = y; pz[ip] = z; }
      if (mode & 7) { vxa[ip] = vx; vya[ip] = vy; vza[ip] = vz; }
    }
  }
}

// ==========================================================================
// Mixed path
// ==========================================================================
__device__ __forceinline__ void unpack_cell(int32_t c, int &i, int &j, int &kk) {
  i = c & 1023;
  j = (c >> 10) & 1023;
  kk = (c >> 20) & 1023;
}

// Ion record ip: two float4 at ions[2 ip], ions[2 ip + 1].  The particle
// arrays are far larger than L2, so they are streamed (evict-first).  The
// last word carries the ion's identity: its index in the host arrays of the
// last upload (or in the device initialisation), which the kernels pass
// through unchanged, so that ions can be matched after the sort reorders
// them (ecs_particles_ids).
struct Ion {
  int32_t c;
  float ox, oy, oz, vx, vy, vz;
  int32_t id;
};
// A record moves as one 256-bit access (sm_100 and later): one load or
// store instruction a record instead of two 128-bit ones, which halves the
// record traffic's share of the SM's L1 data pipe (the tile kernel's busiest
// unit) and took the tile kernel from 3.96 to 3.56 ms at 128^3.
__device__ __forceinline__ void ld_record(const float4 *p, float4 &a, float4 &b) {
  asm volatile("ld.global.cs.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
               : "l"(p));
}
__device__ __forceinline__ Ion load_ion(const float4 *ions, int64_t ip) {
  float4 a, b;
  ld_record(ions + 2 * ip, a, b);
  return {__float_as_int(a.x), a.y, a.z, a.w, b.x, b.y, b.z, __float_as_int(b.w)};
}
__device__ __forceinline__ void store_ion(float4 *ions, int64_t ip, const Ion &q) {
  asm volatile("st.global.cs.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};\n" ::"l"(ions + 2 * ip),
               "f"(__int_as_float(q.c)), "f"(q.ox), "f"(q.oy), "f"(q.oz), "f"(q.vx), "f"(q.vy), "f"(q.vz),
               "f"(__int_as_float(q.id))
               : "memory");
}
__device__ __forceinline__ int32_t ion_cell(const float4 *ions, int64_t ip) {
  return __ldcs(reinterpret_cast<const int32_t *>(ions) + 8 * ip);
}
// Sort key of cell (i, j, k): tile-major (tiles of ECS_TILE_X x ECS_TILE_Y x
// ECS_TILE_Z cells, x fastest), then the cell within its tile.
__device__ __forceinline__ int tile_key(int i, int j, int k, const TileG &t) {
  const int tile = ((k / ECS_TILE_Z) * t.nty + j / ECS_TILE_Y) * t.ntx + i / ECS_TILE_X;
  return tile * ECS_TILE_CELLS + ((k % ECS_TILE_Z) * ECS_TILE_Y + j % ECS_TILE_Y) * ECS_TILE_X + i % ECS_TILE_X;
}
__device__ __forceinline__ int cell_key(int32_t c, const TileG &t) {
  return tile_key(c & 1023, (c >> 10) & 1023, (c >> 20) & 1023, t);
}

// Warp-aggregated count of the lanes' cells (inactive lanes pass key < 0).
__device__ __forceinline__ void count_cells(int32_t *__restrict__ count, int key) {
  const int lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(ECS_FULL_MASK, key);
  if (key >= 0 && lane == __ffs(peers) - 1) atomicAdd(&count[key], __popc(peers));
}

// Corner b (x: bit 0, y: bit 1, z: bit 2) of the cell whose low corner is
// at `base` of a node array with row stride sx and plane stride sxy.
__device__ __forceinline__ int corner_at(int base, int sx, int sxy, int b) {
  return base + (b & 1) + ((b >> 1) & 1) * sx + (b >> 2) * sxy;
}
// Trilinear interpolation of the 8 corner values D at offset (wx, wy, wz).
__device__ __forceinline__ void interp8(const float4 (&D)[8], float wx, float wy, float wz, float f[3]) {
#pragma unroll
  for (int c = 0; c < 3; c++) {
    float v[8];
#pragma unroll
    for (int b = 0; b < 8; b++) v[b] = c == 0 ? D[b].x : (c == 1 ? D[b].y : D[b].z);
    float a00 = v[0] + wy * (v[2] - v[0]);
    float a01 = v[1] + wy * (v[3] - v[1]);
    float a10 = v[4] + wy * (v[6] - v[4]);
    float a11 = v[5] + wy * (v[7] - v[5]);
    float c0 = a00 + wx * (a10 - a00);
    float c1 = a01 + wx * (a11 - a01);
    f[c] = c0 + wz * (c1 - c0);
  }
}
// The same in 2-D (four corners of the z = 0 plane, as gather64).
__device__ __forceinline__ void interp4(const float4 (&D)[8], float wx, float wy, float f[3]) {
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const float v0 = c == 0 ? D[0].x : D[0].y, v1 = c == 0 ? D[1].x : D[1].y;
    const float v2 = c == 0 ? D[2].x : D[2].y, v3 = c == 0 ? D[3].x : D[3].y;
    const float a00 = v0 + wy * (v2 - v0);
    const float a01 = v1 + wy * (v3 - v1);
    f[c] = a00 + wx * (a01 - a00);
  }
  f[2] = 0.0f;
}
__device__ __forceinline__ void gather32(const float4 *__restrict__ E, const PartK &k, int i, int j, int kk,
                                         float wx, float wy, float wz, float f[3]) {
  const int sx = k.Nx + 1, sxy = sx * (k.Ny + 1), base = kk * sxy + j * sx + i;
  float4 D[8];
  if (k.ndim == 2) {
#pragma unroll
    for (int b = 0; b < 4; b++) D[b] = __ldg(&E[corner_at(base, sx, sxy, b)]);
    interp4(D, wx, wy, f);
    return;
  }
#pragma unroll
  for (int b = 0; b < 8; b++) D[b] = __ldg(&E[corner_at(base, sx, sxy, b)]);
  interp8(D, wx, wy, wz, f);
}

// Advance an in-cell offset by du (cell units); returns the cell shift.
__device__ __forceinline__ int advance(float &o, float du) {
  float q = o + du;
  float fl = floorf(q);
  int sh = (int)fl;
  q = q - fl;
  if (q >= 1.0f) {  // q - floor(q) rounded up to 1 for tiny negative q
    q = 0.0f;
    sh += 1;
  }
  o = q;
  return sh;
}

// Apply the boundary condition to an integer cell coordinate along one axis.
__device__ __forceinline__ bool bound_axis(int bc, int N, int &c, float &o, float &v) {
  if (c >= 0 && c < N) return true;
  if (bc == ECS_BC_PERIODIC) {
    c %= N;
    if (c < 0) c += N;
    return true;
  }
  // specular reflection: position c + o mirrored about 0 or N
  if (c < 0) {
    c = -c - 1;
    o = 1.0f - o;
  } else {
    c = 2 * N - c - 1;
    o = 1.0f - o;
  }
  if (o >= 1.0f) { o = 0.0f; c += 1; }
  // a position exactly on the upper wall mirrors onto itself: keep it in the
  // last cell, one FP32 step below the wall
  if (c == N) { c = N - 1; o = 0x1.fffffep-1f; }
  v = -v;
  return c >= 0 && c < N;
}


constexpr int kWX = ECS_TILE_X + 3, kWY = ECS_TILE_Y + 3, kWZ = ECS_TILE_Z + 3;  // window nodes per axis
constexpr int kWNodes = kWX * kWY * kWZ;
// Padded strides of the field window's x and y numerators (a float2 a node;
// the z numerators are kept apart, at the deposit window's strides below).
// An 8-byte shared load is served 16 lanes at a time; with the ions sorted,
// those 16 lanes sit in the 4 x 4 cells of one z plane, and lx + 12 ly takes
// 16 different values mod 16 there, so the eight corner loads are free of
// bank conflicts.  Three words a corner instead of a padded float4 take a
// quarter of the window's load traffic off the shared-memory pipe.
constexpr int kEX = 12, kEXY = kEX * kWY;
static_assert(kWX <= kEX, "field window stride");
// Padded strides of the deposit window: the 32 cells of a tile (one lane
// each when the ions are sorted) map to 32 different shared-memory banks,
// lx + 12 ly + 112 lz taking every value mod 32 once for lx, ly < 4, lz < 2.
constexpr int kSY = 12, kSZ = 112;
constexpr int kWPad = kSZ * kWZ;
static_assert(kWX <= kSY && kWY * kSY <= kSZ, "window strides");
constexpr int kCX = ECS_TILE_X + 2, kCY = ECS_TILE_Y + 2, kCZ = ECS_TILE_Z + 2;  // window cells per axis
constexpr int kWCells = kCX * kCY * kCZ;
// |H| <= 2^19 and |rint(r)| <= 2^18, so 4000 contributions to one word stay
// below 2^31
constexpr int kWindowMax = 4000;  // ions between window flushes (flux words <= 2^19: 4000 x 2^19 < 2^31)

// Push (src/velocities.c:281-371), collisions (src/collisions.c:9-167) and
// move + boundary conditions (src/positions.c:436-472) of one ion, in the
// pass's mode bits.  Returns the ion in cell (i, j, kk) with offsets o*.
struct IonState {
  int i, j, kk;
  float ox, oy, oz, vx, vy, vz;
  int id;
};
// Push (src/velocities.c:281-371) of one ion.  Exy, Ez (nullptr: none) are a
// window of the difference numerators in shared memory, kWX x kWY x kWZ nodes
// from node (wx0, wy0, wz0): x and y at strides kEX, kEXY, z at kSY, kSZ.
__device__ __forceinline__ void ion_push(const PartK &k, const float4 *__restrict__ E, IonState &q,
                                         const float2 *Exy = nullptr, const float *Ez = nullptr, int wx0 = 0,
                                         int wy0 = 0, int wz0 = 0) {
  float f[3];
  const int li = q.i - wx0, lj = q.j - wy0, lk = q.kk - wz0;
  if (Exy && li >= 0 && li < kCX && lj >= 0 && lj < kCY && lk >= 0 && lk < kCZ) {
    const int bxy = lk * kEXY + lj * kEX + li, bz = lk * kSZ + lj * kSY + li;
    float4 D[8];
#pragma unroll
    for (int b = 0; b < 8; b++) {
      const float2 xy = Exy[corner_at(bxy, kEX, kEXY, b)];
      D[b] = make_float4(xy.x, xy.y, Ez[corner_at(bz, kSY, kSZ, b)], 0.f);
    }
    interp8(D, q.ox, q.oy, q.oz, f);
  } else {
    gather32(E, k, q.i, q.j, q.kk, q.ox, q.oy, q.oz, f);
  }
  float vxm = q.vx + k.escf[0] * f[0];
  float vym = q.vy + k.escf[1] * f[1];
  float vzm = q.vz + k.escf[2] * f[2];
  float vxt = vxm + vym * k.tf;
  float vyp = vym - vxt * k.sf;
  float vxp = vxt + vyp * k.tf;
  q.vx = vxp;
  q.vy = vyp;
  q.vz = vzm;
}

// Move + boundary conditions (src/positions.c:436-472, src/boundaries.c:6-34)
// in the pass's mode, then the velocity checks.
__device__ __forceinline__ void ion_move(const PartK &k, int mode, EcsDevStatus *st, IonState &q) {
  if (mode & 4) {
    q.i += advance(q.ox, q.vx * k.dtc[0]);
    q.j += advance(q.oy, q.vy * k.dtc[1]);
    q.kk += advance(q.oz, q.vz * k.dtc[2]);
    const bool inside = bound_axis(k.bc[0], k.Nx, q.i, q.ox, q.vx) & bound_axis(k.bc[1], k.Ny, q.j, q.oy, q.vy) &
                        bound_axis(k.bc[2], k.Nz, q.kk, q.oz, q.vz);
    if (!inside) {
      atomicOr(&st->flags, ECS_FLAG_RANGE);
      q.i = min(max(q.i, 0), k.Nx - 1);
      q.j = min(max(q.j, 0), k.Ny - 1);
      q.kk = min(max(q.kk, 0), k.Nz - 1);
    }
  }
  if (!(isfinite(q.vx) && isfinite(q.vy) && isfinite(q.vz))) atomicOr(&st->flags, ECS_FLAG_NONFINITE);
  if ((mode & 8) && !(fabsf(q.vx) <= k.vmaxf && fabsf(q.vy) <= k.vmaxf && fabsf(q.vz) <= k.vmaxf))
    atomicOr(&st->flags, ECS_FLAG_RANGE);
}

// Push, collisions (src/collisions.c:9-167; keyed by the ion's identity) and
// move of one ion in the pass's mode bits.
__device__ __forceinline__ void ion_update(const PartK &k, int mode, const float4 *__restrict__ E, EcsDevStatus *st,
                                           IonState &q, unsigned int &nacc, unsigned int &nref) {
  if (mode & 1) ion_push(k, E, q);
  if ((mode & 2) && k.collide)
    collide_ion<float>(k, (uint32_t)q.id, kIdTag, (uint32_t)q.id, q.vx, q.vy, q.vz, nacc, nref);
  ion_move(k, mode, st, q);
}
__device__ __forceinline__ IonState ion_state(const Ion &r) {
  IonState q;
  unpack_cell(r.c, q.i, q.j, q.kk);
  q.ox = r.ox; q.oy = r.oy; q.oz = r.oz; q.vx = r.vx; q.vy = r.vy; q.vz = r.vz;
  q.id = r.id;
  return q;
}
__device__ __forceinline__ Ion ion_record(const IonState &q) {
  return {q.i | (q.j << 10) | (q.kk << 20), q.ox, q.oy, q.oz, q.vx, q.vy, q.vz, q.id};
}

// Any ion order: grid-stride over ions, deposit by warp-level cell groups
// (deposit_warp) into global int64 accumulators.
__global__ void __launch_bounds__(kBlock, 3) k_particles32(PartK k, int mode, int64_t np, float4 *ions,
                                                         const float4 *__restrict__ E,
                                                         long long *__restrict__ acc,
                                                         int32_t *__restrict__ count, int32_t *__restrict__ keys,
                                                         EcsDevStatus *st) {
  extern __shared__ long long shm_tiles[];
  long long *tile = shm_tiles + (threadIdx.x >> 5) * 32 * kTileStride;
  const int64_t lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < np;
       base += stride) {
    const int64_t ip = base + lane;
    const bool active = ip < np;
    IonState q = ion_state(active ? load_ion(ions, ip) : Ion{0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0});
    unsigned int nacc = 0, nref = 0;
    if (active) ion_update(k, mode, E, st, q, nacc, nref);
    if ((mode & 2) && k.collide) flush_counts(st, nacc, nref);
    if (count) {
      const int key = active ? tile_key(q.i, q.j, q.kk, k.tg) : -1;
      if (active) keys[ip] = key;
      count_cells(count, key);
    }
    if (mode & 8)
      deposit_warp<float>(acc, tile, k, active, q.i, q.j, q.kk, q.ox, q.oy, q.oz, q.vx, q.vy, q.vz, k.fixn32,
                          k.fixf32);
    if (active && (mode & 7)) store_ion(ions, ip, ion_record(q));
  }
}

// ---- tile kernel: ions ordered by tile ----------------------------------------
// One block per tile of cells processes the ions of the tile's key range
// (the ions that were in the tile at the last sort) in chunks of at most
// kWindowMax.  Each chunk deposits into a shared-memory window of the nodes
// of the tile's cells widened by one cell on every side: five int32 words a
// contribution (the density's two fixed-point words H, rint(r) and one word
// for each flux component), added with shared-memory atomics as biased
// words (bits(bias) + value; the bias of every contribution is taken out at
// the flush from per-cell counts of the window's ions), and the window is
// added to the global int64 accumulators once per chunk.  The chunk is split
// into 32 consecutive segments, one per lane, so the lanes of a warp work on
// different cells and rarely on the same node.  Ions outside the window
// (moved farther, or wrapped around a periodic edge) deposit straight into
// the global accumulators.  The cells of the moved ions are counted the same
// way when a sort follows.
//
// Loads: each thread's next ion record is loaded into registers (one
// 256-bit load) while it works on the current one, with the permutation
// entry of the one after that loaded a step earlier, so the memory latency
// of a record overlaps the arithmetic of the previous ion.  All sums are
// exact integers, so the moments equal those of k_particles32 bit for bit.

// Block shape of the tile kernel: one block a tile.
constexpr int kTileThreads = 256;
constexpr int kTileBlocksPerSM = 4;

struct TileCtx {
  int wx0, wy0, wz0;  // window origin (node and cell index of its corner)
};

__device__ __forceinline__ bool in_cell_window(int li, int lj, int lk) {
  return li >= 0 && li < kCX && lj >= 0 && lj < kCY && lk >= 0 && lk < kCZ;
}

// The rest of one ion's pass after its push and collisions: move + BC and
// checks, the cell count for the next sort, the deposit, and the record.
__device__ __forceinline__ void tile_finish(const PartK &k, int mode, EcsDevStatus *st, IonState &q, int64_t ip,
                                            const TileCtx &tc, unsigned (*win)[kWPad], int *dcnt, int *wcnt,
                                            long long *__restrict__ acc, int32_t *__restrict__ count,
                                            int32_t *__restrict__ keys, float4 *dst) {
  ion_move(k, mode, st, q);
  const int li = q.i - tc.wx0, lj = q.j - tc.wy0, lk = q.kk - tc.wz0;
  const bool inwin = in_cell_window(li, lj, lk);
  if (count) {
    const int key = tile_key(q.i, q.j, q.kk, k.tg);
    keys[ip] = key;
    if (inwin) atomicAdd(&wcnt[(lk * kCY + lj) * kCX + li], 1);
    else atomicAdd(&count[key], 1);
  }
  if (mode & 8) {
    const float wxh = q.ox, wyh = q.oy, wzh = q.oz;
    const float wxl = 1.f - wxh, wyl = 1.f - wyh, wzl = 1.f - wzh;
    // weights w = (wz wy) wx, the product order of deposit_warp
    const float wzy[4] = {wzl * wyl, wzl * wyh, wzh * wyl, wzh * wyh};
    const float s = k.fixf32.s;
    const float vxs = q.vx * s, vys = q.vy * s, vzs = q.vz * s;  // exact: s is a power of two
    if (inwin && fabsf(q.vx) <= k.vwinf && fabsf(q.vy) <= k.vwinf && fabsf(q.vz) <= k.vwinf) {
      const int n0 = lk * kSZ + lj * kSY + li;
      atomicAdd(&dcnt[(lk * kCY + lj) * kCX + li], 1);
#pragma unroll
      for (int bc = 0; bc < 8; bc++) {
        const float w = wzy[bc >> 1] * ((bc & 1) ? wxh : wxl);
        const int nb = n0 + (bc >> 2) * kSZ + ((bc >> 1) & 1) * kSY + (bc & 1);
        const float h = __fmaf_rn(w, k.fixn32.s_hi, kFixBias);
        const float r = __fmaf_rn(__fsub_rn(h, kFixBias), k.fixn32.s_back, w);
        atomicAdd(&win[0][nb], __float_as_uint(h));
        atomicAdd(&win[1][nb], __float_as_uint(__fmaf_rn(r, k.fixn32.s, kFixBias)));
        atomicAdd(&win[2][nb], k.fixf32.biased(vxs, w));
        atomicAdd(&win[3][nb], k.fixf32.biased(vys, w));
        atomicAdd(&win[4][nb], k.fixf32.biased(vzs, w));
      }
    } else {  // outside the window, or fast: straight into the global accumulators
#pragma unroll 1
      for (int bc = 0; bc < 8; bc++) {
        const long long gnode = corner_node(k, q.i, q.j, q.kk, bc);
        if (gnode < 0) continue;
        const float w = (((bc & 4) ? wzh : wzl) * ((bc & 2) ? wyh : wyl)) * ((bc & 1) ? wxh : wxl);
        int hi, lo;
        k.fixn32.split(w, hi, lo);
        atomicAdd((unsigned long long *)&acc[gnode], (unsigned long long)fix_join(hi, lo));
        atomicAdd((unsigned long long *)&acc[k.ncell + gnode], (unsigned long long)(long long)k.fixf32.word(vxs, w));
        atomicAdd((unsigned long long *)&acc[2 * k.ncell + gnode], (unsigned long long)(long long)k.fixf32.word(vys, w));
        atomicAdd((unsigned long long *)&acc[3 * k.ncell + gnode], (unsigned long long)(long long)k.fixf32.word(vzs, w));
      }
    }
  }
  if (mode & 7) store_ion(dst, ip, ion_record(q));
}

__global__ void __launch_bounds__(kTileThreads, kTileBlocksPerSM) k_tiles32(PartK k, int mode, const float4 *src, float4 *dst,
                                                     const int32_t *__restrict__ perm, const float4 *__restrict__ E,
                                                     long long *__restrict__ acc, const int32_t *__restrict__ key_off,
                                                     int32_t *__restrict__ count, int32_t *__restrict__ keys,
                                                     EcsDevStatus *st, int t_begin, int t_end) {
  __shared__ unsigned win[5][kWPad];  // biased words [H, rint(r), flux x, y, z][node, padded strides]
  __shared__ int wcnt[kWCells];       // cells of the moved ions (next sort)
  __shared__ int dcnt[kWCells];       // window deposits a cell (bias removal)
  __shared__ float2 ewxy[kEXY * kWZ];  // x, y difference numerators of the window's nodes (padded strides)
  __shared__ float ewz[kWPad];         // z numerators, at the deposit window's strides
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool collide = (mode & 2) && k.collide;
  unsigned int nacc = 0, nref = 0;  // collision counters of this thread, flushed at the end
  for (int t = t_begin + blockIdx.x; t < t_end; t += gridDim.x) {
    const int tx = t % k.tg.ntx, ty = (t / k.tg.ntx) % k.tg.nty, tz = t / (k.tg.ntx * k.tg.nty);
    // window origin: one cell below the tile on every axis
    const TileCtx tc{tx * ECS_TILE_X - 1, ty * ECS_TILE_Y - 1, tz * ECS_TILE_Z - 1};
    const int a = key_off[t * ECS_TILE_CELLS], b = key_off[(t + 1) * ECS_TILE_CELLS];
    if (a == b) continue;
    for (int ca = a; ca < b; ca += kWindowMax) {
      const int L = min(kWindowMax, b - ca);
      const int seg = (L + 31) >> 5;               // lane segment
      const int sub = (seg + kTileThreads / 32 - 1) / (kTileThreads / 32);  // a warp's run inside each segment
      // this thread's ions: m = 0 .. sub-1 at qi = lane * seg + warp * sub + m
      const int qi0 = lane * seg + warp * sub;
      const int mend = min(sub, min(seg - warp * sub, L - qi0));  // active iterations (may be <= 0)
      auto src_pos = [&](int m) -> int64_t {
        const int64_t ip = (int64_t)ca + qi0 + m;
        return perm ? (int64_t)__ldg(perm + ip) : ip;
      };
      // the chunk's first record (and the permutation entry of the second)
      // are requested before the window set-up, which hides their latency
      int64_t sp_next = 0;
      float4 na = make_float4(0.f, 0.f, 0.f, 0.f), nb4 = na;  // the next record
      if (mend > 0) ld_record(src + 2 * src_pos(0), na, nb4);
      if (mend > 1) sp_next = src_pos(1);
      if ((mode & 1) && ca == a) {  // window nodes outside the extended grid are never read
        const int sx = k.Nx + 1, sxy = sx * (k.Ny + 1);
        for (int e = threadIdx.x; e < kWNodes; e += blockDim.x) {
          const int gx = tc.wx0 + e % kWX, gy = tc.wy0 + (e / kWX) % kWY, gz = tc.wz0 + e / (kWX * kWY);
          const bool in = gx >= 0 && gx <= k.Nx && gy >= 0 && gy <= k.Ny && gz >= 0 && gz <= k.Nz;
          const float4 v = in ? __ldg(&E[gz * sxy + gy * sx + gx]) : make_float4(0.f, 0.f, 0.f, 0.f);
          ewxy[(gz - tc.wz0) * kEXY + (gy - tc.wy0) * kEX + (gx - tc.wx0)] = make_float2(v.x, v.y);
          ewz[(gz - tc.wz0) * kSZ + (gy - tc.wy0) * kSY + (gx - tc.wx0)] = v.z;
        }
      }
      if (mode & 8) {
        for (int e = threadIdx.x; e < 5 * kWPad; e += blockDim.x) (&win[0][0])[e] = 0u;
        for (int e = threadIdx.x; e < kWCells; e += blockDim.x) dcnt[e] = 0;
      }
      if (count)
        for (int e = threadIdx.x; e < kWCells; e += blockDim.x) wcnt[e] = 0;
      __syncthreads();
      for (int m = 0; m < mend; m++) {
        const float4 ra = na, rb = nb4;
        if (m + 1 < mend) {  // the next record, in flight while this one is worked on
          ld_record(src + 2 * sp_next, na, nb4);
          if (m + 2 < mend) sp_next = src_pos(m + 2);
        }
        IonState q = ion_state(Ion{__float_as_int(ra.x), ra.y, ra.z, ra.w, rb.x, rb.y, rb.z, __float_as_int(rb.w)});
        const int64_t ip = (int64_t)ca + qi0 + m;
        if (mode & 1) ion_push(k, E, q, ewxy, ewz, tc.wx0, tc.wy0, tc.wz0);
        if (collide) collide_ion<float>(k, (uint32_t)q.id, kIdTag, (uint32_t)q.id, q.vx, q.vy, q.vz, nacc, nref);
        tile_finish(k, mode, st, q, ip, tc, win, dcnt, wcnt, acc, count, keys, dst);
      }
      __syncthreads();
      // window -> global accumulators
      if (mode & 8) {  // one node per thread, its four fields
        for (int nd = threadIdx.x; nd < kWNodes; nd += blockDim.x) {
          const int wxn = nd % kWX, wyn = (nd / kWX) % kWY, wzn = nd / (kWX * kWY);
          const int np_ = wzn * kSZ + wyn * kSY + wxn;
          int gx = tc.wx0 + wxn, gy = tc.wy0 + wyn, gz = tc.wz0 + wzn;
          // nodes past the last cell wrap (periodic) or are dropped (ghosts)
          if (gx < 0 || gx >= k.Nx) { if (k.bc[0]) continue; gx = gx < 0 ? gx + k.Nx : gx - k.Nx; }
          if (gy < 0 || gy >= k.Ny) { if (k.bc[1]) continue; gy = gy < 0 ? gy + k.Ny : gy - k.Ny; }
          if (gz < 0 || gz >= k.Nz) { if (k.bc[2]) continue; gz = gz < 0 ? gz + k.Nz : gz - k.Nz; }
          // contributions to this node: window deposits of the (up to) 8 cells around it
          int nc = 0;
#pragma unroll
          for (int c = 0; c < 8; c++) {
            const int cx = wxn - (c & 1), cy = wyn - ((c >> 1) & 1), cz = wzn - (c >> 2);
            if (cx >= 0 && cx < kCX && cy >= 0 && cy < kCY && cz >= 0 && cz < kCZ) nc += dcnt[(cz * kCY + cy) * kCX + cx];
          }
          const unsigned bias = (unsigned)nc * kFixBiasBits;
          unsigned long long *g = (unsigned long long *)acc + ((size_t)gz * k.Ny + gy) * k.Nx + gx;
#pragma unroll
          for (int f = 0; f < 4; f++) {
            const long long v = f == 0 ? fix_join((int)(win[0][np_] - bias), (int)(win[1][np_] - bias))
                                       : (long long)(int)(win[1 + f][np_] - bias);
            if (v != 0) atomicAdd(g + (size_t)f * k.ncell, (unsigned long long)v);
          }
        }
      }
      if (count) {
        for (int e = threadIdx.x; e < kWCells; e += blockDim.x) {
          const int n = wcnt[e];
          if (n == 0) continue;
          int gx = tc.wx0 + e % kCX, gy = tc.wy0 + (e / kCX) % kCY, gz = tc.wz0 + e / (kCX * kCY);
          if (gx < 0) gx += k.Nx; else if (gx >= k.Nx) gx -= k.Nx;  // cells of moved ions are in range
          if (gy < 0) gy += k.Ny; else if (gy >= k.Ny) gy -= k.Ny;
          if (gz < 0) gz += k.Nz; else if (gz >= k.Nz) gz -= k.Nz;
          atomicAdd(&count[tile_key(gx, gy, gz, k.tg)], n);
        }
      }
      __syncthreads();
    }
  }
  if (collide) flush_counts(st, nacc, nref);
}

// ---- upload / download conversions ---------------------------------------------
// Host AoS arrays have nd components an ion (3, or 2 for -ndim 2, whose ions
// sit at z = 0 with vz = 0 on the device).
__global__ void k_aos_to_soa64(int64_t n, int nd, const double *__restrict__ pos,
                               const double *__restrict__ vel, double *px, double *py,
                               double *pz, double *vx, double *vy, double *vz) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    px[i] = pos[nd * i]; py[i] = pos[nd * i + 1]; pz[i] = nd == 3 ? pos[3 * i + 2] : 0.0;
    vx[i] = vel[nd * i]; vy[i] = vel[nd * i + 1]; vz[i] = nd == 3 ? vel[3 * i + 2] : 0.0;
  }
}
__global__ void k_soa_to_aos64(int64_t n, int nd, double *__restrict__ pos, double *__restrict__ vel,
                               const double *px, const double *py, const double *pz,
                               const double *vx, const double *vy, const double *vz) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    pos[nd * i] = px[i]; pos[nd * i + 1] = py[i];
    vel[nd * i] = vx[i]; vel[nd * i + 1] = vy[i];
    if (nd == 3) { pos[3 * i + 2] = pz[i]; vel[3 * i + 2] = vz[i]; }
  }
}

// Absolute FP64 coordinate -> (cell, FP32 offset) along one axis.
__device__ __forceinline__ int to_cell(double pos, double d, int N, float &o) {
  double x = pos / d;
  double fl = floor(x);
  int c = (int)fl;
  float of = (float)(x - fl);
  if (of >= 1.0f) { of = 0.0f; c += 1; }
  c %= N;
  if (c < 0) c += N;
  o = of;
  return c;
}

__global__ void k_aos_to_mixed(int64_t n, int nd, PartK k, const double *__restrict__ pos,
                               const double *__restrict__ vel, float4 *__restrict__ ions, int64_t id0) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float a, b, c = 0.0f;
    int ci = to_cell(pos[nd * i], k.dx, k.Nx, a);
    int cj = to_cell(pos[nd * i + 1], k.dy, k.Ny, b);
    int ck = nd == 3 ? to_cell(pos[3 * i + 2], k.dz, k.Nz, c) : 0;
    store_ion(ions, i, {ci | (cj << 10) | (ck << 20), a, b, c, (float)vel[nd * i], (float)vel[nd * i + 1],
                        nd == 3 ? (float)vel[3 * i + 2] : 0.0f, (int32_t)(id0 + i)});
  }
}

__global__ void k_mixed_to_aos(int64_t n, int nd, PartK k, double *__restrict__ pos,
                               double *__restrict__ vel, const float4 *__restrict__ ions) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const Ion q = load_ion(ions, i);
    int ci, cj, ck;
    unpack_cell(q.c, ci, cj, ck);
    pos[nd * i] = ((double)ci + (double)q.ox) * k.dx;
    pos[nd * i + 1] = ((double)cj + (double)q.oy) * k.dy;
    vel[nd * i] = q.vx; vel[nd * i + 1] = q.vy;
    if (nd == 3) {
      pos[3 * i + 2] = ((double)ck + (double)q.oz) * k.dz;
      vel[3 * i + 2] = q.vz;
    }
  }
}

// Download conversion onto whole 256-byte host spans (3-D): the records
// [i0, i1) written as the doubles [d0, d1) of the position array and
// [e0, e1) of the velocity array (ion i holds doubles 3i..3i+2 of each),
// each at its index minus d0 (e0) in the staging regions pos and vel.  The
// first records of the range may belong to the range before, whose span
// ended at the same host boundary.
__global__ void k_mixed_to_aos_span(int64_t i0, int64_t i1, int64_t d0, int64_t d1, int64_t e0, int64_t e1, PartK k,
                                    double *__restrict__ pos, double *__restrict__ vel,
                                    const float4 *__restrict__ ions) {
  for (int64_t i = i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < i1;
       i += (int64_t)gridDim.x * blockDim.x) {
    const Ion q = load_ion(ions, i);
    int ci, cj, ck;
    unpack_cell(q.c, ci, cj, ck);
    const double p3[3] = {((double)ci + (double)q.ox) * k.dx, ((double)cj + (double)q.oy) * k.dy,
                          ((double)ck + (double)q.oz) * k.dz};
    const double v3[3] = {q.vx, q.vy, q.vz};
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const int64_t d = 3 * i + c;
      if (d >= d0 && d < d1) pos[d - d0] = p3[c];
      if (d >= e0 && d < e1) vel[d - e0] = v3[c];
    }
  }
}

// ids[i] = identity of the i-th ion record (the order of a download).
__global__ void k_mixed_ids(int64_t n, const float4 *__restrict__ ions, int32_t *__restrict__ ids) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    ids[i] = __float_as_int(ions[2 * i + 1].w);
}

// out[t] = the first ion of tile t (t <= ntiles; out[ntiles] = np).
__global__ void k_tile_bounds(int ntiles, const int32_t *__restrict__ key_off, int32_t *__restrict__ out) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t <= ntiles; t += gridDim.x * blockDim.x)
    out[t] = key_off[(size_t)t * ECS_TILE_CELLS];
}

// out[t] = the largest perm[j] over tile t's ions j (-1 for an empty tile):
// the last source position a gathering pass reads for the tile.  One warp a
// tile.
__global__ void k_tile_srcmax(int ntiles, const int32_t *__restrict__ key_off, const int32_t *__restrict__ perm,
                              int32_t *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  for (int t = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); t < ntiles; t += (int)((gridDim.x * blockDim.x) >> 5)) {
    const int a = key_off[(size_t)t * ECS_TILE_CELLS], b = key_off[(size_t)(t + 1) * ECS_TILE_CELLS];
    int m = -1;
    for (int j = a + lane; j < b; j += 32) m = max(m, __ldg(perm + j));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) out[t] = m;
  }
}

// ---- counting sort by cell (mixed path) ------------------------------------------
__global__ void k_sort_count(int64_t np, TileG tg, const float4 *__restrict__ ions, int32_t *__restrict__ count,
                             int32_t *__restrict__ keys) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < np;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ip = base + lane;
    const int key = ip < np ? cell_key(ion_cell(ions, ip), tg) : -1;
    if (ip < np) keys[ip] = key;
    count_cells(count, key);
  }
}

// Exclusive scan of count[0..n) into off[0..n], three phases.
constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;
__global__ void k_scan_local(int n, const int32_t *__restrict__ in, int32_t *__restrict__ out,
                             int32_t *__restrict__ sums) {
  __shared__ int32_t warp_tot[32];
  const int tile = kScanBlock * kScanItems;
  const int base = blockIdx.x * tile + threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  int32_t t = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    v[q] = (base + q < n) ? in[base + q] : 0;
    t += v[q];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t incl = t;
#pragma unroll
  for (int s = 1; s < 32; s <<= 1) {
    int32_t y = __shfl_up_sync(ECS_FULL_MASK, incl, s);
    if (lane >= s) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int32_t w = warp_tot[lane];
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
      int32_t y = __shfl_up_sync(ECS_FULL_MASK, w, s);
      if (lane >= s) w += y;
    }
    warp_tot[lane] = w;
  }
  __syncthreads();
  int32_t run = incl - t + (warp > 0 ? warp_tot[warp - 1] : 0);
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    if (base + q < n) out[base + q] = run;
    run += v[q];
  }
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = run;
}
__global__ void k_scan_sums(int nb, int32_t *sums) {
  // single block: serial over chunks of 1024 with a carry
  __shared__ int32_t buf[1024];
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int off = 0; off < nb; off += 1024) {
    int i = off + threadIdx.x;
    int32_t v = i < nb ? sums[i] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int s = 1; s < 1024; s <<= 1) {
      int32_t y = threadIdx.x >= s ? buf[threadIdx.x - s] : 0;
      __syncthreads();
      buf[threadIdx.x] += y;
      __syncthreads();
    }
    if (i < nb) sums[i] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
}
// out[i] += block sums; out[n] = total (the number of ions).
__global__ void k_scan_add(int n, int32_t *__restrict__ out, const int32_t *__restrict__ sums, int total) {
  const int tile = kScanBlock * kScanItems;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += sums[i / tile];
  if (i == 0) out[n] = total;
}

// Every ion record moves whole (32 bytes, one sector) to slot
// off[key] + (its rank among the ions of its cell), ranks handed out by a
// warp-aggregated atomic cursor per cell.
// The counting sort's permutation: perm[d] = the buffer position of the ion
// that goes to position d in key order (keys[ip] from the counting pass).
// Within a key the order follows the atomics; nothing depends on it (the
// moments are exact sums and each ion's random numbers come from its state).
// Only 4-byte indices move: the next particle pass reads the 32-byte records
// through perm and writes them in key order into the other buffer.
__global__ void k_sort_index(int64_t np, const int32_t *__restrict__ keys, const int32_t *__restrict__ off,
                             int32_t *__restrict__ cursor, int32_t *__restrict__ perm) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < np;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ip = base + lane;
    const int key = ip < np ? __ldcs(keys + ip) : -1;
    const unsigned peers = __match_any_sync(ECS_FULL_MASK, key);
    const int leader = __ffs(peers) - 1;
    int slot = 0;
    if (key >= 0 && lane == leader) slot = atomicAdd(&cursor[key], __popc(peers));
    slot = __shfl_sync(ECS_FULL_MASK, slot, leader);
    if (key >= 0) perm[(int64_t)off[key] + slot + __popc(peers & ((1u << lane) - 1u))] = (int32_t)ip;
  }
}

// dst[i] = src[perm[i]]: the records of a pending sort put in key order.
__global__ void k_gather_ions(int64_t np, const int32_t *__restrict__ perm, const float4 *__restrict__ src,
                              float4 *__restrict__ dst) {
  for (int64_t ip = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ip < np; ip += (int64_t)gridDim.x * blockDim.x) {
    const int64_t sp = perm[ip];
    __stcs(dst + 2 * ip, __ldcs(src + 2 * sp));
    __stcs(dst + 2 * ip + 1, __ldcs(src + 2 * sp + 1));
  }
}

// ---- collision-rate estimate (first pass only) -------------------------------------
__global__ void k_estimate64(PartK k, int64_t np, const double *px, const double *py,
                             const double *pz, const double *vxa, const double *vya,
                             const double *vza, EcsDevStatus *st) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < np;
       base += (int64_t)gridDim.x * blockDim.x) {
    int64_t ip = base + lane;
    bool active = ip < np;
    float sample = 0.f;
    if (active) {
      double vx = vxa[ip], vy = vya[ip], vz = vza[ip];
      uint32_t h0, h1;
      hash64(px[ip], py[ip], pz[ip], vx, vy, vz, h0, h1);
      sample = accept_sample<double>(k, h0, h1, vx, vy, vz);
    }
    flush_samples(st, sample, active);
  }
}
__global__ void k_estimate32(PartK k, int64_t np, const float4 *__restrict__ ions, EcsDevStatus *st) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < np;
       base += (int64_t)gridDim.x * blockDim.x) {
    int64_t ip = base + lane;
    bool active = ip < np;
    float sample = 0.f;
    if (active) {
      const Ion q = load_ion(ions, ip);
      sample = accept_sample<float>(k, (uint32_t)q.id, kIdTag, q.vx, q.vy, q.vz);
    }
    flush_samples(st, sample, active);
  }
}

// ---- host helpers -----------------------------------------------------------------
PartK make_k(const EcsCtx *ctx, double dt) {
  const EcsParams &p = ctx->p;
  PartK k;
  memset(&k, 0, sizeof k);
  k.ndim = p.ndim;
  k.Nx = p.Nx; k.Ny = p.Ny; k.Nz = p.Nz;
  for (int d = 0; d < 3; d++) k.bc[d] = p.bc[d] == ECS_BC_PERIODIC ? ECS_BC_PERIODIC : ECS_BC_INJECT_REFLECT;
  k.ncell = ctx->ncell;
  k.dx = p.dx; k.dy = p.dy; k.dz = p.dz;
  k.lo[0] = p.x0; k.lo[1] = p.y0; k.lo[2] = p.z0;
  k.hi[0] = p.x1; k.hi[1] = p.y1; k.hi[2] = p.z1;
  k.L[0] = p.Lx; k.L[1] = p.Ly; k.L[2] = p.Lz;
  // src/velocities.c:307-320, same operation order
  double tscale = 0.5 * (p.qi / p.mi) * dt;
  k.t = tscale * p.B0;
  k.s = 2.0 * k.t / (1 + k.t * k.t);
  double h[3] = {1.0 / p.dx, 1.0 / p.dy, 1.0 / p.dz};
  for (int d = 0; d < 3; d++) {
    k.esc[d] = -0.5 * h[d] * tscale;
    k.escf[d] = (float)k.esc[d];
  }
  k.tf = (float)k.t;
  k.sf = (float)k.s;
  k.dt = dt;
  k.dtc[0] = (float)(dt / p.dx);
  k.dtc[1] = (float)(dt / p.dy);
  k.dtc[2] = (float)(dt / p.dz);
  // src/collisions.c:18-52
  k.collide = p.mn > 0.0 ? 1 : 0;
  double tmp = (p.vi0x - p.vn0x) * (p.vi0x - p.vn0x) + (p.vi0y - p.vn0y) * (p.vi0y - p.vn0y) +
               (p.vi0z - p.vn0z) * (p.vi0z - p.vn0z);
  double vrm = 4.0 * p.viT + sqrt(tmp);
  k.vrm2 = vrm * vrm;
  k.viT = p.viT;
  k.vnT = p.vnT;
  k.vn0[0] = p.vn0x; k.vn0[1] = p.vn0y; k.vn0[2] = p.vn0z;
  k.mi = p.mi; k.mn = p.mn; k.M = p.mn + p.mi;
  k.ivrm2f = (float)(1.0 / k.vrm2);
  k.vnTf = (float)k.vnT;
  for (int d = 0; d < 3; d++) k.vn0f[d] = (float)k.vn0[d];
  k.wif = (float)(k.mi / k.M);
  k.wnf = (float)(k.mn / k.M);
  k.vlimf = (float)(10.0 * k.viT);
  k.key0 = (uint32_t)ctx->seed;
  k.key1 = (uint32_t)(ctx->seed >> 32);
  k.step = (uint32_t)ctx->step_index;
  {
    uint32_t m = (uint32_t)ctx->step_index * 0x9E3779B9u ^ k.key0;
    m ^= m >> 16; m *= 0x7feb352du; m ^= m >> 15; m *= 0x846ca68bu; m ^= m >> 16;
    k.stepmix = m ^ k.key1;
  }
  k.fixn64 = ldexp(1.0, ctx->shift_n);
  k.fixf64 = ldexp(1.0, ctx->shift_f);
  k.fixn32 = {ldexpf(1.0f, ctx->shift_n), ldexpf(1.0f, ctx->shift_n - kFixSplit), -ldexpf(1.0f, kFixSplit - ctx->shift_n)};
  k.fixf32 = {ldexpf(1.0f, ctx->shift_f)};
  // the velocity bound 2^e_v behind the flux scale (ecs_fix_shifts)
  k.vmax = ldexp(1.0, (ctx->prec == ECS_PREC_FP64 ? ECS_FIX_SHIFT_FP64 : ECS_FIX_SHIFT_MIXED_FLUX) - ctx->shift_f);
  k.vmaxf = (float)k.vmax;
  k.vwinf = (float)(k.vmax / 8.0);
  k.tg = {ctx->ntile[0], ctx->ntile[1], ctx->ntile[2]};
  return k;
}

// Reference collision count Nc (src/collisions.c:58-63).
int64_t collision_target(const EcsCtx *ctx, double dt) {
  const EcsParams &p = ctx->p;
  double tmp = (p.vi0x - p.vn0x) * (p.vi0x - p.vn0x) + (p.vi0y - p.vn0y) * (p.vi0y - p.vn0y) +
               (p.vi0z - p.vn0z) * (p.vi0z - p.vn0z);
  double vrm = 4.0 * p.viT + sqrt(tmp);
  double fc = p.nui * dt;
  double nc = ((double)ctx->np * fc * vrm) / ((p.vnT + p.vn0) * sqrt(p.mn / p.mi));
  int64_t Nc = (int64_t)nc;
  if (Nc > ctx->np) Nc = ctx->np;
  if (Nc < 0) Nc = 0;
  return Nc;
}

unsigned int grid_blocks(const EcsCtx *ctx, int64_t n, int per_sm) {
  int64_t want = (n + kBlock - 1) / kBlock;
  int64_t cap = (int64_t)ctx->nsm * per_sm;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  return (unsigned int)want;
}

// ---- initial ions on the device ----------------------------------------------
// Positions (src/positions.c:139-388) and Maxwellian velocities
// (src/velocities.c:14-47), one thread per ion, stored like an upload.
constexpr int kSobolBits = 30;     // MAXBIT of src/random.c
constexpr int kInitTries = 256;    // rejection attempts per ion
constexpr int kInitModes = 16;

struct InitK {
  int dist;
  uint32_t key0, key1;
  double L[3];
  double vT[3], v0[3];
  uint32_t sob[3][kSobolBits];  // direction numbers v_{j}, j = 1..30, of dimensions 1..3
  int nmodes;
  int kv[kInitModes][3];
  double amp[kInitModes], phase[kInitModes];
  double inv_max;  // acceptance scale of the rejection
};

// Sobol direction numbers of the first three dimensions (Bratley-Fox, 30
// bits), with the reference's recurrence: the higher numbers XOR v_{j-1}
// where the published method XORs v_{j-l} (src/random.c:256-266).
void sobol_directions(uint32_t v[3][kSobolBits]) {
  static const int deg[3] = {1, 2, 3};
  static const uint32_t poly[3] = {0, 1, 1};
  static const uint32_t start[3][3] = {{1, 0, 0}, {1, 1, 0}, {1, 3, 7}};
  for (int d = 0; d < 3; d++) {
    uint32_t w[kSobolBits + 1] = {0};
    for (int j = 1; j <= deg[d]; j++) w[j] = start[d][j - 1] << (kSobolBits - j);
    for (int j = deg[d] + 1; j <= kSobolBits; j++) {
      uint32_t x = w[j - deg[d]];
      x ^= x >> deg[d];
      uint32_t c = poly[d];
      for (int l = deg[d] - 1; l >= 1; l--) {
        if (c & 1u) x ^= w[j - 1];
        c >>= 1;
      }
      w[j] = x;
    }
    for (int j = 1; j <= kSobolBits; j++) v[d][j - 1] = w[j];
  }
}

__device__ __forceinline__ double init_density(const InitK &k, const double s[3]) {
  if (k.dist == ECS_INIT_SINUSOIDAL) return 1.0 + 0.25 * sin(2.0 * M_PI * s[0]);  // src/positions.c:236-251
  double w = 1.0;
  for (int m = 0; m < k.nmodes; m++) {
    const double a = (double)k.kv[m][0] * s[0] + (double)k.kv[m][1] * s[1] + (double)k.kv[m][2] * s[2];
    w += k.amp[m] * cos(2.0 * M_PI * a + k.phase[m]);
  }
  return w;
}

// Position of ion i as fractions s of the box; false if the rejection gave up.
__device__ bool init_fraction(const InitK &k, int64_t i, double s[3]) {
  const uint32_t lo = (uint32_t)i, hi = (uint32_t)((uint64_t)i >> 32);
  if (k.dist == ECS_INIT_SOBOL) {
    // after i+1 draws the generator state is the XOR of the direction
    // numbers at the set bits of gray(i+1)
    const uint64_t m = (uint64_t)i + 1;
    const uint32_t g = (uint32_t)(m ^ (m >> 1));
    for (int d = 0; d < 3; d++) {
      uint32_t x = 0;
      for (int b = 0; b < kSobolBits; b++)
        if ((g >> b) & 1u) x ^= k.sob[d][b];
      s[d] = (double)x * (1.0 / 1073741824.0);
    }
    return true;
  }
  for (int a = 0; a < kInitTries; a++) {
    const EcsU4 q1 = ecs_philox({lo, hi, 0x504F5300u + 2u * (uint32_t)a, 0x494E4954u}, k.key0, k.key1);
    const EcsU4 q2 = ecs_philox({lo, hi, 0x504F5301u + 2u * (uint32_t)a, 0x494E4954u}, k.key0, k.key1);
    s[0] = ecs_u01d(q1.x, q1.y);
    s[1] = ecs_u01d(q1.z, q1.w);
    s[2] = ecs_u01d(q2.x, q2.y);
    if (k.dist == ECS_INIT_RANDOM) return true;
    if (init_density(k, s) * k.inv_max > ecs_u01d(q2.z, q2.w)) return true;  // src/positions.c:314-321
  }
  return false;
}

// v_d = vT_d * N(0,1) + v0_d (Box-Muller on the ion's own counter)
__device__ void init_velocity(const InitK &k, int64_t i, double v[3]) {
  const uint32_t lo = (uint32_t)i, hi = (uint32_t)((uint64_t)i >> 32);
  const EcsU4 q1 = ecs_philox({lo, hi, 0x56454C00u, 0x494E4954u}, k.key0, k.key1);
  const EcsU4 q2 = ecs_philox({lo, hi, 0x56454C01u, 0x494E4954u}, k.key0, k.key1);
  const double r1 = sqrt(-2.0 * log(ecs_u01d(q1.x, q1.y)));
  double sn, cs;
  sincospi(2.0 * ecs_u01d(q1.z, q1.w), &sn, &cs);
  const double n2 = sqrt(-2.0 * log(ecs_u01d(q2.x, q2.y))) * cospi(2.0 * ecs_u01d(q2.z, q2.w));
  const double nd[3] = {r1 * cs, r1 * sn, n2};
  for (int d = 0; d < 3; d++) v[d] = k.vT[d] * nd[d] + k.v0[d];
}

__global__ void k_init_ions(InitK ik, PartK k, int64_t n, int fp64, float4 *__restrict__ ions, double *px,
                            double *py, double *pz, double *vx, double *vy, double *vz, EcsDevStatus *st) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s[3], pos[3], vel[3];
    if (!init_fraction(ik, i, s)) {
      atomicOr(&st->flags, ECS_FLAG_RANGE);
      s[0] = s[1] = s[2] = 0.5;
    }
    for (int d = 0; d < 3; d++) {
      pos[d] = s[d] * ik.L[d];  // src/positions.c:174, 318
      if (pos[d] >= ik.L[d]) pos[d] = nextafter(ik.L[d], 0.0);
    }
    init_velocity(ik, i, vel);
    if (k.ndim == 2) pos[2] = vel[2] = 0.0;
    if (fp64) {
      px[i] = pos[0]; py[i] = pos[1]; pz[i] = pos[2];
      vx[i] = vel[0]; vy[i] = vel[1]; vz[i] = vel[2];
    } else {
      float a, b, c;
      const int ci = to_cell(pos[0], k.dx, k.Nx, a);
      const int cj = to_cell(pos[1], k.dy, k.Ny, b);
      const int ck = to_cell(pos[2], k.dz, k.Nz, c);
      store_ion(ions, i, {ci | (cj << 10) | (ck << 20), a, b, c, (float)vel[0], (float)vel[1], (float)vel[2],
                          (int32_t)i});
    }
  }
}

}  // namespace

// ============================================================================
// entry points used by ecs_api.cu
// ============================================================================
int ecs_particles_alloc(EcsCtx *ctx) {
  size_t n = (size_t)ctx->cap;
  if (n == 0) n = 1;
  if (ctx->prec == ECS_PREC_FP64) {
    double **arr[6] = {&ctx->px, &ctx->py, &ctx->pz, &ctx->vx, &ctx->vy, &ctx->vz};
    for (auto a : arr) ECS_CUDA(ctx, cudaMalloc((void **)a, n * sizeof(double)));
  } else {
    for (int b = 0; b < 2; b++) ECS_CUDA(ctx, cudaMalloc((void **)&ctx->ions[b], n * 2 * sizeof(float4)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->sort_keys, n * sizeof(int32_t)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->perm, n * sizeof(int32_t)));
    ctx->ntile[0] = (ctx->p.Nx + ECS_TILE_X - 1) / ECS_TILE_X;
    ctx->ntile[1] = (ctx->p.Ny + ECS_TILE_Y - 1) / ECS_TILE_Y;
    ctx->ntile[2] = (ctx->p.Nz + ECS_TILE_Z - 1) / ECS_TILE_Z;
    ctx->nkeys = (size_t)ctx->ntile[0] * ctx->ntile[1] * ctx->ntile[2] * ECS_TILE_CELLS;
    size_t nb = ecs_div_up(ctx->nkeys, (size_t)kScanBlock * kScanItems);
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->sort_count, ctx->nkeys * sizeof(int32_t)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->sort_offset, (ctx->nkeys + 1) * sizeof(int32_t)));
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->scan_blocks, (nb + 1) * sizeof(int32_t)));
  }
  return ECS_OK;
}

void ecs_part_xfer_free(EcsCtx *ctx);
int ecs_particles_free(EcsCtx *ctx) {
  ecs_part_xfer_free(ctx);
  void *ptrs[] = {ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy, ctx->vz, ctx->ions[0], ctx->ions[1],
                  ctx->sort_keys, ctx->perm, ctx->sort_count, ctx->sort_offset, ctx->scan_blocks};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  return ECS_OK;
}

// ---- host transfers ------------------------------------------------------------
// Ions move between the host's AoS FP64 arrays and the device in chunks
// (ecs_stage_ions) through two staging buffers, so that the copy of one
// chunk overlaps the conversion kernel of the other.

static int ensure_xfer(EcsCtx *ctx) {
  if (ctx->stage[0]) return ECS_OK;
  for (int q = 0; q < 2; q++) {
    ECS_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->xs[q], cudaStreamNonBlocking));
    ECS_CUDA(ctx, cudaEventCreateWithFlags(&ctx->xev_copy[q], cudaEventDisableTiming));
    ECS_CUDA(ctx, cudaEventCreateWithFlags(&ctx->xev_kern[q], cudaEventDisableTiming));
  }
  ECS_CUDA(ctx, cudaEventCreateWithFlags(&ctx->xev_ready, cudaEventDisableTiming));
  const int64_t n = ecs_stage_ions(ctx->cap);
  for (int q = 0; q < 2; q++)
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->stage[q], (size_t)ecs_stage_stride(n) * 2 * sizeof(double)));
  ctx->stage_n = n;
  return ECS_OK;
}

void ecs_part_xfer_free(EcsCtx *ctx) {
  for (int q = 0; q < 2; q++) {
    if (ctx->xs[q]) cudaStreamSynchronize(ctx->xs[q]);
    if (ctx->stage[q]) cudaFree(ctx->stage[q]);
    if (ctx->xev_copy[q]) cudaEventDestroy(ctx->xev_copy[q]);
    if (ctx->xev_kern[q]) cudaEventDestroy(ctx->xev_kern[q]);
    if (ctx->xs[q]) cudaStreamDestroy(ctx->xs[q]);
  }
  if (ctx->xev_ready) cudaEventDestroy(ctx->xev_ready);
  if (ctx->xs_conv) cudaStreamSynchronize(ctx->xs_conv);
  for (int q = 0; q < EcsCtx::kStageDn; q++) {
    if (ctx->stage_dn[q]) cudaFree(ctx->stage_dn[q]);
    if (ctx->xev_tiled[q]) cudaEventDestroy(ctx->xev_tiled[q]);
    if (ctx->xev_dn_conv[q]) cudaEventDestroy(ctx->xev_dn_conv[q]);
    if (ctx->xev_dn_copy[q]) cudaEventDestroy(ctx->xev_dn_copy[q]);
  }
  if (ctx->xs_conv) cudaStreamDestroy(ctx->xs_conv);
  if (ctx->xs_up) {
    cudaStreamSynchronize(ctx->xs_up);
    cudaStreamDestroy(ctx->xs_up);
  }
  for (cudaEvent_t e : ctx->xev_upc) cudaEventDestroy(e);
  ctx->xev_upc.clear();
  if (ctx->tile_tables_dev) cudaFree(ctx->tile_tables_dev);
  if (ctx->tile_bounds) cudaFreeHost(ctx->tile_bounds);
  ctx->tile_tables_dev = ctx->tile_bounds = ctx->tile_srcmax = nullptr;
}

// Host AoS FP64 -> device: copies on xs[1], conversions on ctx->stream.
int ecs_part_upload(EcsCtx *ctx, const double *pos, const double *vel, int64_t np) {
  if (np < 0 || np > ctx->cap) return ecs_fail(ctx, ECS_ERR_INVALID, "np %lld exceeds capacity %lld", (long long)np, (long long)ctx->cap);
  int rc = ensure_xfer(ctx);
  if (rc) return rc;
  const int64_t chunk = ctx->stage_n;
  const int nd = ctx->p.ndim == 2 ? 2 : 3;  // components an ion in the host arrays
  PartK k = make_k(ctx, 0.0);
  // the previous contents of the ion buffer may still be in use
  ECS_CUDA(ctx, cudaEventRecord(ctx->xev_ready, ctx->stream));
  ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->xs[1], ctx->xev_ready, 0));
  int64_t c = 0;
  for (int64_t off = 0; off < np; off += chunk, c++) {
    const int q = (int)(c & 1);
    const int64_t n = np - off < chunk ? np - off : chunk;
    double *st = ctx->stage[q];
    if (c >= 2) ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->xs[1], ctx->xev_kern[q], 0));  // buffer q free
    ECS_CUDA(ctx, cudaMemcpyAsync(st, pos + nd * off, (size_t)n * nd * sizeof(double), cudaMemcpyHostToDevice, ctx->xs[1]));
    ECS_CUDA(ctx, cudaMemcpyAsync(st + nd * n, vel + nd * off, (size_t)n * nd * sizeof(double), cudaMemcpyHostToDevice, ctx->xs[1]));
    ECS_CUDA(ctx, cudaEventRecord(ctx->xev_copy[q], ctx->xs[1]));
    ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->xev_copy[q], 0));
    unsigned int g = grid_blocks(ctx, n, 8);
    if (ctx->prec == ECS_PREC_FP64) {
      k_aos_to_soa64<<<g, kBlock, 0, ctx->stream>>>(n, nd, st, st + nd * n, ctx->px + off, ctx->py + off,
                                                   ctx->pz + off, ctx->vx + off, ctx->vy + off, ctx->vz + off);
    } else {
      k_aos_to_mixed<<<g, kBlock, 0, ctx->stream>>>(n, nd, k, st, st + nd * n, ctx->ions[ctx->cur] + 2 * off, off);
    }
    ECS_LAUNCHED(ctx);
    ECS_CUDA(ctx, cudaEventRecord(ctx->xev_kern[q], ctx->stream));
  }
  ctx->np = np;
  ctx->pgen++;
  ctx->attempt_rate = -1.0;
  ctx->tiles_valid = false;
  ctx->perm_pending = false;
  if (ctx->prec == ECS_PREC_MIXED && ctx->sort_every > 0 && np > 0) {
    rc = ecs_part_sort(ctx);
    if (rc) return rc;
  }
  // the host arrays may be reused once this returns
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->xs[1]));
  return ECS_OK;
}

// Initial ions generated on the device (see InitK); the same bookkeeping as
// an upload.
int ecs_part_init(EcsCtx *ctx, int dist, int64_t np, uint64_t seed, const EcsDensityModes *modes) {
  if (np < 0 || np > ctx->cap) return ecs_fail(ctx, ECS_ERR_INVALID, "np %lld exceeds capacity %lld", (long long)np, (long long)ctx->cap);
  const EcsParams &p = ctx->p;
  InitK ik;
  memset(&ik, 0, sizeof ik);
  ik.dist = dist;
  ik.key0 = (uint32_t)seed ^ 0x52414E44u;
  ik.key1 = (uint32_t)(seed >> 32);
  ik.L[0] = p.Lx; ik.L[1] = p.Ly; ik.L[2] = p.Lz;
  ik.vT[0] = p.viTx; ik.vT[1] = p.viTy; ik.vT[2] = p.viTz;
  ik.v0[0] = p.vi0x; ik.v0[1] = p.vi0y; ik.v0[2] = p.vi0z;
  switch (dist) {
    case ECS_INIT_SOBOL:
      if (np >= ((int64_t)1 << kSobolBits)) return ecs_fail(ctx, ECS_ERR_INVALID, "Sobol positions need np < 2^30");
      sobol_directions(ik.sob);
      break;
    case ECS_INIT_RANDOM:
      break;
    case ECS_INIT_SINUSOIDAL: {
      // the largest density at the grid nodes, src/positions.c:292-303
      double mx = 0.0;
      for (int i = 0; i < p.Nx; i++) mx = std::max(mx, 1.0 + 0.25 * sin(2 * M_PI * ((double)i / p.Nx)));
      ik.inv_max = 1.0 / mx;
      break;
    }
    case ECS_INIT_MODES: {
      if (!modes || modes->nmodes < 0 || modes->nmodes > kInitModes)
        return ecs_fail(ctx, ECS_ERR_INVALID, "density modes: 0..%d modes required", kInitModes);
      double sum = 0.0;
      ik.nmodes = modes->nmodes;
      for (int m = 0; m < modes->nmodes; m++) {
        for (int d = 0; d < 3; d++) ik.kv[m][d] = modes->k[m][d];
        ik.amp[m] = modes->amplitude[m];
        ik.phase[m] = modes->phase[m];
        sum += fabs(modes->amplitude[m]);
      }
      if (!(sum < 1.0)) return ecs_fail(ctx, ECS_ERR_INVALID, "density modes: sum of |amplitude| must be < 1");
      ik.inv_max = 1.0 / (1.0 + sum);
      break;
    }
    default:
      return ecs_fail(ctx, ECS_ERR_UNSUPPORTED, "position distribution %d is not available on the device", dist);
  }
  ECS_CUDA(ctx, cudaMemsetAsync(ctx->dstat, 0, sizeof(EcsDevStatus), ctx->stream));
  const PartK k = make_k(ctx, 0.0);
  const bool fp64 = ctx->prec == ECS_PREC_FP64;
  if (np > 0) {
    k_init_ions<<<grid_blocks(ctx, np, 8), kBlock, 0, ctx->stream>>>(
        ik, k, np, fp64 ? 1 : 0, fp64 ? nullptr : ctx->ions[ctx->cur], ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy,
        ctx->vz, ctx->dstat);
    ECS_LAUNCHED(ctx);
  }
  ECS_CUDA(ctx, cudaMemcpyAsync(ctx->hstat, ctx->dstat, sizeof(EcsDevStatus), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->hstat->flags & ECS_FLAG_RANGE)
    return ecs_fail(ctx, ECS_ERR_RANGE, "rejection sampling gave up after %d attempts for an ion", kInitTries);
  ctx->np = np;
  ctx->pgen++;
  ctx->attempt_rate = -1.0;
  ctx->tiles_valid = false;
  ctx->perm_pending = false;
  if (ctx->prec == ECS_PREC_MIXED && ctx->sort_every > 0 && np > 0) {
    int rc = ecs_part_sort(ctx);
    if (rc) return rc;
  }
  return ECS_OK;
}

// Puts the records of a pending index sort into key order in the other
// buffer (the particle passes read through the permutation instead; the
// host transfers and the order-free kernel need the records themselves).
static int settle_order(EcsCtx *ctx) {
  if (!ctx->perm_pending) return ECS_OK;
  ctx->pgen++;
  if (ctx->np > 0) {
    k_gather_ions<<<grid_blocks(ctx, ctx->np, 8), kBlock, 0, ctx->stream>>>(ctx->np, ctx->perm, ctx->ions[ctx->cur],
                                                                          ctx->ions[1 - ctx->cur]);
    ECS_LAUNCHED(ctx);
    ctx->cur = 1 - ctx->cur;
  }
  ctx->perm_pending = false;
  return ECS_OK;
}

// Device -> host AoS FP64: conversions on xs[0], copies on xs[1], after the
// work enqueued on ctx->stream so far.
int ecs_part_download_async(EcsCtx *ctx, double *pos, double *vel) {
  int rc = ensure_xfer(ctx);
  if (rc) return rc;
  if ((rc = settle_order(ctx))) return rc;
  const int64_t chunk = ctx->stage_n;
  const int nd = ctx->p.ndim == 2 ? 2 : 3;
  const int64_t np = ctx->np;
  PartK k = make_k(ctx, 0.0);
  ECS_CUDA(ctx, cudaEventRecord(ctx->xev_ready, ctx->stream));
  ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->xs[0], ctx->xev_ready, 0));
  int64_t c = 0;
  for (int64_t off = 0; off < np; off += chunk, c++) {
    const int q = (int)(c & 1);
    const int64_t n = np - off < chunk ? np - off : chunk;
    double *st = ctx->stage[q];
    if (c >= 2) ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->xs[0], ctx->xev_copy[q], 0));  // buffer q copied out
    unsigned int g = grid_blocks(ctx, n, 8);
    if (ctx->prec == ECS_PREC_FP64) {
      k_soa_to_aos64<<<g, kBlock, 0, ctx->xs[0]>>>(n, nd, st, st + nd * n, ctx->px + off, ctx->py + off,
                                                  ctx->pz + off, ctx->vx + off, ctx->vy + off, ctx->vz + off);
    } else {
      k_mixed_to_aos<<<g, kBlock, 0, ctx->xs[0]>>>(n, nd, k, st, st + nd * n, ctx->ions[ctx->cur] + 2 * off);
    }
    ECS_LAUNCHED(ctx);
    ECS_CUDA(ctx, cudaEventRecord(ctx->xev_kern[q], ctx->xs[0]));
    ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->xs[1], ctx->xev_kern[q], 0));
    if (pos) ECS_CUDA(ctx, cudaMemcpyAsync(pos + nd * off, st, (size_t)n * nd * sizeof(double), cudaMemcpyDeviceToHost, ctx->xs[1]));
    if (vel) ECS_CUDA(ctx, cudaMemcpyAsync(vel + nd * off, st + nd * n, (size_t)n * nd * sizeof(double), cudaMemcpyDeviceToHost, ctx->xs[1]));
    ECS_CUDA(ctx, cudaEventRecord(ctx->xev_copy[q], ctx->xs[1]));
  }
  return ECS_OK;
}

int ecs_part_xfer_wait(EcsCtx *ctx) {
  if (!ctx->xs[1]) return ECS_OK;
  if (ctx->xs_conv) ECS_CUDA(ctx, cudaStreamSynchronize(ctx->xs_conv));
  if (ctx->xs_up) ECS_CUDA(ctx, cudaStreamSynchronize(ctx->xs_up));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->xs[0]));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->xs[1]));
  return ECS_OK;
}

int ecs_part_download(EcsCtx *ctx, double *pos, double *vel) {
  int rc = ecs_part_download_async(ctx, pos, vel);
  if (rc) return rc;
  return ecs_part_xfer_wait(ctx);
}

// The identity of every ion, in the order ecs_part_download returns them.
int ecs_part_ids(EcsCtx *ctx, int32_t *ids) {
  const int64_t np = ctx->np;
  if (np == 0) return ECS_OK;
  if (ctx->prec == ECS_PREC_FP64) {  // the FP64 path never reorders its ions
    for (int64_t i = 0; i < np; i++) ids[i] = (int32_t)i;
    return ECS_OK;
  }
  int rc = settle_order(ctx);
  if (rc) return rc;
  int32_t *d = nullptr;
  ECS_CUDA(ctx, cudaMallocAsync((void **)&d, (size_t)np * sizeof(int32_t), ctx->stream));
  k_mixed_ids<<<grid_blocks(ctx, np, 8), kBlock, 0, ctx->stream>>>(np, ctx->ions[ctx->cur], d);
  ECS_LAUNCHED(ctx);
  ECS_CUDA(ctx, cudaMemcpyAsync(ids, d, (size_t)np * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaFreeAsync(d, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return ECS_OK;
}

// Parameters of one particle pass in `mode` (the collision bit dropped when
// mn = 0).  The collision attempt rate is estimated from the ions' state at
// the start of the first pass that pushes or collides, so that a step run as
// separate push and collide passes (the reference's UpdateVelocities) and
// the same step as one fused pass start from the same rate.
static int pass_params(EcsCtx *ctx, double dt, int &mode, PartK &k) {
  int rc0 = ecs_part_settle(ctx);  // a rate update still pending from a fused pass
  if (rc0) return rc0;
  k = make_k(ctx, dt);
  if ((mode & 3) && k.collide && ctx->attempt_rate < 0) {
    int rc = ecs_part_estimate_rate(ctx, dt);
    if (rc) return rc;
  }
  if ((mode & 2) && k.collide) {
    k.rate = ctx->attempt_rate;
    k.ratef = (float)k.rate;
    k.p0f = (float)exp(-k.rate);
    ECS_CUDA(ctx, cudaMemsetAsync(ctx->dstat, 0, sizeof(EcsDevStatus), ctx->stream));
  }
  if (!k.collide) mode &= ~2;
  return ECS_OK;
}

// One pass of the particle kernel over all ions.  With `count_for_sort` the
// pass also counts the ions' (new) cells for the counting sort that follows.
static int launch_particles(EcsCtx *ctx, double dt, int mode, bool count_for_sort = false) {
  if (ctx->np == 0) return ECS_OK;
  PartK k;
  int rc = pass_params(ctx, dt, mode, k);
  if (rc) return rc;
  ctx->pgen++;
  const size_t shm = (size_t)(kBlock / 32) * 32 * kTileStride * sizeof(long long);
  static std::atomic<bool> attr_set{false};
  if (!attr_set) {
    cudaFuncSetAttribute(k_particles64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
    cudaFuncSetAttribute(k_particles32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
    attr_set = true;
  }
  int32_t *count = nullptr;
  if (count_for_sort && ctx->prec == ECS_PREC_MIXED) {
    ECS_CUDA(ctx, cudaMemsetAsync(ctx->sort_count, 0, ctx->nkeys * sizeof(int32_t), ctx->stream));
    count = ctx->sort_count;
  }
  unsigned int g = grid_blocks(ctx, ctx->np, 3);
  if (ctx->ev[0]) cudaEventRecord(ctx->ev[0], ctx->stream);
  if (ctx->prec == ECS_PREC_FP64) {
    k_particles64<<<g, kBlock, shm, ctx->stream>>>(k, mode, ctx->np, ctx->px, ctx->py, ctx->pz, ctx->vx,
                                                ctx->vy, ctx->vz, ctx->eext64, ctx->acc, ctx->dstat);
  } else if (ctx->tiles_valid) {
    // after an index sort the pass reads the records through the permutation
    // and, if it writes them, leaves them in key order in the other buffer
    const int ntiles = ctx->ntile[0] * ctx->ntile[1] * ctx->ntile[2];
    const bool gather = ctx->perm_pending, writes = (mode & 7) != 0;
    float4 *src = ctx->ions[ctx->cur];
    float4 *dst = gather ? ctx->ions[1 - ctx->cur] : src;
    k_tiles32<<<ntiles, kTileThreads, 0, ctx->stream>>>(k, mode, src, dst, gather ? ctx->perm : nullptr, ctx->eext32,
                                                  ctx->acc, ctx->sort_offset, count, ctx->sort_keys, ctx->dstat, 0,
                                                  ntiles);
    if (gather && writes) {
      ctx->cur = 1 - ctx->cur;
      ctx->perm_pending = false;
    }
  } else {
    rc = settle_order(ctx);
    if (rc) return rc;
    k_particles32<<<g, kBlock, shm, ctx->stream>>>(k, mode, ctx->np, ctx->ions[ctx->cur], ctx->eext32, ctx->acc,
                                                count, ctx->sort_keys, ctx->dstat);
  }
  ECS_LAUNCHED(ctx);
  if (ctx->ev[1]) {
    cudaEventRecord(ctx->ev[1], ctx->stream);
    ctx->ev_particle = true;
  }
  return ECS_OK;
}

// After a collision pass, from its counters in hstat: the next pass's rate.
static int collisions_update(EcsCtx *ctx, double dt) {
  const EcsDevStatus &s = *ctx->hstat;
  // Attempt rate of the next pass: the expected number of accepted
  // collisions is rate * sum_i P_accept(v_i), so scale the rate by
  // Nc / accepted (damped by a square root against Poisson noise).  The
  // accepted count is a sum over ions, independent of their order.
  int64_t Nc = collision_target(ctx, dt);
  if (s.collisions > 0 && Nc > 0) {
    double f = sqrt((double)Nc / (double)s.collisions);
    if (f > 2.0) f = 2.0;
    if (f < 0.5) f = 0.5;
    ctx->attempt_rate *= f;
  } else if (Nc > 0 && ctx->attempt_rate > 0) {
    ctx->attempt_rate *= 2.0;
  }
  if (s.refused >= 10) return ecs_fail(ctx, ECS_ERR_COLLISION, "%llu collisions refused (final speed > 10 viT)", s.refused);
  return ECS_OK;
}
// After a collision pass: read the counters, update the next pass's rate.
static int finish_collisions(EcsCtx *ctx, double dt) {
  ECS_CUDA(ctx, cudaMemcpyAsync(ctx->hstat, ctx->dstat, sizeof(EcsDevStatus), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return collisions_update(ctx, dt);
}

int ecs_part_status_async(EcsCtx *ctx) {
  if (!ctx->ev_stat) ECS_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_stat, cudaEventDisableTiming));
  ECS_CUDA(ctx, cudaMemcpyAsync(ctx->hstat, ctx->dstat, sizeof(EcsDevStatus), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaEventRecord(ctx->ev_stat, ctx->stream));
  ctx->stat_queued = true;
  return ECS_OK;
}

// The counters in hstat: wait for their queued copy, or copy them now.
static int status_to_host(EcsCtx *ctx) {
  if (ctx->stat_queued) {
    ECS_CUDA(ctx, cudaEventSynchronize(ctx->ev_stat));
  } else {
    ECS_CUDA(ctx, cudaMemcpyAsync(ctx->hstat, ctx->dstat, sizeof(EcsDevStatus), cudaMemcpyDeviceToHost, ctx->stream));
    ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  ctx->stat_queued = false;
  return ECS_OK;
}

int ecs_part_settle(EcsCtx *ctx) {
  if (!ctx->coll_pending) return ECS_OK;
  int rc = status_to_host(ctx);
  if (rc) return rc;
  ctx->coll_pending = false;
  return collisions_update(ctx, ctx->coll_dt);
}

int ecs_part_status_finish(EcsCtx *ctx) {
  int rc = status_to_host(ctx);
  if (rc) return rc;
  if (ctx->coll_pending) {
    ctx->coll_pending = false;
    rc = collisions_update(ctx, ctx->coll_dt);
  }
  const unsigned int f = ctx->hstat->flags;
  if (f & ECS_FLAG_NONFINITE) return ecs_fail(ctx, ECS_ERR_NONFINITE, "non-finite particle velocity");
  if (f & ECS_FLAG_RANGE) return ecs_fail(ctx, ECS_ERR_RANGE, "particle outside the domain or deposit range exceeded");
  return rc;
}

int ecs_part_estimate_rate(EcsCtx *ctx, double dt) {
  PartK k = make_k(ctx, dt);
  ECS_CUDA(ctx, cudaMemsetAsync(ctx->dstat, 0, sizeof(EcsDevStatus), ctx->stream));
  unsigned int g = grid_blocks(ctx, ctx->np, 8);
  if (ctx->prec == ECS_PREC_FP64) {
    k_estimate64<<<g, kBlock, 0, ctx->stream>>>(k, ctx->np, ctx->px, ctx->py, ctx->pz, ctx->vx, ctx->vy,
                                               ctx->vz, ctx->dstat);
  } else {
    k_estimate32<<<g, kBlock, 0, ctx->stream>>>(k, ctx->np, ctx->ions[ctx->cur], ctx->dstat);
  }
  ECS_LAUNCHED(ctx);
  ECS_CUDA(ctx, cudaMemcpyAsync(ctx->hstat, ctx->dstat, sizeof(EcsDevStatus), cudaMemcpyDeviceToHost, ctx->stream));
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double mean = ctx->hstat->acc_count ? (double)ctx->hstat->acc_fix / 16777216.0 / (double)ctx->hstat->acc_count : 0.0;
  int64_t Nc = collision_target(ctx, dt);
  ctx->attempt_rate = (mean > 0 && ctx->np > 0) ? (double)Nc / ((double)ctx->np * mean) : 0.0;
  return ECS_OK;
}

int ecs_part_push(EcsCtx *ctx, double dt) { return launch_particles(ctx, dt, 1); }
int ecs_part_collide(EcsCtx *ctx, double dt) {
  if (ctx->p.mn <= 0.0) return ECS_OK;
  int rc = launch_particles(ctx, dt, 2);
  if (rc) return rc;
  rc = finish_collisions(ctx, dt);
  ctx->step_index++;
  return rc;
}

// Whether the pass that moves the ions now is followed by a cell sort.
// The tile kernel's windows are 3-D, so 2-D ions stay unsorted (order-free
// kernel).
static bool sort_due(const EcsCtx *ctx) {
  return ctx->prec == ECS_PREC_MIXED && ctx->p.ndim == 3 && ctx->sort_every > 0 &&
         ctx->steps_since_sort + 1 >= ctx->sort_every;
}

// Scan of the cell counts and the permutation into key order (the next
// particle pass moves the records).
static int sort_counted(EcsCtx *ctx) {
  const int n = (int)ctx->nkeys;
  const int nb = (int)ecs_div_up(ctx->nkeys, (size_t)kScanBlock * kScanItems);
  k_scan_local<<<nb, kScanBlock, 0, ctx->stream>>>(n, ctx->sort_count, ctx->sort_offset, ctx->scan_blocks);
  ECS_LAUNCHED(ctx);
  k_scan_sums<<<1, 1024, 0, ctx->stream>>>(nb, ctx->scan_blocks);
  ECS_LAUNCHED(ctx);
  k_scan_add<<<ecs_div_up(ctx->nkeys, 256), 256, 0, ctx->stream>>>(n, ctx->sort_offset, ctx->scan_blocks,
                                                                  (int)ctx->np);
  ECS_LAUNCHED(ctx);
  ECS_CUDA(ctx, cudaMemsetAsync(ctx->sort_count, 0, ctx->nkeys * sizeof(int32_t), ctx->stream));
  k_sort_index<<<grid_blocks(ctx, ctx->np, 8), kBlock, 0, ctx->stream>>>(ctx->np, ctx->sort_keys, ctx->sort_offset,
                                                                        ctx->sort_count, ctx->perm);
  ECS_LAUNCHED(ctx);
  ctx->perm_pending = true;
  ctx->steps_since_sort = 0;
  ctx->tiles_valid = true;
  ctx->bounds_valid = false;
  ctx->pgen++;
  return ECS_OK;
}

static int sort_after_pass(EcsCtx *ctx, bool counted) {
  if (!counted) {
    ctx->steps_since_sort++;
    return ECS_OK;
  }
  if (ctx->ev[2]) cudaEventRecord(ctx->ev[2], ctx->stream);
  int rc = sort_counted(ctx);
  if (rc) return rc;
  if (ctx->ev[3]) {
    cudaEventRecord(ctx->ev[3], ctx->stream);
    ctx->ev_sort = true;
  }
  return ECS_OK;
}

// UpdatePositions + ApplyBC, then (DMSwarmMigrate analogue,
// src/boundaries.c:92) the cell sort when it is due.
int ecs_part_move(EcsCtx *ctx, double dt) {
  const bool counted = sort_due(ctx) && ctx->np > 0;
  int rc = launch_particles(ctx, dt, 4, counted);
  if (rc) return rc;
  return sort_after_pass(ctx, counted);
}
int ecs_part_collect(EcsCtx *ctx) {
  int rc = ecs_grid_clear_acc(ctx);
  if (rc) return rc;
  return launch_particles(ctx, 0.0, 8);
}
int ecs_part_fused(EcsCtx *ctx, double dt, int do_collide, int *sorted) {
  int rc = ecs_grid_clear_acc(ctx);
  if (rc) return rc;
  int collide = do_collide && ctx->p.mn > 0.0;
  const bool counted = sort_due(ctx) && ctx->np > 0;
  rc = launch_particles(ctx, dt, 1 | (collide ? 2 : 0) | 4 | 8, counted);
  if (rc) return rc;
  if ((rc = sort_after_pass(ctx, counted))) return rc;
  if (sorted) *sorted = counted ? 1 : 0;
  if (collide) {  // the rate update waits for the counters (ecs_part_status_finish)
    ctx->coll_pending = true;
    ctx->coll_dt = dt;
    ctx->step_index++;
  }
  return rc;
}

// ---- the particle pass of ecs_step_host, pipelined with the host copies ---------
// When the host arrays hold the ions as the previous ecs_step_host call
// returned them (the generation count has not moved since), they are in the
// order of the device records, so the upload, the fused pass and the
// download run chunk by chunk:
//   uploads   fixed chunks of stage_n ions: copies in on xs[1], conversion
//             into the records on xs_up (two staging buffers), all issued
//             at once;
//   the pass  by ranges of whole tiles (at most stage_n ions) on the
//             context's stream, each range after the upload chunks it reads
//             have been converted;
//   downloads by the same ranges: conversion on xs_conv, copies out on
//             xs[0] (three staging buffers).
// The copies in never wait for the copies out, so both directions of the
// host link stay busy.  After a cell sort (pending permutation) the pass
// gathers each range's ions from their old positions (the host arrays'
// order) into the other record buffer in key order: a range then waits for
// the upload chunks of its largest source position (tile_srcmax) and of its
// own host span, which its download overwrites.  The pass that counts cells
// for a sort downloads in its own order; the next call gathers.  The
// identities become the host indices, as in an upload.
//
// The copies start and end on 256-byte host boundaries: a copy of host
// memory that starts inside a 256-byte block moves about a quarter less per
// second over the host link while copies run both ways.  An upload reads
// from the boundary at or below its chunk's first double to the one at or
// above its last (bytes of the neighbours, not converted); a download
// writes from the boundary at or below its range's first double to the
// boundary at or below the next range's, so the few ions before that
// boundary go out with the next range (their records are final by then).
constexpr uintptr_t kXferAlign = 256;
static inline double *xfer_lo(double *P, int64_t A, int64_t np) {
  if (A <= 0) return P;
  if (A >= np) return P + 3 * np;
  if ((uintptr_t)P % sizeof(double)) return P + 3 * A;
  const uintptr_t a = (uintptr_t)(P + 3 * A) & ~(kXferAlign - 1);
  return a > (uintptr_t)P ? (double *)a : P;
}
static inline double *xfer_hi(double *P, int64_t A, int64_t np) {
  if (A >= np) return P + 3 * np;
  if ((uintptr_t)P % sizeof(double)) return P + 3 * A;
  const uintptr_t a = ((uintptr_t)(P + 3 * A) + kXferAlign - 1) & ~(kXferAlign - 1);
  return a < (uintptr_t)(P + 3 * np) ? (double *)a : P + 3 * np;
}

// Download of the records [A, A + n) of recs as the whole host spans from
// xfer_lo(A) to xfer_lo(A + n): conversion on xs_conv into staging buffer
// qd, copies on xs[0].
static int host_span_out(EcsCtx *ctx, const PartK &k, double *pos, double *vel, int64_t np, int64_t A, int64_t n,
                         const float4 *recs, int qd) {
  const int64_t stride = ecs_stage_stride(ctx->stage_n);
  double *out = ctx->stage_dn[qd];
  double *p0 = xfer_lo(pos, A, np), *p1 = xfer_lo(pos, A + n, np);
  double *v0 = xfer_lo(vel, A, np), *v1 = xfer_lo(vel, A + n, np);
  const int64_t d0 = p0 - pos, d1 = p1 - pos, e0 = v0 - vel, e1 = v1 - vel;
  const int64_t i0 = std::min(d0 / 3, e0 / 3), i1 = A + n;
  k_mixed_to_aos_span<<<grid_blocks(ctx, i1 - i0, 8), kBlock, 0, ctx->xs_conv>>>(i0, i1, d0, d1, e0, e1, k, out,
                                                                               out + stride, recs);
  ECS_LAUNCHED(ctx);
  ECS_CUDA(ctx, cudaEventRecord(ctx->xev_dn_conv[qd], ctx->xs_conv));
  ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->xs[0], ctx->xev_dn_conv[qd], 0));
  if (d1 > d0)
    ECS_CUDA(ctx, cudaMemcpyAsync(p0, out, (size_t)(d1 - d0) * sizeof(double), cudaMemcpyDeviceToHost, ctx->xs[0]));
  if (e1 > e0)
    ECS_CUDA(ctx, cudaMemcpyAsync(v0, out + stride, (size_t)(e1 - e0) * sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx->xs[0]));
  ECS_CUDA(ctx, cudaEventRecord(ctx->xev_dn_copy[qd], ctx->xs[0]));
  return ECS_OK;
}

// The current sort's first ion of every tile (tile_bounds) and, with a
// gather pending, every tile's largest source position (tile_srcmax).
// The tables and their device buffer are allocated once per context, so that
// no step allocates or frees memory.
static int host_tile_tables(EcsCtx *ctx, int ntiles, bool gather) {
  const bool want_b = !ctx->bounds_valid;
  if (!want_b && !gather) return ECS_OK;
  const size_t nb = (size_t)ntiles + 1, words = nb + (size_t)ntiles;
  if (!ctx->tile_tables_dev) {
    ECS_CUDA(ctx, cudaMalloc((void **)&ctx->tile_tables_dev, words * sizeof(int32_t)));
    ECS_CUDA(ctx, cudaMallocHost((void **)&ctx->tile_bounds, words * sizeof(int32_t)));
    ctx->tile_srcmax = ctx->tile_bounds + nb;
  }
  int32_t *d = ctx->tile_tables_dev;
  if (want_b) {
    k_tile_bounds<<<ecs_div_up(nb, 256), 256, 0, ctx->stream>>>(ntiles, ctx->sort_offset, d);
    ECS_LAUNCHED(ctx);
    ECS_CUDA(ctx, cudaMemcpyAsync(ctx->tile_bounds, d, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (gather) {
    k_tile_srcmax<<<ecs_div_up((size_t)ntiles * 32, 256), 256, 0, ctx->stream>>>(ntiles, ctx->sort_offset, ctx->perm,
                                                                                  d + nb);
    ECS_LAUNCHED(ctx);
    ECS_CUDA(ctx, cudaMemcpyAsync(ctx->tile_srcmax, d + nb, (size_t)ntiles * sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, ctx->stream));
  }
  ECS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->bounds_valid = true;
  return ECS_OK;
}

int ecs_part_host_pass(EcsCtx *ctx, double *pos, double *vel, int64_t np, double dt, int *sorted) {
  if (ctx->prec != ECS_PREC_MIXED || ctx->p.ndim != 3 || np != ctx->np || np == 0 || !ctx->tiles_valid ||
      ctx->host_gen != ctx->pgen)
    return ECS_ERR_STATE;
  int rc = ensure_xfer(ctx);
  if (rc) return rc;
  const int64_t chunk = ctx->stage_n;
  const int ntiles = ctx->ntile[0] * ctx->ntile[1] * ctx->ntile[2];
  const bool gather = ctx->perm_pending;
  if ((rc = host_tile_tables(ctx, ntiles, gather))) return rc;
  const int32_t *tb = ctx->tile_bounds;
  if (tb[ntiles] != np) return ECS_ERR_STATE;
  for (int t = 0; t < ntiles; t++)
    if (tb[t + 1] - tb[t] > chunk) return ECS_ERR_STATE;  // a tile larger than a staging chunk
  const int64_t nup = ecs_div_up(np, chunk);
  if (!ctx->stage_dn[0]) {
    ECS_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->xs_conv, cudaStreamNonBlocking));
    ECS_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->xs_up, cudaStreamNonBlocking));
    for (int q = 0; q < EcsCtx::kStageDn; q++) {
      ECS_CUDA(ctx, cudaMalloc((void **)&ctx->stage_dn[q], (size_t)ecs_stage_stride(chunk) * 2 * sizeof(double)));
      ECS_CUDA(ctx, cudaEventCreateWithFlags(&ctx->xev_tiled[q], cudaEventDisableTiming));
      ECS_CUDA(ctx, cudaEventCreateWithFlags(&ctx->xev_dn_conv[q], cudaEventDisableTiming));
      ECS_CUDA(ctx, cudaEventCreateWithFlags(&ctx->xev_dn_copy[q], cudaEventDisableTiming));
    }
  }
  while ((int64_t)ctx->xev_upc.size() < nup) {
    cudaEvent_t e;
    ECS_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ctx->xev_upc.push_back(e);
  }
  constexpr int ND = EcsCtx::kStageDn;
  const int64_t stride = ecs_stage_stride(chunk);
  const int collide = ctx->p.mn > 0.0;
  int mode = 1 | (collide ? 2 : 0) | 4 | 8;
  PartK k;
  if ((rc = pass_params(ctx, dt, mode, k))) return rc;
  const bool counted = sort_due(ctx);
  if ((rc = ecs_grid_clear_acc(ctx))) return rc;
  if (counted) ECS_CUDA(ctx, cudaMemsetAsync(ctx->sort_count, 0, ctx->nkeys * sizeof(int32_t), ctx->stream));
  int32_t *count = counted ? ctx->sort_count : nullptr;
  const int nd = 3;
  ctx->pgen++;
  float4 *src = ctx->ions[ctx->cur];
  float4 *dst = gather ? ctx->ions[1 - ctx->cur] : src;
  ECS_CUDA(ctx, cudaEventRecord(ctx->xev_ready, ctx->stream));  // earlier work on the buffers
  for (cudaStream_t s : {ctx->xs[0], ctx->xs[1], ctx->xs_conv, ctx->xs_up})
    ECS_CUDA(ctx, cudaStreamWaitEvent(s, ctx->xev_ready, 0));
  if (ctx->ev[0]) cudaEventRecord(ctx->ev[0], ctx->stream);
  // every upload chunk: copies in, then its conversion into the records
  for (int64_t u = 0; u < nup; u++) {
    const int q = (int)(u & 1);
    const int64_t A = u * chunk, n = std::min(chunk, np - A);
    double *in = ctx->stage[q];
    if (u >= 2) ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->xs[1], ctx->xev_upc[u - 2], 0));  // staging in free
    double *p0 = xfer_lo(pos, A, np), *p1 = xfer_hi(pos, A + n, np);
    double *v0 = xfer_lo(vel, A, np), *v1 = xfer_hi(vel, A + n, np);
    ECS_CUDA(ctx, cudaMemcpyAsync(in, p0, (size_t)(p1 - p0) * sizeof(double), cudaMemcpyHostToDevice, ctx->xs[1]));
    ECS_CUDA(ctx, cudaMemcpyAsync(in + stride, v0, (size_t)(v1 - v0) * sizeof(double), cudaMemcpyHostToDevice,
                                  ctx->xs[1]));
    ECS_CUDA(ctx, cudaEventRecord(ctx->xev_copy[q], ctx->xs[1]));
    ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->xs_up, ctx->xev_copy[q], 0));
    k_aos_to_mixed<<<grid_blocks(ctx, n, 8), kBlock, 0, ctx->xs_up>>>(n, nd, k, in + (pos + nd * A - p0),
                                                                    in + stride + (vel + nd * A - v0), src + 2 * A, A);
    ECS_LAUNCHED(ctx);
    ECS_CUDA(ctx, cudaEventRecord(ctx->xev_upc[u], ctx->xs_up));
  }
  // the pass and the download by ranges of whole tiles; a range waits for
  // the upload chunk of the last ion it reads (gathered sources) or
  // overwrites on the host (its own span)
  struct Range {
    int t0, t1;
    int64_t A, n, need;
  };
  std::vector<Range> rg;
  const int32_t *smax = gather ? ctx->tile_srcmax : nullptr;
  for (int t0 = 0; t0 < ntiles;) {
    int t1 = t0 + 1;
    while (t1 < ntiles && (int64_t)tb[t1 + 1] - tb[t0] <= chunk) t1++;
    const int64_t A = tb[t0], n = (int64_t)tb[t1] - A;
    if (n > 0) {
      int64_t last = A + n - 1;
      if (smax)
        for (int t = t0; t < t1; t++) last = std::max(last, (int64_t)smax[t]);
      rg.push_back({t0, t1, A, n, std::min(last / chunk, nup - 1)});
    }
    t0 = t1;
  }
  // The kernels run in the order of the chunks they wait for (after a sort,
  // ions that crossed a periodic face come from the far end of the old
  // order: their ranges go last).  A range's download also carries the last
  // few ions of the range before it, so it goes out once both are done.
  const int R = (int)rg.size();
  std::vector<int> order(R);
  for (int r = 0; r < R; r++) order[r] = r;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return rg[a].need < rg[b].need; });
  std::vector<char> done(R, 0), out(R, 0);
  int64_t waited = -1, c = 0;
  for (int r : order) {
    const Range &g = rg[r];
    if (g.need > waited) {
      ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->xev_upc[g.need], 0));
      waited = g.need;
    }
    k_tiles32<<<g.t1 - g.t0, kTileThreads, 0, ctx->stream>>>(k, mode, src, dst, gather ? ctx->perm : nullptr,
                                                          ctx->eext32, ctx->acc, ctx->sort_offset, count,
                                                          ctx->sort_keys, ctx->dstat, g.t0, g.t1);
    ECS_LAUNCHED(ctx);
    done[r] = 1;
    for (int d = r; d <= r + 1 && d < R; d++) {
      if (out[d] || !done[d] || (d > 0 && !done[d - 1])) continue;
      const int qd = (int)(c % ND);
      ECS_CUDA(ctx, cudaEventRecord(ctx->xev_tiled[qd], ctx->stream));
      ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->xs_conv, ctx->xev_tiled[qd], 0));
      if (c >= ND) ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->xs_conv, ctx->xev_dn_copy[qd], 0));  // staging out free
      if ((rc = host_span_out(ctx, k, pos, vel, np, rg[d].A, rg[d].n, dst, qd))) return rc;
      out[d] = 1;
      c++;
    }
  }
  if (waited < nup - 1) ECS_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->xev_upc[nup - 1], 0));
  if (ctx->ev[1]) {
    cudaEventRecord(ctx->ev[1], ctx->stream);
    ctx->ev_particle = true;
  }
  if (gather) {
    ctx->cur = 1 - ctx->cur;
    ctx->perm_pending = false;
  }
  if ((rc = sort_after_pass(ctx, counted))) return rc;
  if (sorted) *sorted = counted ? 1 : 0;
  if (mode & 2) {  // the rate update waits for the counters (ecs_part_status_finish)
    ctx->coll_pending = true;
    ctx->coll_dt = dt;
    ctx->step_index++;
  }
  return rc;
}

// Full counting sort (count pass included), used after an upload.
int ecs_part_sort(EcsCtx *ctx) {
  if (ctx->prec != ECS_PREC_MIXED || ctx->np == 0 || ctx->p.ndim != 3) return ECS_OK;
  int rc = settle_order(ctx);
  if (rc) return rc;
  ECS_CUDA(ctx, cudaMemsetAsync(ctx->sort_count, 0, ctx->nkeys * sizeof(int32_t), ctx->stream));
  const PartK k = make_k(ctx, 0.0);
  k_sort_count<<<grid_blocks(ctx, ctx->np, 8), kBlock, 0, ctx->stream>>>(ctx->np, k.tg, ctx->ions[ctx->cur],
                                                                        ctx->sort_count, ctx->sort_keys);
  ECS_LAUNCHED(ctx);
  return sort_counted(ctx);
}
