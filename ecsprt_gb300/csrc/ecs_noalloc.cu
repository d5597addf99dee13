// ecs_rhs_noalloc: the right-hand side of the quasineutral potential equation
// (ComputeFullRHS3D src/rhs.c:259-373 / ComputeFullRHS2D src/rhs.c:151-256,
// or the -rhs constant / sinusoidal options src/rhs.c:6-148, each with the
// reference's mean removal) for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at the point where they need the RHS:
// a host framework that reserves its whole device-memory budget in its own
// pool at start-up and forbids allocations inside its time-step loop, or a
// latency-critical loop that cannot accept the implicit device
// synchronisation an allocation may cause.  They own the input and output
// buffers; this entry point needs only a small reduction scratch, which lives
// in a file-scope __device__ array instead of an allocation.
//
// Scratch: ECS_NOALLOC_RHS_MAX_BLOCKS FP64 block partial sums plus one slot
// for the mean (32 KiB + 8 B), present on every device that loads the
// library until the process exits.  Each thread block reduces
// ECS_NOALLOC_RHS_CELLS_PER_BLOCK cells, so grids of at most
// ECS_NOALLOC_RHS_MAX_CELLS cells (256 x 256 x 128) are accepted.
//
// Every call shares the array: each call writes every partial and the mean
// before it reads them, so nothing from an earlier call is used, but two
// calls that overlap on the GPU (different streams without ordering) race on
// it.
//
// The array's device address is looked up once per device, the first time a
// call runs with that device current, and cached for the life of the
// process.  The cache does not survive cudaDeviceReset (or anything else that
// replaces the device's primary context): a process that resets a device
// must not call this entry point on it afterwards.
#include <math.h>

#include <algorithm>
#include <mutex>

#include "ecs_internal.cuh"

#define ECS_NOALLOC_RHS_MAX_BLOCKS 4096
#define ECS_NOALLOC_RHS_CELLS_PER_BLOCK 2048
#define ECS_NOALLOC_RHS_MAX_CELLS (ECS_NOALLOC_RHS_MAX_BLOCKS * ECS_NOALLOC_RHS_CELLS_PER_BLOCK)
#define ECS_NOALLOC_MAX_DEVICES 64

// [0, MAX_BLOCKS): block partial sums of b; [MAX_BLOCKS]: the mean of b.
static __device__ __align__(256) double g_rhs_scratch[ECS_NOALLOC_RHS_MAX_BLOCKS + 1];

namespace {

constexpr int kThreads = 256;

struct rdn {
  double v;
};
__device__ __forceinline__ rdn operator+(rdn a, rdn b) { return {__dadd_rn(a.v, b.v)}; }
__device__ __forceinline__ rdn operator-(rdn a, rdn b) { return {__dsub_rn(a.v, b.v)}; }
__device__ __forceinline__ rdn operator*(rdn a, rdn b) { return {__dmul_rn(a.v, b.v)}; }

struct RhsNoAllocK {
  int nx, ny, nz;
  int bc[3];
  int ndim;
  size_t n;
  double kappa, hx, hy, hz, hxx, hyy, hzz, E0, cth, cG, scale;
  double dx, dy, dz, n0;  // -rhs sinusoidal
};

// Moment c of node (k,j,i) from FluidNode{n,Gx,Gy,Gz} storage, with the
// reference's ghost semantics (periodic wrap, zero outside ghosted axes).
__device__ __forceinline__ double node_moment(const double *__restrict__ m, const RhsNoAllocK &g, int k,
                                              int j, int i, int c) {
  if (i < 0 || i >= g.nx) { if (g.bc[0]) return 0.0; i = i < 0 ? i + g.nx : i - g.nx; }
  if (j < 0 || j >= g.ny) { if (g.bc[1]) return 0.0; j = j < 0 ? j + g.ny : j - g.ny; }
  if (k < 0 || k >= g.nz) { if (g.bc[2]) return 0.0; k = k < 0 ? k + g.nz : k - g.nz; }
  return m[(((size_t)k * g.ny + j) * g.nx + i) * 4 + c];
}

// b of the full RHS (src/rhs.c:321-354) at node (k, j, i).  A 2-D grid is
// one node deep with a unit, periodic z cell, so every z term is exactly 0.
__device__ __forceinline__ double full_rhs(const double *__restrict__ mom, const RhsNoAllocK &g, int k, int j,
                                           int i) {
  rdn nijk{node_moment(mom, g, k, j, i, 0)};
  rdn npjk{node_moment(mom, g, k, j, i + 1, 0)}, nmjk{node_moment(mom, g, k, j, i - 1, 0)};
  rdn nipk{node_moment(mom, g, k, j + 1, i, 0)}, nimk{node_moment(mom, g, k, j - 1, i, 0)};
  rdn nijp{node_moment(mom, g, k + 1, j, i, 0)}, nijm{node_moment(mom, g, k - 1, j, i, 0)};
  rdn two{2.0}, one{1.0}, kap{g.kappa};
  rdn dndx = rdn{g.hx} * (npjk - nmjk);
  rdn dndy = rdn{g.hy} * (nipk - nimk);
  rdn d2ndxx = rdn{g.hxx} * ((npjk - two * nijk) + nmjk);
  rdn d2ndyy = rdn{g.hyy} * ((nipk - two * nijk) + nimk);
  rdn d2ndzz = rdn{g.hzz} * ((nijp - two * nijk) + nijm);
  rdn dGxdx = rdn{g.hx} * (rdn{node_moment(mom, g, k, j, i + 1, 1)} - rdn{node_moment(mom, g, k, j, i - 1, 1)});
  rdn dGydy = rdn{g.hy} * (rdn{node_moment(mom, g, k, j + 1, i, 2)} - rdn{node_moment(mom, g, k, j - 1, i, 2)});
  rdn dGzdz = rdn{g.hz} * (rdn{node_moment(mom, g, k + 1, j, i, 3)} - rdn{node_moment(mom, g, k - 1, j, i, 3)});
  rdn Eterm = (dndy - kap * dndx) * rdn{g.E0};
  rdn Pterm = rdn{g.cth} * ((d2ndxx + d2ndyy) + (one + kap * kap) * d2ndzz);
  rdn Gterm = rdn{g.cG} * ((dGxdx + dGydy) + dGzdz);
  return (rdn{g.scale} * ((Eterm + Pterm) + Gterm)).v;
}

// b of -rhs sinusoidal (src/rhs.c:82-148; 2-D src/rhs.c:26-79): n0 cos(2 pi
// x) cos(2 pi y) [cos(2 pi z)] scale at the cell centres in grid units.
__device__ __forceinline__ double sin_rhs(const RhsNoAllocK &g, int k, int j, int i) {
  const double twopi = 2 * M_PI;
  const double cx = cos(__dmul_rn(twopi, __dmul_rn(__dadd_rn((double)i, 0.5), g.dx)));
  const double cy = cos(__dmul_rn(twopi, __dmul_rn(__dadd_rn((double)j, 0.5), g.dy)));
  const double cxy = __dmul_rn(cx, cy);
  const double val =
      g.ndim == 2 ? cxy : __dmul_rn(cxy, cos(__dmul_rn(twopi, __dmul_rn(__dadd_rn((double)k, 0.5), g.dz))));
  return __dmul_rn(__dmul_rn(g.n0, val), g.scale);
}

// One block per ECS_NOALLOC_RHS_CELLS_PER_BLOCK consecutive cells; each
// block writes its partial sum of b into partials[blockIdx.x].
template <bool kSinusoidal>
__global__ void __launch_bounds__(kThreads) k_rhs_noalloc(RhsNoAllocK g, const double *__restrict__ mom,
                                                          double *__restrict__ b, double *__restrict__ partials) {
  __shared__ double sh[kThreads / 32];
  double local = 0.0;
  const size_t c0 = (size_t)blockIdx.x * ECS_NOALLOC_RHS_CELLS_PER_BLOCK;
  for (int q = threadIdx.x; q < ECS_NOALLOC_RHS_CELLS_PER_BLOCK; q += blockDim.x) {
    const size_t c = c0 + q;
    if (c >= g.n) break;
    const int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / ((size_t)g.nx * g.ny));
    const double v = kSinusoidal ? sin_rhs(g, k, j, i) : full_rhs(mom, g, k, j, i);
    b[c] = v;
    local += v;
  }
  for (int s = 16; s >= 1; s >>= 1) local += __shfl_xor_sync(ECS_FULL_MASK, local, s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kThreads / 32; w++) t += sh[w];
    partials[blockIdx.x] = t;
  }
}

// The mean, once: one block sums the nb partials in a fixed order (strided
// per thread, warp tree, then the warps in order) into partials[MAX_BLOCKS].
__global__ void __launch_bounds__(1024) k_mean_noalloc(int nb, double n, double *__restrict__ partials) {
  __shared__ double sh[32];
  double t = 0.0;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) t += partials[q];
  for (int s = 16; s >= 1; s >>= 1) t += __shfl_xor_sync(ECS_FULL_MASK, t, s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) u += sh[w];
    partials[ECS_NOALLOC_RHS_MAX_BLOCKS] = u / n;
  }
}

__global__ void __launch_bounds__(kThreads) k_sub_mean_noalloc(size_t n, double *__restrict__ b,
                                                               const double *__restrict__ partials) {
  const double mean = partials[ECS_NOALLOC_RHS_MAX_BLOCKS];
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    b[c] -= mean;
}

// -rhs constant (src/rhs.c:6-23): b = n0 scale everywhere, no projection.
__global__ void __launch_bounds__(kThreads) k_fill_noalloc(size_t n, double v, double *__restrict__ b) {
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    b[c] = v;
}

// Device address of the scratch array, looked up once per device.
std::mutex g_setup_mutex;
double *g_scratch_addr[ECS_NOALLOC_MAX_DEVICES] = {nullptr};

cudaError_t scratch_for_current_device(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= ECS_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    double *ptr = nullptr;
    e = cudaGetSymbolAddress((void **)&ptr, g_rhs_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = ptr;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

int launched(const char *what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return ecs_fail(nullptr, ECS_ERR_CUDA, "ecs_rhs_noalloc: %s launch: %s", what, cudaGetErrorString(e));
  return ECS_OK;
}

}  // namespace

extern "C" int ecs_rhs_noalloc(const EcsParams *params, const double *d_moments, double *d_rhs, void *stream) {
  if (!params || !d_rhs) return ecs_fail(nullptr, ECS_ERR_INVALID, "ecs_rhs_noalloc: NULL argument");
  int rc = ecs_validate_params(params);  // the checks of ecs_ctx_create
  if (rc) return rc;
  if (params->rhs_type == ECS_RHS_FULL && !d_moments)
    return ecs_fail(nullptr, ECS_ERR_INVALID, "ecs_rhs_noalloc: NULL moments for -rhs full");
  // 2-D runs on a one-node-deep grid with a unit, periodic z cell, as a
  // context does (the reference's 2-D parameters have dz = 0)
  EcsParams p = *params;
  if (p.ndim == 2) {
    p.dz = 1.0;
    p.bc[2] = ECS_BC_PERIODIC;
  }
  const size_t n = (size_t)p.Nx * p.Ny * p.Nz;
  if (n > (size_t)ECS_NOALLOC_RHS_MAX_CELLS)
    return ecs_fail(nullptr, ECS_ERR_INVALID,
                    "ecs_rhs_noalloc: %zu grid nodes exceed the fixed scratch limit of %d nodes "
                    "(256x256x128); use ecs_rhs on a context for larger grids",
                    n, ECS_NOALLOC_RHS_MAX_CELLS);
  double *scratch = nullptr;
  cudaError_t e = scratch_for_current_device(&scratch);
  if (e != cudaSuccess)
    return ecs_fail(nullptr, ECS_ERR_CUDA, "ecs_rhs_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
  cudaStream_t s = (cudaStream_t)stream;
  const int nb_elem = (int)std::min<size_t>((n + kThreads - 1) / kThreads, 4096);
  if (p.rhs_type == ECS_RHS_CONSTANT) {
    k_fill_noalloc<<<nb_elem, kThreads, 0, s>>>(n, p.n0 * p.scale, d_rhs);
    return launched("fill");
  }
  RhsNoAllocK g;
  g.nx = p.Nx; g.ny = p.Ny; g.nz = p.Nz;
  for (int d = 0; d < 3; d++) g.bc[d] = p.bc[d] == ECS_BC_PERIODIC ? 0 : 1;
  g.ndim = p.ndim;
  g.n = n;
  g.kappa = p.kappa_e;
  g.hx = 1.0 / (2.0 * p.dx); g.hy = 1.0 / (2.0 * p.dy); g.hz = 1.0 / (2.0 * p.dz);
  g.hxx = 1.0 / (p.dx * p.dx); g.hyy = 1.0 / (p.dy * p.dy); g.hzz = 1.0 / (p.dz * p.dz);
  g.E0 = p.E0; g.cth = p.cth; g.cG = p.cG; g.scale = p.scale;
  g.dx = p.dx; g.dy = p.dy; g.dz = p.dz; g.n0 = p.n0;
  const int nb = (int)((n + ECS_NOALLOC_RHS_CELLS_PER_BLOCK - 1) / ECS_NOALLOC_RHS_CELLS_PER_BLOCK);
  if (p.rhs_type == ECS_RHS_SINUSOIDAL)
    k_rhs_noalloc<true><<<nb, kThreads, 0, s>>>(g, d_moments, d_rhs, scratch);
  else
    k_rhs_noalloc<false><<<nb, kThreads, 0, s>>>(g, d_moments, d_rhs, scratch);
  if ((rc = launched("rhs"))) return rc;
  k_mean_noalloc<<<1, 1024, 0, s>>>(nb, (double)n, scratch);
  if ((rc = launched("mean"))) return rc;
  k_sub_mean_noalloc<<<nb_elem, kThreads, 0, s>>>(n, d_rhs, scratch);
  return launched("mean removal");
}
