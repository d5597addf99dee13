// ecs_rhs_noalloc: the quasineutral RHS (src/rhs.c:259-373, mean removed as
// src/rhs.c:363-366 does) for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at the point where they need the RHS:
// a host framework that reserves its whole device-memory budget in its own
// pool at start-up and forbids allocations inside its time-step loop, or a
// latency-critical loop that cannot accept the implicit device
// synchronisation an allocation may cause.  They own the input and output
// buffers; this entry point needs only a small reduction scratch, which lives
// in a file-scope __device__ array instead of an allocation.
//
// Scratch: ECS_NOALLOC_RHS_MAX_BLOCKS FP64 block partial sums (32 KiB),
// present on every device that loads the library until the process exits.
// Each thread block reduces ECS_NOALLOC_RHS_CELLS_PER_BLOCK cells, so grids
// of at most ECS_NOALLOC_RHS_MAX_CELLS cells (256 x 256 x 128) are accepted.
//
// Every call shares the array: each call writes every partial it reads, so
// nothing from an earlier call is used, but two calls that overlap on the GPU
// (different streams without ordering) race on it.
#include <algorithm>
#include <mutex>

#include "ecs_internal.cuh"

#define ECS_NOALLOC_RHS_MAX_BLOCKS 4096
#define ECS_NOALLOC_RHS_CELLS_PER_BLOCK 2048
#define ECS_NOALLOC_RHS_MAX_CELLS (ECS_NOALLOC_RHS_MAX_BLOCKS * ECS_NOALLOC_RHS_CELLS_PER_BLOCK)
#define ECS_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_rhs_partials[ECS_NOALLOC_RHS_MAX_BLOCKS];

namespace {

struct rdn {
  double v;
};
__device__ __forceinline__ rdn operator+(rdn a, rdn b) { return {__dadd_rn(a.v, b.v)}; }
__device__ __forceinline__ rdn operator-(rdn a, rdn b) { return {__dsub_rn(a.v, b.v)}; }
__device__ __forceinline__ rdn operator*(rdn a, rdn b) { return {__dmul_rn(a.v, b.v)}; }

struct RhsNoAllocK {
  int nx, ny, nz;
  int bc[3];
  size_t n;
  double kappa, hx, hy, hz, hxx, hyy, hzz, E0, cth, cG, scale;
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

// One block per ECS_NOALLOC_RHS_CELLS_PER_BLOCK consecutive cells; each
// block writes its partial sum of b into partials[blockIdx.x].
__global__ void __launch_bounds__(256) k_rhs_noalloc(RhsNoAllocK g, const double *__restrict__ mom,
                                                     double *__restrict__ b, double *__restrict__ partials) {
  __shared__ double sh[8];
  double local = 0.0;
  const size_t c0 = (size_t)blockIdx.x * ECS_NOALLOC_RHS_CELLS_PER_BLOCK;
  for (int q = threadIdx.x; q < ECS_NOALLOC_RHS_CELLS_PER_BLOCK; q += blockDim.x) {
    size_t c = c0 + q;
    if (c >= g.n) break;
    int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / ((size_t)g.nx * g.ny));
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
    double v = (rdn{g.scale} * ((Eterm + Pterm) + Gterm)).v;
    b[c] = v;
    local += v;
  }
  for (int s = 16; s >= 1; s >>= 1) local += __shfl_xor_sync(ECS_FULL_MASK, local, s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    partials[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(256) k_sub_mean_noalloc(size_t n, double *__restrict__ b,
                                                          const double *__restrict__ partials, int nb) {
  __shared__ double mean;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < nb; q++) t += partials[q];
    mean = t / (double)n;
  }
  __syncthreads();
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    b[c] -= mean;
}

// Device address of the scratch array, looked up once per device.
std::mutex g_setup_mutex;
double *g_partials_addr[ECS_NOALLOC_MAX_DEVICES] = {nullptr};

cudaError_t scratch_for_current_device(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= ECS_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_partials_addr[dev]) {
    double *ptr = nullptr;
    e = cudaGetSymbolAddress((void **)&ptr, g_rhs_partials);
    if (e != cudaSuccess) return e;
    g_partials_addr[dev] = ptr;
  }
  *out = g_partials_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int ecs_rhs_noalloc(const EcsParams *p, const double *d_moments, double *d_rhs, void *stream) {
  if (!p || !d_moments || !d_rhs) return ecs_fail(nullptr, ECS_ERR_INVALID, "ecs_rhs_noalloc: NULL argument");
  if (p->Nx < 1 || p->Ny < 1 || p->Nz < 1) return ecs_fail(nullptr, ECS_ERR_INVALID, "ecs_rhs_noalloc: empty grid");
  const size_t n = (size_t)p->Nx * p->Ny * p->Nz;
  if (n > (size_t)ECS_NOALLOC_RHS_MAX_CELLS)
    return ecs_fail(nullptr, ECS_ERR_INVALID,
                    "ecs_rhs_noalloc: %zu grid nodes exceed the fixed scratch limit of %d nodes "
                    "(256x256x128); use ecs_rhs on a context for larger grids",
                    n, ECS_NOALLOC_RHS_MAX_CELLS);
  double *partials = nullptr;
  cudaError_t e = scratch_for_current_device(&partials);
  if (e != cudaSuccess)
    return ecs_fail(nullptr, ECS_ERR_CUDA, "ecs_rhs_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
  RhsNoAllocK g;
  g.nx = p->Nx; g.ny = p->Ny; g.nz = p->Nz;
  for (int d = 0; d < 3; d++) g.bc[d] = p->bc[d] == ECS_BC_PERIODIC ? 0 : 1;
  g.n = n;
  g.kappa = p->kappa_e;
  g.hx = 1.0 / (2.0 * p->dx); g.hy = 1.0 / (2.0 * p->dy); g.hz = 1.0 / (2.0 * p->dz);
  g.hxx = 1.0 / (p->dx * p->dx); g.hyy = 1.0 / (p->dy * p->dy); g.hzz = 1.0 / (p->dz * p->dz);
  g.E0 = p->E0; g.cth = p->cth; g.cG = p->cG; g.scale = p->scale;
  const int nb = (int)((n + ECS_NOALLOC_RHS_CELLS_PER_BLOCK - 1) / ECS_NOALLOC_RHS_CELLS_PER_BLOCK);
  cudaStream_t s = (cudaStream_t)stream;
  k_rhs_noalloc<<<nb, 256, 0, s>>>(g, d_moments, d_rhs, partials);
  e = cudaGetLastError();
  if (e != cudaSuccess) return ecs_fail(nullptr, ECS_ERR_CUDA, "ecs_rhs_noalloc launch: %s", cudaGetErrorString(e));
  const int nb2 = (int)std::min<size_t>((n + 255) / 256, 4096);
  k_sub_mean_noalloc<<<nb2, 256, 0, s>>>(n, d_rhs, partials, nb);
  e = cudaGetLastError();
  if (e != cudaSuccess) return ecs_fail(nullptr, ECS_ERR_CUDA, "ecs_rhs_noalloc launch: %s", cudaGetErrorString(e));
  return ECS_OK;
}
