/*
 * ecs_serve.h -- request loop of libecsgpu: stand-alone potential solves and
 * small simulation instances served concurrently on one GPU.
 *
 * The reference runs one solve per process (src/solver.c:107-203: load a
 * density, fluxes = flux_scale * density in LoadFluidQuantities
 * src/file-io.c:8-75, ComputePotential, write the potential) and one
 * simulation per process (src/pic.c).  A server keeps many of these resident
 * on the device at once:
 *
 *   - Each admitted request owns a slot: a context (ecsgpu.h) whose device
 *     state stays resident for the request's lifetime.  Solve slots are kept
 *     after their request and reused by the next request with the same
 *     parameters, so their CUDA graphs are built once.
 *   - A solve request runs as ONE captured CUDA graph on its slot's stream:
 *     density copy in, fluxes, RHS, operator set-up, the FP32 multigrid-FGMRES
 *     solve inside FP64 iterative refinement (device-side loops), potential
 *     copy out.  Requests of different grid sizes run on different streams at
 *     the same time, so their kernels overlap on the GPU.
 *   - A simulation request is stepped with ecs_step, one step per turn; its
 *     next step is queued behind the work that arrived meanwhile, so
 *     instances and solves interleave (continuous batching).
 *   - Admission is first come, first served against an HBM budget: a request
 *     starts when a worker is free and its slot fits in the budget (idle
 *     solve slots of other parameters are evicted, least recently used
 *     first).  A request larger than the whole budget is rejected at submit.
 *   - Results are bit-identical to the same request run alone: every slot
 *     computes in a fixed order with fixed-point deposition, independent of
 *     what else is on the GPU.
 *
 * Host buffers of a request belong to the caller until its result is polled.
 * Page-locked buffers (ecs_host_alloc, cudaHostAlloc or registered memory)
 * are copied by DMA directly; other buffers go through the slot's staging
 * buffers.  A server's functions may be called from any host thread.
 */
#ifndef ECS_SERVE_H
#define ECS_SERVE_H

#include "ecsgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct EcsServer EcsServer;

enum { ECS_SERVE_SOLVE = 0, ECS_SERVE_SIM = 1 };

typedef struct EcsServeConfig {
  int64_t hbm_budget_bytes; /* device bytes the slots may hold together */
  int32_t max_inflight;     /* worker threads = requests on the GPU at once.  Streams
                               overlap on the device only as far as its hardware work
                               queues allow: set CUDA_DEVICE_MAX_CONNECTIONS (CUDA's
                               default 8) to at least this before the process first
                               uses CUDA, else at most about 4 requests overlap. */
  int32_t precision;        /* ECS_PREC_MIXED or ECS_PREC_FP64 */
  double timeout_seconds;   /* per solve request (<= 0: 60 s); ECS_ERR_TIMEOUT after it */
} EcsServeConfig;

/* A stand-alone solve (src/solver.c:107-170). */
typedef struct EcsSolveRequest {
  const double *density; /* [Nz][Ny][Nx] */
  double flux_scale[3];  /* --x/y/z-flux-scale (src/solver.c:50-68), default 1 */
  double rtol;           /* relative FP64 residual target */
  int32_t max_it;        /* inner Krylov iterations over all refinements */
  double *phi_out;       /* [Nz][Ny][Nx] */
} EcsSolveRequest;

/* A simulation instance advanced nsteps steps of src/pic.c:238-269. */
typedef struct EcsSimRequest {
  const double *pos, *vel; /* AoS FP64 [np][3], read at admission */
  int64_t np;
  uint64_t seed;           /* collision RNG seed (ecs_set_seed) */
  int32_t nsteps;
  int32_t sort_every;      /* cell-sort cadence of the mixed path (0: default) */
  double dt, rtol;
  int32_t max_it;
  double *step_seconds;    /* [nsteps] host wall time of each step, or NULL */
  double *phi_out;         /* final potential [Nz][Ny][Nx], or NULL */
  double *pos_out, *vel_out; /* final ions [np][3], or NULL */
} EcsSimRequest;

typedef struct EcsServeResult {
  int64_t id;
  int32_t kind;          /* ECS_SERVE_SOLVE or ECS_SERVE_SIM */
  int32_t status;        /* ECS_OK or the request's error */
  double latency;        /* seconds from submit to completion */
  double queued;         /* seconds from submit to admission */
  double device_seconds; /* solve: its graph's device time; sim: sum of solve times */
  EcsSolveStats solve;   /* solve: its stats; sim: the last step's solve */
  int32_t steps;         /* sim: steps taken */
  int32_t slot_reused;   /* 1 if the request ran on an existing slot */
  char message[160];     /* error message when status != ECS_OK */
} EcsServeResult;

typedef struct EcsServeStats {
  int64_t submitted, completed, failed;
  int64_t solves;               /* completed solve requests */
  double solve_p50, solve_p99;  /* their latency percentiles, seconds */
  double solve_mean, solve_max;
  int64_t steps;                /* simulation steps taken */
  double step_p50, step_p99;    /* their wall-time percentiles, seconds */
  int64_t device_bytes;         /* slot bytes held now */
  int64_t peak_device_bytes;
  int32_t peak_inflight;        /* most requests on the GPU at once */
  int32_t slots;                /* slots held now */
  int64_t slots_created, slot_hits, evictions;
  int64_t gpu_launches;         /* kernels launched by the server's slots */
  double busy_seconds;          /* wall time with at least one request running */
} EcsServeStats;

int ecs_serve_create(const EcsServeConfig *config, EcsServer **out);
/* Stops the server: requests being run finish; queued requests and
   simulations with steps left are dropped without a result; frees all slots. */
int ecs_serve_destroy(EcsServer *server);
/* Queue a request; returns at once with its id (ECS_ERR_NOMEM if its slot
   alone exceeds the budget, ECS_ERR_INVALID for bad arguments). */
int ecs_serve_submit_solve(EcsServer *server, const EcsParams *params, const EcsSolveRequest *req, int64_t *id);
int ecs_serve_submit_sim(EcsServer *server, const EcsParams *params, const EcsSimRequest *req, int64_t *id);
/* Up to max finished results, waiting up to timeout_ms for the first one
   (0: do not wait).  Returns the number written, or a negative status. */
int ecs_serve_poll(EcsServer *server, EcsServeResult *out, int max, int timeout_ms);
/* Requests submitted and not yet polled. */
int64_t ecs_serve_pending(EcsServer *server);
int ecs_serve_stats(EcsServer *server, EcsServeStats *stats);
/* Clear the latency samples and counters (not the slots). */
int ecs_serve_reset_stats(EcsServer *server);
/* Device bytes of the slot a request needs (the admission charge). */
int64_t ecs_serve_request_bytes(const EcsParams *params, int precision, int kind, int64_t np);

/* Stand-alone solve on one context, synchronously, through the same graph
   as a served solve request (src/solver.c:158-163). */
int ecs_solve_density(EcsCtx *ctx, const double *density, const double flux_scale[3], double rtol,
                      int max_it, double *phi_out, EcsSolveStats *stats);

/* Page-locked host memory for request buffers. */
void *ecs_host_alloc(size_t bytes);
void ecs_host_free(void *ptr);

#ifdef __cplusplus
}
#endif

#endif /* ECS_SERVE_H */
