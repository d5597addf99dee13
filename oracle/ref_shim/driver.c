/*
 * ctypes-facing driver around the reference's own functions, compiled with
 * the PETSc-API shim into oracle/_ref/libecsref.so.
 *
 * TEST INFRASTRUCTURE ONLY.  Each entry point calls the reference exactly the
 * way its programs do (src/pic.c:148-269, src/solver.c:107-167): options are
 * parsed by ProcessOptions (src/parameters.c:25), the context is built by
 * SetUpContext / CreateSwarmDM / CreatePotentialDM (src/setup.c:13,466,411),
 * and the operators are called through the bound function pointers
 * (ctx.ions.push/collide/collect, ctx.potential.lhs/rhs).
 */
#include <setjmp.h>

#include "petsc.h"
#include "ecsprt.h"
#include "parameters.h"
#include "setup.h"
#include "positions.h"
#include "velocities.h"
#include "potential.h"
#include "random.h"

extern jmp_buf g_shim_abort_jmp;
extern int g_shim_abort_armed;
extern int g_shim_abort_code;
extern int g_shim_verbose;
int shim_options_set(const char *text);
const char *shim_last_error(void);
KSP shim_ksp_create(DM dm);
Mat shim_ksp_mat(KSP k);
Vec shim_ksp_rhs(KSP k);
int shim_mat_size(Mat A);
void shim_mat_dense(Mat A, double *out);
int shim_mat_has_nullspace(Mat A);
double *shim_vec_data(Vec v);
size_t shim_vec_size(Vec v);
Vec shim_new_global(DM dm);

static Context g_ctx;
static CLI g_cli;
static KSP g_ksp;
static int g_ready = 0;

#define ARMED_CALL(expr)                                                       \
  do {                                                                         \
    if (setjmp(g_shim_abort_jmp)) {                                            \
      g_shim_abort_armed = 0;                                                  \
      return -1000 - g_shim_abort_code;                                        \
    }                                                                          \
    g_shim_abort_armed = 1;                                                    \
    int rc_ = (int)(expr);                                                     \
    g_shim_abort_armed = 0;                                                    \
    return rc_;                                                                \
  } while (0)

const char *ref_last_error(void) { return shim_last_error(); }
void ref_set_verbose(int v) { g_shim_verbose = v; }

/* Build the reference context from an options string and a total ion count. */
int ref_setup(const char *opts, int Np) {
  PetscErrorCode ierr;
  memset(&g_ctx, 0, sizeof g_ctx);
  memset(&g_cli, 0, sizeof g_cli);
  shim_options_set(opts);
  g_ctx.log.world = printNone;
  g_ctx.log.self = printNone;
  g_ctx.log.ranks = printNone;
  g_ctx.log.checkpoint = printNone;
  g_ctx.log.status = printNone;
  g_ctx.mpi.rank = 0;
  g_ctx.mpi.size = 1;
  if ((ierr = ProcessOptions(&g_cli))) return ierr;
  if ((ierr = SetUpContext(g_cli, &g_ctx))) return ierr;
  if ((ierr = CreateSwarmDM(g_cli.ndim, Np, &g_ctx))) return ierr;
  if ((ierr = CreatePotentialDM(g_cli.ndim, &g_ctx))) return ierr;
  g_ksp = shim_ksp_create(g_ctx.potential.dm);
  g_ctx.potential.solution = shim_new_global(g_ctx.potential.dm);
  g_ready = 1;
  return 0;
}

/* Derived context values, in the order of ref_param_names(). */
static const char *k_param_names =
    "ndim,Nx,Ny,Nz,dx,dy,dz,Lx,Ly,Lz,x0,y0,z0,x1,y1,z1,"
    "qi,mi,B0,E0,n0,nui,viT,viTx,viTy,viTz,vi0x,vi0y,vi0z,vi0,Ti,Omega_i,kappa_i,"
    "qe,me,nue,Te,kappa_e,Omega_e,mn,Tn,vnT,vn0x,vn0y,vn0z,vn0,scale,gammaT,"
    "stencilSize,lhsType,rhsType,xBC,yBC,zBC";
const char *ref_param_names(void) { return k_param_names; }
int ref_params(double *out) {
  int i = 0;
  if (!g_ready) return -1;
  out[i++] = g_cli.ndim;
  out[i++] = g_ctx.grid.Nx; out[i++] = g_ctx.grid.Ny; out[i++] = g_ctx.grid.Nz;
  out[i++] = g_ctx.grid.dx; out[i++] = g_ctx.grid.dy; out[i++] = g_ctx.grid.dz;
  out[i++] = g_ctx.grid.Lx; out[i++] = g_ctx.grid.Ly; out[i++] = g_ctx.grid.Lz;
  out[i++] = g_ctx.grid.x0; out[i++] = g_ctx.grid.y0; out[i++] = g_ctx.grid.z0;
  out[i++] = g_ctx.grid.x1; out[i++] = g_ctx.grid.y1; out[i++] = g_ctx.grid.z1;
  out[i++] = g_ctx.ions.q; out[i++] = g_ctx.ions.m; out[i++] = g_ctx.plasma.B0;
  out[i++] = g_ctx.plasma.E0; out[i++] = g_ctx.plasma.n0; out[i++] = g_ctx.ions.nu;
  out[i++] = g_ctx.ions.vT; out[i++] = g_ctx.ions.vTx; out[i++] = g_ctx.ions.vTy;
  out[i++] = g_ctx.ions.vTz; out[i++] = g_ctx.ions.v0x; out[i++] = g_ctx.ions.v0y;
  out[i++] = g_ctx.ions.v0z; out[i++] = g_ctx.ions.v0; out[i++] = g_ctx.ions.T;
  out[i++] = g_ctx.ions.Omega; out[i++] = g_ctx.ions.kappa;
  out[i++] = g_ctx.electrons.q; out[i++] = g_ctx.electrons.m; out[i++] = g_ctx.electrons.nu;
  out[i++] = g_ctx.electrons.T; out[i++] = g_ctx.electrons.kappa; out[i++] = g_ctx.electrons.Omega;
  out[i++] = g_ctx.neutrals.m; out[i++] = g_ctx.neutrals.T; out[i++] = g_ctx.neutrals.vT;
  out[i++] = g_ctx.neutrals.v0x; out[i++] = g_ctx.neutrals.v0y; out[i++] = g_ctx.neutrals.v0z;
  out[i++] = g_ctx.neutrals.v0; out[i++] = g_ctx.potential.scale; out[i++] = g_ctx.gammaT;
  out[i++] = g_ctx.potential.stencilSize; out[i++] = g_cli.lhsType; out[i++] = g_cli.rhsType;
  out[i++] = g_ctx.ions.xBC; out[i++] = g_ctx.ions.yBC; out[i++] = g_ctx.ions.zBC;
  return i;
}

int ref_np(void) {
  PetscInt np = 0;
  DMSwarmGetLocalSize(g_ctx.swarmDM, &np);
  return np;
}

int ref_set_particles(const double *pos, const double *vel, int np) {
  double *p, *v;
  int nd = g_cli.ndim;
  if (np != ref_np()) DMSwarmSetLocalSizes(g_ctx.swarmDM, np, 0);
  DMSwarmGetField(g_ctx.swarmDM, DMSwarmPICField_coor, NULL, NULL, (void **)&p);
  DMSwarmGetField(g_ctx.swarmDM, "velocity", NULL, NULL, (void **)&v);
  memcpy(p, pos, sizeof(double) * (size_t)np * nd);
  memcpy(v, vel, sizeof(double) * (size_t)np * nd);
  return 0;
}

int ref_get_particles(double *pos, double *vel) {
  double *p, *v;
  int np = ref_np(), nd = g_cli.ndim;
  DMSwarmGetField(g_ctx.swarmDM, DMSwarmPICField_coor, NULL, NULL, (void **)&p);
  DMSwarmGetField(g_ctx.swarmDM, "velocity", NULL, NULL, (void **)&v);
  memcpy(pos, p, sizeof(double) * (size_t)np * nd);
  memcpy(vel, v, sizeof(double) * (size_t)np * nd);
  return np;
}

int ref_set_phi(const double *phi) {
  Vec s = g_ctx.potential.solution;
  memcpy(shim_vec_data(s), phi, sizeof(double) * shim_vec_size(s));
  return 0;
}

int ref_set_moments(const double *m) {
  memcpy(shim_vec_data(g_ctx.moments), m, sizeof(double) * shim_vec_size(g_ctx.moments));
  return 0;
}
int ref_get_moments(double *m) {
  memcpy(m, shim_vec_data(g_ctx.moments), sizeof(double) * shim_vec_size(g_ctx.moments));
  return 0;
}

/* Operators, called through the same pointers the reference binds. */
int ref_push(double dt) { ARMED_CALL(g_ctx.ions.push(dt, &g_ctx)); }
int ref_collide(double dt) { ARMED_CALL(g_ctx.ions.collide(g_cli.ndim, dt, &g_ctx)); }
int ref_update_velocities(double dt) { ARMED_CALL(UpdateVelocities(g_cli.ndim, dt, &g_ctx)); }
int ref_update_positions(double dt) { ARMED_CALL(UpdatePositions(g_cli.ndim, dt, &g_ctx)); }
int ref_collect(void) { ARMED_CALL(g_ctx.ions.collect(&g_ctx)); }
int ref_init_positions(int pdist) { ARMED_CALL(InitializePositions(g_cli.ndim, (PDistType)pdist, &g_ctx)); }
int ref_init_velocities(void) { ARMED_CALL(InitializeVelocities(g_cli.ndim, VDIST_NORMAL, &g_ctx)); }

/* RHS through ComputeRHS (src/potential.c:33), written to b (global order). */
int ref_rhs(double *b) {
  Vec v = shim_ksp_rhs(g_ksp);
  int rc = ComputeRHS(g_ksp, v, &g_ctx);
  if (rc) return rc;
  memcpy(b, shim_vec_data(v), sizeof(double) * shim_vec_size(v));
  return 0;
}

/* Operator through ComputeLHS (src/potential.c:46) as a dense n x n matrix. */
int ref_lhs_size(void) { return shim_mat_size(shim_ksp_mat(g_ksp)); }
int ref_lhs_dense(double *A) {
  Mat M = shim_ksp_mat(g_ksp);
  int rc = ComputeLHS(g_ksp, M, M, &g_ctx);
  if (rc) return rc;
  shim_mat_dense(M, A);
  return shim_mat_has_nullspace(M);
}

/* Write the options log exactly as EchoOptions (src/parameters.c:354) does. */
int ref_echo_options(const char *path) {
  PetscStrcpy(g_ctx.optionsLog, path);
  return EchoOptions(g_ctx);
}

/* Raw RNG streams (src/random.c:24,94,172,233) with their static state. */
int ref_ran1(long *idum, int n, float *out) {
  for (int i = 0; i < n; i++) out[i] = ran1(idum);
  return 0;
}
int ref_ran3(long *idum, int n, float *out) {
  for (int i = 0; i < n; i++) out[i] = ran3(idum);
  return 0;
}
int ref_gasdev(long *idum, int n, float *out) {
  for (int i = 0; i < n; i++) out[i] = gasdev(idum);
  return 0;
}
int ref_sobseq(int ndim, int n, double *out) {
  PetscInt init = -1, nd = ndim;
  PetscReal x[8];
  Sobseq(&init, x - 1 + 1);
  for (int i = 0; i < n; i++) {
    Sobseq(&nd, x - 1);
    for (int d = 0; d < ndim; d++) out[i * ndim + d] = x[d];
  }
  return 0;
}
