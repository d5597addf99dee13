/*
 * Options database and parameter derivation of the GB300 ECSPRT host.
 *
 * Option names, defaults and derived quantities follow ProcessOptions
 * (src/parameters.c:25-346), SetUpContext (src/setup.c:13-277),
 * NormalizeGrid (src/setup.c:296-346), ProcessPICOptions (src/pic.c:32-115)
 * and ProcessSolverOptions (src/solver.c:29-74).  Each derived value is
 * evaluated with the same operations in the same order as the reference, so
 * the resulting EcsParams equal the reference's context values exactly.
 */
#include <ctype.h>
#include <errno.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include "ecs_host.h"

/* Physical constants of src/constants.h:4-7 (SI). */
#define ECS_Q 1.6022e-19
#define ECS_MP 1.6726e-27
#define ECS_ME 9.1094e-31
#define ECS_KB 1.3807e-23

#define MAX_OPTS 512

struct EcsOptions {
  int n;
  char *key[MAX_OPTS];
  char *val[MAX_OPTS];
};

EcsOptions *ecs_options_create(void) { return calloc(1, sizeof(EcsOptions)); }

void ecs_options_destroy(EcsOptions *o) {
  if (!o) return;
  for (int i = 0; i < o->n; i++) {
    free(o->key[i]);
    free(o->val[i]);
  }
  free(o);
}

static int is_number(const char *s) {
  char *end;
  if (!s || !*s) return 0;
  errno = 0;
  strtod(s, &end);
  return *end == '\0';
}

static int set_opt(EcsOptions *o, const char *key, const char *val) {
  for (int i = 0; i < o->n; i++)
    if (strcmp(o->key[i], key) == 0) {
      free(o->val[i]);
      o->val[i] = val ? strdup(val) : NULL;
      return ECS_OK;
    }
  if (o->n >= MAX_OPTS) return ECS_ERR_INVALID;
  o->key[o->n] = strdup(key);
  o->val[o->n] = val ? strdup(val) : NULL;
  o->n++;
  return ECS_OK;
}

int ecs_options_parse(EcsOptions *o, const char *text) {
  if (!o) return ECS_ERR_INVALID;
  if (!text) return ECS_OK;
  char *buf = strdup(text);
  /* drop comments: '#' to end of line */
  for (char *p = buf; *p; p++) {
    if (*p == '#') {
      while (*p && *p != '\n') *p++ = ' ';
      if (!*p) break;
    }
  }
  char *tok[2 * MAX_OPTS];
  int nt = 0;
  for (char *p = strtok(buf, " \t\r\n"); p && nt < 2 * MAX_OPTS; p = strtok(NULL, " \t\r\n")) tok[nt++] = p;
  int rc = ECS_OK;
  for (int i = 0; i < nt && rc == ECS_OK; i++) {
    if (tok[i][0] != '-' || is_number(tok[i])) continue;
    const char *key = tok[i], *val = NULL;
    if (i + 1 < nt && (tok[i + 1][0] != '-' || is_number(tok[i + 1]))) val = tok[++i];
    rc = set_opt(o, key, val);
  }
  free(buf);
  return rc;
}

int ecs_options_load_file(EcsOptions *o, const char *path) {
  FILE *f = fopen(path, "rb");
  if (!f) return ECS_ERR_INVALID;
  fseek(f, 0, SEEK_END);
  long len = ftell(f);
  fseek(f, 0, SEEK_SET);
  char *buf = malloc((size_t)len + 1);
  size_t got = fread(buf, 1, (size_t)len, f);
  buf[got] = '\0';
  fclose(f);
  int rc = ecs_options_parse(o, buf);
  free(buf);
  return rc;
}

const char *ecs_options_get(const EcsOptions *o, const char *key, int *found) {
  for (int i = 0; o && i < o->n; i++)
    if (strcmp(o->key[i], key) == 0) {
      if (found) *found = 1;
      return o->val[i];
    }
  if (found) *found = 0;
  return NULL;
}

static void fail(char *err, int errlen, const char *fmt, ...) {
  if (!err || errlen <= 0) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(err, (size_t)errlen, fmt, ap);
  va_end(ap);
}

static int get_real(const EcsOptions *o, const char *key, double *v) {
  int found;
  const char *s = ecs_options_get(o, key, &found);
  if (!found || !s) return 0;
  *v = strtod(s, NULL);
  return 1;
}
static int get_int(const EcsOptions *o, const char *key, int *v) {
  int found;
  const char *s = ecs_options_get(o, key, &found);
  if (!found || !s) return 0;
  *v = (int)strtol(s, NULL, 10);
  return 1;
}
static int get_bool(const EcsOptions *o, const char *key, int *v) {
  int found;
  const char *s = ecs_options_get(o, key, &found);
  if (!found) return 0;
  if (!s) {
    *v = 1;
    return 1;
  }
  *v = !(strcasecmp(s, "false") == 0 || strcasecmp(s, "no") == 0 || strcmp(s, "0") == 0 ||
         strcasecmp(s, "off") == 0);
  return 1;
}
/* Returns index in names (NULL-terminated), -1 absent, -2 unknown value. */
static int get_enum(const EcsOptions *o, const char *key, const char *const *names) {
  int found;
  const char *s = ecs_options_get(o, key, &found);
  if (!found) return -1;
  for (int i = 0; names[i]; i++)
    if (s && strcasecmp(s, names[i]) == 0) return i;
  return -2;
}

static const char *const k_rhs_names[] = {"constant", "sinusoidal", "full", NULL};
static const char *const k_lhs_names[] = {"identity", "laplacian", "full", NULL};
static const char *const k_bc_names[] = {"periodic", "inject-reflect", "inject-advect", NULL};
static const char *const k_pdist_names[] = {"sobol", "reverse", "normal", "uniform", "sinusoidal", "gaussian", NULL};
static const char *const k_vdist_names[] = {"normal", NULL};

static double mag3(double x, double y, double z) { return sqrt(x * x + y * y + z * z); }

int ecs_params_from_options(const EcsOptions *o, EcsParams *p, char *err, int errlen) {
  memset(p, 0, sizeof *p);
  int e, iv;
  /* ---- ProcessOptions (src/parameters.c:36-343) ---- */
  e = get_enum(o, "-rhs", k_rhs_names);
  if (e == -2) { fail(err, errlen, "unknown -rhs"); return ECS_ERR_INVALID; }
  p->rhs_type = e >= 0 ? e : ECS_RHS_FULL;
  e = get_enum(o, "-lhs", k_lhs_names);
  if (e == -2) { fail(err, errlen, "unknown -lhs"); return ECS_ERR_INVALID; }
  p->lhs_type = e >= 0 ? e : ECS_LHS_FULL;
  p->ndim = get_int(o, "-ndim", &iv) ? iv : 3;
  int Nx = -1, Ny = -1, Nz = -1;
  if (get_int(o, "-Nx", &iv)) Nx = iv;
  if (get_int(o, "-Ny", &iv)) Ny = iv;
  if (get_int(o, "-Nz", &iv)) Nz = iv;
  if (get_int(o, "-da_grid_x", &iv)) Nx = iv;
  if (get_int(o, "-da_grid_y", &iv)) Ny = iv;
  if (get_int(o, "-da_grid_z", &iv)) Nz = iv;
  double dx = -1.0, dy = -1.0, dz = -1.0, x0 = 0.0, y0 = 0.0, z0 = 0.0, x1 = 1.0, y1 = 1.0, z1 = 1.0;
  get_real(o, "-dx", &dx); get_real(o, "-dy", &dy); get_real(o, "-dz", &dz);
  get_real(o, "-x0", &x0); get_real(o, "-y0", &y0); get_real(o, "-z0", &z0);
  get_real(o, "-x1", &x1); get_real(o, "-y1", &y1); get_real(o, "-z1", &z1);
  const char *bckeys[3] = {"-xBC", "-yBC", "-zBC"};
  for (int d = 0; d < 3; d++) {
    e = get_enum(o, bckeys[d], k_bc_names);
    if (e == -2) { fail(err, errlen, "unknown %s", bckeys[d]); return ECS_ERR_INVALID; }
    p->bc[d] = e >= 0 ? e : ECS_BC_PERIODIC;
  }
  double n0 = 1.0, qi = ECS_Q, mi = ECS_MP, nue = 1.0, nui = 1.0;
  get_real(o, "-n0", &n0); get_real(o, "-qi", &qi); get_real(o, "-mi", &mi);
  get_real(o, "-nue", &nue); get_real(o, "-nui", &nui);
  double ve0[3] = {0, 0, 0}, vi0[3] = {0, 0, 0}, veT[3] = {0, 0, 0}, viT[3] = {0, 0, 0}, vn0[3] = {0, 0, 0};
  double v;
  if (get_real(o, "-ve0", &v)) ve0[0] = ve0[1] = ve0[2] = v;
  get_real(o, "-ve0x", &ve0[0]); get_real(o, "-ve0y", &ve0[1]); get_real(o, "-ve0z", &ve0[2]);
  if (get_real(o, "-vi0", &v)) vi0[0] = vi0[1] = vi0[2] = v;
  get_real(o, "-vi0x", &vi0[0]); get_real(o, "-vi0y", &vi0[1]); get_real(o, "-vi0z", &vi0[2]);
  if (get_real(o, "-veT", &v)) veT[0] = veT[1] = veT[2] = v;
  get_real(o, "-veTx", &veT[0]); get_real(o, "-veTy", &veT[1]); get_real(o, "-veTz", &veT[2]);
  double Te = 0.0, Ti = 0.0;
  get_real(o, "-Te", &Te);
  if (get_real(o, "-viT", &v)) viT[0] = viT[1] = viT[2] = v;
  get_real(o, "-viTx", &viT[0]); get_real(o, "-viTy", &viT[1]); get_real(o, "-viTz", &viT[2]);
  get_real(o, "-Ti", &Ti);
  double mn = mi, Tn = -1.0;
  get_real(o, "-mn", &mn);
  get_real(o, "-Tn", &Tn);
  if (get_real(o, "-vn0", &v)) vn0[0] = vn0[1] = vn0[2] = v;
  get_real(o, "-vn0x", &vn0[0]); get_real(o, "-vn0y", &vn0[1]); get_real(o, "-vn0z", &vn0[2]);
  double B0 = 0.0, E0 = 0.0;
  get_real(o, "-B0", &B0);
  get_real(o, "-E0", &E0);

  /* ---- SetUpContext (src/setup.c:116-271) ---- */
  p->qe = -ECS_Q;
  p->me = ECS_ME;
  p->n0 = n0; p->B0 = B0; p->E0 = E0;
  p->qi = qi; p->mi = mi;
  p->vi0x = vi0[0]; p->vi0y = vi0[1]; p->vi0z = vi0[2];
  p->viTx = viT[0]; p->viTy = viT[1]; p->viTz = viT[2];
  p->Ti = Ti; p->nui = nui;
  p->veTx = veT[0]; p->veTy = veT[1]; p->veTz = veT[2];
  p->Te = Te; p->nue = nue;
  p->ve0x = ve0[0]; p->ve0y = ve0[1]; p->ve0z = ve0[2];
  p->mn = mn;
  p->vn0x = vn0[0]; p->vn0y = vn0[1]; p->vn0z = vn0[2];
  p->Tn = Tn;
  p->Nx = Nx > 0 ? Nx : 7;
  p->Ny = Ny > 0 ? Ny : 7;
  p->dx = dx; p->dy = dy;
  p->x0 = x0; p->x1 = x1; p->y0 = y0; p->y1 = y1;
  if (p->ndim == 3) {
    p->Nz = Nz > 0 ? Nz : 7;
    p->dz = dz;
    p->z0 = z0; p->z1 = z1;
  } else {
    p->Nz = 1;
    p->dz = 0.0;
  }
  p->Omega_e = fabs(p->qe * p->B0 / p->me);
  p->Omega_i = fabs(p->qi * p->B0 / p->mi);
  p->kappa_e = p->Omega_e / p->nue;
  p->kappa_i = p->Omega_i / p->nui;
  p->scale = 1.0 / (1 + p->kappa_e * p->kappa_e);
  p->ve0 = mag3(p->ve0x, p->ve0y, p->ve0z);
  p->vi0 = mag3(p->vi0x, p->vi0y, p->vi0z);
  p->vn0 = mag3(p->vn0x, p->vn0y, p->vn0z);
  if (p->veTx != 0.0 || p->veTy != 0.0 || p->veTz != 0.0) {
    p->veT = mag3(p->veTx, p->veTy, p->veTz);
    p->Te = (0.5 * p->me / ECS_KB) * (p->veT * p->veT);
  } else {
    double tmp = sqrt(2.0 * ECS_KB * p->Te / p->me) / 3.0;
    p->veTx = p->veTy = p->veTz = tmp;
    p->veT = mag3(p->veTx, p->veTy, p->veTz);
  }
  if (p->viTx != 0.0 || p->viTy != 0.0 || p->viTz != 0.0) {
    p->viT = mag3(p->viTx, p->viTy, p->viTz);
    p->Ti = (0.5 * p->mi / ECS_KB) * (p->viT * p->viT);
  } else {
    double tmp = sqrt(2.0 * ECS_KB * p->Ti / p->mi) / 3.0;
    p->viTx = p->viTy = p->viTz = tmp;
    p->viT = mag3(p->viTx, p->viTy, p->viTz);
  }
  if (p->Tn == -1.0) p->Tn = p->Ti;
  p->vnT = sqrt(2.0 * ECS_KB * p->Tn / p->mn);
  p->gammaT = 1.0;

  /* ---- NormalizeGrid (src/setup.c:319-342) ---- */
  if (p->Nx < 0 || p->Ny < 0 || p->Nz < 0) { fail(err, errlen, "negative grid size"); return ECS_ERR_INVALID; }
  if (p->dx <= 0.0) { p->Lx = p->x1 - p->x0; p->dx = p->Lx / (double)p->Nx; }
  else { p->Lx = p->dx * (double)p->Nx; p->x0 = 0.0; p->x1 = p->Lx; }
  if (p->dy <= 0.0) { p->Ly = p->y1 - p->y0; p->dy = p->Ly / (double)p->Ny; }
  else { p->Ly = p->dy * (double)p->Ny; p->y0 = 0.0; p->y1 = p->Ly; }
  if (p->dz <= 0.0) { p->Lz = p->z1 - p->z0; p->dz = p->Lz / (double)p->Nz; }
  else { p->Lz = p->dz * (double)p->Nz; p->z0 = 0.0; p->z1 = p->Lz; }

  /* ---- RHS coefficients (src/rhs.c:291-292) ---- */
  p->cth = p->gammaT * ECS_KB * p->Te / ECS_Q;
  p->cG = (1 + p->kappa_e * p->kappa_e) * p->me * p->nue / ECS_Q;
  return ECS_OK;
}

int ecs_pic_app_from_options(const EcsOptions *o, const EcsParams *p, EcsPicApp *app, char *err, int errlen) {
  memset(app, 0, sizeof *app);
  int e = get_enum(o, "--position-dist", k_pdist_names);
  if (e == -2) { fail(err, errlen, "unknown --position-dist"); return ECS_ERR_INVALID; }
  app->pdist = e >= 0 ? e : ECS_PDIST_SOBOL;
  e = get_enum(o, "--velocity-dist", k_vdist_names);
  if (e == -2) { fail(err, errlen, "unknown --velocity-dist"); return ECS_ERR_INVALID; }
  app->vdist = e >= 0 ? e : 0;
  int iv;
  int Np = get_int(o, "-Np", &iv) ? iv : 0;
  app->Nt = get_int(o, "-Nt", &iv) ? iv : 1;
  app->every = get_int(o, "--every", &iv) ? iv : 1;
  double dt;
  app->dt = get_real(o, "-dt", &dt) ? dt : 1.0 / p->nui;
  int b;
  app->output_particles = get_bool(o, "--output-particles", &b) ? b : 0;
  int64_t ncell = (int64_t)p->Nx * p->Ny * p->Nz;
  if (Np > 0) app->Np = Np;
  else if (Np < 0) app->Np = (int64_t)(-Np) * ncell;
  else app->Np = ncell;
  if (app->Np <= 0) { fail(err, errlen, "Failed to set Np > 0"); return ECS_ERR_INVALID; }
  return ECS_OK;
}

int ecs_solver_app_from_options(const EcsOptions *o, EcsSolverApp *app) {
  memset(app, 0, sizeof *app);
  int found;
  const char *s = ecs_options_get(o, "--input", &found);
  if (found && s) snprintf(app->input, sizeof app->input, "%s", s);
  int b;
  app->view_lhs = get_bool(o, "--view-lhs", &b) ? b : 0;
  double v = 1.0;
  get_real(o, "--flux-scale", &v);
  app->flux_scale[0] = app->flux_scale[1] = app->flux_scale[2] = v;
  get_real(o, "--x-flux-scale", &app->flux_scale[0]);
  get_real(o, "--y-flux-scale", &app->flux_scale[1]);
  get_real(o, "--z-flux-scale", &app->flux_scale[2]);
  return ECS_OK;
}

int ecs_echo_options(const char *path, const EcsOptions *o, const EcsParams *p) {
  FILE *f = fopen(path, "w");
  if (!f) return ECS_ERR_INVALID;
  static const char *const bcn[] = {"periodic", "inject-reflect", "inject-advect"};
  fprintf(f, "#PETSc Option Table entries:\n");
  for (int i = 0; o && i < o->n; i++) {
    if (o->val[i]) fprintf(f, "%s %s\n", o->key[i], o->val[i]);
    else fprintf(f, "%s\n", o->key[i]);
  }
  fprintf(f, "#End of PETSc Option Table entries\n");
  fprintf(f, "\n\n#Common Parameter Values\n");
  fprintf(f, "Nx = %d\n", p->Nx);
  fprintf(f, "Ny = %d\n", p->Ny);
  fprintf(f, "Nz = %d\n", p->Nz);
  fprintf(f, "x0 = %f [m]\n", p->x0);
  fprintf(f, "y0 = %f [m]\n", p->y0);
  fprintf(f, "z0 = %f [m]\n", p->z0);
  fprintf(f, "x1 = %f [m]\n", p->x1);
  fprintf(f, "y1 = %f [m]\n", p->y1);
  fprintf(f, "z1 = %f [m]\n", p->z1);
  fprintf(f, "Lx = %f [m]\n", p->Lx);
  fprintf(f, "Ly = %f [m]\n", p->Ly);
  fprintf(f, "Lz = %f [m]\n", p->Lz);
  fprintf(f, "dx = %f [m]\n", p->dx);
  fprintf(f, "dy = %f [m]\n", p->dy);
  fprintf(f, "dz = %f [m]\n", p->dz);
  fprintf(f, "xBC = %s\n", bcn[p->bc[0]]);
  fprintf(f, "yBC = %s\n", bcn[p->bc[1]]);
  fprintf(f, "zBC = %s\n", bcn[p->bc[2]]);
  fprintf(f, "stencil type = %s\n", p->lhs_type == ECS_LHS_FULL ? "box" : "star");
  fprintf(f, "stencil size = %d\n", p->lhs_type == ECS_LHS_FULL ? (p->ndim == 3 ? 11 : 9)
                                     : p->lhs_type == ECS_LHS_LAPLACIAN ? (p->ndim == 3 ? 7 : 5) : 1);
  fprintf(f, "B0 = %g [T]\n", p->B0);
  fprintf(f, "E0 = %g [N/C]\n", p->E0);
  fprintf(f, "qe = %e [C]\n", p->qe);
  fprintf(f, "me = %e [kg]\n", p->me);
  fprintf(f, "nue = %g [s^-1]\n", p->nue);
  fprintf(f, "ve0x = %f [m/s]\n", p->ve0x);
  fprintf(f, "ve0y = %f [m/s]\n", p->ve0y);
  fprintf(f, "ve0z = %f [m/s]\n", p->ve0z);
  fprintf(f, "veTx = %f [m/s]\n", p->veTx);
  fprintf(f, "veTy = %f [m/s]\n", p->veTy);
  fprintf(f, "veTz = %f [m/s]\n", p->veTz);
  fprintf(f, "Te = %f [K]\n", p->Te);
  fprintf(f, "gamma_e = %f\n", p->gammaT);
  fprintf(f, "Omega_e = %g [s^-1]\n", p->Omega_e);
  fprintf(f, "kappa_e = %g\n", p->kappa_e);
  fprintf(f, "qi = %e [C]\n", p->qi);
  fprintf(f, "mi = %e [kg]\n", p->mi);
  fprintf(f, "nui = %g [s^-1]\n", p->nui);
  fprintf(f, "vi0x = %f [m/s]\n", p->vi0x);
  fprintf(f, "vi0y = %f [m/s]\n", p->vi0y);
  fprintf(f, "vi0z = %f [m/s]\n", p->vi0z);
  fprintf(f, "viTx = %f [m/s]\n", p->viTx);
  fprintf(f, "viTy = %f [m/s]\n", p->viTy);
  fprintf(f, "viTz = %f [m/s]\n", p->viTz);
  fprintf(f, "Ti = %f [K]\n", p->Ti);
  fprintf(f, "Omega_i = %g [s^-1]\n", p->Omega_i);
  fprintf(f, "kappa_i = %g\n", p->kappa_i);
  fprintf(f, "mn = %e\n", p->mn);
  fprintf(f, "Tn = %f\n", p->Tn);
  fprintf(f, "vnT = %f\n", p->vnT);
  fprintf(f, "vn0x = %f\n", p->vn0x);
  fprintf(f, "vn0y = %f\n", p->vn0y);
  fprintf(f, "vn0z = %f\n", p->vn0z);
  fprintf(f, "#End of Common Parameter Values\n");
  fclose(f);
  return ECS_OK;
}
