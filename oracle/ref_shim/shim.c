/*
 * Single-rank implementation of the PETSc-API subset declared in petsc.h.
 * TEST INFRASTRUCTURE ONLY: it exists so that the reference's unmodified
 * hot-path sources can be compiled into oracle/_ref/ and used to pin the
 * oracle restatement.  Nothing in the product links it.
 */
#include "petsc.h"

#include <ctype.h>
#include <setjmp.h>

const char DMSwarmPICField_coor[] = "DMSwarmPIC_coor";

/* ---------------------------------------------------------------------- */
/* error reporting and abort capture                                      */
/* ---------------------------------------------------------------------- */
static char g_errmsg[1024];
jmp_buf g_shim_abort_jmp;
int g_shim_abort_armed = 0;
int g_shim_abort_code = 0;
int g_shim_verbose = 0;

PetscErrorCode ShimSetError(PetscErrorCode code, const char *file, int line,
                            const char *fmt, ...) {
  va_list ap;
  int n = snprintf(g_errmsg, sizeof g_errmsg, "%s:%d: ", file, line);
  va_start(ap, fmt);
  vsnprintf(g_errmsg + n, sizeof g_errmsg - (size_t)n, fmt, ap);
  va_end(ap);
  if (g_shim_verbose) fprintf(stderr, "[shim] error %d %s\n", code, g_errmsg);
  return code;
}

const char *shim_last_error(void) { return g_errmsg; }

int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return 0; }
int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm) {
  (void)buf; (void)count; (void)t; (void)root; (void)comm;
  return 0;
}
int MPI_Abort(MPI_Comm comm, int code) {
  (void)comm;
  g_shim_abort_code = code;
  if (g_shim_abort_armed) longjmp(g_shim_abort_jmp, 1);
  fprintf(stderr, "[shim] MPI_Abort(%d) outside an armed driver call\n", code);
  exit(code);
}

/* ---------------------------------------------------------------------- */
/* system                                                                 */
/* ---------------------------------------------------------------------- */
PetscErrorCode PetscInitialize(int *argc, char ***args, const char file[],
                               const char help[]) {
  (void)argc; (void)args; (void)file; (void)help;
  return 0;
}
PetscErrorCode PetscFinalize(void) { return 0; }
PetscErrorCode PetscEnd(void) { return 0; }

static PetscErrorCode vprint(const char *fmt, va_list ap) {
  if (g_shim_verbose) vfprintf(stdout, fmt, ap);
  return 0;
}
PetscErrorCode PetscPrintf(MPI_Comm comm, const char fmt[], ...) {
  va_list ap; (void)comm;
  va_start(ap, fmt); vprint(fmt, ap); va_end(ap);
  return 0;
}
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm comm, const char fmt[], ...) {
  va_list ap; (void)comm;
  va_start(ap, fmt); vprint(fmt, ap); va_end(ap);
  return 0;
}
PetscErrorCode PetscSynchronizedFlush(MPI_Comm comm, FILE *fd) {
  (void)comm; if (g_shim_verbose) fflush(fd);
  return 0;
}
PetscErrorCode PetscStrcpy(char s[], const char t[]) { strcpy(s, t); return 0; }
PetscErrorCode PetscStrcat(char s[], const char t[]) { strcat(s, t); return 0; }
PetscErrorCode PetscStrcmp(const char a[], const char b[], PetscBool *flg) {
  *flg = (strcmp(a, b) == 0) ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscGetFullPath(const char path[], char fullpath[], size_t flen) {
  snprintf(fullpath, flen, "%s", path);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* options database: "-key value" pairs from a string                     */
/* ---------------------------------------------------------------------- */
#define MAX_OPTS 256
static char *g_keys[MAX_OPTS];
static char *g_vals[MAX_OPTS];
static int g_nopts = 0;

static int looks_numeric(const char *s) {
  char *end;
  if (!s || !*s) return 0;
  strtod(s, &end);
  return *end == '\0';
}

void shim_options_clear(void) {
  for (int i = 0; i < g_nopts; i++) { free(g_keys[i]); free(g_vals[i]); }
  g_nopts = 0;
}

/* Parse whitespace-separated tokens; a token starting with '-' that is not a
   number opens a key, and the following token is its value unless it opens
   another key.  Later occurrences override earlier ones, as in PETSc. */
int shim_options_set(const char *text) {
  shim_options_clear();
  if (!text) return 0;
  char *buf = strdup(text);
  char *tok[2 * MAX_OPTS];
  int nt = 0;
  for (char *p = strtok(buf, " \t\r\n"); p && nt < 2 * MAX_OPTS; p = strtok(NULL, " \t\r\n"))
    tok[nt++] = p;
  for (int i = 0; i < nt; i++) {
    if (tok[i][0] != '-' || looks_numeric(tok[i])) continue;
    const char *key = tok[i];
    const char *val = NULL;
    if (i + 1 < nt && (tok[i + 1][0] != '-' || looks_numeric(tok[i + 1]))) val = tok[++i];
    int slot = -1;
    for (int k = 0; k < g_nopts; k++)
      if (strcmp(g_keys[k], key) == 0) slot = k;
    if (slot < 0) {
      if (g_nopts >= MAX_OPTS) break;
      slot = g_nopts++;
      g_keys[slot] = strdup(key);
    } else {
      free(g_vals[slot]);
    }
    g_vals[slot] = val ? strdup(val) : NULL;
  }
  free(buf);
  return 0;
}

static int find_opt(const char *name) {
  for (int k = 0; k < g_nopts; k++)
    if (strcmp(g_keys[k], name) == 0) return k;
  return -1;
}

PetscErrorCode PetscOptionsGetReal(PetscOptions o, const char pre[], const char name[],
                                   PetscReal *v, PetscBool *set) {
  (void)o; (void)pre;
  int k = find_opt(name);
  *set = PETSC_FALSE;
  if (k < 0) return 0;
  if (!g_vals[k]) SETERRQ(0, PETSC_ERR_ARG_WRONG, "missing value for %s", name);
  *v = strtod(g_vals[k], NULL);
  *set = PETSC_TRUE;
  return 0;
}
PetscErrorCode PetscOptionsGetInt(PetscOptions o, const char pre[], const char name[],
                                  PetscInt *v, PetscBool *set) {
  (void)o; (void)pre;
  int k = find_opt(name);
  *set = PETSC_FALSE;
  if (k < 0) return 0;
  if (!g_vals[k]) SETERRQ(0, PETSC_ERR_ARG_WRONG, "missing value for %s", name);
  *v = (PetscInt)strtol(g_vals[k], NULL, 10);
  *set = PETSC_TRUE;
  return 0;
}
PetscErrorCode PetscOptionsGetBool(PetscOptions o, const char pre[], const char name[],
                                   PetscBool *v, PetscBool *set) {
  (void)o; (void)pre;
  int k = find_opt(name);
  *set = PETSC_FALSE;
  if (k < 0) return 0;
  *set = PETSC_TRUE;
  if (!g_vals[k]) { *v = PETSC_TRUE; return 0; }
  const char *s = g_vals[k];
  *v = (!strcasecmp(s, "false") || !strcasecmp(s, "no") || !strcmp(s, "0")) ? PETSC_FALSE
                                                                              : PETSC_TRUE;
  return 0;
}
PetscErrorCode PetscOptionsGetEnum(PetscOptions o, const char pre[], const char name[],
                                   const char *const *list, PetscEnum *v, PetscBool *set) {
  (void)o; (void)pre;
  int k = find_opt(name);
  int n = 0;
  *set = PETSC_FALSE;
  if (k < 0) return 0;
  while (list[n]) n++;
  n -= 2; /* trailing entries before the NULL: enum type name, prefix */
  for (int i = 0; i < n; i++) {
    if (g_vals[k] && !strcasecmp(g_vals[k], list[i])) {
      *v = i;
      *set = PETSC_TRUE;
      return 0;
    }
  }
  SETERRQ(0, PETSC_ERR_ARG_UNKNOWN_TYPE, "unknown value %s for %s", g_vals[k] ? g_vals[k] : "", name);
}

/* ---------------------------------------------------------------------- */
/* viewers: plain FILE*                                                   */
/* ---------------------------------------------------------------------- */
struct _p_PetscViewer {
  FILE *fp;
  PetscFileMode mode;
};
PetscErrorCode PetscViewerASCIIOpen(MPI_Comm comm, const char name[], PetscViewer *v) {
  (void)comm;
  *v = calloc(1, sizeof(**v));
  (*v)->fp = fopen(name, "w");
  return (*v)->fp ? 0 : 65;
}
PetscErrorCode PetscViewerCreate(MPI_Comm comm, PetscViewer *v) {
  (void)comm;
  *v = calloc(1, sizeof(**v));
  (*v)->mode = FILE_MODE_WRITE;
  return 0;
}
PetscErrorCode PetscViewerSetType(PetscViewer v, PetscViewerType t) { (void)v; (void)t; return 0; }
PetscErrorCode PetscViewerFileSetMode(PetscViewer v, PetscFileMode m) { v->mode = m; return 0; }
PetscErrorCode PetscViewerFileSetName(PetscViewer v, const char name[]) {
  v->fp = fopen(name, v->mode == FILE_MODE_APPEND ? "a" : "w");
  return v->fp ? 0 : 65;
}
PetscErrorCode PetscViewerASCIIPrintf(PetscViewer v, const char fmt[], ...) {
  va_list ap;
  if (!v || !v->fp) return 0;
  va_start(ap, fmt);
  vfprintf(v->fp, fmt, ap);
  va_end(ap);
  return 0;
}
PetscErrorCode PetscViewerDestroy(PetscViewer *v) {
  if (*v) {
    if ((*v)->fp) fclose((*v)->fp);
    free(*v);
    *v = NULL;
  }
  return 0;
}
PetscErrorCode PetscOptionsView(PetscOptions o, PetscViewer v) {
  (void)o;
  PetscViewerASCIIPrintf(v, "#PETSc Option Table entries:\n");
  for (int k = 0; k < g_nopts; k++) {
    if (g_vals[k]) PetscViewerASCIIPrintf(v, "%s %s\n", g_keys[k], g_vals[k]);
    else PetscViewerASCIIPrintf(v, "%s\n", g_keys[k]);
  }
  PetscViewerASCIIPrintf(v, "#End of PETSc Option Table entries\n");
  return 0;
}

PetscErrorCode PetscObjectSetOptionsPrefix(PetscObject obj, const char prefix[]) {
  (void)obj; (void)prefix;
  return 0;
}
PetscErrorCode PetscObjectSetName(PetscObject obj, const char name[]) {
  (void)obj; (void)name;
  return 0;
}

/* ---------------------------------------------------------------------- */
/* DM                                                                     */
/* ---------------------------------------------------------------------- */
struct _p_DM {
  int isswarm;
  int dim;
  int M, N, P;
  int dof, sw;
  DMBoundaryType bx, by, bz;
  DMDAStencilType st;
  /* swarm */
  DM celldm;
  int np;
  int veldim;
  double *coor;
  double *vel;
  void *appctx;
};

struct _p_Vec {
  DM dm;
  int local;
  size_t n;
  double *a;
  void *views[4]; /* allocations that back the most recent array view */
};

static int gext(DM dm, int d) { /* ghosted extent along dimension d */
  int n = d == 0 ? dm->M : (d == 1 ? dm->N : dm->P);
  DMBoundaryType b = d == 0 ? dm->bx : (d == 1 ? dm->by : dm->bz);
  if (d >= dm->dim) return 1;
  return n + ((b == DM_BOUNDARY_NONE) ? 0 : 2 * dm->sw);
}
static int gstart(DM dm, int d) {
  DMBoundaryType b = d == 0 ? dm->bx : (d == 1 ? dm->by : dm->bz);
  if (d >= dm->dim) return 0;
  return (b == DM_BOUNDARY_NONE) ? 0 : -dm->sw;
}

static PetscErrorCode create_da(int dim, DMBoundaryType bx, DMBoundaryType by,
                                DMBoundaryType bz, DMDAStencilType st, int M, int N, int P,
                                int dof, int s, DM *da) {
  DM dm = calloc(1, sizeof(*dm));
  dm->dim = dim; dm->M = M; dm->N = N; dm->P = dim == 3 ? P : 1;
  dm->dof = dof; dm->sw = s;
  dm->bx = bx; dm->by = by; dm->bz = dim == 3 ? bz : DM_BOUNDARY_NONE;
  dm->st = st;
  *da = dm;
  return 0;
}
PetscErrorCode DMDACreate2d(MPI_Comm comm, DMBoundaryType bx, DMBoundaryType by,
                            DMDAStencilType st, PetscInt M, PetscInt N, PetscInt m,
                            PetscInt n, PetscInt dof, PetscInt s, const PetscInt lx[],
                            const PetscInt ly[], DM *da) {
  (void)comm; (void)m; (void)n; (void)lx; (void)ly;
  return create_da(2, bx, by, DM_BOUNDARY_NONE, st, M, N, 1, dof, s, da);
}
PetscErrorCode DMDACreate3d(MPI_Comm comm, DMBoundaryType bx, DMBoundaryType by,
                            DMBoundaryType bz, DMDAStencilType st, PetscInt M,
                            PetscInt N, PetscInt P, PetscInt m, PetscInt n, PetscInt p,
                            PetscInt dof, PetscInt s, const PetscInt lx[],
                            const PetscInt ly[], const PetscInt lz[], DM *da) {
  (void)comm; (void)m; (void)n; (void)p; (void)lx; (void)ly; (void)lz;
  return create_da(3, bx, by, bz, st, M, N, P, dof, s, da);
}
PetscErrorCode DMDASetElementType(DM dm, DMDAElementType t) { (void)dm; (void)t; return 0; }
PetscErrorCode DMSetFromOptions(DM dm) { (void)dm; return 0; }
PetscErrorCode DMSetUp(DM dm) { (void)dm; return 0; }
PetscErrorCode DMDASetUniformCoordinates(DM dm, PetscReal x0, PetscReal x1, PetscReal y0,
                                         PetscReal y1, PetscReal z0, PetscReal z1) {
  (void)dm; (void)x0; (void)x1; (void)y0; (void)y1; (void)z0; (void)z1;
  return 0;
}
PetscErrorCode DMDASetFieldName(DM dm, PetscInt nf, const char name[]) {
  (void)dm; (void)nf; (void)name;
  return 0;
}
PetscErrorCode DMSetApplicationContext(DM dm, void *ctx) { dm->appctx = ctx; return 0; }
PetscErrorCode DMCreate(MPI_Comm comm, DM *dm) {
  (void)comm;
  *dm = calloc(1, sizeof(**dm));
  return 0;
}
PetscErrorCode DMSetType(DM dm, DMType type) {
  dm->isswarm = strcmp(type, DMSWARM) == 0;
  return 0;
}
PetscErrorCode DMGetDimension(DM dm, PetscInt *dim) { *dim = dm->dim; return 0; }
PetscErrorCode DMSetDimension(DM dm, PetscInt dim) { dm->dim = dim; return 0; }
PetscErrorCode DMDestroy(DM *dm) {
  if (*dm) {
    free((*dm)->coor);
    free((*dm)->vel);
    free(*dm);
    *dm = NULL;
  }
  return 0;
}
PetscErrorCode DMView(DM dm, PetscViewer v) { (void)dm; (void)v; return 0; }
PetscErrorCode DMDAGetCorners(DM dm, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m,
                              PetscInt *n, PetscInt *p) {
  if (x) *x = 0;
  if (y) *y = 0;
  if (z) *z = 0;
  if (m) *m = dm->M;
  if (n) *n = dm->N;
  if (p) *p = dm->P;
  return 0;
}
PetscErrorCode DMDAGetLocalInfo(DM dm, DMDALocalInfo *info) {
  memset(info, 0, sizeof *info);
  info->dim = dm->dim; info->dof = dm->dof; info->sw = dm->sw;
  info->mx = dm->M; info->my = dm->N; info->mz = dm->P;
  info->xm = dm->M; info->ym = dm->N; info->zm = dm->P;
  info->gxs = gstart(dm, 0); info->gys = gstart(dm, 1); info->gzs = gstart(dm, 2);
  info->gxm = gext(dm, 0); info->gym = gext(dm, 1); info->gzm = gext(dm, 2);
  info->bx = dm->bx; info->by = dm->by; info->bz = dm->bz;
  info->st = dm->st; info->da = dm;
  return 0;
}

static Vec new_vec(DM dm, int local) {
  Vec v = calloc(1, sizeof(*v));
  v->dm = dm;
  v->local = local;
  if (local) v->n = (size_t)gext(dm, 0) * gext(dm, 1) * gext(dm, 2) * dm->dof;
  else v->n = (size_t)dm->M * dm->N * dm->P * dm->dof;
  v->a = calloc(v->n ? v->n : 1, sizeof(double));
  return v;
}
PetscErrorCode DMCreateGlobalVector(DM dm, Vec *v) { *v = new_vec(dm, 0); return 0; }
PetscErrorCode DMGetGlobalVector(DM dm, Vec *v) { *v = new_vec(dm, 0); return 0; }
PetscErrorCode DMRestoreGlobalVector(DM dm, Vec *v) { (void)dm; return VecDestroy(v); }
PetscErrorCode DMGetLocalVector(DM dm, Vec *v) { *v = new_vec(dm, 1); return 0; }
PetscErrorCode DMRestoreLocalVector(DM dm, Vec *v) { (void)dm; return VecDestroy(v); }

/* Map a (possibly ghost) index along dimension d to its owner, or -1 when it
   falls outside a non-periodic dimension. */
static int owner_index(DM dm, int d, int i) {
  int n = d == 0 ? dm->M : (d == 1 ? dm->N : dm->P);
  DMBoundaryType b = d == 0 ? dm->bx : (d == 1 ? dm->by : dm->bz);
  if (d >= dm->dim) return 0;
  if (i >= 0 && i < n) return i;
  if (b == DM_BOUNDARY_PERIODIC) return ((i % n) + n) % n;
  return -1;
}

PetscErrorCode DMGlobalToLocal(DM dm, Vec g, InsertMode mode, Vec l) {
  (void)mode;
  int gx = gext(dm, 0), gy = gext(dm, 1), gz = gext(dm, 2);
  int sx = gstart(dm, 0), sy = gstart(dm, 1), sz = gstart(dm, 2);
  int dof = dm->dof;
  for (int kk = 0; kk < gz; kk++) {
    int k = owner_index(dm, 2, kk + sz);
    for (int jj = 0; jj < gy; jj++) {
      int j = owner_index(dm, 1, jj + sy);
      for (int ii = 0; ii < gx; ii++) {
        int i = owner_index(dm, 0, ii + sx);
        double *dst = l->a + (((size_t)kk * gy + jj) * gx + ii) * dof;
        if (i < 0 || j < 0 || k < 0) {
          for (int c = 0; c < dof; c++) dst[c] = 0.0;
          continue;
        }
        const double *src = g->a + (((size_t)k * dm->N + j) * dm->M + i) * dof;
        for (int c = 0; c < dof; c++) dst[c] = src[c];
      }
    }
  }
  return 0;
}
PetscErrorCode DMGlobalToLocalBegin(DM dm, Vec g, InsertMode mode, Vec l) {
  return DMGlobalToLocal(dm, g, mode, l);
}
PetscErrorCode DMGlobalToLocalEnd(DM dm, Vec g, InsertMode mode, Vec l) {
  (void)dm; (void)g; (void)mode; (void)l;
  return 0;
}
PetscErrorCode DMLocalToGlobal(DM dm, Vec l, InsertMode mode, Vec g) {
  int gx = gext(dm, 0), gy = gext(dm, 1), gz = gext(dm, 2);
  int sx = gstart(dm, 0), sy = gstart(dm, 1), sz = gstart(dm, 2);
  int dof = dm->dof;
  for (int kk = 0; kk < gz; kk++) {
    int kraw = kk + sz;
    int k = owner_index(dm, 2, kraw);
    for (int jj = 0; jj < gy; jj++) {
      int jraw = jj + sy;
      int j = owner_index(dm, 1, jraw);
      for (int ii = 0; ii < gx; ii++) {
        int iraw = ii + sx;
        int i = owner_index(dm, 0, iraw);
        if (i < 0 || j < 0 || k < 0) continue;
        int owned = (iraw == i) && (jraw == j) && (dm->dim < 3 || kraw == k);
        if (mode == INSERT_VALUES && !owned) continue;
        const double *src = l->a + (((size_t)kk * gy + jj) * gx + ii) * dof;
        double *dst = g->a + (((size_t)k * dm->N + j) * dm->M + i) * dof;
        for (int c = 0; c < dof; c++) {
          if (mode == ADD_VALUES) dst[c] += src[c];
          else dst[c] = src[c];
        }
      }
    }
  }
  return 0;
}

/* Array views addressed with global indices (see petsc.h header comment). */
static void free_views(Vec v) {
  for (int i = 0; i < 4; i++) { free(v->views[i]); v->views[i] = NULL; }
}
static PetscErrorCode get_array(DM dm, Vec v, void *array, int perdof) {
  int gx, gy, gz, sx, sy, sz, dof = dm->dof;
  if (v->local) {
    gx = gext(dm, 0); gy = gext(dm, 1); gz = gext(dm, 2);
    sx = gstart(dm, 0); sy = gstart(dm, 1); sz = gstart(dm, 2);
  } else {
    gx = dm->M; gy = dm->N; gz = dm->P; sx = sy = sz = 0;
  }
  free_views(v);
  size_t es = sizeof(double) * (size_t)dof; /* element stride in bytes */
  char *base = (char *)v->a;
  if (dm->dim == 3) {
    if (!perdof) {
      char **rows = malloc(sizeof(char *) * (size_t)gz * gy);
      char ***planes = malloc(sizeof(char **) * (size_t)gz);
      for (int kk = 0; kk < gz; kk++) {
        for (int jj = 0; jj < gy; jj++)
          rows[(size_t)kk * gy + jj] = base + (((size_t)kk * gy + jj) * gx) * es - (ptrdiff_t)sx * (ptrdiff_t)es;
        planes[kk] = rows + (size_t)kk * gy - sy;
      }
      v->views[0] = rows; v->views[1] = planes;
      *(char ****)array = planes - sz;
    } else {
      double **nodes = malloc(sizeof(double *) * (size_t)gz * gy * gx);
      double ***rows = malloc(sizeof(double **) * (size_t)gz * gy);
      double ****planes = malloc(sizeof(double ***) * (size_t)gz);
      for (size_t idx = 0; idx < (size_t)gz * gy * gx; idx++) nodes[idx] = v->a + idx * dof;
      for (int kk = 0; kk < gz; kk++) {
        for (int jj = 0; jj < gy; jj++)
          rows[(size_t)kk * gy + jj] = nodes + ((size_t)kk * gy + jj) * gx - sx;
        planes[kk] = rows + (size_t)kk * gy - sy;
      }
      v->views[0] = nodes; v->views[1] = rows; v->views[2] = planes;
      *(double *****)array = planes - sz;
    }
  } else {
    if (!perdof) {
      char **rows = malloc(sizeof(char *) * (size_t)gy);
      for (int jj = 0; jj < gy; jj++)
        rows[jj] = base + ((size_t)jj * gx) * es - (ptrdiff_t)sx * (ptrdiff_t)es;
      v->views[0] = rows;
      *(char ***)array = rows - sy;
    } else {
      double **nodes = malloc(sizeof(double *) * (size_t)gy * gx);
      double ***rows = malloc(sizeof(double **) * (size_t)gy);
      for (size_t idx = 0; idx < (size_t)gy * gx; idx++) nodes[idx] = v->a + idx * dof;
      for (int jj = 0; jj < gy; jj++) rows[jj] = nodes + (size_t)jj * gx - sx;
      v->views[0] = nodes; v->views[1] = rows;
      *(double ****)array = rows - sy;
    }
  }
  return 0;
}
PetscErrorCode DMDAVecGetArray(DM dm, Vec v, void *array) { return get_array(dm, v, array, 0); }
PetscErrorCode DMDAVecRestoreArray(DM dm, Vec v, void *array) {
  (void)dm; (void)array; free_views(v);
  return 0;
}
PetscErrorCode DMDAVecGetArrayDOF(DM dm, Vec v, void *array) { return get_array(dm, v, array, 1); }
PetscErrorCode DMDAVecRestoreArrayDOF(DM dm, Vec v, void *array) {
  (void)dm; (void)array; free_views(v);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* DMSwarm                                                                */
/* ---------------------------------------------------------------------- */
PetscErrorCode DMSwarmSetCellDM(DM sw, DM cell) { sw->celldm = cell; return 0; }
PetscErrorCode DMSwarmGetCellDM(DM sw, DM *cell) { *cell = sw->celldm; return 0; }
PetscErrorCode DMSwarmSetType(DM sw, DMSwarmType t) { (void)sw; (void)t; return 0; }
PetscErrorCode DMSwarmInitializeFieldRegister(DM sw) { (void)sw; return 0; }
PetscErrorCode DMSwarmRegisterPetscDatatypeField(DM sw, const char name[], PetscInt bs,
                                                 PetscDataType t) {
  (void)t;
  if (strcmp(name, "velocity") == 0) sw->veldim = bs;
  return 0;
}
PetscErrorCode DMSwarmFinalizeFieldRegister(DM sw) { (void)sw; return 0; }
PetscErrorCode DMSwarmSetLocalSizes(DM sw, PetscInt n, PetscInt buf) {
  (void)buf;
  int nd = sw->dim, vd = sw->veldim ? sw->veldim : sw->dim;
  double *c = calloc((size_t)(n ? n : 1) * nd, sizeof(double));
  double *w = calloc((size_t)(n ? n : 1) * vd, sizeof(double));
  int keep = sw->np < n ? sw->np : n;
  if (sw->coor) memcpy(c, sw->coor, sizeof(double) * (size_t)keep * nd);
  if (sw->vel) memcpy(w, sw->vel, sizeof(double) * (size_t)keep * vd);
  free(sw->coor); free(sw->vel);
  sw->coor = c; sw->vel = w; sw->np = n;
  return 0;
}
PetscErrorCode DMSwarmGetLocalSize(DM sw, PetscInt *n) { *n = sw->np; return 0; }
PetscErrorCode DMSwarmGetSize(DM sw, PetscInt *n) { *n = sw->np; return 0; }
PetscErrorCode DMSwarmGetField(DM sw, const char name[], PetscInt *bs, PetscDataType *t,
                               void **data) {
  if (t) *t = PETSC_REAL;
  if (strcmp(name, DMSwarmPICField_coor) == 0) {
    if (bs) *bs = sw->dim;
    *data = sw->coor;
    return 0;
  }
  if (strcmp(name, "velocity") == 0) {
    if (bs) *bs = sw->veldim;
    *data = sw->vel;
    return 0;
  }
  SETERRQ(0, PETSC_ERR_ARG_WRONG, "unknown swarm field %s", name);
}
PetscErrorCode DMSwarmRestoreField(DM sw, const char name[], PetscInt *bs,
                                   PetscDataType *t, void **data) {
  (void)sw; (void)name; (void)bs; (void)t;
  *data = NULL;
  return 0;
}
PetscErrorCode DMSwarmMigrate(DM sw, PetscBool remove) { (void)sw; (void)remove; return 0; }
PetscErrorCode DMSwarmSetPointsUniformCoordinates(DM sw, PetscReal min[], PetscReal max[],
                                                  PetscInt npoints[], InsertMode mode) {
  (void)sw; (void)min; (void)max; (void)npoints; (void)mode;
  SETERRQ(0, PETSC_ERR_SUP, "DMSwarmSetPointsUniformCoordinates is outside the shim");
}

/* ---------------------------------------------------------------------- */
/* Vec / Mat / nullspace / KSP                                            */
/* ---------------------------------------------------------------------- */
PetscErrorCode VecZeroEntries(Vec v) { memset(v->a, 0, sizeof(double) * v->n); return 0; }
PetscErrorCode VecSet(Vec v, PetscScalar a) {
  for (size_t i = 0; i < v->n; i++) v->a[i] = a;
  return 0;
}
PetscErrorCode VecCopy(Vec x, Vec y) {
  if (x->n != y->n) SETERRQ(0, PETSC_ERR_ARG_WRONG, "VecCopy size mismatch");
  memcpy(y->a, x->a, sizeof(double) * x->n);
  return 0;
}
PetscErrorCode VecDestroy(Vec *v) {
  if (*v) {
    free_views(*v);
    free((*v)->a);
    free(*v);
    *v = NULL;
  }
  return 0;
}

#define SHIM_MAXNZ 27
struct _p_Mat {
  DM dm;
  int n;
  int *nnz;
  int *cols;
  double *vals;
  int has_nullspace;
};
PetscErrorCode DMCreateMatrix(DM dm, Mat *A) {
  Mat m = calloc(1, sizeof(*m));
  m->dm = dm;
  m->n = dm->M * dm->N * dm->P * dm->dof;
  m->nnz = calloc((size_t)m->n, sizeof(int));
  m->cols = calloc((size_t)m->n * SHIM_MAXNZ, sizeof(int));
  m->vals = calloc((size_t)m->n * SHIM_MAXNZ, sizeof(double));
  *A = m;
  return 0;
}
static void mat_insert(Mat A, int row, int col, double v, int add) {
  int *c = A->cols + (size_t)row * SHIM_MAXNZ;
  double *x = A->vals + (size_t)row * SHIM_MAXNZ;
  for (int e = 0; e < A->nnz[row]; e++) {
    if (c[e] == col) {
      x[e] = add ? x[e] + v : v;
      return;
    }
  }
  if (A->nnz[row] < SHIM_MAXNZ) {
    c[A->nnz[row]] = col;
    x[A->nnz[row]] = v;
    A->nnz[row]++;
  }
}
static int stencil_index(DM dm, MatStencil s) {
  int i = owner_index(dm, 0, s.i);
  int j = owner_index(dm, 1, s.j);
  int k = owner_index(dm, 2, dm->dim == 3 ? s.k : 0);
  if (i < 0 || j < 0 || k < 0) return -1;
  /* PETSc reads the component field only when dof > 1; callers with dof 1
     (src/lhs.c) leave it unset. */
  return ((k * dm->N + j) * dm->M + i) * dm->dof + (dm->dof > 1 ? s.c : 0);
}
PetscErrorCode MatSetValuesStencil(Mat A, PetscInt m, const MatStencil idxm[], PetscInt n,
                                   const MatStencil idxn[], const PetscScalar v[],
                                   InsertMode mode) {
  for (int r = 0; r < m; r++) {
    int row = stencil_index(A->dm, idxm[r]);
    if (row < 0) continue;
    for (int c = 0; c < n; c++) {
      int col = stencil_index(A->dm, idxn[c]);
      if (col < 0) continue;
      mat_insert(A, row, col, v[(size_t)r * n + c], mode == ADD_VALUES);
    }
  }
  return 0;
}
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
PetscErrorCode MatZeroEntries(Mat A) {
  for (size_t e = 0; e < (size_t)A->n * SHIM_MAXNZ; e++) A->vals[e] = 0.0;
  return 0;
}
PetscErrorCode MatShift(Mat A, PetscScalar a) {
  for (int r = 0; r < A->n; r++) mat_insert(A, r, r, a, 1);
  return 0;
}
PetscErrorCode MatMult(Mat A, Vec x, Vec y) {
  for (int r = 0; r < A->n; r++) {
    double s = 0.0;
    for (int e = 0; e < A->nnz[r]; e++) s += A->vals[(size_t)r * SHIM_MAXNZ + e] * x->a[A->cols[(size_t)r * SHIM_MAXNZ + e]];
    y->a[r] = s;
  }
  return 0;
}
PetscErrorCode MatCreateVecs(Mat A, Vec *r, Vec *l) {
  if (r) *r = new_vec(A->dm, 0);
  if (l) *l = new_vec(A->dm, 0);
  return 0;
}
int shim_mat_size(Mat A) { return A->n; }
/* Dense copy of the captured operator (row-major n x n). */
void shim_mat_dense(Mat A, double *out) {
  memset(out, 0, sizeof(double) * (size_t)A->n * A->n);
  for (int r = 0; r < A->n; r++)
    for (int e = 0; e < A->nnz[r]; e++)
      out[(size_t)r * A->n + A->cols[(size_t)r * SHIM_MAXNZ + e]] += A->vals[(size_t)r * SHIM_MAXNZ + e];
}
int shim_mat_has_nullspace(Mat A) { return A->has_nullspace; }

struct _p_MatNullSpace {
  int has_cnst;
};
PetscErrorCode MatNullSpaceCreate(MPI_Comm comm, PetscBool has_cnst, PetscInt n,
                                  const Vec vecs[], MatNullSpace *sp) {
  (void)comm; (void)n; (void)vecs;
  *sp = calloc(1, sizeof(**sp));
  (*sp)->has_cnst = has_cnst;
  return 0;
}
PetscErrorCode MatSetNullSpace(Mat A, MatNullSpace sp) { A->has_nullspace = sp->has_cnst; return 0; }
/* Remove the constant component: v <- v - mean(v). */
PetscErrorCode MatNullSpaceRemove(MatNullSpace sp, Vec v) {
  if (!sp->has_cnst) return 0;
  double s = 0.0;
  for (size_t i = 0; i < v->n; i++) s += v->a[i];
  s /= (double)v->n;
  for (size_t i = 0; i < v->n; i++) v->a[i] -= s;
  return 0;
}
PetscErrorCode MatNullSpaceDestroy(MatNullSpace *sp) { free(*sp); *sp = NULL; return 0; }

struct _p_KSP {
  DM dm;
  Mat A;
  Vec b, x;
};
KSP shim_ksp_create(DM dm) {
  KSP k = calloc(1, sizeof(*k));
  k->dm = dm;
  DMCreateMatrix(dm, &k->A);
  k->b = new_vec(dm, 0);
  k->x = new_vec(dm, 0);
  return k;
}
Mat shim_ksp_mat(KSP k) { return k->A; }
Vec shim_ksp_rhs(KSP k) { return k->b; }
PetscErrorCode KSPGetDM(KSP ksp, DM *dm) { *dm = ksp->dm; return 0; }
PetscErrorCode KSPSolve(KSP ksp, Vec b, Vec x) {
  (void)ksp; (void)b; (void)x;
  SETERRQ(0, PETSC_ERR_SUP, "KSPSolve is outside the shim; solve the captured system");
}
PetscErrorCode KSPGetSolution(KSP ksp, Vec *x) { *x = ksp->x; return 0; }
PetscErrorCode KSPGetOperators(KSP ksp, Mat *A, Mat *P) {
  if (A) *A = ksp->A;
  if (P) *P = ksp->A;
  return 0;
}

/* Raw data access for the driver. */
double *shim_vec_data(Vec v) { return v->a; }
size_t shim_vec_size(Vec v) { return v->n; }
Vec shim_new_global(DM dm) { return new_vec(dm, 0); }

PetscErrorCode PetscRandomCreate(MPI_Comm comm, PetscRandom *r) {
  (void)comm; (void)r;
  SETERRQ(0, PETSC_ERR_SUP, "PetscRandom is outside the shim");
}
PetscErrorCode PetscRandomSetInterval(PetscRandom r, PetscReal lo, PetscReal hi) {
  (void)r; (void)lo; (void)hi; return PETSC_ERR_SUP;
}
PetscErrorCode PetscRandomSetSeed(PetscRandom r, unsigned long seed) { (void)r; (void)seed; return PETSC_ERR_SUP; }
PetscErrorCode PetscRandomSeed(PetscRandom r) { (void)r; return PETSC_ERR_SUP; }
PetscErrorCode PetscRandomGetValueReal(PetscRandom r, PetscReal *v) { (void)r; (void)v; return PETSC_ERR_SUP; }
PetscErrorCode PetscRandomGetValuesReal(PetscRandom r, PetscInt n, PetscReal *v) {
  (void)r; (void)n; (void)v; return PETSC_ERR_SUP;
}
PetscErrorCode PetscRandomDestroy(PetscRandom *r) { (void)r; return 0; }
