/*
 * Minimal single-rank stand-in for the PETSc public API.
 *
 * TEST INFRASTRUCTURE ONLY.  This header lets the reference's own hot-path C
 * sources (src/velocities.c, src/vector-math.c, src/moments.c,
 * src/collisions.c, src/boundaries.c, src/positions.c, src/lhs.c, src/rhs.c,
 * src/random.c, src/setup.c, src/parameters.c, src/potential.c,
 * src/logging.c, src/common.c) compile UNMODIFIED into oracle/_ref/, so that
 * their outputs can pin the oracle restatement.  It is written from PETSc's
 * documented names and signatures; it is not PETSc and it does not distribute.
 *
 * Semantics kept from PETSc 3.20 (the version the reference's setup.sh:42
 * installs):
 *   - PetscReal = double, PetscInt = 32-bit int (PETSc's default build).
 *   - PetscSqr is the function-like macro ((a)*(a)); an argument with side
 *     effects is therefore evaluated twice, exactly as under PETSc.
 *   - DMDA arrays are addressed with global indices, ghosted local arrays
 *     reach `stencil width` points past each end, and periodic ghosts hold the
 *     wrapped values after DMGlobalToLocal.
 *   - DMLocalToGlobal(ADD_VALUES) folds ghost contributions into their owners.
 *   - MatSetValuesStencil(INSERT_VALUES) wraps periodic column indices and
 *     overwrites duplicates; out-of-range columns of ghosted dimensions are
 *     dropped.
 */
#ifndef ECS_SHIM_PETSC_H
#define ECS_SHIM_PETSC_H

#include <math.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int PetscErrorCode;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef double PetscReal;
typedef double PetscScalar;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef int PetscEnum;
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef FILE *PetscFILE;

#define PETSC_COMM_WORLD 0
#define PETSC_COMM_SELF 1
#define PETSC_STDOUT stdout
#define MPIU_REAL 1
#define PETSC_SUCCESS 0
#define PETSC_ERR_ARG_WRONG 62
#define PETSC_ERR_ARG_UNKNOWN_TYPE 86
#define PETSC_ERR_SUP 56
#define PETSC_DECIDE (-1)
#define PETSC_DEFAULT (-2)
#define PETSC_MAX_PATH_LEN 4096
#define PETSC_PI 3.14159265358979323846264338327950288419716939937510582
#define PETSC_MACHINE_EPSILON 2.2204460492503131e-16

#define PetscSqr(a) ((a) * (a))
#define PetscSqrtReal(a) sqrt(a)
#define PetscCosReal(a) cos(a)
#define PetscSinReal(a) sin(a)
#define PetscCosScalar(a) cos(a)
#define PetscAbsReal(a) fabs(a)
#define PetscLog10Real(a) log10(a)
#define PetscRealPart(a) (a)
#define PetscImaginaryPart(a) ((PetscReal)0.0)
#define PetscMin(a, b) (((a) < (b)) ? (a) : (b))
#define PetscMax(a, b) (((a) < (b)) ? (b) : (a))

#define PetscFunctionBeginUser
#define PetscFunctionReturn(a) return (a)
#define PetscCall(...)                                                         \
  do {                                                                         \
    PetscErrorCode ierr_shim_ = (__VA_ARGS__);                                 \
    if (ierr_shim_ != 0) return ierr_shim_;                                    \
  } while (0)
#define PetscCallMPI(...) PetscCall(__VA_ARGS__)
#define SETERRQ(comm, code, ...)                                               \
  return ShimSetError((code), __FILE__, __LINE__, __VA_ARGS__)

PetscErrorCode ShimSetError(PetscErrorCode code, const char *file, int line,
                            const char *fmt, ...);

/* ---- opaque objects -------------------------------------------------- */
typedef struct _p_DM *DM;
typedef struct _p_Vec *Vec;
typedef struct _p_Mat *Mat;
typedef struct _p_KSP *KSP;
typedef struct _p_MatNullSpace *MatNullSpace;
typedef struct _p_PetscViewer *PetscViewer;
typedef struct _p_PetscRandom *PetscRandom;
typedef struct _p_PetscObject *PetscObject;
typedef void *PetscOptions;

typedef enum {
  DM_BOUNDARY_NONE,
  DM_BOUNDARY_GHOSTED,
  DM_BOUNDARY_MIRROR,
  DM_BOUNDARY_PERIODIC,
  DM_BOUNDARY_TWIST
} DMBoundaryType;
typedef enum { DMDA_STENCIL_STAR, DMDA_STENCIL_BOX } DMDAStencilType;
typedef enum { DMDA_ELEMENT_P1, DMDA_ELEMENT_Q1 } DMDAElementType;
typedef enum { NOT_SET_VALUES, INSERT_VALUES, ADD_VALUES } InsertMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { DMSWARM_BASIC = 0, DMSWARM_PIC } DMSwarmType;
typedef enum { PETSC_INT = 0, PETSC_REAL = 1 } PetscDataType;
typedef enum { FILE_MODE_READ, FILE_MODE_WRITE, FILE_MODE_APPEND } PetscFileMode;
typedef const char *DMType;
typedef const char *PetscViewerType;
#define DMSWARM "swarm"
#define PETSCVIEWERASCII "ascii"
#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)

typedef struct {
  PetscInt k, j, i, c;
} MatStencil;

typedef struct {
  PetscInt dim, dof, sw;
  PetscInt mx, my, mz;
  PetscInt xs, ys, zs;
  PetscInt xm, ym, zm;
  PetscInt gxs, gys, gzs;
  PetscInt gxm, gym, gzm;
  DMBoundaryType bx, by, bz;
  DMDAStencilType st;
  DM da;
} DMDALocalInfo;

extern const char DMSwarmPICField_coor[];

/* ---- MPI ---------------------------------------------------------------- */
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int errorcode);

/* ---- system ------------------------------------------------------------- */
PetscErrorCode PetscInitialize(int *argc, char ***args, const char file[],
                               const char help[]);
PetscErrorCode PetscFinalize(void);
PetscErrorCode PetscEnd(void);
PetscErrorCode PetscPrintf(MPI_Comm comm, const char fmt[], ...);
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm comm, const char fmt[], ...);
PetscErrorCode PetscSynchronizedFlush(MPI_Comm comm, FILE *fd);
PetscErrorCode PetscStrcpy(char s[], const char t[]);
PetscErrorCode PetscStrcat(char s[], const char t[]);
PetscErrorCode PetscStrcmp(const char a[], const char b[], PetscBool *flg);
PetscErrorCode PetscGetFullPath(const char path[], char fullpath[], size_t flen);
#define PetscMalloc1(n, p) (((*(p)) = calloc((size_t)(n) + 1, sizeof(**(p)))) ? 0 : 55)
#define PetscFree(p) (free(p), (p) = NULL, 0)

/* ---- options ------------------------------------------------------------ */
PetscErrorCode PetscOptionsGetReal(PetscOptions o, const char pre[], const char name[],
                                   PetscReal *v, PetscBool *set);
PetscErrorCode PetscOptionsGetInt(PetscOptions o, const char pre[], const char name[],
                                  PetscInt *v, PetscBool *set);
PetscErrorCode PetscOptionsGetBool(PetscOptions o, const char pre[], const char name[],
                                   PetscBool *v, PetscBool *set);
PetscErrorCode PetscOptionsGetEnum(PetscOptions o, const char pre[], const char name[],
                                   const char *const *list, PetscEnum *v, PetscBool *set);
PetscErrorCode PetscOptionsView(PetscOptions o, PetscViewer viewer);

/* ---- viewers ------------------------------------------------------------ */
PetscErrorCode PetscViewerASCIIOpen(MPI_Comm comm, const char name[], PetscViewer *v);
PetscErrorCode PetscViewerCreate(MPI_Comm comm, PetscViewer *v);
PetscErrorCode PetscViewerSetType(PetscViewer v, PetscViewerType t);
PetscErrorCode PetscViewerFileSetMode(PetscViewer v, PetscFileMode m);
PetscErrorCode PetscViewerFileSetName(PetscViewer v, const char name[]);
PetscErrorCode PetscViewerASCIIPrintf(PetscViewer v, const char fmt[], ...);
PetscErrorCode PetscViewerDestroy(PetscViewer *v);

/* ---- objects ------------------------------------------------------------ */
PetscErrorCode PetscObjectSetOptionsPrefix(PetscObject obj, const char prefix[]);
PetscErrorCode PetscObjectSetName(PetscObject obj, const char name[]);

/* ---- DM / DMDA ---------------------------------------------------------- */
PetscErrorCode DMDACreate2d(MPI_Comm comm, DMBoundaryType bx, DMBoundaryType by,
                            DMDAStencilType st, PetscInt M, PetscInt N, PetscInt m,
                            PetscInt n, PetscInt dof, PetscInt s, const PetscInt lx[],
                            const PetscInt ly[], DM *da);
PetscErrorCode DMDACreate3d(MPI_Comm comm, DMBoundaryType bx, DMBoundaryType by,
                            DMBoundaryType bz, DMDAStencilType st, PetscInt M,
                            PetscInt N, PetscInt P, PetscInt m, PetscInt n, PetscInt p,
                            PetscInt dof, PetscInt s, const PetscInt lx[],
                            const PetscInt ly[], const PetscInt lz[], DM *da);
PetscErrorCode DMDASetElementType(DM dm, DMDAElementType t);
PetscErrorCode DMSetFromOptions(DM dm);
PetscErrorCode DMSetUp(DM dm);
PetscErrorCode DMDASetUniformCoordinates(DM dm, PetscReal x0, PetscReal x1, PetscReal y0,
                                         PetscReal y1, PetscReal z0, PetscReal z1);
PetscErrorCode DMDASetFieldName(DM dm, PetscInt nf, const char name[]);
PetscErrorCode DMSetApplicationContext(DM dm, void *ctx);
PetscErrorCode DMCreate(MPI_Comm comm, DM *dm);
PetscErrorCode DMSetType(DM dm, DMType type);
PetscErrorCode DMGetDimension(DM dm, PetscInt *dim);
PetscErrorCode DMSetDimension(DM dm, PetscInt dim);
PetscErrorCode DMDestroy(DM *dm);
PetscErrorCode DMView(DM dm, PetscViewer v);
PetscErrorCode DMDAGetCorners(DM dm, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m,
                              PetscInt *n, PetscInt *p);
PetscErrorCode DMDAGetLocalInfo(DM dm, DMDALocalInfo *info);
PetscErrorCode DMCreateGlobalVector(DM dm, Vec *v);
PetscErrorCode DMGetGlobalVector(DM dm, Vec *v);
PetscErrorCode DMRestoreGlobalVector(DM dm, Vec *v);
PetscErrorCode DMGetLocalVector(DM dm, Vec *v);
PetscErrorCode DMRestoreLocalVector(DM dm, Vec *v);
PetscErrorCode DMGlobalToLocal(DM dm, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMGlobalToLocalBegin(DM dm, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMGlobalToLocalEnd(DM dm, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMLocalToGlobal(DM dm, Vec l, InsertMode mode, Vec g);
PetscErrorCode DMDAVecGetArray(DM dm, Vec v, void *array);
PetscErrorCode DMDAVecRestoreArray(DM dm, Vec v, void *array);
PetscErrorCode DMDAVecGetArrayDOF(DM dm, Vec v, void *array);
PetscErrorCode DMDAVecRestoreArrayDOF(DM dm, Vec v, void *array);
PetscErrorCode DMCreateMatrix(DM dm, Mat *A);

/* ---- DMSwarm ------------------------------------------------------------ */
PetscErrorCode DMSwarmSetCellDM(DM sw, DM cell);
PetscErrorCode DMSwarmGetCellDM(DM sw, DM *cell);
PetscErrorCode DMSwarmSetType(DM sw, DMSwarmType t);
PetscErrorCode DMSwarmInitializeFieldRegister(DM sw);
PetscErrorCode DMSwarmRegisterPetscDatatypeField(DM sw, const char name[], PetscInt bs,
                                                 PetscDataType t);
PetscErrorCode DMSwarmFinalizeFieldRegister(DM sw);
PetscErrorCode DMSwarmSetLocalSizes(DM sw, PetscInt n, PetscInt buf);
PetscErrorCode DMSwarmGetLocalSize(DM sw, PetscInt *n);
PetscErrorCode DMSwarmGetSize(DM sw, PetscInt *n);
PetscErrorCode DMSwarmGetField(DM sw, const char name[], PetscInt *bs, PetscDataType *t,
                               void **data);
PetscErrorCode DMSwarmRestoreField(DM sw, const char name[], PetscInt *bs,
                                   PetscDataType *t, void **data);
PetscErrorCode DMSwarmMigrate(DM sw, PetscBool remove);
PetscErrorCode DMSwarmSetPointsUniformCoordinates(DM sw, PetscReal min[], PetscReal max[],
                                                  PetscInt npoints[], InsertMode mode);

/* ---- Vec / Mat / KSP ---------------------------------------------------- */
PetscErrorCode VecZeroEntries(Vec v);
PetscErrorCode VecSet(Vec v, PetscScalar a);
PetscErrorCode VecCopy(Vec x, Vec y);
PetscErrorCode VecDestroy(Vec *v);
PetscErrorCode MatSetValuesStencil(Mat A, PetscInt m, const MatStencil idxm[], PetscInt n,
                                   const MatStencil idxn[], const PetscScalar v[],
                                   InsertMode mode);
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t);
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t);
PetscErrorCode MatZeroEntries(Mat A);
PetscErrorCode MatShift(Mat A, PetscScalar a);
PetscErrorCode MatMult(Mat A, Vec x, Vec y);
PetscErrorCode MatCreateVecs(Mat A, Vec *r, Vec *l);
PetscErrorCode MatNullSpaceCreate(MPI_Comm comm, PetscBool has_cnst, PetscInt n,
                                  const Vec vecs[], MatNullSpace *sp);
PetscErrorCode MatSetNullSpace(Mat A, MatNullSpace sp);
PetscErrorCode MatNullSpaceRemove(MatNullSpace sp, Vec v);
PetscErrorCode MatNullSpaceDestroy(MatNullSpace *sp);
PetscErrorCode KSPGetDM(KSP ksp, DM *dm);
PetscErrorCode KSPSolve(KSP ksp, Vec b, Vec x);
PetscErrorCode KSPGetSolution(KSP ksp, Vec *x);
PetscErrorCode KSPGetOperators(KSP ksp, Mat *A, Mat *P);

/* ---- PetscRandom (not exercised by the hot path) ------------------------ */
PetscErrorCode PetscRandomCreate(MPI_Comm comm, PetscRandom *r);
PetscErrorCode PetscRandomSetInterval(PetscRandom r, PetscReal lo, PetscReal hi);
PetscErrorCode PetscRandomSetSeed(PetscRandom r, unsigned long seed);
PetscErrorCode PetscRandomSeed(PetscRandom r);
PetscErrorCode PetscRandomGetValueReal(PetscRandom r, PetscReal *v);
PetscErrorCode PetscRandomGetValuesReal(PetscRandom r, PetscInt n, PetscReal *v);
PetscErrorCode PetscRandomDestroy(PetscRandom *r);

#endif /* ECS_SHIM_PETSC_H */
