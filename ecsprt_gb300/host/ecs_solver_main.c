/*
 * solver -- the reference's stand-alone potential solver (src/solver.c:107-203)
 * on libecsgpu.
 *
 * Options as the reference's (src/parameters.c:25-346, src/solver.c:29-74),
 * read as pic reads them.  LoadFluidQuantities (src/file-io.c:8-75) reads
 * the density from the HDF5 dataset "density-kji" of --input; this build has
 * no HDF5, so --input names a PETSc binary Vec of the same Nz x Ny x Nx
 * values (i fastest, the order of "density-kji").  The fluxes are
 * flux_scale x density (src/file-io.c:51-59, --flux-scale and
 * --{x,y,z}-flux-scale), the potential is solved to -ksp_rtol (default
 * 1e-5) within -ksp_max_it iterations, and OutputFluidHDF5("") becomes
 * fluid.bin: density, x flux, y flux, z flux, rhs and potential as
 * consecutive PETSc binary Vecs.  --view-lhs and --lhs-eigenvalues (PETSc
 * matrix and SLEPc output) are not available and are refused.
 *
 * Extra options as pic: --precision fp64|mixed (default mixed).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ecs_driver.h"
#include "ecs_serve.h"

int main(int argc, char **argv) {
  EcsOptions *o = ecs_options_create();
  char err[512] = "";
  int rc = ecs_drv_load_options(argc, argv, o);
  if (rc) return ecs_drv_fail(rc, "cannot read the options file");
  if (ecs_drv_version(o, "solver")) return 0;
  ecs_drv_log_level(o);
  ecs_drv_status("[solver] Running on 1 GPU\n\n**************** START *****************\n\n");
  EcsParams p;
  ecs_drv_status("Processing common options\n");
  if ((rc = ecs_params_from_options(o, &p, err, sizeof err))) return ecs_drv_fail(rc, err);
  EcsSolverApp app;
  ecs_drv_status("Processing application-specific options\n");
  ecs_solver_app_from_options(o, &app);
  EcsDrvExtra x;
  ecs_drv_extra(o, &x);
  int found = 0;
  ecs_options_get(o, "--lhs-eigenvalues", &found);
  if (app.view_lhs || found)
    return ecs_drv_fail(ECS_ERR_UNSUPPORTED, "--view-lhs and --lhs-eigenvalues are not available in this build");
  if (!app.input[0]) return ecs_drv_fail(ECS_ERR_INVALID, "--input is required");

  ecs_drv_status("Echoing parameter values to options.log\n");
  if ((rc = ecs_echo_options("options.log", o, &p))) return ecs_drv_fail(rc, "cannot write options.log");
  const int64_t n = (int64_t)p.Nx * p.Ny * p.Nz;
  double *dens = malloc(sizeof(double) * n), *phi = malloc(sizeof(double) * n);
  double *mom = malloc(sizeof(double) * 4 * n), *rhs = malloc(sizeof(double) * n);
  if (!dens || !phi || !mom || !rhs) return ecs_drv_fail(ECS_ERR_NOMEM, "host allocation failed");
  ecs_drv_status("Loading fluid quantities\n");
  if ((rc = ecs_read_petsc_vec(app.input, dens, n)))
    return ecs_drv_fail(rc, "--input must be a PETSc binary Vec of Nx*Ny*Nz densities");

  EcsCtx *ctx = NULL;
  if ((rc = ecs_ctx_create(&p, x.precision, 0, NULL, &ctx))) return ecs_drv_fail(rc, ecs_last_error(NULL));
  ecs_drv_status("Computing initial potential\n");
  EcsSolveStats st;
  memset(&st, 0, sizeof st);
  rc = ecs_solve_density(ctx, dens, app.flux_scale, x.rtol, x.max_it, phi, &st);
  if (rc) return ecs_drv_fail(rc, ecs_last_error(ctx));
  ecs_drv_detail("  solve: %d iterations, relative residual %.3e\n", st.iterations, st.relres);
  if ((rc = ecs_moments_download(ctx, mom)) || (rc = ecs_rhs_download(ctx, rhs)))
    return ecs_drv_fail(rc, ecs_last_error(ctx));
  ecs_drv_status("Writing fluid quantities to fluid.bin\n");
  if ((rc = ecs_write_fluid("fluid.bin", mom, rhs, phi, n))) return ecs_drv_fail(rc, "output failed");
  ecs_drv_status("Freeing objects\n");
  ecs_ctx_destroy(ctx);
  free(dens); free(phi); free(mom); free(rhs);
  ecs_options_destroy(o);
  ecs_drv_status("\n***************** END ******************\n");
  return 0;
}
