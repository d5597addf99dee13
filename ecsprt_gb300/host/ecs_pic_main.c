/*
 * pic -- the reference's PIC program (src/pic.c:148-287) on libecsgpu.
 *
 * The same options file and command line as the reference: the options
 * file is argv[1] when that names an existing file, else ./petsc.ini when it
 * exists (src/common.c:16-22); options given on the command line override
 * the file's.  The same program order: options (src/parameters.c:25-346,
 * src/pic.c:32-115), options.log (src/parameters.c:354-433), initial ions,
 * initial moments and potential, then -Nt steps of UpdateVelocities,
 * UpdatePositions, collect and ComputePotential (src/pic.c:238-258) through
 * the reference's operator slots (include/ecs_compat.h), with output at
 * step 0 and every --every steps after it, and at the start and the end:
 *
 *   fluid-initial.bin, fluid-NNN.bin, fluid-final.bin: the datasets of the
 *     reference's fluid*.hdf (density, x flux, y flux, z flux, rhs,
 *     potential) as consecutive PETSc binary Vecs (no HDF5 in this build)
 *   position*.bin, velocity*.bin (--output-particles): PETSc binary Vecs
 *     of the AoS FP64 arrays, as OutputSwarmBinary (src/file-io.c:103-161)
 *
 * NNN has 1 + floor(log10(Nt)) digits (src/pic.c:216-220).
 *
 * Options without a reference counterpart:
 *   --precision fp64|mixed   the plain FP64 path or the FP32 + FP64-refined
 *                            path (default mixed)
 *   --sort-every N           cell-sort cadence of the mixed path (default 2)
 *   --seed S                 seed of the device-side initial ions and of the
 *                            collision streams (default 20261203)
 * The potential solve stops at -ksp_rtol (PETSc's default 1e-5) or after
 * -ksp_max_it iterations (default 10000), the PETSc KSP options the
 * reference's solver reads.
 *
 * Exit status 0 on success; on failure the library's message is printed and
 * the status is the negated ECS_ERR_* code.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ecs_compat.h"
#include "ecs_host.h"
#include "ecs_driver.h"

typedef struct PicRun {
  EcsCtx *ctx;
  EcsParams p;
  EcsPicApp app;
  int nd;
  double *moments, *rhs, *phi, *pos, *vel;
} PicRun;

/* OutputFluidHDF5 + particleFunc (src/file-io.c:103-222) for one insert. */
static int output(PicRun *r, const char *insert) {
  char path[4200];
  const int64_t n = (int64_t)r->p.Nx * r->p.Ny * r->p.Nz;
  int rc = ecs_moments_download(r->ctx, r->moments);
  if (!rc) rc = ecs_rhs_download(r->ctx, r->rhs);
  if (!rc) rc = ecs_phi_download(r->ctx, r->phi);
  if (rc) return rc;
  snprintf(path, sizeof path, "fluid%s.bin", insert);
  ecs_drv_status("Writing %s\n", path);
  if ((rc = ecs_write_fluid(path, r->moments, r->rhs, r->phi, n))) return rc;
  if (!r->app.output_particles) return ECS_OK;
  const int64_t np = ecs_particles_count(r->ctx);
  if ((rc = ecs_particles_download(r->ctx, r->pos, r->vel))) return rc;
  snprintf(path, sizeof path, "position%s.bin", insert);
  ecs_drv_status("Writing %s\n", path);
  if ((rc = ecs_write_petsc_vec(path, r->pos, np * r->nd))) return rc;
  snprintf(path, sizeof path, "velocity%s.bin", insert);
  ecs_drv_status("Writing %s\n", path);
  return ecs_write_petsc_vec(path, r->vel, np * r->nd);
}

int main(int argc, char **argv) {
  EcsOptions *o = ecs_options_create();
  char err[512] = "";
  int rc = ecs_drv_load_options(argc, argv, o);
  if (rc) return ecs_drv_fail(rc, "cannot read the options file");
  if (ecs_drv_version(o, "pic")) return 0;
  ecs_drv_log_level(o);
  ecs_drv_status("[pic] Running on 1 GPU\n\n**************** START *****************\n\n");

  PicRun r;
  memset(&r, 0, sizeof r);
  ecs_drv_status("Processing common options\n");
  if ((rc = ecs_params_from_options(o, &r.p, err, sizeof err))) return ecs_drv_fail(rc, err);
  ecs_drv_status("Processing application-specific options\n");
  if ((rc = ecs_pic_app_from_options(o, &r.p, &r.app, err, sizeof err))) return ecs_drv_fail(rc, err);
  EcsDrvExtra x;
  ecs_drv_extra(o, &x);
  r.nd = r.p.ndim == 2 ? 2 : 3;

  ecs_drv_status("Echoing parameter values to options.log\n");
  if ((rc = ecs_echo_options("options.log", o, &r.p))) return ecs_drv_fail(rc, "cannot write options.log");

  if ((rc = ecs_ctx_create(&r.p, x.precision, r.app.Np, NULL, &r.ctx))) return ecs_drv_fail(rc, ecs_last_error(NULL));
  ecs_set_sort_every(r.ctx, x.sort_every);
  ecs_set_seed(r.ctx, x.seed);
  const int64_t n = (int64_t)r.p.Nx * r.p.Ny * r.p.Nz;
  r.moments = malloc(sizeof(double) * 4 * n);
  r.rhs = malloc(sizeof(double) * n);
  r.phi = malloc(sizeof(double) * n);
  if (r.app.output_particles) {
    r.pos = malloc(sizeof(double) * r.nd * r.app.Np);
    r.vel = malloc(sizeof(double) * r.nd * r.app.Np);
  }
  if (!r.moments || !r.rhs || !r.phi || (r.app.output_particles && (!r.pos || !r.vel)))
    return ecs_drv_fail(ECS_ERR_NOMEM, "host allocation failed");

  ecs_drv_status("\n=== Initial stage ===\n\n");
  ecs_drv_status("Initializing positions\n");
  ecs_drv_status("Initializing velocities\n");
  if (r.app.vdist != 0) return ecs_drv_fail(ECS_ERR_UNSUPPORTED, "only --velocity-dist normal exists");
  if ((rc = ecs_particles_init(r.ctx, r.app.pdist, r.app.Np, x.seed, NULL)))
    return ecs_drv_fail(rc, ecs_last_error(r.ctx));

  /* the reference's operator slots, bound as SetUpContext binds them */
  EcsOperators ops;
  if ((rc = EcsGpuBindOperatorsFor(&ops, &r.p))) return ecs_drv_fail(rc, "unknown -lhs / -rhs");
  EcsGpuContext g;
  memset(&g, 0, sizeof g);
  g.ctx = r.ctx;
  g.params = r.p;
  g.rtol = x.rtol;
  g.max_it = x.max_it;

  ecs_drv_status("Collecting initial moments\n");
  if ((rc = ops.collect(&g))) return ecs_drv_fail(rc, ecs_last_error(r.ctx));
  ecs_drv_status("Computing initial potential\n");
  if ((rc = EcsGpuComputePotential(&ops, &g))) return ecs_drv_fail(rc, ecs_last_error(r.ctx));
  if ((rc = output(&r, "-initial"))) return ecs_drv_fail(rc, "output failed");

  const int width = 1 + (int)log10((double)(r.app.Nt > 0 ? r.app.Nt : 1));
  ecs_drv_status("\n\n=== Main time-step loop ===\n\n");
  for (int it = 0; it < r.app.Nt; it++) {
    ecs_drv_status("< Time step %0*d >\n", width, it);
    ecs_drv_status("Updating velocities\n");
    if ((rc = EcsGpuUpdateVelocities(&ops, r.p.ndim, r.app.dt, &g))) return ecs_drv_fail(rc, ecs_last_error(r.ctx));
    ecs_drv_status("Updating positions\n");
    if ((rc = EcsGpuUpdatePositions(&ops, r.p.ndim, r.app.dt, &g))) return ecs_drv_fail(rc, ecs_last_error(r.ctx));
    ecs_drv_status("Collecting moments\n");
    if ((rc = ops.collect(&g))) return ecs_drv_fail(rc, ecs_last_error(r.ctx));
    ecs_drv_status("Computing potential\n");
    if ((rc = EcsGpuComputePotential(&ops, &g))) return ecs_drv_fail(rc, ecs_last_error(r.ctx));
    ecs_drv_detail("  solve: %d iterations, relative residual %.3e\n", g.last_solve.iterations, g.last_solve.relres);
    if (r.app.every > 0 && it % r.app.every == 0) {
      char insert[32];
      snprintf(insert, sizeof insert, "-%0*d", width, it);
      if ((rc = output(&r, insert))) return ecs_drv_fail(rc, "output failed");
    }
    ecs_drv_status("\n");
  }
  ecs_drv_status("\n=== Final stage ===\n\n");
  if ((rc = output(&r, "-final"))) return ecs_drv_fail(rc, "output failed");
  ecs_drv_status("Freeing objects\n");
  ecs_ctx_destroy(r.ctx);
  free(r.moments); free(r.rhs); free(r.phi); free(r.pos); free(r.vel);
  ecs_options_destroy(o);
  ecs_drv_status("\n***************** END ******************\n");
  return 0;
}
