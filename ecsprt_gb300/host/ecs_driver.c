/*
 * Helpers of the re-hosted programs (ecs_driver.h).
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <unistd.h>

#include "ecs_driver.h"

static int g_level = 1;

static int parse_argv(EcsOptions *o, int argc, char **argv, int first) {
  size_t len = 1;
  for (int i = first; i < argc; i++) len += strlen(argv[i]) + 1;
  char *buf = malloc(len);
  if (!buf) return ECS_ERR_NOMEM;
  buf[0] = '\0';
  for (int i = first; i < argc; i++) {
    strcat(buf, argv[i]);
    strcat(buf, " ");
  }
  int rc = ecs_options_parse(o, buf);
  free(buf);
  return rc;
}

int ecs_drv_load_options(int argc, char **argv, EcsOptions *o) {
  int first = 1, rc = ECS_OK;
  if (argc > 1 && access(argv[1], F_OK) == 0) {
    rc = ecs_options_load_file(o, argv[1]);
    first = 2;
  } else if (access("petsc.ini", F_OK) == 0) {
    rc = ecs_options_load_file(o, "petsc.ini");
  }
  if (rc) return rc;
  return parse_argv(o, argc, argv, first);
}

int ecs_drv_version(const EcsOptions *o, const char *name) {
  int found = 0;
  ecs_options_get(o, "--version", &found);
  if (!found) return 0;
  printf("ECSPRT: Electrostatic Collisional Space Plasma Research Toolkit\n");
  printf("[%s] Version 0.6.0 (%s)\n\n", name, ecs_version());
  return 1;
}

void ecs_drv_log_level(const EcsOptions *o) {
  int found = 0;
  const char *s = ecs_options_get(o, "--log-level", &found);
  if (found && s) g_level = atoi(s);
}

void ecs_drv_status(const char *fmt, ...) {
  if (g_level < 1) return;
  va_list ap;
  va_start(ap, fmt);
  vprintf(fmt, ap);
  va_end(ap);
  fflush(stdout);
}

void ecs_drv_detail(const char *fmt, ...) {
  if (g_level < 2) return;
  va_list ap;
  va_start(ap, fmt);
  vprintf(fmt, ap);
  va_end(ap);
  fflush(stdout);
}

int ecs_drv_fail(int code, const char *msg) {
  fprintf(stderr, "error: %s (%s)\n", msg && msg[0] ? msg : "failure", ecs_status_string(code));
  return code < 0 ? -code : 1;
}

void ecs_drv_extra(const EcsOptions *o, EcsDrvExtra *x) {
  int found = 0;
  const char *s;
  x->precision = ECS_PREC_MIXED;
  x->sort_every = 2;
  x->seed = 20261203ull;
  x->rtol = 1e-5;
  x->max_it = 10000;
  s = ecs_options_get(o, "--precision", &found);
  if (found && s && strcasecmp(s, "fp64") == 0) x->precision = ECS_PREC_FP64;
  s = ecs_options_get(o, "--sort-every", &found);
  if (found && s) x->sort_every = atoi(s);
  s = ecs_options_get(o, "--seed", &found);
  if (found && s) x->seed = strtoull(s, NULL, 10);
  s = ecs_options_get(o, "-ksp_rtol", &found);
  if (found && s) x->rtol = strtod(s, NULL);
  s = ecs_options_get(o, "-ksp_max_it", &found);
  if (found && s) x->max_it = atoi(s);
}
