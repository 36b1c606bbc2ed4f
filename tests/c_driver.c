/*
 * c_driver.c -- the C ABI used from C (C99), as a host program that is not Python would use
 * it: namelist, host set-up, a restart snapshot written and read back, read_boundaries' file
 * name, and context creation (LGAME_ERR_NO_DEVICE without a GPU; created and destroyed, no
 * step, where there is one).  Built and run by tests/test_library.py:
 *   c_driver <namelist file> <scratch directory>
 * Prints "ok" and exits 0 when every check holds.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "lgame_emulator.h"
#include "lgame_gpu.h"
#include "lgame_host.h"

#define CHECK(call)                                                                       \
  do {                                                                                    \
    int rc_ = (call);                                                                     \
    if (rc_ != LGAME_OK) {                                                                \
      fprintf(stderr, "%s: %d (%s)\n", #call, rc_, lgame_gpu_last_error());               \
      return 1;                                                                           \
    }                                                                                     \
  } while (0)

int main(int argc, char** argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: c_driver <namelist> <scratch dir>\n");
    return 2;
  }
  lgame_namelist nml;
  CHECK(lgame_namelist_read_file(argv[1], &nml));
  lgame_config cfg;
  CHECK(lgame_config_from_namelist(&nml, &cfg));
  lgame_host_model* hm = NULL;
  CHECK(lgame_host_setup(&nml, &hm));

  /* snapshot of the initial state (both slots) and diagnostics, then read back */
  const double* st[LGAME_STATE_NFIELDS];
  const double* dg[LGAME_DIAG_NFIELDS];
  double* st2[2][LGAME_STATE_NFIELDS];
  double* dg2[LGAME_DIAG_NFIELDS];
  size_t nst[LGAME_STATE_NFIELDS], ndg[LGAME_DIAG_NFIELDS];
  for (int f = 0; f < LGAME_STATE_NFIELDS; ++f) {
    st[f] = lgame_host_state_field(hm, f, &nst[f]);
    st2[0][f] = malloc(nst[f] * sizeof(double));
    st2[1][f] = malloc(nst[f] * sizeof(double));
    if (!st[f] || !st2[0][f] || !st2[1][f]) return 1;
  }
  for (int f = 0; f < LGAME_DIAG_NFIELDS; ++f) {
    dg[f] = lgame_host_diag_field(hm, f, &ndg[f]);
    dg2[f] = malloc(ndg[f] * sizeof(double));
    if (!dg[f] || !dg2[f]) return 1;
  }
  char path[1024];
  snprintf(path, sizeof path, "%s/c_driver.snap", argv[2]);
  CHECK(lgame_host_write_snapshot(path, cfg.ny, cfg.nx, cfg.n_layers, nml.n_constituents, 7, st, st, dg));
  long long step = -1;
  CHECK(lgame_host_read_snapshot(path, cfg.ny, cfg.nx, cfg.n_layers, nml.n_constituents, &step, st2[0], st2[1],
                                 dg2));
  if (step != 7) return 1;
  for (int f = 0; f < LGAME_STATE_NFIELDS; ++f)
    for (int s = 0; s < 2; ++s)
      if (memcmp(st[f], st2[s][f], nst[f] * sizeof(double)) != 0) {
        fprintf(stderr, "state field %d of slot %d differs\n", f, s);
        return 1;
      }
  for (int f = 0; f < LGAME_DIAG_NFIELDS; ++f)
    if (memcmp(dg[f], dg2[f], ndg[f] * sizeof(double)) != 0) {
      fprintf(stderr, "diagnostic %d differs\n", f);
      return 1;
    }
  /* a snapshot of other dimensions is refused */
  if (lgame_host_read_snapshot(path, cfg.ny + 2, cfg.nx, cfg.n_layers, nml.n_constituents, &step, st2[0], st2[1],
                               dg2) != LGAME_ERR_BAD_DIMS)
    return 1;

  char name[256];
  CHECK(lgame_host_bc_filename(nml.bc_root_filename, 10800.0, 0.0, name, (int)sizeof name));
  char expect[256];
  snprintf(expect, sizeof expect, "%s+10800s.bin", nml.bc_root_filename);
  if (strcmp(name, expect) != 0) return 1;

  lgame_gpu* g = NULL;
  const int rc = lgame_gpu_create(&cfg, &g);
  if (rc == LGAME_OK) {
    lgame_gpu_destroy(g);
  } else if (rc != LGAME_ERR_NO_DEVICE) {
    fprintf(stderr, "lgame_gpu_create: %d (%s)\n", rc, lgame_gpu_last_error());
    return 1;
  }
  printf("%s\n", lgame_gpu_version());

  for (int f = 0; f < LGAME_STATE_NFIELDS; ++f) {
    free(st2[0][f]);
    free(st2[1][f]);
  }
  for (int f = 0; f < LGAME_DIAG_NFIELDS; ++f) free(dg2[f]);
  lgame_host_destroy(hm);
  printf("ok\n");
  return 0;
}
