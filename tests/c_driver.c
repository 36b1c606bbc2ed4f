/*
 * c_driver.c -- the C ABI used from C (C99), as a host program that is not Python would use
 * it: namelist, host set-up, a restart snapshot written and read back, read_boundaries' file
 * name, and context creation (LGAME_ERR_NO_DEVICE without a GPU; created and destroyed where
 * there is one).  With a third argument "step" (a GPU is then required) it also steps: two
 * lgame_gpu_pchevi calls on device-resident state against two lgame_gpu_pchevi_host calls with
 * host arrays, in FP64 and in split precision, bit for bit.  Built and run by
 * tests/test_library.py:
 *   c_driver <namelist file> <scratch directory> [step]
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

/* Two steps of the device-resident lgame_gpu_pchevi in one context against two steps of
 * lgame_gpu_pchevi_host (host state in, host state out) in a second context, from the same
 * initial state and diagnostics: every field of the final state finite and bit-equal. */
static int step_both_ways(lgame_host_model* hm, const lgame_config* cfg0, int precision, const double** st,
                          const double** dg, const size_t* nst) {
  lgame_config cfg = *cfg0;
  cfg.precision = precision;
  const double* grid[LGAME_GRID_NFIELDS];
  for (int f = 0; f < LGAME_GRID_NFIELDS; ++f) {
    size_t n = 0;
    grid[f] = lgame_host_grid_field(hm, f, &n);
    if (!grid[f] && n) return 1;
  }
  double* dev_out[LGAME_STATE_NFIELDS];
  double* host_mid[LGAME_STATE_NFIELDS];
  double* host_out[LGAME_STATE_NFIELDS];
  for (int f = 0; f < LGAME_STATE_NFIELDS; ++f) {
    dev_out[f] = malloc((nst[f] ? nst[f] : 1) * sizeof(double));
    host_mid[f] = malloc((nst[f] ? nst[f] : 1) * sizeof(double));
    host_out[f] = malloc((nst[f] ? nst[f] : 1) * sizeof(double));
    if (!dev_out[f] || !host_mid[f] || !host_out[f]) return 1;
  }
  lgame_gpu* a = NULL;
  lgame_gpu* b = NULL;
  CHECK(lgame_gpu_create(&cfg, &a));
  CHECK(lgame_gpu_create(&cfg, &b));
  lgame_gpu* both[2] = {a, b};
  for (int k = 0; k < 2; ++k) {
    CHECK(lgame_gpu_set_grid(both[k], grid, LGAME_GRID_NFIELDS));
    CHECK(lgame_gpu_set_state(both[k], 0, st, LGAME_STATE_NFIELDS));
    CHECK(lgame_gpu_set_state(both[k], 1, st, LGAME_STATE_NFIELDS));
    CHECK(lgame_gpu_set_diag(both[k], dg, LGAME_DIAG_NFIELDS));
  }
  CHECK(lgame_gpu_pchevi(a, 0, 1, 0, 0, 0.0));
  CHECK(lgame_gpu_pchevi(a, 1, 0, 1, 0, 0.0));
  CHECK(lgame_gpu_get_state(a, 0, dev_out, LGAME_STATE_NFIELDS));
  CHECK(lgame_gpu_pchevi_host(b, st, host_mid, LGAME_STATE_NFIELDS, 0, 0, 0.0));
  CHECK(lgame_gpu_pchevi_host(b, (const double* const*)host_mid, host_out, LGAME_STATE_NFIELDS, 1, 0, 0.0));
  int bad = 0;
  for (int f = 0; f < LGAME_STATE_NFIELDS; ++f) {
    for (size_t e = 0; e < nst[f]; ++e)
      if (!(dev_out[f][e] - dev_out[f][e] == 0.0)) {
        fprintf(stderr, "precision %d: non-finite value in state field %d\n", precision, f);
        bad = 1;
        break;
      }
    if (memcmp(dev_out[f], host_out[f], nst[f] * sizeof(double)) != 0) {
      fprintf(stderr, "precision %d: state field %d differs between pchevi and pchevi_host\n", precision, f);
      bad = 1;
    }
  }
  lgame_gpu_destroy(a);
  lgame_gpu_destroy(b);
  for (int f = 0; f < LGAME_STATE_NFIELDS; ++f) {
    free(dev_out[f]);
    free(host_mid[f]);
    free(host_out[f]);
  }
  if (!bad) printf("stepped: precision %d, 2 steps, pchevi == pchevi_host\n", precision);
  return bad;
}

int main(int argc, char** argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: c_driver <namelist> <scratch dir> [step]\n");
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
    st2[0][f] = malloc((nst[f] ? nst[f] : 1) * sizeof(double));
    st2[1][f] = malloc((nst[f] ? nst[f] : 1) * sizeof(double));
    if ((!st[f] && nst[f]) || !st2[0][f] || !st2[1][f]) return 1;
  }
  for (int f = 0; f < LGAME_DIAG_NFIELDS; ++f) {
    dg[f] = lgame_host_diag_field(hm, f, &ndg[f]);
    dg2[f] = malloc(ndg[f] * sizeof(double));
    if (!dg[f] || !dg2[f]) return 1;
  }
  char path[1024];
  snprintf(path, sizeof path, "%s/c_driver.snap", argv[2]);
  CHECK(lgame_host_write_snapshot(path, cfg.ny, cfg.nx, cfg.n_layers, nml.n_constituents, nml.nsoillays, 7, st, st,
                                  dg));
  long long step = -1;
  CHECK(lgame_host_read_snapshot(path, cfg.ny, cfg.nx, cfg.n_layers, nml.n_constituents, nml.nsoillays, &step, st2[0],
                                 st2[1], dg2));
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
  if (lgame_host_read_snapshot(path, cfg.ny + 2, cfg.nx, cfg.n_layers, nml.n_constituents, nml.nsoillays, &step,
                               st2[0], st2[1], dg2) != LGAME_ERR_BAD_DIMS)
    return 1;

  char name[256];
  CHECK(lgame_host_bc_filename(nml.bc_root_filename, 10800.0, 0.0, name, (int)sizeof name));
  char expect[256];
  snprintf(expect, sizeof expect, "%s+10800s.bin", nml.bc_root_filename);
  if (strcmp(name, expect) != 0) return 1;

  lgame_gpu* g = NULL;
  const int stepping = argc > 3 && strcmp(argv[3], "step") == 0;
  const int rc = lgame_gpu_create(&cfg, &g);
  if (rc == LGAME_OK) {
    lgame_gpu_destroy(g);
  } else if (rc != LGAME_ERR_NO_DEVICE || stepping) {
    fprintf(stderr, "lgame_gpu_create: %d (%s)\n", rc, lgame_gpu_last_error());
    return 1;
  }
  printf("%s\n", lgame_gpu_version());
  if (stepping) {
    for (int prec = LGAME_PRECISION_FP64; prec <= LGAME_PRECISION_SPLIT; ++prec)
      if (step_both_ways(hm, &cfg, prec, st, dg, nst)) return 1;
  }

  for (int f = 0; f < LGAME_STATE_NFIELDS; ++f) {
    free(st2[0][f]);
    free(st2[1][f]);
  }
  for (int f = 0; f < LGAME_DIAG_NFIELDS; ++f) free(dg2[f]);
  lgame_host_destroy(hm);
  printf("ok\n");
  return 0;
}
