/*
 * lgame_oracle.h -- CPU FP64 restatement of L-GAME's HEVI step (TEST INFRASTRUCTURE).
 *
 * This is the correctness oracle and the timed CPU baseline of the GPU library.  It is
 * a line-by-line restatement in C of the reference's Fortran (src/time_stepping/,
 * src/spatial_operators/, src/constituents/mo_derived.F90, mo_dictionary.F90,
 * src/io/mo_write_out.F90:226-304): same loops, same operation order, same boundary
 * handling, same quirks.  It is never linked into the product; only the tests, the
 * smoke check and the CPU-baseline leg of bench.py load it.
 *
 * Parity against the Fortran binary itself is unpinned: the reference cannot be
 * compiled here (no Fortran compiler, no netCDF-Fortran, no RTE+RRTMGP) and ships no
 * tests or golden outputs.  The restatement is pinned instead by analytic invariants
 * (tests/test_oracle_*.py) and by committed golden vectors of this restatement.
 *
 * The interface mirrors lgame_gpu.h (same lgame_config, same field enums and the same
 * reference-layout arrays) so that a test can feed identical inputs to both.
 */
#ifndef LGAME_ORACLE_H
#define LGAME_ORACLE_H

#include "../include/lgame_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

int  oracle_create(const lgame_config* cfg, oracle_ctx** out);
void oracle_destroy(oracle_ctx* o);
int  oracle_set_grid(oracle_ctx* o, const double* const* fields, int nfields);
/* diag%heating_diss of the last step (ny,nx,nl), the dissipative heating power density */
int  oracle_heating_diss(const oracle_ctx* o, double* out);
/* the scalar diffusion of the last step: mass_diff_tendency (ny,nx,nl,ncons) and
 * temp_diff_heating (ny,nx,nl) */
int  oracle_scalar_diffusion(const oracle_ctx* o, double* mass_diff_tendency, double* temp_diff_heating);
int  oracle_set_state(oracle_ctx* o, int slot, const double* const* fields, int nfields);
int  oracle_get_state(oracle_ctx* o, int slot, double* const* fields, int nfields);
int  oracle_set_diag(oracle_ctx* o, const double* const* fields, int nfields);
int  oracle_get_diag(oracle_ctx* o, double* const* fields, int nfields);
/* one step, exactly mo_manage_pchevi.F90:27-118; a non-periodic run with boundary data set
 * up ends with oracle_update_boundaries(o, new_slot, (total_step_counter+1)*dtime) */
int  oracle_pchevi(oracle_ctx* o, int old_slot, int new_slot, int total_step_counter);
/* lateral boundary relaxation, mo_boundaries.F90 (same contract as lgame_gpu_bc_setup,
 * lgame_gpu_set_bc, lgame_gpu_update_boundaries and lgame_gpu_bc_state) */
int  oracle_bc_setup(oracle_ctx* o, int n_swamp, int dtime_bc, double t_latest_bc, lgame_bc_loader loader,
                     void* user);
int  oracle_set_bc(oracle_ctx* o, int time_index, const double* rho, const double* rhotheta_v,
                   const double* wind_u, const double* wind_v, const double* wind_w);
int  oracle_update_boundaries(oracle_ctx* o, int slot, double t_now);
int  oracle_bc_state(oracle_ctx* o, int* index_old, int* index_new, double* t_latest_bc);
/* the output fields of write_output for coeff_1*state[slot_1] + coeff_2*state[slot_2]
 * (same contract as lgame_gpu_output) */
int  oracle_output(oracle_ctx* o, int slot_1, int slot_2, double coeff_1, double coeff_2, float* const* fields,
                   int nfields, int* crashed);
/* the rescale factors of setup_bc_factor (mo_boundaries.F90:125-170) after oracle_bc_setup:
 * scalar (ny x nx), u (ny x (nx+1)), v ((ny+1) x nx), column-major */
int  oracle_bc_factors(oracle_ctx* o, double* scalar_f, double* u_f, double* v_f);
int  oracle_budgets(oracle_ctx* o, int slot, double* out, int nout);
/* number of OpenMP threads the oracle runs with */
int  oracle_num_threads(void);
/* the Thomas algorithm of mo_column_solvers.F90:606-640, for unit tests */
void oracle_thomas(const double* c, const double* d, const double* e, const double* r,
                   double* solution, int n);

#ifdef __cplusplus
}
#endif
#endif
