/*
 * lgame_host.h -- host side of the drop-in driver: namelist, grid and initial state.
 *
 * In the reference these steps run in Fortran before the time loop
 * (src/control.F90:64-91 namelists, :453 grid_setup, :466 bg_setup, :476 ideal_init).
 * A Fortran host keeps doing them itself and only binds lgame_gpu.h.  This header
 * is for hosts without a Fortran compiler (the C++ driver lgame_gpu_run, the Python
 * bindings): it produces the same grid, background state and idealised initial
 * state, in the reference's array layout, ready for lgame_gpu_set_grid/set_state.
 */
#ifndef LGAME_HOST_H
#define LGAME_HOST_H

#include <stddef.h>
#include "lgame_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Every variable of the seven namelist groups of the reference with its default
 * (mo_run_nml.F90:55-80, mo_io_nml.F90:251-257, mo_constituents_nml.F90:236-238,
 * mo_diff_nml.F90:39-53, mo_surface_nml.F90:148-154, mo_bc_nml.F90:293-298,
 * mo_rad_nml.F90:206-211), the derived quantities the reference computes after
 * reading them, and one extension group &gpu whose defaults leave the reference
 * behaviour unchanged. */
typedef struct lgame_namelist {
  /* &run */
  int    ny, nx, n_layers, n_oro_layers;
  double dy, dx;
  int    run_span_min;
  double stretching_parameter;
  int    theta_adv_order;
  double toa;
  char   scenario[64];
  int    llinear;
  char   run_id[64];
  int    lcorio;
  double lat_center, lon_center;
  int    start_year, start_month, start_day, start_hour, start_minute;
  int    lplane, luse_bg_state;
  /* &io */
  int    dt_write_min, lread_geo, lwrite_grid;
  char   grid_filename[64], restart_filename[64];
  int    lwrite_integrals;
  /* &constituents */
  int    lmoist;
  /* &diff */
  int    lmom_diff_h, lmom_diff_v, ltemp_diff_h, ltemp_diff_v, lmass_diff_h, lmass_diff_v;
  double h_prandtl, karman;
  int    lklemp;
  double klemp_damp_max, klemp_begin_rel;
  char   diff_coeff_scheme_h[16], diff_coeff_scheme_v[16];
  double bg_shear, c_s;
  /* &surface */
  int    orography_id, lprog_soil_temp, nsoillays, lsfc_sensible_heat_flux, lsfc_phase_trans, lpbl, lsleve;
  /* &bc */
  int    n_swamp, lperiodic, lfreeslip, dtime_bc;
  char   bc_root_filename[64];
  /* &rad */
  int    lrad;
  double dtime_rad;
  char   rrtmgp_coefficients_file_sw[128], rrtmgp_coefficients_file_lw[128];
  char   cloud_coefficients_file_sw[128], cloud_coefficients_file_lw[128];
  /* &gpu (extension; no reference counterpart) */
  int    precision;          /* 0 fp64, 1 split                                        */
  double dtime_override;     /* > 0: use this time step instead of 1.61*sqrt(dx*dy)/1000 */
  int    strict_reference;   /* 1: keep the reference's odd-nx/ny check                */
  long long seed;            /* seed of the random orography and the moist jet state   */
  int    n_hills;            /* orography_id=5: number of Gaussian hills               */
  double hill_height_min, hill_height_max, hill_width_min, hill_width_max;
  double jet_speed, jet_pressure;  /* scenario "baroclinic_jet" */
  double t_pert_sigma, rh_mean;
  int    check_finite;
  int    lphase_trans;       /* 1: the phase transitions the reference never calls (lgame_config) */
  /* derived (mo_run_nml.F90:89-101, mo_constituents_nml.F90:246-253, mo_io_nml.F90:266) */
  int    n_levels, n_flat_layers, n_condensed_constituents, n_constituents;
  double eff_hor_res, dtime, dt_write, t_init;
} lgame_namelist;

/* Fills every field with the reference default. */
void lgame_namelist_defaults(lgame_namelist* nml);
/* Reads the Fortran namelist groups from text (the file namelist.nml of the reference,
 * e.g. run_scripts/schaer.sh:12-65) over the current contents of nml, then derives
 * n_levels, dtime, ... and runs the reference's sanity checks (mo_run_nml.F90:103-141,
 * mo_diff_nml.F90:91-98, mo_surface_nml.F90:163-166, control.F90:94-97).  Returns 0 or
 * LGAME_ERR_BAD_CONFIG / LGAME_ERR_BAD_DIMS with lgame_gpu_last_error() set; never exits. */
int  lgame_namelist_parse(const char* text, lgame_namelist* nml);
/* Reads a namelist file (defaults first, then the file). */
int  lgame_namelist_read_file(const char* path, lgame_namelist* nml);
/* Translates a namelist into the run configuration of lgame_gpu_create. */
int  lgame_config_from_namelist(const lgame_namelist* nml, lgame_config* cfg);

/* Host model: grid, background and initial state in the reference's layout. */
typedef struct lgame_host_model lgame_host_model;
/* grid_setup + bg_setup + ideal_init (mo_grid_generator.F90:29-1457,
 * mo_set_initial_state.F90:22-382).  Orography ids 0, 2, 3, 4 as in the reference;
 * 5 = sum of n_hills seeded Gaussian hills.  Scenarios standard, seabreeze, advection,
 * schaer, mountain_rest as in the reference; baroclinic_jet = seeded moist jet. */
int  lgame_host_setup(const lgame_namelist* nml, lgame_host_model** out);
void lgame_host_destroy(lgame_host_model* m);
/* Pointers into the model's arrays (owned by the model); *n receives the element count. */
double* lgame_host_grid_field(lgame_host_model* m, int field, size_t* n);
double* lgame_host_state_field(lgame_host_model* m, int field, size_t* n);
double* lgame_host_diag_field(lgame_host_model* m, int field, size_t* n);
/* 2-D surface fields: 0 oro, 1 sfc_albedo, 2 lat_geo_scalar, 3 lon_geo_scalar */
double* lgame_host_surface_field(lgame_host_model* m, int field, size_t* n);

/* ---- raw binary files where the reference uses netCDF (absent here) ------------------------
 * A 64-byte little-endian header (magic "LGAMESNP" or "LGAMEBCL", int32 version 4, int32 ny,
 * nx, n_layers, n_constituents, then the int64 step counter or the FP64 valid time, then int32
 * nsoillays (0 in a boundary level)) followed by
 * FP64 arrays in the reference layout (column-major, reference extents).  Readers check the
 * magic, the version, the dimensions and the length, and fail with LGAME_ERR_BAD_DIMS or
 * LGAME_ERR_INVALID_ARG. */

/* Restart snapshot: the LGAME_STATE_NFIELDS fields of state slot 0 and of slot 1 (enum
 * lgame_state_field order, as lgame_gpu_get_state returns them; the soil temperature has
 * nsoillays layers and may be NULL when nsoillays is 0), the LGAME_DIAG_NFIELDS carried diagnostics (as
 * lgame_gpu_get_diag returns them) and the step counter: a run resumed from it with
 * lgame_gpu_set_state, lgame_gpu_set_diag and the next step number continues bit for bit.
 * Replaces restart() (mo_set_initial_state.F90:259-320), which reads one state's rho,
 * rhotheta_v and winds from netCDF and is unreachable in the reference (no lrestart in the
 * namelist). */
int  lgame_host_write_snapshot(const char* path, int ny, int nx, int n_layers, int n_constituents, int nsoillays,
                               long long step, const double* const* slot0, const double* const* slot1,
                               const double* const* diag);
int  lgame_host_read_snapshot(const char* path, int ny, int nx, int n_layers, int n_constituents, int nsoillays,
                              long long* step, double* const* slot0, double* const* slot1, double* const* diag);

/* Lateral boundary level: the t_bc arrays of one time index (rho, rhotheta_v, wind_u, wind_v,
 * wind_w, extents as lgame_gpu_set_bc takes them) and their valid time (s); what
 * read_boundaries (mo_boundaries.F90:99-123) reads from netCDF. */
int  lgame_host_write_bc_level(const char* path, int ny, int nx, int n_layers, int n_constituents, double t_valid,
                               const double* rho, const double* rhotheta_v, const double* wind_u,
                               const double* wind_v, const double* wind_w);
int  lgame_host_read_bc_level(const char* path, int ny, int nx, int n_layers, int n_constituents, double* t_valid,
                              double* rho, double* rhotheta_v, double* wind_u, double* wind_v, double* wind_w);
/* read_boundaries' file name (mo_boundaries.F90:112-113) with a .bin suffix:
 * "<root>+<int(t_update - t_init)>s.bin" (seconds truncated toward zero) into out[n]. */
int  lgame_host_bc_filename(const char* root, double t_update, double t_init, char* out, int n);

/* A ready-made lgame_bc_loader for lgame_gpu_bc_setup: user points to an lgame_bc_files; a new
 * level comes from the file lgame_host_bc_filename(root, t_update, t_init) and goes to the
 * context with lgame_gpu_set_bc. */
typedef struct lgame_bc_files {
  lgame_gpu*  ctx;
  const char* root;
  double      t_init;
  int         ny, nx, n_layers, n_constituents;
} lgame_bc_files;
int  lgame_bc_file_loader(void* user, double t_update, int time_index);

#ifdef __cplusplus
}
#endif
#endif
