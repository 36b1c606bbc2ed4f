/*
 * lgame_oracle.c -- CPU FP64 restatement of L-GAME's HEVI time step (TEST INFRASTRUCTURE).
 *
 * Only tests/, the smoke check and bench.py's CPU-baseline leg load this file.  Each
 * function restates the Fortran routine cited in its comment: same loop nests, same
 * left-to-right evaluation order of every expression (Fortran evaluates a*b/c*d as
 * ((a*b)/c)*d and -a*b as -(a*b)), same boundary branches, and the same "keep the
 * previous value" behaviour of arrays that an operator does not write (all arrays
 * start at zero as in src/control.F90:274-444).  Integer powers x**2, x**3, x**4 are
 * written as x*x, (x*x)*x, (x*x)*(x*x), the multiplication chains gfortran emits.
 * Compile with -O2 -ffp-contract=off so that no multiply-add is fused.
 *
 * Array layout: Fortran column-major with the reference's extents, 1-based index
 * macros so that the code reads like the Fortran.
 */
#include "lgame_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants, src/mo_constants.F90:12-37 ------------------------------- */
static const double r_e = 6371000.789927;
static const double k_b = 1.380649e-23;
static const double n_a = 6.02214076e23;
static const double t_0 = 273.15;
static const double rho_h2o = 1024.0;
static const double r_d = 287.057811;
static const double c_d_v = 717.942189;
static const double c_v_v = 1396.475121;
static const double c_d_p = 1005.0;
#define M_D (6.02214076e23 * 0.004810e-23)  /* n_a*0.004810e-23_wp */
#define M_V (6.02214076e23 * 0.002991e-23)  /* n_a*0.002991e-23_wp */
#define IMPL_THERMO_WEIGHT (717.942189 / 1005.0)
static const double M_PI_ = 3.14159265358979323846;  /* 4._wp*atan(1._wp) */
static const double p_0 = 100000.0;
static const double r_v = 461.524879;
#define GRAVITY 9.80616                               /* gravity, mo_constants.F90:21 */

struct oracle_ctx {
  int ny, nx, nl, n_levels, n_oro_layers, n_flat_layers;
  int nc;      /* n_condensed_constituents */
  int ncons;   /* n_constituents */
  int lmoist, lperiodic, lfreeslip, lcorio, llinear, luse_bg_state, lklemp, theta_adv_order;
  double dtime, toa, dx, dy, klemp_damp_max, klemp_begin_rel;
  int n_damping_levels;  /* levels whose highest z_w lies above klemp_begin_rel*toa */
  /* &diff (mo_diff_nml.F90:12-26) and the derived scalars of the diffusion closure:
   * eff_hor_res = sqrt(dx*dy) (mo_run_nml.F90:93), mean_velocity_area =
   * 2*sum(area_z(:,:,n_levels))/(ny*nx) (mo_grid_generator.F90:1111) */
  int lmom_diff_h, lmom_diff_v, ltemp_diff_h, ltemp_diff_v, lmass_diff_h, lmass_diff_v, diff_h_tke;
  double bg_shear, c_s, eff_hor_res, mean_velocity_area;
  /* &surface (mo_surface_nml.F90:12-20) and the surface-layer constants of &diff; the soil grid's
   * depth of the constant temperature (mo_grid_generator.F90:1363) */
  int lprog_soil_temp, lsfc_sensible_heat_flux, lsfc_phase_trans, lpbl, nsoil;
  int lphase_trans;  /* extension: calc_h2otracers_source_rates at the first substep */
  double h_prandtl, karman, z_t_const;
  /* grid */
  double *z_scalar, *z_u, *z_v, *z_w, *gdx, *gdy, *gdz, *volume, *area_x, *area_y, *area_z;
  double *area_dual_x, *area_dual_y, *area_dual_z, *z_area_dual_z, *slope_x, *slope_y, *ipw;
  double *theta_v_bg, *exner_bg, *exner_bg_grad_u, *exner_bg_grad_v, *exner_bg_grad_w;
  double *gravity_m_v, *gravity_potential, *fvec_x, *fvec_y, *fvec_z, *trsk_u, *trsk_v;
  /* two states */
  double *rho[2], *rhotheta_v[2], *theta_v_pert[2], *exner_pert[2], *wind_u[2], *wind_v[2], *wind_w[2];
  /* tendencies */
  double *t_rho, *t_rhotheta_v, *t_wind_u, *t_wind_v, *t_wind_w;
  /* diagnostics */
  double *v_squared, *pg_l_u, *pg_l_v, *pg_l_w, *pg_nl_u, *pg_nl_v, *pg_nl_w, *p_grad_condensates_w;
  double *pg_old_u, *pg_old_v, *vsg_x, *vsg_y, *vsg_z, *pvt_x, *pvt_y, *pvt_z;
  double *scalar_placeholder, *temperature, *u_placeholder, *v_placeholder, *w_placeholder;
  double *theta_v_u, *theta_v_v, *zeta_x, *zeta_y, *zeta_z, *eta_x, *eta_y, *eta_z;
  double *radiation_tendency, *flux_density_u, *flux_density_v, *flux_density_div;
  double *p_grad_decel_factor, *mom_diff_tend_x, *mom_diff_tend_y, *mom_diff_tend_z;
  double *heating_diss, *phase_trans_rates, *phase_trans_heating_rate, *temp_diff_heating;
  /* diffusion closure: the grid's dual distances and layer thicknesses; its diagnostics */
  double *dx_dual, *dy_dual, *layer_thickness;
  double *tke, *viscosity, *viscosity_molecular, *viscosity_dual, *n_squared, *du_dz, *dv_dz;
  double *vert_hor_viscosity_u, *vert_hor_viscosity_v, *mass_diff_coeff_eff_h, *mass_diff_coeff_eff_v;
  double *temp_diff_coeff_eff_h, *temp_diff_coeff_eff_v, *flux_density_w;
  double *condensates_sediment_heat, *mass_diff_tendency;
  /* the surface and the soil: grid (roughness_length_grid is grid%roughness_length), the soil
   * temperature of the two states, the surface diagnostics (roughness_length is
   * diag%roughness_length) */
  double *land_fraction, *lake_fraction, *roughness_length_grid, *sfc_rho_c, *t_conduc_soil, *t_const_soil;
  double *z_soil_interface, *z_soil_center, *temperature_soil[2];
  double *roughness_length, *roughness_velocity, *monin_obukhov_length, *scalar_flux_resistance;
  double *sens_soil, *sens_sea, *sst, *sfc_sw_in, *sfc_lw_out, *lat_lake, *lat_sea;
  double *a_rain;
  /* lateral boundary conditions (t_bc, mo_definitions.F90:117-131): two time levels, the
   * rescale factors, the level indices (1-based) and the time of the older level */
  int bc_on, bc_index_old, bc_index_new, dtime_bc;
  double t_latest_bc;
  double *bc_rho[2], *bc_rhotheta_v[2], *bc_wind_u[2], *bc_wind_v[2], *bc_wind_w[2];
  double *scalar_bc_factor, *u_bc_factor, *v_bc_factor;
  lgame_bc_loader bc_loader;
  void* bc_user;
};

/* extents */
#define DIMS const int ny = o->ny, nx = o->nx, nl = o->nl; (void)ny; (void)nx; (void)nl
#define IS(i,j,k) ((size_t)((i)-1) + (size_t)ny*((size_t)((j)-1) + (size_t)nx*(size_t)((k)-1)))
#define IU(i,j,k) ((size_t)((i)-1) + (size_t)ny*((size_t)((j)-1) + (size_t)(nx+1)*(size_t)((k)-1)))
#define IV(i,j,k) ((size_t)((i)-1) + (size_t)(ny+1)*((size_t)((j)-1) + (size_t)nx*(size_t)((k)-1)))
#define IZ(i,j,k) ((size_t)((i)-1) + (size_t)(ny+1)*((size_t)((j)-1) + (size_t)(nx+1)*(size_t)((k)-1)))
#define IRHO(i,j,k,c) (IS(i,j,k) + (size_t)ny*(size_t)nx*(size_t)nl*(size_t)((c)-1))
#define IPW(n,i,j,k) ((size_t)((n)-1) + 6*IS(i,j,k))
#define W(n,i,j,k) (o->ipw[IPW(n,i,j,k)])
#define TRSKU(n,i) (o->trsk_u[(size_t)((n)-1) + 3*(size_t)((i)-1)])
#define TRSKV(n,i) (o->trsk_v[(size_t)((n)-1) + 2*(size_t)((i)-1)])

/* ---- allocation ---------------------------------------------------------- */
static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int oracle_create(const lgame_config* cfg, oracle_ctx** out) {
  if (!cfg || !out) return LGAME_ERR_INVALID_ARG;
  if (cfg->ny < 3 || cfg->nx < 3 || cfg->n_layers < 3 || cfg->n_oro_layers < 1 ||
      cfg->n_oro_layers >= cfg->n_layers || cfg->n_layers > 250) return LGAME_ERR_BAD_DIMS;
  if (cfg->theta_adv_order != 2 && cfg->theta_adv_order != 3) return LGAME_ERR_BAD_CONFIG;
  if (cfg->lphase_trans && !cfg->lmoist) return LGAME_ERR_BAD_CONFIG;
  oracle_ctx* o = (oracle_ctx*)calloc(1, sizeof(oracle_ctx));
  if (!o) return LGAME_ERR_ALLOC;
  o->ny = cfg->ny; o->nx = cfg->nx; o->nl = cfg->n_layers; o->n_levels = cfg->n_layers + 1;
  o->n_oro_layers = cfg->n_oro_layers; o->n_flat_layers = cfg->n_layers - cfg->n_oro_layers;
  o->lmoist = cfg->lmoist; o->nc = cfg->lmoist ? 5 : 0; o->ncons = o->nc + (cfg->lmoist ? 2 : 1);
  o->lperiodic = cfg->lperiodic; o->lfreeslip = cfg->lfreeslip; o->lcorio = cfg->lcorio;
  o->llinear = cfg->llinear; o->luse_bg_state = cfg->luse_bg_state; o->lklemp = cfg->lklemp;
  o->theta_adv_order = cfg->theta_adv_order; o->dtime = cfg->dtime; o->toa = cfg->toa;
  o->dx = cfg->dx; o->dy = cfg->dy; o->klemp_damp_max = cfg->klemp_damp_max;
  o->klemp_begin_rel = cfg->klemp_begin_rel;
  o->lmom_diff_h = cfg->lmom_diff_h; o->lmom_diff_v = cfg->lmom_diff_v; o->ltemp_diff_h = cfg->ltemp_diff_h;
  o->ltemp_diff_v = cfg->ltemp_diff_v; o->lmass_diff_h = cfg->lmass_diff_h; o->lmass_diff_v = cfg->lmass_diff_v;
  o->diff_h_tke = cfg->diff_coeff_scheme_h == LGAME_DIFF_COEFF_TKE;
  o->bg_shear = cfg->bg_shear; o->c_s = cfg->c_s; o->eff_hor_res = sqrt(cfg->dx*cfg->dy);
  o->lprog_soil_temp = cfg->lprog_soil_temp; o->lsfc_sensible_heat_flux = cfg->lsfc_sensible_heat_flux;
  o->lsfc_phase_trans = cfg->lsfc_phase_trans; o->lpbl = cfg->lpbl;
  o->nsoil = cfg->nsoillays > 0 ? cfg->nsoillays : 0;
  o->h_prandtl = cfg->h_prandtl; o->karman = cfg->karman; o->lphase_trans = cfg->lphase_trans;
  if (o->nsoil > LGAME_MAX_SOIL_LAYERS) { free(o); return LGAME_ERR_BAD_CONFIG; }
  DIMS;
  const size_t nS = (size_t)ny*nx*nl, nU = (size_t)ny*(nx+1)*nl, nV = (size_t)(ny+1)*nx*nl;
  const size_t nW = (size_t)ny*nx*(nl+1), nZ = (size_t)(ny+1)*(nx+1)*nl;
  const size_t nEX = (size_t)(ny+1)*nx*(nl+1), nEY = (size_t)ny*(nx+1)*(nl+1);
  o->z_scalar = zalloc(nS); o->z_u = zalloc(nU); o->z_v = zalloc(nV); o->z_w = zalloc(nW);
  o->gdx = zalloc(nU); o->gdy = zalloc(nV); o->gdz = zalloc(nW); o->volume = zalloc(nS);
  o->area_x = zalloc(nU); o->area_y = zalloc(nV); o->area_z = zalloc(nW);
  o->area_dual_x = zalloc(nEX); o->area_dual_y = zalloc(nEY); o->area_dual_z = zalloc(nZ);
  o->z_area_dual_z = zalloc(nZ); o->slope_x = zalloc(nU); o->slope_y = zalloc(nV);
  o->ipw = zalloc(6*nS); o->theta_v_bg = zalloc(nS); o->exner_bg = zalloc(nS);
  o->exner_bg_grad_u = zalloc(nU); o->exner_bg_grad_v = zalloc(nV); o->exner_bg_grad_w = zalloc(nW);
  o->gravity_m_v = zalloc(nW); o->gravity_potential = zalloc(nS);
  o->fvec_x = zalloc((size_t)(ny+1)*nx); o->fvec_y = zalloc((size_t)ny*(nx+1));
  o->fvec_z = zalloc((size_t)(ny+1)*(nx+1)); o->trsk_u = zalloc(3*(size_t)ny); o->trsk_v = zalloc(2*(size_t)(ny+1));
  for (int s = 0; s < 2; ++s) {
    o->rho[s] = zalloc(nS*o->ncons); o->rhotheta_v[s] = zalloc(nS); o->theta_v_pert[s] = zalloc(nS);
    o->exner_pert[s] = zalloc(nS); o->wind_u[s] = zalloc(nU); o->wind_v[s] = zalloc(nV); o->wind_w[s] = zalloc(nW);
  }
  o->t_rho = zalloc(nS*o->ncons); o->t_rhotheta_v = zalloc(nS); o->t_wind_u = zalloc(nU);
  o->t_wind_v = zalloc(nV); o->t_wind_w = zalloc(nW);
  o->v_squared = zalloc(nS); o->pg_l_u = zalloc(nU); o->pg_l_v = zalloc(nV); o->pg_l_w = zalloc(nW);
  o->pg_nl_u = zalloc(nU); o->pg_nl_v = zalloc(nV); o->pg_nl_w = zalloc(nW);
  o->p_grad_condensates_w = zalloc(nW); o->pg_old_u = zalloc(nU); o->pg_old_v = zalloc(nV);
  o->vsg_x = zalloc(nU); o->vsg_y = zalloc(nV); o->vsg_z = zalloc(nW);
  o->pvt_x = zalloc(nU); o->pvt_y = zalloc(nV); o->pvt_z = zalloc(nW);
  o->scalar_placeholder = zalloc(nS); o->temperature = zalloc(nS);
  o->u_placeholder = zalloc(nU); o->v_placeholder = zalloc(nV); o->w_placeholder = zalloc(nW);
  o->theta_v_u = zalloc(nU); o->theta_v_v = zalloc(nV);
  o->zeta_x = zalloc(nEX); o->zeta_y = zalloc(nEY); o->zeta_z = zalloc(nZ);
  o->eta_x = zalloc(nEX); o->eta_y = zalloc(nEY); o->eta_z = zalloc(nZ);
  o->radiation_tendency = zalloc(nS); o->flux_density_u = zalloc(nU); o->flux_density_v = zalloc(nV);
  o->flux_density_div = zalloc(nS); o->p_grad_decel_factor = zalloc(nS);
  o->mom_diff_tend_x = zalloc(nU); o->mom_diff_tend_y = zalloc(nV); o->mom_diff_tend_z = zalloc(nW);
  o->heating_diss = zalloc(nS); o->phase_trans_rates = zalloc(nS*(o->nc+1));
  o->phase_trans_heating_rate = zalloc(nS); o->temp_diff_heating = zalloc(nS);
  o->condensates_sediment_heat = zalloc(nS); o->mass_diff_tendency = zalloc(nS*o->ncons);
  o->dx_dual = zalloc(nV); o->dy_dual = zalloc(nU); o->layer_thickness = zalloc(nS);
  o->tke = zalloc(nS); o->viscosity = zalloc(nS); o->viscosity_molecular = zalloc(nS);
  o->viscosity_dual = zalloc(nZ); o->n_squared = zalloc(nS);
  o->du_dz = zalloc((size_t)ny*(nx+1)*(nl+1)); o->dv_dz = zalloc((size_t)(ny+1)*nx*(nl+1));
  o->vert_hor_viscosity_u = zalloc((size_t)ny*(nx+1)*(nl+1)); o->vert_hor_viscosity_v = zalloc((size_t)(ny+1)*nx*(nl+1));
  o->mass_diff_coeff_eff_h = zalloc(nS); o->mass_diff_coeff_eff_v = zalloc(nS);
  o->temp_diff_coeff_eff_h = zalloc(nS); o->temp_diff_coeff_eff_v = zalloc(nS); o->flux_density_w = zalloc(nW);
  {
    const size_t n2 = (size_t)ny*nx;
    o->land_fraction = zalloc(n2); o->lake_fraction = zalloc(n2); o->roughness_length_grid = zalloc(n2);
    o->sfc_rho_c = zalloc(n2); o->t_conduc_soil = zalloc(n2); o->t_const_soil = zalloc(n2);
    o->z_soil_interface = zalloc((size_t)o->nsoil + 1); o->z_soil_center = zalloc((size_t)o->nsoil);
    o->temperature_soil[0] = zalloc(n2*(size_t)o->nsoil); o->temperature_soil[1] = zalloc(n2*(size_t)o->nsoil);
    o->roughness_length = zalloc(n2); o->roughness_velocity = zalloc(n2); o->monin_obukhov_length = zalloc(n2);
    o->scalar_flux_resistance = zalloc(n2); o->sens_soil = zalloc(n2); o->sens_sea = zalloc(n2);
    o->sst = zalloc(n2); o->sfc_sw_in = zalloc(n2); o->sfc_lw_out = zalloc(n2);
    o->lat_lake = zalloc(n2); o->lat_sea = zalloc(n2);
  }
  o->a_rain = zalloc(nS);
  for (double** q = &o->z_scalar; q <= &o->a_rain; ++q)
    if (!*q) { oracle_destroy(o); return LGAME_ERR_ALLOC; }
  *out = o;
  return LGAME_OK;
}

void oracle_destroy(oracle_ctx* o) {
  if (!o) return;
  double** p = &o->z_scalar;
  double** end = &o->a_rain;
  for (; p <= end; ++p) free(*p);
  for (int i = 0; i < 2; ++i) {
    free(o->bc_rho[i]); free(o->bc_rhotheta_v[i]); free(o->bc_wind_u[i]); free(o->bc_wind_v[i]);
    free(o->bc_wind_w[i]);
  }
  free(o->scalar_bc_factor); free(o->u_bc_factor); free(o->v_bc_factor);
  free(o);
}

/* sizes of the interface arrays, in the order of the lgame_gpu.h enums */
static size_t grid_size(const oracle_ctx* o, int f) {
  DIMS;
  const size_t nS = (size_t)ny*nx*nl, nU = (size_t)ny*(nx+1)*nl, nV = (size_t)(ny+1)*nx*nl;
  const size_t nW = (size_t)ny*nx*(nl+1), nZ = (size_t)(ny+1)*(nx+1)*nl;
  switch (f) {
    case LGAME_GRID_Z_SCALAR: case LGAME_GRID_VOLUME: case LGAME_GRID_THETA_V_BG:
    case LGAME_GRID_EXNER_BG: case LGAME_GRID_GRAVITY_POTENTIAL: return nS;
    case LGAME_GRID_Z_U: case LGAME_GRID_DX: case LGAME_GRID_AREA_X: case LGAME_GRID_SLOPE_X:
    case LGAME_GRID_EXNER_BG_GRAD_U: return nU;
    case LGAME_GRID_Z_V: case LGAME_GRID_DY: case LGAME_GRID_AREA_Y: case LGAME_GRID_SLOPE_Y:
    case LGAME_GRID_EXNER_BG_GRAD_V: return nV;
    case LGAME_GRID_Z_W: case LGAME_GRID_DZ: case LGAME_GRID_AREA_Z: case LGAME_GRID_EXNER_BG_GRAD_W:
    case LGAME_GRID_GRAVITY_M_V: return nW;
    case LGAME_GRID_AREA_DUAL_X: return (size_t)(ny+1)*nx*(nl+1);
    case LGAME_GRID_AREA_DUAL_Y: return (size_t)ny*(nx+1)*(nl+1);
    case LGAME_GRID_AREA_DUAL_Z: case LGAME_GRID_Z_AREA_DUAL_Z: return nZ;
    case LGAME_GRID_INNER_PRODUCT_WEIGHTS: return 6*nS;
    case LGAME_GRID_FVEC_X: return (size_t)(ny+1)*nx;
    case LGAME_GRID_FVEC_Y: return (size_t)ny*(nx+1);
    case LGAME_GRID_FVEC_Z: return (size_t)(ny+1)*(nx+1);
    case LGAME_GRID_TRSK_WEIGHTS_U: return 3*(size_t)ny;
    case LGAME_GRID_TRSK_WEIGHTS_V: return 2*(size_t)(ny+1);
    case LGAME_GRID_DX_DUAL: return nV;
    case LGAME_GRID_DY_DUAL: return nU;
    case LGAME_GRID_LAYER_THICKNESS: return nS;
    case LGAME_GRID_LAND_FRACTION: case LGAME_GRID_LAKE_FRACTION: case LGAME_GRID_ROUGHNESS_LENGTH:
    case LGAME_GRID_SFC_RHO_C: case LGAME_GRID_T_CONDUC_SOIL: case LGAME_GRID_T_CONST_SOIL: return (size_t)ny*nx;
    case LGAME_GRID_Z_SOIL_INTERFACE: return (size_t)o->nsoil + 1;
    case LGAME_GRID_Z_SOIL_CENTER: return (size_t)o->nsoil;
    case LGAME_GRID_Z_T_CONST: return 1;
  }
  return 0;
}

int oracle_set_grid(oracle_ctx* o, const double* const* f, int nfields) {
  if (!o || !f || nfields != LGAME_GRID_NFIELDS) return LGAME_ERR_INVALID_ARG;
  double* dst[LGAME_GRID_NFIELDS] = {
    o->z_scalar, o->z_u, o->z_v, o->z_w, o->gdx, o->gdy, o->gdz, o->volume, o->area_x, o->area_y,
    o->area_z, o->area_dual_x, o->area_dual_y, o->area_dual_z, o->z_area_dual_z, o->slope_x,
    o->slope_y, o->ipw, o->theta_v_bg, o->exner_bg, o->exner_bg_grad_u, o->exner_bg_grad_v,
    o->exner_bg_grad_w, o->gravity_m_v, o->gravity_potential, o->fvec_x, o->fvec_y, o->fvec_z,
    o->trsk_u, o->trsk_v, o->dx_dual, o->dy_dual, o->layer_thickness, o->land_fraction, o->lake_fraction,
    o->roughness_length_grid, o->sfc_rho_c, o->t_conduc_soil, o->t_const_soil, o->z_soil_interface,
    o->z_soil_center, &o->z_t_const};
  const int sfc_on = o->lprog_soil_temp || o->lsfc_sensible_heat_flux || o->lsfc_phase_trans || o->lpbl;
  for (int i = 0; i < LGAME_GRID_NFIELDS; ++i) {
    if (!f[i]) {
      if (i >= LGAME_GRID_LAND_FRACTION && !sfc_on) continue;  /* surface fields, surface off */
      return LGAME_ERR_INVALID_ARG;
    }
    memcpy(dst[i], f[i], grid_size(o, i)*sizeof(double));
  }
  /* diag%roughness_length = grid%roughness_length, control.F90:458 */
  memcpy(o->roughness_length, o->roughness_length_grid, (size_t)o->ny*o->nx*sizeof(double));
  /* mean_velocity_area, mo_grid_generator.F90:1111: the surface areas summed in array order */
  {
    const size_t n2 = (size_t)o->ny*o->nx, base = n2*(size_t)o->nl;
    double sum = 0.0;
    for (size_t c = 0; c < n2; ++c) sum = sum + o->area_z[base + c];
    o->mean_velocity_area = 2.0*sum/(double)n2;
  }
  /* n_damping_levels, mo_grid_generator.F90:1049-1058 */
  o->n_damping_levels = 0;
  for (int jl = 1; jl <= o->n_levels; ++jl) {
    double max_z = -1e300;
    for (size_t c = 0; c < (size_t)o->ny*o->nx; ++c) {
      const double z = o->z_w[c + (size_t)o->ny*o->nx*(jl - 1)];
      if (z > max_z) max_z = z;
    }
    if (max_z > o->klemp_begin_rel*o->toa) o->n_damping_levels = o->n_damping_levels + 1;
  }
  return LGAME_OK;
}

int oracle_scalar_diffusion(const oracle_ctx* o, double* mass_diff_tendency, double* temp_diff_heating) {
  if (!o || !mass_diff_tendency || !temp_diff_heating) return LGAME_ERR_INVALID_ARG;
  const size_t nS = (size_t)o->ny*o->nx*o->nl;
  memcpy(mass_diff_tendency, o->mass_diff_tendency, nS*(size_t)o->ncons*sizeof(double));
  memcpy(temp_diff_heating, o->temp_diff_heating, nS*sizeof(double));
  return LGAME_OK;
}

int oracle_heating_diss(const oracle_ctx* o, double* out) {
  if (!o || !out) return LGAME_ERR_INVALID_ARG;
  memcpy(out, o->heating_diss, (size_t)o->ny*o->nx*o->nl*sizeof(double));
  return LGAME_OK;
}

static void state_ptrs(oracle_ctx* o, int s, double** p, size_t* n) {
  DIMS;
  const size_t nS = (size_t)ny*nx*nl;
  p[0] = o->rho[s]; n[0] = nS*o->ncons;
  p[1] = o->rhotheta_v[s]; n[1] = nS;
  p[2] = o->theta_v_pert[s]; n[2] = nS;
  p[3] = o->exner_pert[s]; n[3] = nS;
  p[4] = o->wind_u[s]; n[4] = (size_t)ny*(nx+1)*nl;
  p[5] = o->wind_v[s]; n[5] = (size_t)(ny+1)*nx*nl;
  p[6] = o->wind_w[s]; n[6] = (size_t)ny*nx*(nl+1);
  p[7] = o->temperature_soil[s]; n[7] = (size_t)ny*nx*(size_t)o->nsoil;
}

int oracle_set_state(oracle_ctx* o, int slot, const double* const* f, int nfields) {
  if (!o || !f || slot < 0 || slot > 1 || (nfields != LGAME_STATE_NFIELDS && nfields != LGAME_STATE_NFIELDS_ATMOS))
    return LGAME_ERR_INVALID_ARG;
  double* p[LGAME_STATE_NFIELDS]; size_t n[LGAME_STATE_NFIELDS];
  state_ptrs(o, slot, p, n);
  for (int i = 0; i < nfields; ++i) {
    if (!f[i]) {
      if (i == LGAME_STATE_TEMPERATURE_SOIL && n[i] == 0) continue;
      return LGAME_ERR_INVALID_ARG;
    }
    memcpy(p[i], f[i], n[i]*sizeof(double));
  }
  return LGAME_OK;
}

int oracle_get_state(oracle_ctx* o, int slot, double* const* f, int nfields) {
  if (!o || !f || slot < 0 || slot > 1 || (nfields != LGAME_STATE_NFIELDS && nfields != LGAME_STATE_NFIELDS_ATMOS))
    return LGAME_ERR_INVALID_ARG;
  double* p[LGAME_STATE_NFIELDS]; size_t n[LGAME_STATE_NFIELDS];
  state_ptrs(o, slot, p, n);
  for (int i = 0; i < nfields; ++i)
    if (f[i]) memcpy(f[i], p[i], n[i]*sizeof(double));
  return LGAME_OK;
}

static void diag_ptrs(oracle_ctx* o, double** p, size_t* n) {
  DIMS;
  const size_t nS = (size_t)ny*nx*nl, nU = (size_t)ny*(nx+1)*nl, nV = (size_t)(ny+1)*nx*nl;
  const size_t nW = (size_t)ny*nx*(nl+1);
  p[LGAME_DIAG_P_GRAD_ACC_NEG_NL_U] = o->pg_nl_u; n[LGAME_DIAG_P_GRAD_ACC_NEG_NL_U] = nU;
  p[LGAME_DIAG_P_GRAD_ACC_NEG_NL_V] = o->pg_nl_v; n[LGAME_DIAG_P_GRAD_ACC_NEG_NL_V] = nV;
  p[LGAME_DIAG_P_GRAD_ACC_NEG_NL_W] = o->pg_nl_w; n[LGAME_DIAG_P_GRAD_ACC_NEG_NL_W] = nW;
  p[LGAME_DIAG_P_GRAD_ACC_NEG_L_U] = o->pg_l_u; n[LGAME_DIAG_P_GRAD_ACC_NEG_L_U] = nU;
  p[LGAME_DIAG_P_GRAD_ACC_NEG_L_V] = o->pg_l_v; n[LGAME_DIAG_P_GRAD_ACC_NEG_L_V] = nV;
  p[LGAME_DIAG_P_GRAD_ACC_NEG_L_W] = o->pg_l_w; n[LGAME_DIAG_P_GRAD_ACC_NEG_L_W] = nW;
  p[LGAME_DIAG_P_GRAD_ACC_OLD_U] = o->pg_old_u; n[LGAME_DIAG_P_GRAD_ACC_OLD_U] = nU;
  p[LGAME_DIAG_P_GRAD_ACC_OLD_V] = o->pg_old_v; n[LGAME_DIAG_P_GRAD_ACC_OLD_V] = nV;
  p[LGAME_DIAG_POT_VORT_TEND_X] = o->pvt_x; n[LGAME_DIAG_POT_VORT_TEND_X] = nU;
  p[LGAME_DIAG_POT_VORT_TEND_Y] = o->pvt_y; n[LGAME_DIAG_POT_VORT_TEND_Y] = nV;
  p[LGAME_DIAG_POT_VORT_TEND_Z] = o->pvt_z; n[LGAME_DIAG_POT_VORT_TEND_Z] = nW;
  p[LGAME_DIAG_V_SQUARED_GRAD_X] = o->vsg_x; n[LGAME_DIAG_V_SQUARED_GRAD_X] = nU;
  p[LGAME_DIAG_V_SQUARED_GRAD_Y] = o->vsg_y; n[LGAME_DIAG_V_SQUARED_GRAD_Y] = nV;
  p[LGAME_DIAG_V_SQUARED_GRAD_Z] = o->vsg_z; n[LGAME_DIAG_V_SQUARED_GRAD_Z] = nW;
  p[LGAME_DIAG_CONDENSATES_SEDIMENT_HEAT] = o->condensates_sediment_heat; n[LGAME_DIAG_CONDENSATES_SEDIMENT_HEAT] = nS;
  p[LGAME_DIAG_RADIATION_TENDENCY] = o->radiation_tendency; n[LGAME_DIAG_RADIATION_TENDENCY] = nS;
  p[LGAME_DIAG_TEMPERATURE] = o->temperature; n[LGAME_DIAG_TEMPERATURE] = nS;
  p[LGAME_DIAG_TEND_RHO] = o->t_rho; n[LGAME_DIAG_TEND_RHO] = nS*o->ncons;
  p[LGAME_DIAG_TEND_RHOTHETA_V] = o->t_rhotheta_v; n[LGAME_DIAG_TEND_RHOTHETA_V] = nS;
  p[LGAME_DIAG_TEND_WIND_U] = o->t_wind_u; n[LGAME_DIAG_TEND_WIND_U] = nU;
  p[LGAME_DIAG_TEND_WIND_V] = o->t_wind_v; n[LGAME_DIAG_TEND_WIND_V] = nV;
  p[LGAME_DIAG_TEND_WIND_W] = o->t_wind_w; n[LGAME_DIAG_TEND_WIND_W] = nW;
  p[LGAME_DIAG_TKE] = o->tke; n[LGAME_DIAG_TKE] = nS;
  p[LGAME_DIAG_VISCOSITY] = o->viscosity; n[LGAME_DIAG_VISCOSITY] = nS;
  p[LGAME_DIAG_HEATING_DISS] = o->heating_diss; n[LGAME_DIAG_HEATING_DISS] = nS;
  p[LGAME_DIAG_MOM_DIFF_TEND_X] = o->mom_diff_tend_x; n[LGAME_DIAG_MOM_DIFF_TEND_X] = nU;
  p[LGAME_DIAG_MOM_DIFF_TEND_Y] = o->mom_diff_tend_y; n[LGAME_DIAG_MOM_DIFF_TEND_Y] = nV;
  p[LGAME_DIAG_MOM_DIFF_TEND_Z] = o->mom_diff_tend_z; n[LGAME_DIAG_MOM_DIFF_TEND_Z] = nW;
  const size_t n2 = (size_t)ny*nx;
  p[LGAME_DIAG_V_SQUARED] = o->v_squared; n[LGAME_DIAG_V_SQUARED] = nS;
  p[LGAME_DIAG_ROUGHNESS_LENGTH] = o->roughness_length; n[LGAME_DIAG_ROUGHNESS_LENGTH] = n2;
  p[LGAME_DIAG_ROUGHNESS_VELOCITY] = o->roughness_velocity; n[LGAME_DIAG_ROUGHNESS_VELOCITY] = n2;
  p[LGAME_DIAG_MONIN_OBUKHOV_LENGTH] = o->monin_obukhov_length; n[LGAME_DIAG_MONIN_OBUKHOV_LENGTH] = n2;
  p[LGAME_DIAG_SCALAR_FLUX_RESISTANCE] = o->scalar_flux_resistance; n[LGAME_DIAG_SCALAR_FLUX_RESISTANCE] = n2;
  p[LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SOIL] = o->sens_soil; n[LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SOIL] = n2;
  p[LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SEA] = o->sens_sea; n[LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SEA] = n2;
  p[LGAME_DIAG_SST] = o->sst; n[LGAME_DIAG_SST] = n2;
  p[LGAME_DIAG_SFC_SW_IN] = o->sfc_sw_in; n[LGAME_DIAG_SFC_SW_IN] = n2;
  p[LGAME_DIAG_SFC_LW_OUT] = o->sfc_lw_out; n[LGAME_DIAG_SFC_LW_OUT] = n2;
  p[LGAME_DIAG_PHASE_TRANS_RATES] = o->phase_trans_rates; n[LGAME_DIAG_PHASE_TRANS_RATES] = nS*(size_t)(o->nc+1);
  p[LGAME_DIAG_PHASE_TRANS_HEATING_RATE] = o->phase_trans_heating_rate; n[LGAME_DIAG_PHASE_TRANS_HEATING_RATE] = nS;
  p[LGAME_DIAG_POWER_FLUX_DENSITY_LAT_LAKE] = o->lat_lake; n[LGAME_DIAG_POWER_FLUX_DENSITY_LAT_LAKE] = n2;
  p[LGAME_DIAG_POWER_FLUX_DENSITY_LAT_SEA] = o->lat_sea; n[LGAME_DIAG_POWER_FLUX_DENSITY_LAT_SEA] = n2;
  p[LGAME_DIAG_TEMP_DIFF_HEATING] = o->temp_diff_heating; n[LGAME_DIAG_TEMP_DIFF_HEATING] = nS;
  p[LGAME_DIAG_MASS_DIFF_TENDENCY] = o->mass_diff_tendency;
  n[LGAME_DIAG_MASS_DIFF_TENDENCY] = nS*(size_t)o->ncons;
}

int oracle_set_diag(oracle_ctx* o, const double* const* f, int nfields) {
  if (!o || !f || nfields != LGAME_DIAG_NFIELDS) return LGAME_ERR_INVALID_ARG;
  double* p[LGAME_DIAG_NFIELDS]; size_t n[LGAME_DIAG_NFIELDS];
  diag_ptrs(o, p, n);
  for (int i = 0; i < LGAME_DIAG_NFIELDS; ++i)
    if (f[i]) memcpy(p[i], f[i], n[i]*sizeof(double));
  return LGAME_OK;
}

int oracle_get_diag(oracle_ctx* o, double* const* f, int nfields) {
  if (!o || !f || nfields != LGAME_DIAG_NFIELDS) return LGAME_ERR_INVALID_ARG;
  double* p[LGAME_DIAG_NFIELDS]; size_t n[LGAME_DIAG_NFIELDS];
  diag_ptrs(o, p, n);
  for (int i = 0; i < LGAME_DIAG_NFIELDS; ++i)
    if (f[i]) memcpy(f[i], p[i], n[i]*sizeof(double));
  return LGAME_OK;
}

/* ---- lateral boundary conditions, src/io/mo_boundaries.F90 ------------------------- */

/* setup_bc_factor, mo_boundaries.F90:125-170.  dist_from_boundary is real(wp) in the
 * Fortran: the integer minimum converts to double before the division by n_swamp. */
static void setup_bc_factor(oracle_ctx* o, int n_swamp) {
  DIMS;
  for (int ji = 1; ji <= ny; ++ji)
    for (int jk = 1; jk <= nx; ++jk) {
      int d = ji - 1; if (jk - 1 < d) d = jk - 1; if (ny - ji < d) d = ny - ji; if (nx - jk < d) d = nx - jk;
      double f = 1.0 - (double)d/n_swamp;
      if (f < 0.0) f = 0.0;
      const double sn = sin(0.5*M_PI_*f);
      o->scalar_bc_factor[(ji-1) + (size_t)ny*(jk-1)] = sn*sn;
    }
  for (int ji = 1; ji <= ny; ++ji)
    for (int jk = 1; jk <= nx+1; ++jk) {
      int d = ji - 1; if (jk - 1 < d) d = jk - 1; if (ny - ji < d) d = ny - ji; if (nx + 1 - jk < d) d = nx + 1 - jk;
      double f = 1.0 - (double)d/n_swamp;
      if (f < 0.0) f = 0.0;
      const double sn = sin(0.5*M_PI_*f);
      o->u_bc_factor[(ji-1) + (size_t)ny*(jk-1)] = sn*sn;
    }
  for (int ji = 1; ji <= ny+1; ++ji)
    for (int jk = 1; jk <= nx; ++jk) {
      int d = ji - 1; if (jk - 1 < d) d = jk - 1; if (ny + 1 - ji < d) d = ny + 1 - ji; if (nx - jk < d) d = nx - jk;
      double f = 1.0 - (double)d/n_swamp;
      if (f < 0.0) f = 0.0;
      const double sn = sin(0.5*M_PI_*f);
      o->v_bc_factor[(ji-1) + (size_t)(ny+1)*(jk-1)] = sn*sn;
    }
}

int oracle_bc_setup(oracle_ctx* o, int n_swamp, int dtime_bc, double t_latest_bc, lgame_bc_loader loader,
                    void* user) {
  if (!o || n_swamp < 1 || dtime_bc < 1) return LGAME_ERR_INVALID_ARG;
  if (o->lperiodic) return LGAME_ERR_STATE;
  DIMS;
  const size_t nS = (size_t)ny*nx*nl, nU = (size_t)ny*(nx+1)*nl, nV = (size_t)(ny+1)*nx*nl;
  const size_t nW = (size_t)ny*nx*(nl+1);
  if (!o->scalar_bc_factor) {
    for (int i = 0; i < 2; ++i) {
      o->bc_rho[i] = zalloc(nS*o->ncons); o->bc_rhotheta_v[i] = zalloc(nS); o->bc_wind_u[i] = zalloc(nU);
      o->bc_wind_v[i] = zalloc(nV); o->bc_wind_w[i] = zalloc(nW);
    }
    o->scalar_bc_factor = zalloc((size_t)ny*nx); o->u_bc_factor = zalloc((size_t)ny*(nx+1));
    o->v_bc_factor = zalloc((size_t)(ny+1)*nx);
  }
  setup_bc_factor(o, n_swamp);
  o->bc_index_old = 1;  /* control.F90:358-359 */
  o->bc_index_new = 2;
  o->dtime_bc = dtime_bc;
  o->t_latest_bc = t_latest_bc;
  o->bc_loader = loader;
  o->bc_user = user;
  o->bc_on = 1;
  return LGAME_OK;
}

int oracle_set_bc(oracle_ctx* o, int time_index, const double* rho, const double* rhotheta_v,
                  const double* wind_u, const double* wind_v, const double* wind_w) {
  if (!o || !o->bc_on || time_index < 1 || time_index > 2 || !rho || !rhotheta_v || !wind_u || !wind_v || !wind_w)
    return LGAME_ERR_INVALID_ARG;
  DIMS;
  const size_t nS = (size_t)ny*nx*nl, nU = (size_t)ny*(nx+1)*nl, nV = (size_t)(ny+1)*nx*nl;
  const size_t nW = (size_t)ny*nx*(nl+1);
  const int t = time_index - 1;
  memcpy(o->bc_rho[t], rho, nS*o->ncons*sizeof(double));
  memcpy(o->bc_rhotheta_v[t], rhotheta_v, nS*sizeof(double));
  memcpy(o->bc_wind_u[t], wind_u, nU*sizeof(double));
  memcpy(o->bc_wind_v[t], wind_v, nV*sizeof(double));
  memcpy(o->bc_wind_w[t], wind_w, nW*sizeof(double));
  return LGAME_OK;
}

/* update_boundaries, mo_boundaries.F90:19-97 */
int oracle_update_boundaries(oracle_ctx* o, int slot, double t_now) {
  if (!o || !o->bc_on || slot < 0 || slot > 1) return LGAME_ERR_INVALID_ARG;
  DIMS;
  const int nc = o->nc, ncons = o->ncons;
  const double old_weight = 1.0 - (t_now - o->t_latest_bc)/o->dtime_bc;
  if (old_weight < 0.0) {
    /* read_boundaries(bc, t_latest_bc+dtime_bc, bc%index_old), then the index swap */
    if (!o->bc_loader || o->bc_loader(o->bc_user, o->t_latest_bc + o->dtime_bc, o->bc_index_old) != 0)
      return LGAME_ERR_STATE;
    o->bc_index_old = o->bc_index_new;
    o->bc_index_new = 1;
    if (o->bc_index_old == 1) o->bc_index_new = 2;
    o->t_latest_bc = o->t_latest_bc + o->dtime_bc;
  }
  const double new_weight = 1.0 - old_weight;
  const int io = o->bc_index_old - 1, in = o->bc_index_new - 1;
  double* rho = o->rho[slot]; double* rt = o->rhotheta_v[slot];
  double* u = o->wind_u[slot]; double* v = o->wind_v[slot]; double* w = o->wind_w[slot];
  #pragma omp parallel for
  for (int ji = 1; ji <= ny; ++ji)
    for (int jk = 1; jk <= nx; ++jk) {
      const double f = o->scalar_bc_factor[(ji-1) + (size_t)ny*(jk-1)];
      for (int jl = 1; jl <= nl; ++jl) {
        for (int jc = 1; jc <= ncons; ++jc) {
          const size_t q = IRHO(ji,jk,jl,jc);
          rho[q] = f*(old_weight*o->bc_rho[io][q] + new_weight*o->bc_rho[in][q]) + (1.0 - f)*rho[q];
        }
        const size_t q = IS(ji,jk,jl);
        rt[q] = f*(old_weight*o->bc_rhotheta_v[io][q] + new_weight*o->bc_rhotheta_v[in][q]) + (1.0 - f)*rt[q];
      }
      for (int jl = 1; jl <= nl+1; ++jl) {
        const size_t q = IS(ji,jk,jl);
        w[q] = f*(old_weight*o->bc_wind_w[io][q] + new_weight*o->bc_wind_w[in][q]) + (1.0 - f)*w[q];
      }
    }
  #pragma omp parallel for
  for (int ji = 1; ji <= ny; ++ji)
    for (int jk = 1; jk <= nx+1; ++jk) {
      const double f = o->u_bc_factor[(ji-1) + (size_t)ny*(jk-1)];
      for (int jl = 1; jl <= nl; ++jl) {
        const size_t q = IU(ji,jk,jl);
        u[q] = f*(old_weight*o->bc_wind_u[io][q] + new_weight*o->bc_wind_u[in][q]) + (1.0 - f)*u[q];
      }
    }
  #pragma omp parallel for
  for (int ji = 1; ji <= ny+1; ++ji)
    for (int jk = 1; jk <= nx; ++jk) {
      const double f = o->v_bc_factor[(ji-1) + (size_t)(ny+1)*(jk-1)];
      for (int jl = 1; jl <= nl; ++jl) {
        const size_t q = IV(ji,jk,jl);
        v[q] = f*(old_weight*o->bc_wind_v[io][q] + new_weight*o->bc_wind_v[in][q]) + (1.0 - f)*v[q];
      }
    }
  /* theta_v_pert and exner_pert from the relaxed state, mo_boundaries.F90:92-95 */
  const size_t nS = (size_t)ny*nx*nl;
  const double* rho_g = rho + nS*(size_t)nc;
  double* tp = o->theta_v_pert[slot]; double* ep = o->exner_pert[slot];
  #pragma omp parallel for
  for (size_t i = 0; i < nS; ++i) {
    tp[i] = rt[i]/rho_g[i] - o->theta_v_bg[i];
    ep[i] = pow(r_d*rt[i]/p_0, r_d/c_d_v) - o->exner_bg[i];
  }
  return LGAME_OK;
}

int oracle_bc_state(oracle_ctx* o, int* index_old, int* index_new, double* t_latest_bc) {
  if (!o || !o->bc_on) return LGAME_ERR_STATE;
  if (index_old) *index_old = o->bc_index_old;
  if (index_new) *index_new = o->bc_index_new;
  if (t_latest_bc) *t_latest_bc = o->t_latest_bc;
  return LGAME_OK;
}

int oracle_bc_factors(oracle_ctx* o, double* scalar_f, double* u_f, double* v_f) {
  if (!o || !o->bc_on) return LGAME_ERR_STATE;
  DIMS;
  if (scalar_f) memcpy(scalar_f, o->scalar_bc_factor, (size_t)ny*nx*sizeof(double));
  if (u_f) memcpy(u_f, o->u_bc_factor, (size_t)ny*(nx+1)*sizeof(double));
  if (v_f) memcpy(v_f, o->v_bc_factor, (size_t)(ny+1)*nx*sizeof(double));
  return LGAME_OK;
}

/* ---- output fields, mo_write_out.F90:167-217 after linear_combine_two_states ---------- */

/* saturation_pressure_over_water (mo_dictionary.F90:256-291) for temperatures above t_0,
 * the only ones rel_humidity passes to it (temp_c > 0: Huang's formula) */
static double sat_water_warm(double temperature) {
  double temp_c = temperature - t_0;
  if (temp_c > 100.0) temp_c = 100.0;
  return exp(34.494 - 4924.99/(temp_c + 237.1))/pow(temp_c + 105.0, 1.57);
}
/* saturation_pressure_ice_huang and _murphy, mo_dictionary.F90:416-442 */
static double sat_ice_huang(double temperature) {
  const double temp_c = temperature - t_0;
  const double d = temp_c + 868.0;
  return exp(43.494 - 6545.8/(temp_c + 278.0))/(d*d);
}
static double sat_ice_murphy(double temperature) {
  return exp(9.550426 - 5723.265/temperature + 3.53068*log(temperature) - 0.00728332*temperature);
}
/* saturation_pressure_over_ice, mo_dictionary.F90:318-353 (with its "+ (1-w) +" blend) */
static double sat_ice(double temperature) {
  double t_local = temperature;
  const double temp_c = t_local - t_0;
  if (temp_c >= -80.0) {
    if (t_local > t_0) t_local = t_0;
    return sat_ice_huang(t_local);
  } else if (temp_c >= -100.0) {
    const double huang_weight = (temp_c + 100.0)/20.0;
    return huang_weight*sat_ice_huang(t_local) + (1.0 - huang_weight) + sat_ice_murphy(t_local);
  }
  if (t_local < 110.0) t_local = 110.0;
  return sat_ice_murphy(t_local);
}
/* rel_humidity, mo_derived.F90:131-155 */
static double rel_humidity(double abs_humidity, double temperature) {
  const double vapour_pressure = abs_humidity*r_v*temperature;
  double saturation_pressure = 0.0;
  if (temperature > t_0) saturation_pressure = sat_water_warm(temperature);
  if (temperature <= t_0) saturation_pressure = sat_ice(temperature);
  return vapour_pressure/saturation_pressure;
}

int oracle_output(oracle_ctx* o, int slot_1, int slot_2, double coeff_1, double coeff_2, float* const* fields,
                  int nfields, int* crashed) {
  if (!o || !fields || nfields != LGAME_OUTPUT_NFIELDS || slot_1 < 0 || slot_1 > 1 || slot_2 < 0 || slot_2 > 1)
    return LGAME_ERR_INVALID_ARG;
  DIMS;
  const int nc = o->nc, ncons = o->ncons;
  const size_t nS = (size_t)ny*nx*nl;
  /* state_write = linear_combine_two_states(state_1, state_2, ...), mo_linear_combination.F90:26-35 */
  double* rho = (double*)malloc(nS*ncons*sizeof(double));
  double* rt = (double*)malloc(nS*sizeof(double));
  double* tp = (double*)malloc(nS*sizeof(double));
  double* ep = (double*)malloc(nS*sizeof(double));
  double* u = (double*)malloc((size_t)ny*(nx+1)*nl*sizeof(double));
  double* v = (double*)malloc((size_t)(ny+1)*nx*nl*sizeof(double));
  double* w = (double*)malloc((size_t)ny*nx*(nl+1)*sizeof(double));
  if (!rho || !rt || !tp || !ep || !u || !v || !w) {
    free(rho); free(rt); free(tp); free(ep); free(u); free(v); free(w);
    return LGAME_ERR_ALLOC;
  }
  for (size_t i = 0; i < nS*ncons; ++i) rho[i] = coeff_1*o->rho[slot_1][i] + coeff_2*o->rho[slot_2][i];
  for (size_t i = 0; i < nS; ++i) rt[i] = coeff_1*o->rhotheta_v[slot_1][i] + coeff_2*o->rhotheta_v[slot_2][i];
  for (size_t i = 0; i < nS; ++i) tp[i] = rt[i]/rho[nS*(size_t)nc + i] - o->theta_v_bg[i];
  for (size_t i = 0; i < nS; ++i) ep[i] = coeff_1*o->exner_pert[slot_1][i] + coeff_2*o->exner_pert[slot_2][i];
  for (size_t i = 0; i < (size_t)ny*(nx+1)*nl; ++i) u[i] = coeff_1*o->wind_u[slot_1][i] + coeff_2*o->wind_u[slot_2][i];
  for (size_t i = 0; i < (size_t)(ny+1)*nx*nl; ++i) v[i] = coeff_1*o->wind_v[slot_1][i] + coeff_2*o->wind_v[slot_2][i];
  for (size_t i = 0; i < (size_t)ny*nx*(nl+1); ++i) w[i] = coeff_1*o->wind_w[slot_1][i] + coeff_2*o->wind_w[slot_2][i];
  /* the crash check of write_output, mo_write_out.F90:60-67 */
  int nan = 0;
  for (size_t i = 0; i < nS; ++i) nan |= isnan(ep[i]);
  if (crashed) *crashed = nan;
  /* the fields as stored (NF90_REAL: rounded to float) */
  if (fields[0]) for (size_t i = 0; i < nS*ncons; ++i) fields[0][i] = (float)rho[i];
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji) {
        const size_t q = IS(ji,jk,jl);
        const double temperature = (o->theta_v_bg[q] + tp[q])*(o->exner_bg[q] + ep[q]);
        if (fields[1]) fields[1][q] = (float)temperature;
        if (fields[2] && ncons > 1) fields[2][q] = (float)rel_humidity(rho[IRHO(ji,jk,jl,nc+2)], temperature);
        if (fields[3]) fields[3][q] = (float)(0.5*(u[IU(ji,jk,jl)] + u[IU(ji,jk+1,jl)]));
        if (fields[4]) fields[4][q] = (float)(0.5*(v[IV(ji,jk,jl)] + v[IV(ji+1,jk,jl)]));
        if (fields[5]) {
          const double upper_weight = (o->z_scalar[q] - o->z_w[IS(ji,jk,jl+1)])/(o->z_w[IS(ji,jk,jl)] - o->z_w[IS(ji,jk,jl+1)]);
          fields[5][q] = (float)(upper_weight*w[IS(ji,jk,jl)] + (1.0 - upper_weight)*w[IS(ji,jk,jl+1)]);
        }
      }
  free(rho); free(rt); free(tp); free(ep); free(u); free(v); free(w);
  return LGAME_OK;
}

#include "lgame_oracle_ops.inc"
#include "lgame_oracle_step.inc"
