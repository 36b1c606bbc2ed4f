/*
 * lgame_gpu.h -- C ABI of the GB300 (sm_103a) HEVI time step of L-GAME.
 *
 * The library replaces one Fortran module procedure of the reference model:
 *
 *   subroutine pchevi(state_old,state_new,tend,bc,grid,diag,total_step_counter,lrad_update,t_0)
 *   (src/time_stepping/mo_manage_pchevi.F90:27-118, called from src/control.F90:520-524)
 *
 * The reference passes Fortran derived types with allocatable components
 * (src/mo_definitions.F90:29-212), which are not C-interoperable.  This ABI
 * therefore passes every array as a plain pointer to a contiguous column-major
 * (Fortran-order) double array with exactly the reference's extents; the array
 * kinds and their order are fixed by the enums below.  A Fortran host binds it
 * with iso_c_binding (c_loc of each contiguous allocatable); a C or C++ host
 * passes pointers directly.
 *
 * Index conventions (identical to the reference, src/mo_grid_generator.F90:129-133):
 *   ji = 1..ny  (y, north to south, fastest varying)
 *   jk = 1..nx  (x, west to east)
 *   jl = 1..n_layers (layer 1 = top), levels 1..n_layers+1 (level n_layers+1 = surface)
 * Staggered extents:
 *   scalar (ny,nx,nl)      u (ny,nx+1,nl)       v (ny+1,nx,nl)       w (ny,nx,nl+1)
 *   zeta_x/eta_x (ny+1,nx,nl+1)   zeta_y/eta_y (ny,nx+1,nl+1)   zeta_z/eta_z (ny+1,nx+1,nl)
 *
 * Every entry point returns 0 on success or a negative LGAME_ERR_* code and never
 * calls exit(); lgame_gpu_last_error() describes the last failure of the calling
 * thread.  The library owns device copies of the grid, two state slots, the
 * tendencies and the diagnostics that are carried from one step to the next; host
 * pointers are borrowed for the duration of a call only.
 */
#ifndef LGAME_GPU_H
#define LGAME_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define LGAME_OK                 0
#define LGAME_ERR_INVALID_ARG   -1  /* null pointer, bad slot, bad field count          */
#define LGAME_ERR_BAD_DIMS      -2  /* ny/nx/n_layers/n_oro_layers out of range          */
#define LGAME_ERR_BAD_CONFIG    -3  /* theta_adv_order, precision, dtime ...             */
#define LGAME_ERR_UNSUPPORTED   -4  /* a physics switch outside the GPU path is on       */
#define LGAME_ERR_ALLOC         -5  /* device or pinned allocation failed                */
#define LGAME_ERR_CUDA          -6  /* a CUDA runtime call failed                        */
#define LGAME_ERR_NONFINITE     -7  /* NaN/Inf found in the new state (check enabled)    */
#define LGAME_ERR_NO_DEVICE     -8  /* no CUDA device, or not an sm_103 device           */
#define LGAME_ERR_STATE         -9  /* call out of order (e.g. step before set_grid)     */

/* ---- precision modes ---------------------------------------------------- */
#define LGAME_PRECISION_FP64   0  /* every operation in FP64, reference operation order */
#define LGAME_PRECISION_SPLIT  1  /* FP32 explicit stencils, tracer fluxes and the
                                     coefficients and multipliers of the column solves;
                                     FP64 right-hand side and substitutions of the vertical
                                     acoustic solve, background subtraction in the pressure
                                     gradient, state accumulation and budgets */
#define LGAME_PRECISION_SPLIT_FP64_COLUMN 2  /* as LGAME_PRECISION_SPLIT, with the vertical
                                     acoustic solve wholly in FP64 (coefficients,
                                     multipliers, quotients from the FP64 state) */

/* ---- run configuration ----------------------------------------------------
 * One field per namelist variable the HEVI step reads (the src/namelists modules),
 * plus the derived quantities the reference computes once at start-up
 * (n_levels, n_flat_layers, dtime: mo_run_nml.F90:89-94; n_constituents:
 * mo_constituents_nml.F90:246-253).  Logical switches are 0/1 ints.
 * Combinations of switches that the reference cannot run as specified (see
 * lgame_gpu_create) are rejected with LGAME_ERR_UNSUPPORTED or LGAME_ERR_BAD_CONFIG. */
typedef struct lgame_config {
  /* &run (mo_run_nml.F90:44-46) */
  int    ny, nx, n_layers, n_oro_layers;
  double dx, dy, toa;
  double dtime;                 /* seconds; the reference derives 1.61*sqrt(dx*dy)/1000 */
  int    theta_adv_order;       /* 2 or 3 */
  int    llinear, lcorio, luse_bg_state, lplane;
  /* &constituents (mo_constituents_nml.F90:227) */
  int    lmoist;                /* 1: 5 condensates + 2 gases (7 constituents); 0: dry (1) */
  /* &diff (mo_diff_nml.F90:28-29): only the Klemp layer is in the step */
  int    lklemp;
  double klemp_damp_max, klemp_begin_rel;
  int    lmom_diff_h, lmom_diff_v, ltemp_diff_h, ltemp_diff_v, lmass_diff_h, lmass_diff_v;
  /* &surface (mo_surface_nml.F90:138) */
  int    lprog_soil_temp, lsfc_sensible_heat_flux, lsfc_phase_trans, lpbl;
  /* &bc (mo_bc_nml.F90:283) */
  int    lperiodic, lfreeslip;
  /* extension: precision and checks (no reference counterpart) */
  int    precision;             /* LGAME_PRECISION_* */
  int    check_finite;          /* 1: scan the new state for NaN/Inf after every step */
  int    device;                /* CUDA device ordinal the context lives on          */
  /* &diff, the diffusion closure (mo_diff_nml.F90:12-26; appended, so that the fields above
   * keep their offsets): the horizontal coefficient scheme (the vertical one is always tke),
   * the minimum background shear (1/s) and the Smagorinsky parameter */
  int    diff_coeff_scheme_h;   /* LGAME_DIFF_COEFF_SMAG or LGAME_DIFF_COEFF_TKE */
  double bg_shear, c_s;
  /* &surface and the surface-layer constants of &diff (mo_surface_nml.F90:14, mo_diff_nml.F90:
   * 18-19; appended): the number of soil layers (2..LGAME_MAX_SOIL_LAYERS when the soil or the
   * sensible heat flux is on), the height of the Prandtl layer (m) and von Karman's constant */
  int    nsoillays;
  double h_prandtl, karman;
  /* extension (appended): the phase transitions of the water constituents
   * (calc_h2otracers_source_rates, mo_phase_trans.F90:22-330), which the reference compiles but
   * never calls, so its rates stay zero there.  1: formed at the first substep of every step
   * from state_old and its temperature, read by both substeps' scalar tendencies as the
   * reference's scalar_tend_expl reads them (mo_scalar_tend_expl.F90:127, 163, 170), with the
   * surface evaporation of lsfc_phase_trans and the latent heat flux over lakes into the soil.
   * Needs lmoist. */
  int    lphase_trans;
} lgame_config;

#define LGAME_MAX_SOIL_LAYERS 16

#define LGAME_DIFF_COEFF_SMAG 0  /* diff_coeff_scheme_h = "smag" */
#define LGAME_DIFF_COEFF_TKE  1  /* diff_coeff_scheme_h = "tke"  */

/* ---- grid arrays (t_grid, src/mo_definitions.F90:29-91) --------------------
 * Extents in brackets; all double, column-major.  These are exactly the grid
 * quantities pchevi reads. */
enum lgame_grid_field {
  LGAME_GRID_Z_SCALAR = 0,          /* (ny,nx,nl)      */
  LGAME_GRID_Z_U,                   /* (ny,nx+1,nl)    */
  LGAME_GRID_Z_V,                   /* (ny+1,nx,nl)    */
  LGAME_GRID_Z_W,                   /* (ny,nx,nl+1)    */
  LGAME_GRID_DX,                    /* (ny,nx+1,nl)    */
  LGAME_GRID_DY,                    /* (ny+1,nx,nl)    */
  LGAME_GRID_DZ,                    /* (ny,nx,nl+1)    */
  LGAME_GRID_VOLUME,                /* (ny,nx,nl)      */
  LGAME_GRID_AREA_X,                /* (ny,nx+1,nl)    */
  LGAME_GRID_AREA_Y,                /* (ny+1,nx,nl)    */
  LGAME_GRID_AREA_Z,                /* (ny,nx,nl+1)    */
  LGAME_GRID_AREA_DUAL_X,           /* (ny+1,nx,nl+1)  */
  LGAME_GRID_AREA_DUAL_Y,           /* (ny,nx+1,nl+1)  */
  LGAME_GRID_AREA_DUAL_Z,           /* (ny+1,nx+1,nl)  */
  LGAME_GRID_Z_AREA_DUAL_Z,         /* (ny+1,nx+1,nl)  */
  LGAME_GRID_SLOPE_X,               /* (ny,nx+1,nl)    */
  LGAME_GRID_SLOPE_Y,               /* (ny+1,nx,nl)    */
  LGAME_GRID_INNER_PRODUCT_WEIGHTS, /* (6,ny,nx,nl)    */
  LGAME_GRID_THETA_V_BG,            /* (ny,nx,nl)      */
  LGAME_GRID_EXNER_BG,              /* (ny,nx,nl)      */
  LGAME_GRID_EXNER_BG_GRAD_U,       /* (ny,nx+1,nl)    */
  LGAME_GRID_EXNER_BG_GRAD_V,       /* (ny+1,nx,nl)    */
  LGAME_GRID_EXNER_BG_GRAD_W,       /* (ny,nx,nl+1)    */
  LGAME_GRID_GRAVITY_M_V,           /* (ny,nx,nl+1)    */
  LGAME_GRID_GRAVITY_POTENTIAL,     /* (ny,nx,nl)      */
  LGAME_GRID_FVEC_X,                /* (ny+1,nx)       */
  LGAME_GRID_FVEC_Y,                /* (ny,nx+1)       */
  LGAME_GRID_FVEC_Z,                /* (ny+1,nx+1)     */
  LGAME_GRID_TRSK_WEIGHTS_U,        /* (3,ny)          */
  LGAME_GRID_TRSK_WEIGHTS_V,        /* (2,ny+1)        */
  /* the metrics of the diffusion closure (mo_grid_generator.F90:1012-1031, 1060-1064) */
  LGAME_GRID_DX_DUAL,               /* (ny+1,nx,nl)    */
  LGAME_GRID_DY_DUAL,               /* (ny,nx+1,nl)    */
  LGAME_GRID_LAYER_THICKNESS,       /* (ny,nx,nl)      */
  /* the surface and the soil (mo_definitions.F90:70-88; mo_grid_generator.F90:746-813, 1360-1378) */
  LGAME_GRID_LAND_FRACTION,         /* (ny,nx)         */
  LGAME_GRID_LAKE_FRACTION,         /* (ny,nx)         */
  LGAME_GRID_ROUGHNESS_LENGTH,      /* (ny,nx)  m, of the land                      */
  LGAME_GRID_SFC_RHO_C,             /* (ny,nx)  volumetric heat capacity of the soil */
  LGAME_GRID_T_CONDUC_SOIL,         /* (ny,nx)  temperature conductivity of the soil */
  LGAME_GRID_T_CONST_SOIL,          /* (ny,nx)  K, temperature at depth z_t_const    */
  LGAME_GRID_Z_SOIL_INTERFACE,      /* (nsoillays+1) m, 0 at the surface, downward negative */
  LGAME_GRID_Z_SOIL_CENTER,         /* (nsoillays)   m                               */
  LGAME_GRID_Z_T_CONST,             /* (1)      m, depth of the constant soil temperature */
  LGAME_GRID_NFIELDS
};

/* ---- prognostic state (t_state, src/mo_definitions.F90:94-105) ----------- */
enum lgame_state_field {
  LGAME_STATE_RHO = 0,        /* (ny,nx,nl,n_constituents) */
  LGAME_STATE_RHOTHETA_V,     /* (ny,nx,nl)     */
  LGAME_STATE_THETA_V_PERT,   /* (ny,nx,nl)     */
  LGAME_STATE_EXNER_PERT,     /* (ny,nx,nl)     */
  LGAME_STATE_WIND_U,         /* (ny,nx+1,nl)   */
  LGAME_STATE_WIND_V,         /* (ny+1,nx,nl)   */
  LGAME_STATE_WIND_W,         /* (ny,nx,nl+1)   */
  LGAME_STATE_TEMPERATURE_SOIL, /* (ny,nx,nsoillays) */
  LGAME_STATE_NFIELDS
};
/* The state calls take either all LGAME_STATE_NFIELDS arrays or only the first
 * LGAME_STATE_NFIELDS_ATMOS (the atmosphere; the soil temperature on the device is then left
 * as it is, which a run without prognostic soil and sensible heat flux never reads). */
#define LGAME_STATE_NFIELDS_ATMOS 7

/* ---- diagnostics carried between steps (t_diag, t_tend) -------------------
 * These are the arrays whose values survive from one call of pchevi to the next
 * (or that the host provides), i.e. what a restart needs besides the state. */
enum lgame_diag_field {
  LGAME_DIAG_P_GRAD_ACC_NEG_NL_U = 0, /* (ny,nx+1,nl)   */
  LGAME_DIAG_P_GRAD_ACC_NEG_NL_V,     /* (ny+1,nx,nl)   */
  LGAME_DIAG_P_GRAD_ACC_NEG_NL_W,     /* (ny,nx,nl+1)   */
  LGAME_DIAG_P_GRAD_ACC_NEG_L_U,      /* (ny,nx+1,nl)   */
  LGAME_DIAG_P_GRAD_ACC_NEG_L_V,      /* (ny+1,nx,nl)   */
  LGAME_DIAG_P_GRAD_ACC_NEG_L_W,      /* (ny,nx,nl+1)   */
  LGAME_DIAG_P_GRAD_ACC_OLD_U,        /* (ny,nx+1,nl)   */
  LGAME_DIAG_P_GRAD_ACC_OLD_V,        /* (ny+1,nx,nl)   */
  LGAME_DIAG_POT_VORT_TEND_X,         /* (ny,nx+1,nl)   */
  LGAME_DIAG_POT_VORT_TEND_Y,         /* (ny+1,nx,nl)   */
  LGAME_DIAG_POT_VORT_TEND_Z,         /* (ny,nx,nl+1)   */
  LGAME_DIAG_V_SQUARED_GRAD_X,        /* (ny,nx+1,nl)   */
  LGAME_DIAG_V_SQUARED_GRAD_Y,        /* (ny+1,nx,nl)   */
  LGAME_DIAG_V_SQUARED_GRAD_Z,        /* (ny,nx,nl+1)   */
  LGAME_DIAG_CONDENSATES_SEDIMENT_HEAT,/* (ny,nx,nl)    */
  LGAME_DIAG_RADIATION_TENDENCY,      /* (ny,nx,nl)  W m^-3, provided by the host   */
  LGAME_DIAG_TEMPERATURE,             /* (ny,nx,nl)  of state_old of the last step  */
  LGAME_DIAG_TEND_RHO,                /* (ny,nx,nl,n_constituents)                  */
  LGAME_DIAG_TEND_RHOTHETA_V,         /* (ny,nx,nl)     */
  LGAME_DIAG_TEND_WIND_U,             /* (ny,nx+1,nl)   */
  LGAME_DIAG_TEND_WIND_V,             /* (ny+1,nx,nl)   */
  LGAME_DIAG_TEND_WIND_W,             /* (ny,nx,nl+1)   */
  /* carried by the diffusion closure (a step's first substep reads them before it forms them
   * anew), and the swamp layer's dissipation */
  LGAME_DIAG_TKE,                     /* (ny,nx,nl)  specific turbulent kinetic energy (J/kg) */
  LGAME_DIAG_VISCOSITY,               /* (ny,nx,nl)  horizontal dynamic viscosity (kg m^-1 s^-1) */
  LGAME_DIAG_HEATING_DISS,            /* (ny,nx,nl)  dissipative heating power density (W m^-3) */
  LGAME_DIAG_MOM_DIFF_TEND_X,         /* (ny,nx+1,nl) momentum diffusion acceleration, x  */
  LGAME_DIAG_MOM_DIFF_TEND_Y,         /* (ny+1,nx,nl) momentum diffusion acceleration, y  */
  LGAME_DIAG_MOM_DIFF_TEND_Z,         /* (ny,nx,nl+1) momentum diffusion acceleration, z  */
  /* the surface layer (mo_definitions.F90:137, 172-181, 185): v_squared and the roughness length
   * are carried (the next step's surface update reads them before they are formed anew); the
   * sea surface temperature and the surface radiation fluxes are provided by the host */
  LGAME_DIAG_V_SQUARED,               /* (ny,nx,nl)  specific kinetic energy (m^2 s^-2)   */
  LGAME_DIAG_ROUGHNESS_LENGTH,        /* (ny,nx)  m, actual (sea: from the 10 m wind)     */
  LGAME_DIAG_ROUGHNESS_VELOCITY,      /* (ny,nx)  m/s                                     */
  LGAME_DIAG_MONIN_OBUKHOV_LENGTH,    /* (ny,nx)  m                                       */
  LGAME_DIAG_SCALAR_FLUX_RESISTANCE,  /* (ny,nx)  s/m                                     */
  LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SOIL, /* (ny,nx) W m^-2, sensible heat into the soil */
  LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SEA,  /* (ny,nx) W m^-2, sensible heat into the sea  */
  LGAME_DIAG_SST,                     /* (ny,nx)  K, sea surface temperature (host)       */
  LGAME_DIAG_SFC_SW_IN,               /* (ny,nx)  W m^-2, shortwave into the surface (host) */
  LGAME_DIAG_SFC_LW_OUT,              /* (ny,nx)  W m^-2, longwave out of the surface (host) */
  /* the phase transitions (lphase_trans; zero otherwise, as in the reference's step) */
  LGAME_DIAG_PHASE_TRANS_RATES,       /* (ny,nx,nl,n_condensed_constituents+1) kg m^-3 s^-1 */
  LGAME_DIAG_PHASE_TRANS_HEATING_RATE,/* (ny,nx,nl)  W m^-3                                 */
  LGAME_DIAG_POWER_FLUX_DENSITY_LAT_LAKE, /* (ny,nx) W m^-2, latent heat into lakes       */
  LGAME_DIAG_POWER_FLUX_DENSITY_LAT_SEA,  /* (ny,nx) W m^-2, latent heat into the sea     */
  /* the temperature and mass diffusion (mo_definitions.F90:207-209), formed at each step's first
   * substep from state_old (zero when ltemp_diff_h / lmass_diff_h is off) */
  LGAME_DIAG_TEMP_DIFF_HEATING,       /* (ny,nx,nl)  W m^-3, heating by temperature diffusion */
  LGAME_DIAG_MASS_DIFF_TENDENCY,      /* (ny,nx,nl,n_constituents) kg m^-3 s^-1, mass diffusion */
  LGAME_DIAG_NFIELDS
};

/* ---- output fields (write_output, src/io/mo_write_out.F90:167-217) -------------------
 * The variables of an output file, at the scalar points, as the file stores them (NF90_REAL:
 * the FP64 values rounded to float), column-major host arrays. */
enum lgame_output_field {
  LGAME_OUTPUT_RHO = 0,          /* (ny,nx,nl,n_constituents)  mass densities          */
  LGAME_OUTPUT_TEMPERATURE,      /* (ny,nx,nl)  (theta_v_bg + theta_v_pert)*(exner_bg + exner_pert) */
  LGAME_OUTPUT_REL_HUMIDITY,     /* (ny,nx,nl)  rel_humidity (moist runs only)         */
  LGAME_OUTPUT_WIND_U,           /* (ny,nx,nl)  0.5*(u(jk) + u(jk+1))                  */
  LGAME_OUTPUT_WIND_V,           /* (ny,nx,nl)  0.5*(v(ji) + v(ji+1))                  */
  LGAME_OUTPUT_WIND_W,           /* (ny,nx,nl)  w interpolated to the layer's z_scalar */
  LGAME_OUTPUT_NFIELDS
};

/* Budget vector of lgame_gpu_budgets (mo_write_out.F90:226-304):
 *   out[0 .. n_constituents-1]  sum(rho(:,:,:,jc)*volume)        (masses)
 *   out[n_constituents]         sum(rhotheta_v*volume)
 *   out[n_constituents+1]       0.5*sum(rho_g*|v|^2 *volume)     (kinetic)
 *   out[n_constituents+2]       sum(rho_g*gravity_potential*volume)
 *   out[n_constituents+3]       sum(c_d_v*rho_g*temperature*volume) (internal) */
#define LGAME_BUDGETS_MAX 11

typedef struct lgame_gpu lgame_gpu;   /* opaque context, one per model instance */

/* Supplier of boundary data for the lateral relaxation (the role of read_boundaries,
 * mo_boundaries.F90:99-123): called when a boundary update needs a new level, with the
 * valid time the reference would read (t_update, seconds) and the time index (1 or 2)
 * the level goes to.  It must hand the level over with lgame_gpu_set_bc (or, for the
 * oracle, oracle_set_bc) before it returns, and returns 0, or nonzero to fail the step. */
typedef int (*lgame_bc_loader)(void* user, double t_update, int time_index);

/* Creates a context on the current CUDA device and allocates its device memory.
 * Replaces the allocation block of src/control.F90:99-444 for the arrays pchevi uses. */
int  lgame_gpu_create(const lgame_config* cfg, lgame_gpu** out);

/* Copies the grid (host, reference layout) to the device once, precomputing nothing
 * that changes the arithmetic of the FP64 path.  Replaces the grid argument of pchevi
 * (mo_manage_pchevi.F90:35) for the lifetime of the context.  nfields must equal
 * LGAME_GRID_NFIELDS.  The surface and soil fields may be NULL when the surface switches
 * (lprog_soil_temp, lsfc_sensible_heat_flux, lsfc_phase_trans, lpbl) are all off.  The call
 * also sets the carried roughness length to the grid's (diag%roughness_length =
 * grid%roughness_length, control.F90:458). */
int  lgame_gpu_set_grid(lgame_gpu* ctx, const double* const* fields, int nfields);

/* Host -> device copy of one state slot (slot 0 or 1, the reference's state_1/state_2,
 * control.F90:30-31).  nfields must be LGAME_STATE_NFIELDS, or LGAME_STATE_NFIELDS_ATMOS
 * to leave the soil temperature as it is (get_state: not to copy it). */
int  lgame_gpu_set_state(lgame_gpu* ctx, int slot, const double* const* fields, int nfields);
/* Device -> host copy of one state slot; synchronises. */
int  lgame_gpu_get_state(lgame_gpu* ctx, int slot, double* const* fields, int nfields);

/* Host <-> device copies of the carried diagnostics (restart, parity checks, and the
 * host-provided radiation tendency).  nfields must equal LGAME_DIAG_NFIELDS; a NULL
 * pointer in set_diag leaves that field unchanged, in get_diag skips it. */
int  lgame_gpu_set_diag(lgame_gpu* ctx, const double* const* fields, int nfields);
int  lgame_gpu_get_diag(lgame_gpu* ctx, double* const* fields, int nfields);

/* One HEVI predictor-corrector step entirely on the device: state[new_slot] is
 * computed from state[old_slot].  Equivalent of
 *   call pchevi(state_old,state_new,tend,bc,grid,diag,total_step_counter,lrad_update,t_0)
 * In a non-periodic run with boundary data set up (lgame_gpu_bc_setup), the step ends
 * with lgame_gpu_update_boundaries(ctx, new_slot, (total_step_counter+1)*dtime), as the
 * reference's does (mo_manage_pchevi.F90:114-116).  With a radiation emulator attached
 * (lgame_gpu_rad_attach, lgame_emulator.h), lrad_update = 1 runs the emulator's radiation
 * update on state_old before the substeps, at t_0 + dtime_rad/2, as the reference's
 * update_rad_fluxes (mo_manage_pchevi.F90:56-58); without one, lrad_update is ignored and
 * the radiation tendency is whatever the host last set.  Stream-ordered: returns after
 * enqueueing unless check_finite is on, a boundary level has to be loaded or a radiation
 * update ran. */
int  lgame_gpu_pchevi(lgame_gpu* ctx, int old_slot, int new_slot,
                      int total_step_counter, int lrad_update, double t_0);

/* The same step with host buffers: copies state_old from host memory to the device,
 * runs lgame_gpu_pchevi into slot 1, and copies the new state back to state_new
 * (host).  This is what a Fortran pchevi_gpu shim with pchevi's exact argument list
 * would call when the host keeps the authoritative state (mo_manage_pchevi.F90:27).
 * When every array is page-locked and mapped (cudaHostAlloc / cudaHostRegister with
 * mapping; on Grace systems the GPU then reaches it over the coherent CPU-GPU link), the
 * GPU reads and writes the host arrays itself and fills the FP32 state mirror in the
 * same pass; otherwise the copy engines move the state.  In split precision (without a
 * boundary relaxation), fields of the new state that are final before the step ends are
 * copied out on a second stream while the step still runs.  Slots 0 and 1 are used.
 * nfields is LGAME_STATE_NFIELDS, or LGAME_STATE_NFIELDS_ATMOS when neither the soil
 * temperature nor the sensible heat flux is on (the soil temperature is then not moved). */
int  lgame_gpu_pchevi_host(lgame_gpu* ctx, const double* const* state_old,
                           double* const* state_new, int nfields,
                           int total_step_counter, int lrad_update, double t_0);

/* FP64 domain integrals of one slot (mo_write_out.F90:226-304); out must hold
 * n_constituents+4 doubles.  Uses the temperature diagnosed at the start of the last
 * step, as the reference's write_out_integrals does (control.F90:529-535).
 * Synchronises. */
int  lgame_gpu_budgets(lgame_gpu* ctx, int slot, double* out, int nout);

/* The same budget vector as lgame_gpu_budgets (bit for bit), computed without allocating
 * any memory, host or device.  No counterpart in the reference.
 *
 * For hosts that must not allocate inside their time loop: drivers that reserve all
 * memory at start-up and run the loop under an allocation guard (a malloc hook, or a
 * device memory pool with a fixed cap), and hosts whose device memory is fully committed
 * to model state (a 1024x1024x80 split-precision context holds about 108 GB, so a few
 * ensemble members fill a GPU).  lgame_gpu_budgets allocates a small host array on every
 * call; this entry point uses a fixed scratch array compiled into the library instead:
 * 1024*11 + 11 doubles (90,200 bytes) per device, which is why at most LGAME_BUDGETS_MAX
 * (11) quantities, i.e. n_constituents <= 7, are accepted (more: LGAME_ERR_INVALID_ARG).
 *
 * - lgame_gpu_create loads the module that holds the scratch array and the two reduction
 *   kernels on its device (under CUDA's lazy loading that load takes device memory), so
 *   the calls of this function inside a time loop allocate nothing.  Every call looks the
 *   scratch address up again (cudaGetSymbolAddress, with the context's device current):
 *   after a cudaDeviceReset the next context loads the module anew and the address may
 *   change, so nothing is cached across calls.
 * - There is one scratch array per device, shared by all contexts on that device: calls
 *   that overlap in time on one device (several host threads, or several contexts of the
 *   same device used concurrently) race on it and return wrong sums.  Calls from a single
 *   host thread never overlap, since the function returns after the result is copied.
 * - The context's device is made current for the call and the caller's device restored.
 * Synchronises. */
int  lgame_gpu_budgets_static(lgame_gpu* ctx, int slot, double* out, int nout);

/* Blocks until all work of the context has finished. */
int  lgame_gpu_synchronize(lgame_gpu* ctx);

/* Number of kernels launched by the last lgame_gpu_pchevi call. */
int  lgame_gpu_kernels_per_step(const lgame_gpu* ctx);

/* The CUDA stream (cudaStream_t) on which the context launches all its work, so that a
 * host can record its own CUDA events around the step.  Tracing aid; no reference
 * counterpart (the reference's only instrumentation is cpu_time, control.F90:545-547). */
void* lgame_gpu_stream(const lgame_gpu* ctx);

/* Per-kernel tracing: when enabled, every kernel launch of the step is bracketed by a
 * pair of CUDA events on the context's stream.  lgame_gpu_profile_report synchronises,
 * writes a JSON object {"kernel name": {"launches": n, "ms": total}, ...} accumulated
 * since the last report (or since tracing was enabled) into buf, and resets the counts.
 * Returns the length of the JSON text (or the length needed if len is too small). */
int  lgame_gpu_set_profiling(lgame_gpu* ctx, int enable);
int  lgame_gpu_profile_report(lgame_gpu* ctx, char* buf, int len);

/* The step as a CUDA graph (on by default): after step 0 every call of lgame_gpu_pchevi for
 * a given (old_slot, new_slot) pair launches the same kernels with the same arguments, so the
 * library captures that sequence once per pair, at its first use, and then launches the
 * graph: one host launch instead of about 30 (the split step: 31), which matters where the
 * kernels are short (small grids).  Results are the same bits either way.  Graphs are not
 * used while per-kernel tracing is on.  No counterpart in the reference (a CPU program). */
int  lgame_gpu_set_graphs(lgame_gpu* ctx, int enable);

/* The output of the reference's time loop (control.F90:535-537): the state
 *   state_write = coeff_1*state[slot_1] + coeff_2*state[slot_2]
 * (linear_combine_two_states, mo_linear_combination.F90:15-37, which recomputes theta_v_pert
 * from the combined rho and rhotheta_v), then the fields write_output puts in the file
 * (mo_write_out.F90:167-217), in the order of enum lgame_output_field, as floats.  NULL
 * entries are skipped; LGAME_OUTPUT_REL_HUMIDITY is not written in dry runs.  *crashed
 * (if given) becomes 1 when the combined exner_pert holds a NaN, the reference's "model
 * crashed" check (mo_write_out.F90:60-67), else 0.  Synchronous. */
int  lgame_gpu_output(lgame_gpu* ctx, int slot_1, int slot_2, double coeff_1, double coeff_2,
                      float* const* fields, int nfields, int* crashed);

/* ---- lateral boundary relaxation (src/io/mo_boundaries.F90) --------------------------
 * Turns on the relaxation of a non-periodic run (lperiodic = 0; else LGAME_ERR_STATE):
 * the rescale factors of a swamp layer n_swamp points wide (setup_bc_factor,
 * mo_boundaries.F90:125-170: sin^2 of pi/2*max(1 - d/n_swamp, 0), d the index distance
 * from the edge), the interval dtime_bc (s) between boundary levels, t_latest_bc (s) the
 * valid time of the level in time index 1 on the clock of the step's t_now, i.e. time
 * since the start (the reference's default, 0), and the loader of later levels.  Level
 * indices start as old = 1, new = 2 (control.F90:358-359); both levels are zero until set.
 * Without this call the step applies no relaxation (the reference would relax toward
 * all-zero boundary data in idealised non-periodic runs, which empties the outer ring). */
int  lgame_gpu_bc_setup(lgame_gpu* ctx, int n_swamp, int dtime_bc, double t_latest_bc,
                        lgame_bc_loader loader, void* user);
/* One boundary level into time index 1 or 2 (bc%rho(:,:,:,:,i) ... bc%wind_w(:,:,:,i)):
 * rho (ny,nx,n_layers,n_constituents), rhotheta_v (ny,nx,n_layers), wind_u
 * (ny,nx+1,n_layers), wind_v (ny+1,nx,n_layers), wind_w (ny,nx,n_layers+1), host arrays
 * in the reference layout. */
int  lgame_gpu_set_bc(lgame_gpu* ctx, int time_index, const double* rho, const double* rhotheta_v,
                      const double* wind_u, const double* wind_v, const double* wind_w);
/* update_boundaries(state, bc, t_now, grid), mo_boundaries.F90:19-97, on state slot `slot`:
 * time weights old = 1 - (t_now - t_latest_bc)/dtime_bc and new = 1 - old; if old < 0
 * the loader is asked for the level of t_latest_bc + dtime_bc into the old index, the
 * indices swap and t_latest_bc advances by dtime_bc (the weights are not recomputed, as in
 * the reference); then every point becomes factor*(old*bc_old + new*bc_new) +
 * (1 - factor)*state for rho, rhotheta_v, u, v, w, and theta_v_pert and exner_pert are
 * recomputed from rho and rhotheta_v over the whole domain. */
int  lgame_gpu_update_boundaries(lgame_gpu* ctx, int slot, double t_now);
/* The boundary bookkeeping: level indices (1-based) and t_latest_bc. */
int  lgame_gpu_bc_state(lgame_gpu* ctx, int* index_old, int* index_new, double* t_latest_bc);

/* Bytes of device memory held by the context. */
long long lgame_gpu_device_bytes(const lgame_gpu* ctx);

/* Frees all device memory of the context. */
void lgame_gpu_destroy(lgame_gpu* ctx);

/* Human-readable description of the last error of the calling thread. */
const char* lgame_gpu_last_error(void);

/* Library version string. */
const char* lgame_gpu_version(void);

#ifdef __cplusplus
}
#endif
#endif /* LGAME_GPU_H */
