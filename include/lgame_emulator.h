/*
 * lgame_emulator.h -- C ABI of the radiation emulator and its coupling to the HEVI step.
 *
 * No counterpart in the reference beyond the seam it plugs into.  The reference calls
 * RTE+RRTMGP every dtime_rad seconds (update_rad_fluxes, src/radiation/
 * mo_manage_radiation_calls.F90:17-59, and calc_radiative_flux_convergence,
 * src/radiation/mo_rterrtmgp_coupler.F90:56-493), which writes the radiative power density
 * diag%radiation_tendency (W m^-3) that the scalar tendency turns into a rho*theta_v
 * tendency (src/time_stepping/mo_scalar_tend_expl.F90:157-166).  Here a small MLP predicts
 * the shortwave and longwave heating-rate profiles of every column from its state, on the
 * GPU, with BF16 tensor-core (tcgen05) kernels for training and inference; a CPU scheme
 * (lgame_rad_teacher) stands in for RRTMGP as the source of training targets, the check of
 * sampled columns and the fallback.
 *
 * Column features (float, one row of 4*nlev+2 per column, layer 1 = top):
 *   [0, nlev)         temperature (K)
 *   [nlev, 2 nlev)    dry-air pressure r_d*rho_dry*T (Pa), mo_rterrtmgp_coupler.F90:166
 *   [2 nlev, 3 nlev)  water vapour density (kg m^-3), the last constituent
 *   [3 nlev, 4 nlev)  ozone density (kg m^-3): calc_o3_vmr(z) (mo_dictionary.F90:66-86)
 *                     times rho_dry times M_O3/M_dry
 *   4 nlev            surface albedo
 *   4 nlev + 1        cosine of the solar zenith angle, coszenith
 *                     (mo_rterrtmgp_coupler.F90:550-629), 0 at night
 * Heating rates (float, one row of 2*nlev per column): shortwave then longwave, K/day.
 * Conversion to the reference's power density: Q = rate/86400 * rho * c_d_p with rho the
 * gas density (dry air + vapour) of the layer.
 *
 * All functions return LGAME_OK (0) or a negative LGAME_ERR_* code of lgame_gpu.h.
 */
#ifndef LGAME_EMULATOR_H
#define LGAME_EMULATOR_H

#include "lgame_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LGAME_RAD_NLEV_MAX 128

/* ---- stand-in radiation scheme (CPU, OpenMP) ------------------------------- */
/* Heating rates of ncol columns from their features; the scheme is described in
 * l-game_gb300/csrc/host/teacher.cpp (Lacis-Hansen shortwave absorption by water vapour
 * and ozone, semi-gray two-stream longwave). */
int lgame_rad_teacher(const float* features, long long ncol, int nlev, float* heating);

/* ---- the MLP ------------------------------------------------------------------
 * (4*nlev+2) -> hidden -> hidden -> hidden -> 2*nlev, GELU after the hidden layers.
 * Parameters in FP32 (Adam master copy) and BF16 (tensor-core operands); GEMMs in BF16
 * with FP32 accumulation in tensor memory.  Inputs and targets are standardised with the
 * statistics given by lgame_emu_set_normalization (identity by default). */
typedef struct lgame_emu lgame_emu;

/* nlev <= LGAME_RAD_NLEV_MAX; hidden a multiple of 256; batch_max a multiple of 128. */
int  lgame_emu_create(int nlev, int hidden, int batch_max, unsigned long long seed, int device, lgame_emu** out);
void lgame_emu_destroy(lgame_emu* emu);
/* number of parameters and their order: W1 (hidden x nin), b1, W2, b2, W3, b3, W4 (nout x hidden), b4 */
long long lgame_emu_num_params(const lgame_emu* emu);
int  lgame_emu_get_params(lgame_emu* emu, float* params);
int  lgame_emu_set_params(lgame_emu* emu, const float* params);
int  lgame_emu_set_normalization(lgame_emu* emu, const float* x_mean, const float* x_std,
                                 const float* y_mean, const float* y_std);
/* Mean squared error (standardised targets) of one batch and its gradient with respect to
 * every parameter (host arrays; grads in the order of lgame_emu_get_params). */
int  lgame_emu_loss_grad(lgame_emu* emu, const float* x, const float* y, int batch, float* loss, float* grads);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on one batch of host data. */
int  lgame_emu_train_step(lgame_emu* emu, const float* x, const float* y, int batch, float lr, float* loss);
/* Training data resident on the device: upload once, then epochs over shuffled batches. */
int  lgame_emu_set_dataset(lgame_emu* emu, const float* x, const float* y, long long n);
int  lgame_emu_train_epoch(lgame_emu* emu, int batch, float lr, unsigned long long seed, float* mean_loss);
/* Heating rates of n columns (host arrays, any n; processed in batches of batch_max).
 * Page-locked x and y are read and written by the GPU directly over the CPU-GPU link;
 * other host arrays are copied through device buffers.  Both give the same bits. */
int  lgame_emu_infer(lgame_emu* emu, const float* x, long long n, float* y);
/* Tensor-core GEMM C = A * B^T (BF16 bit patterns in, FP32 out, host arrays), A: M x K,
 * B: N x K, both row-major; M % 128 == 0, K % 64 == 0, N % 64 == 0.  Exposed for tests. */
int  lgame_emu_gemm_bf16(lgame_emu* emu, const unsigned short* a, const unsigned short* b, float* c,
                         int m, int n, int k);
/* Launches of tensor-core GEMM kernels and their floating-point operations since the last call. */
int  lgame_emu_stats(lgame_emu* emu, long long* gemm_launches, double* gemm_flop);

/* ---- coupling to the HEVI step (a lgame_gpu context) ------------------------------ */
/* Surface albedo, geographic latitude and longitude of the columns (ny x nx, column-major,
 * radians), copied to the device once. */
int  lgame_gpu_rad_set_surface(lgame_gpu* ctx, const double* albedo, const double* lat_geo, const double* lon_geo);
/* Features of every column of state slot `slot` at time t (Unix seconds; the zenith angle
 * is taken at t).  Computed on the device; copied to `features` (ny*nx rows, column index
 * ji + ny*(jk-1)) when it is not NULL. */
int  lgame_gpu_rad_features(lgame_gpu* ctx, int slot, double t, float* features);
/* Radiation tendency (W m^-3) of state slot `slot` from heating rates of every column
 * (host array in the row order of lgame_gpu_rad_features). */
int  lgame_gpu_rad_apply_heating(lgame_gpu* ctx, int slot, const float* heating);

/* One radiation update with the emulator: features, inference, radiation tendency, all on
 * the device.  A sample of the columns (every `sample_stride`-th, 0: none) is also computed
 * by lgame_rad_teacher on the CPU; if the RMS difference of the sampled heating rates
 * exceeds bound_k_per_day, the teacher's rates are used for every column instead.
 * report (may be NULL): [0] sampled RMS error (K/day), [1] 1 if the fallback was taken,
 * [2] columns sampled, [3] wall time of the update (s). */
int  lgame_gpu_rad_update(lgame_gpu* ctx, lgame_emu* emu, int slot, double t, int sample_stride,
                          double bound_k_per_day, double* report);

/* Attaches an emulator to the context (NULL detaches it), so that the step's own radiation
 * switch drives it: lgame_gpu_pchevi(ctx, old, new, counter, lrad_update = 1, t_0) then runs
 * lgame_gpu_rad_update(ctx, emu, old, t_0 + dtime_rad/2, sample_stride, bound_k_per_day)
 * before the substeps, as the reference's pchevi calls update_rad_fluxes(state_old, grid,
 * diag, t_0) (src/time_stepping/mo_manage_pchevi.F90:56-58), which evaluates the zenith angle
 * at t_0 + 0.5*dtime_rad (src/radiation/mo_manage_radiation_calls.F90:46-51).  The radiation
 * update synchronises (the sampled check runs on the CPU), so a step with lrad_update = 1
 * returns after its radiation update has finished.  Without an attached emulator
 * lrad_update is ignored and the radiation tendency stays what the host last set. */
int  lgame_gpu_rad_attach(lgame_gpu* ctx, lgame_emu* emu, double dtime_rad, int sample_stride,
                          double bound_k_per_day);
/* The report of the last radiation update lgame_gpu_pchevi ran (the layout of
 * lgame_gpu_rad_update's report) and the number of such updates since the attach. */
int  lgame_gpu_rad_last_report(const lgame_gpu* ctx, double* report, int* updates);

#ifdef __cplusplus
}
#endif
#endif /* LGAME_EMULATOR_H */
