// surface.cuh -- the surface layer, the planetary boundary layer and the soil of the HEVI step:
//
//   k_sfc_turb     update_sfc_turb_quantities, mo_pbl.F90:19-108 (once per step, before the
//                  substeps: roughness length over the sea, roughness velocity, Monin-Obukhov
//                  length, scalar flux resistance)
//   k_pbl          pbl_wind_tendency, mo_pbl.F90:110-251 (first substep: the surface friction of
//                  the lowest layer's u and v, added to the momentum diffusion acceleration)
//   k_sfc_column   the sensible heat flux of three_band_solver_ver (mo_column_solvers.F90:80-120)
//                  and its soil rows (:128-133, 228-300, 335-340), every substep
//
// All of it is two-dimensional (one thread per column or per lowest-layer vector point) and runs
// in FP64 in both precision modes, on the FP64 state; T is the type of the arrays it adds to
// (the rhotheta_v tendency and the momentum diffusion acceleration: double in the FP64 step,
// float in the split step).  Surface fields are single padded planes (IX(D, ji, jk, 1)); the
// soil temperature has one plane per soil layer.
//
// The reference solves the soil rows in the same tridiagonal system as the vertical acoustic
// rows, but their coupling entries c(n_layers-1) and e(n_layers-1) are zero
// (mo_column_solvers.F90:289-290): the downward sweep then enters the first soil row with
// d - e'*0 = d and r - r'*0 = r, and the upward sweep leaves the atmosphere's last unknown as
// r' - 0*x = r', so solving the soil rows as a system of their own gives the same values.
#pragma once

#include "dev.cuh"
#include "lgame_gpu.h"

namespace lg {

constexpr double kGRAVITY = 9.80616;        // mo_constants.F90:21
constexpr double kEPSILON_SECURITY = 1e-10;  // mo_constants.F90:34

struct SfcPar {
  double h_prandtl, karman, dtime, z_t_const;
  int ns;         // soil layers
  int prog_soil;  // lprog_soil_temp
  int sens;       // lsfc_sensible_heat_flux
  double zi[LGAME_MAX_SOIL_LAYERS + 1], zc[LGAME_MAX_SOIL_LAYERS];  // z_soil_interface, z_soil_center
};

// grid fields (read-only) and surface diagnostics, one padded plane each
struct SfcBuf {
  const double *land, *lake, *rl_grid, *rhoc, *tcond, *tconst;
  double *rl, *rv, *mol, *sfr, *sens_soil, *sens_sea, *sst, *sw_in, *lw_out;
  double *lat_lake, *lat_sea;  // latent heat flux densities (formed by the phase transitions)
};

// roughness_length_from_u10_sea, mo_pbl.F90:253-282
__device__ __forceinline__ double sfc_rl_sea(double u10) {
  const double swh = 0.0248 * (u10 * u10);
  const double period = 0.729 * u10;
  const double wavelength = kGRAVITY * (period * period) / (2.0 * kPI);
  const double r = 1200.0 * swh * pow(swh / fmax(wavelength, kEPSILON_SECURITY), 4.5);
  return fmax(0.0001, r);
}

// psi_h and psi_m, mo_pbl.F90:382-433
__device__ __forceinline__ double sfc_psi_h(double eff, double l) {
  const double ll = fabs(l) < kEPSILON_SECURITY ? kEPSILON_SECURITY : l;
  if (ll < 0.0) {
    const double x = pow(1.0 - 15.0 * eff / ll, 0.25);
    return 2.0 * log((1.0 + x * x) / 2.0);
  }
  return -4.0 * eff / ll;
}
__device__ __forceinline__ double sfc_psi_m(double eff, double l) {
  const double ll = fabs(l) < kEPSILON_SECURITY ? kEPSILON_SECURITY : l;
  if (ll < 0.0) {
    const double x = pow(1.0 - 15.0 * eff / ll, 0.25);
    return 2.0 * log((1.0 + x) / 2.0) + log((1.0 + x * x) / 2.0) - 2.0 * atan(x) + kPI / 2.0;
  }
  return -4.7 * eff / ll;
}

// roughness_velocity, mo_pbl.F90:358-380
__device__ __forceinline__ double sfc_rough_vel(const SfcPar& P, double wind_speed, double z_agl, double rl) {
  double den = log(z_agl / rl);
  if (fabs(den) < kEPSILON_SECURITY) den = kEPSILON_SECURITY;
  return fmax(kEPSILON_SECURITY, wind_speed * P.karman / den);
}

// scalar_flux_resistance and momentum_flux_resistance, mo_pbl.F90:284-356
__device__ __forceinline__ double sfc_scalar_res(const SfcPar& P, double rv, double z_agl, double rl, double mol) {
  const double h = fmin(z_agl, P.h_prandtl);
  double r = 1.0 / (P.karman * rv) * (log(h / rl) - sfc_psi_h(h, mol) + log(7.0));
  if (r < P.dtime / z_agl) r = P.dtime / z_agl;
  return r;
}
__device__ __forceinline__ double sfc_mom_res(const SfcPar& P, double wind, double z_agl, double rl, double mol) {
  const double h = fmin(z_agl, P.h_prandtl);
  double r = 1.0 / (P.karman * sfc_rough_vel(P, wind, z_agl, rl)) * (log(h / rl) - sfc_psi_m(h, mol));
  if (r < P.dtime / z_agl) r = P.dtime / z_agl;
  return r;
}

// update_sfc_turb_quantities, mo_pbl.F90:19-108, one thread per column; vsq is the v_squared
// the previous step's second substep left (zero before the first step)
static __global__ void k_sfc_turb(Dims D, Grid<double> G, State S, const double* __restrict__ vsq, SfcBuf B, SfcPar P) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const int nl = D.nl;
  const long long c = IX(D, ji, jk, 1), iN = IX(D, ji, jk, nl), iN1 = IX(D, ji, jk, nl - 1);
  const double agl = G.z_scalar[iN] - G.z_w[IX(D, ji, jk, D.NL)];
  const double u_low = sqrt(vsq[iN]);  // v_squared**0.5_wp
  double rl = B.rl[c];
  const double u10 = u_low * log(10.0 / rl) / log(agl / rl);
  const double land = B.land[c];
  if (land < 1.0) rl = land * B.rl_grid[c] + (1.0 - land) * sfc_rl_sea(u10);
  B.rl[c] = rl;
  const double rv = sfc_rough_vel(P, u_low, agl, rl);
  B.rv[c] = rv;
  const double tv1 = G.theta_v_bg[iN] + S.tp[iN];
  const double tv2 = G.theta_v_bg[iN1] + S.tp[iN1];
  const double dz = G.z_scalar[iN1] - G.z_scalar[iN];
  const double dtvdz = (tv2 - tv1) / dz;
  const double w_pert = u10 * fmax(0.001, 0.02 * (1.0 - dtvdz / 0.01));
  const double tv_pert = -(0.2 * P.dtime * w_pert * dtvdz);
  double wt = 0.2 * w_pert * tv_pert;
  if (fabs(wt) < kEPSILON_SECURITY) wt = kEPSILON_SECURITY;
  const double mol = -(tv1 * ((rv * rv) * rv)) / (P.karman * kGRAVITY * wt);
  B.mol[c] = mol;
  if (P.prog_soil) B.sfr[c] = sfc_scalar_res(P, rv, agl, rl, mol);
}

// the friction of one lowest-layer vector point between the columns (a1,b1) and (a2,b2),
// mo_pbl.F90:133-156: the acceleration that is subtracted
__device__ __forceinline__ double sfc_friction(const Dims& D, const Grid<double>& G, const double* vsq, const SfcBuf& B,
                                               const SfcPar& P, double z_vec, double wind, int a1, int b1, int a2,
                                               int b2) {
  const int nl = D.nl, NL = D.NL;
  const double ws = 0.5 * (sqrt(vsq[IX(D, a1, b1, nl)]) + sqrt(vsq[IX(D, a2, b2, nl)]));
  const double zs1 = G.z_w[IX(D, a1, b1, NL)], zs2 = G.z_w[IX(D, a2, b2, NL)];
  const double z_agl = z_vec - 0.5 * (zs1 + zs2);
  const double lt = 0.5 * (G.z_w[IX(D, a1, b1, nl)] + G.z_w[IX(D, a2, b2, nl)]) - 0.5 * (zs1 + zs2);
  const long long c1 = IX(D, a1, b1, 1), c2 = IX(D, a2, b2, 1);
  const double rl = 0.5 * (B.rl[c1] + B.rl[c2]);
  const double mol = 0.5 * (B.mol[c1] + B.mol[c2]);
  const double fr = sfc_mom_res(P, ws, z_agl, rl, mol);
  double wrf = 1.0;
  if (z_agl > P.h_prandtl) wrf = log(P.h_prandtl / rl) / log(z_agl / rl);
  return wrf * wind / fr / lt;
}

// pbl_wind_tendency, mo_pbl.F90:110-251: one thread per lowest-layer u point (ji <= ny) and v
// point (jk <= nx).  With periodic boundaries the thread of the first column (row) forms the
// wrap point and writes its copy at nx+1 (ny+1), as the reference copies it.
template <class T>
__global__ void k_pbl(Dims D, Grid<double> G, State S, const double* __restrict__ vsq, SfcBuf B, SfcPar P,
                      T* __restrict__ mdtx, T* __restrict__ mdty) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  const int ny = D.ny, nx = D.nx, nl = D.nl;
  if (ji <= ny && jk <= nx) {
    const long long i = IX(D, ji, jk, nl);
    if (jk >= 2) {
      const double f = sfc_friction(D, G, vsq, B, P, G.z_u[i], S.u[i], ji, jk - 1, ji, jk);
      mdtx[i] = cvt<T>(cvt<double>(mdtx[i]) - f);
    } else if (D.periodic) {
      const double f = sfc_friction(D, G, vsq, B, P, G.z_u[i], S.u[i], ji, nx, ji, 1);
      const T v = cvt<T>(cvt<double>(mdtx[i]) - f);
      mdtx[i] = v;
      mdtx[IX(D, ji, nx + 1, nl)] = v;
    }
    if (ji >= 2) {
      const double f = sfc_friction(D, G, vsq, B, P, G.z_v[i], S.v[i], ji - 1, jk, ji, jk);
      mdty[i] = cvt<T>(cvt<double>(mdty[i]) - f);
    } else if (D.periodic) {
      const double f = sfc_friction(D, G, vsq, B, P, G.z_v[i], S.v[i], ny, jk, 1, jk);
      const T v = cvt<T>(cvt<double>(mdty[i]) - f);
      mdty[i] = v;
      mdty[IX(D, ny + 1, jk, nl)] = v;
    }
  }
}

// The surface part of three_band_solver_ver, one thread per column: with the sensible heat flux
// on, the power flux densities into the soil and the sea (from state_old and state_new_used,
// Snu) and their heating of the lowest layer, added to its rhotheta_v tendency; with the
// prognostic soil, the soil temperature of state_new from its own tridiagonal system.
template <class T>
__global__ void k_sfc_column(Dims D, Grid<double> G, State So, State Snu, T* __restrict__ trt, SfcBuf B, SfcPar P,
                             const double* __restrict__ ts_o, const double* ts_nu, double* ts_n) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const int nl = D.nl;
  const long long c = IX(D, ji, jk, 1), i = IX(D, ji, jk, nl);
  const long long pl = D.plane;
  if (P.sens) {
    const long long gd = (long long)(D.g - 1) * D.fstride, gv = (long long)D.g * D.fstride;
    const double rg_o = So.rho[i + gd], rg_n = Snu.rho[i + gd];
    double t_old = (G.exner_bg[i] + So.ep[i]) * (G.theta_v_bg[i] + So.tp[i]);
    double t_new = (G.exner_bg[i] + Snu.ep[i]) * (G.theta_v_bg[i] + Snu.tp[i]);
    if (D.lmoist) {
      t_old = t_old / (1.0 + So.rho[i + gv] / rg_o * (kM_D / kM_V - 1.0));
      t_new = t_new / (1.0 + Snu.rho[i + gv] / rg_n * (kM_D / kM_V - 1.0));
    }
    const double sfr = B.sfr[c], land = B.land[c], lake = B.lake[c], sst = B.sst[c];
    const double ss = (land + lake) * 0.5 * kC_D_V * (rg_n * (t_old - ts_o[c]) + rg_o * (t_new - ts_nu[c])) / sfr;
    const double se = (1.0 - land - lake) * 0.5 * kC_D_V * (rg_n * (t_old - sst) + rg_o * (t_new - sst)) / sfr;
    B.sens_soil[c] = ss;
    B.sens_sea[c] = se;
    trt[i] = cvt<T>(cvt<double>(trt[i]) - G.area_z[IX(D, ji, jk, D.NL)] * (ss + se) /
                                                ((G.exner_bg[i] + Snu.ep[i]) * kC_D_P) / G.volume[i]);
  }
  if (!P.prog_soil) return;
  // soil rows, mo_column_solvers.F90:228-300, 1-based like the reference (index 0 unused)
  const int ns = P.ns;
  const double dt = P.dtime, rc = B.rhoc[c], tc = B.tcond[c];
  double h[LGAME_MAX_SOIL_LAYERS + 1], cv[LGAME_MAX_SOIL_LAYERS + 1], dv[LGAME_MAX_SOIL_LAYERS + 1];
  double ev[LGAME_MAX_SOIL_LAYERS + 1], rv[LGAME_MAX_SOIL_LAYERS + 1];
  const double* zi = P.zi - 1;
  const double* zc = P.zc - 1;
#pragma unroll 1
  for (int jl = 1; jl <= ns - 1; ++jl)
    h[jl] = -(rc * tc * (ts_o[c + (jl - 1) * pl] - ts_o[c + jl * pl]) / (zc[jl] - zc[jl + 1]));
  h[ns] = -(rc * tc * (ts_o[c + (ns - 1) * pl] - B.tconst[c]) / (2.0 * (zc[ns] - P.z_t_const)));
  // the latent heat flux over lakes is formed only by the phase transitions, which the
  // reference's step never calls (its initial zero then; with lphase_trans, their value)
  const double lat_lake = B.lat_lake[c];
  rv[1] = ts_o[c] + (B.sens_soil[c] + lat_lake + B.sw_in[c] - B.lw_out[c] + 0.5 * h[1]) / ((zi[1] - zi[2]) * rc) * dt;
#pragma unroll 1
  for (int jl = 2; jl <= ns; ++jl)
    rv[jl] = ts_o[c + (jl - 1) * pl] + 0.5 * (-h[jl - 1] + h[jl]) / ((zi[jl] - zi[jl + 1]) * rc) * dt;
#pragma unroll 1
  for (int jl = 1; jl <= ns; ++jl) {
    const double q = 0.5 * dt * rc * tc / ((zi[jl] - zi[jl + 1]) * rc);
    if (jl == 1) dv[jl] = 1.0 + q * 1.0 / (zc[jl] - zc[jl + 1]);
    else if (jl == ns) dv[jl] = 1.0 + q * 1.0 / (zc[jl - 1] - zc[jl]);
    else dv[jl] = 1.0 + q * (1.0 / (zc[jl - 1] - zc[jl]) + 1.0 / (zc[jl] - zc[jl + 1]));
  }
#pragma unroll 1
  for (int jl = 1; jl <= ns - 1; ++jl) {
    cv[jl] = -(0.5 * dt * rc * tc / ((zi[jl + 1] - zi[jl + 2]) * rc) / (zc[jl] - zc[jl + 1]));
    ev[jl] = -(0.5 * dt * rc * tc / ((zi[jl] - zi[jl + 1]) * rc) / (zc[jl] - zc[jl + 1]));
  }
  // thomas_algorithm, mo_column_solvers.F90:606-640 (e' into ev, r' into rv)
  ev[1] = ev[1] / dv[1];
#pragma unroll 1
  for (int jl = 2; jl <= ns - 1; ++jl) ev[jl] = ev[jl] / (dv[jl] - ev[jl - 1] * cv[jl - 1]);
  rv[1] = rv[1] / dv[1];
#pragma unroll 1
  for (int jl = 2; jl <= ns; ++jl) rv[jl] = (rv[jl] - rv[jl - 1] * cv[jl - 1]) / (dv[jl] - ev[jl - 1] * cv[jl - 1]);
  double x = rv[ns];
  ts_n[c + (ns - 1) * pl] = x;
#pragma unroll 1
  for (int jl = ns - 1; jl >= 1; --jl) {
    x = rv[jl] - ev[jl] * x;
    ts_n[c + (jl - 1) * pl] = x;
  }
}

}  // namespace lg
