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
  // reciprocals of the soil grid's spacings, formed once on the host for the split step's
  // soil solve: 1/(zi(l) - zi(l+1)), 1/(zc(l) - zc(l+1)), 1/(2*(zc(ns) - z_t_const))
  double idzi[LGAME_MAX_SOIL_LAYERS], idzc[LGAME_MAX_SOIL_LAYERS], i2dzt;
};

// grid fields (read-only) and surface diagnostics, one padded plane each
struct SfcBuf {
  const double *land, *lake, *rl_grid, *rhoc, *tcond, *tconst;
  double *rl, *rv, *mol, *sfr, *sens_soil, *sens_sea, *sst, *sw_in, *lw_out;
  double *lat_lake, *lat_sea;  // latent heat flux densities (formed by the phase transitions)
};

// The helpers and the two kernels below are templated on the arithmetic type R: the FP64 step
// evaluates them in double in the reference's order; the split step evaluates them in float,
// as its other explicit terms (they are two-dimensional and otherwise bound by the FP64 pipe).

// roughness_length_from_u10_sea, mo_pbl.F90:253-282
template <class R>
__device__ __forceinline__ R sfc_rl_sea(R u10) {
  const R swh = R(0.0248) * (u10 * u10);
  const R period = R(0.729) * u10;
  const R wavelength = R(kGRAVITY) * (period * period) / (R(2.0) * R(kPI));
  const R r = R(1200.0) * swh * pow(swh / fmax(wavelength, R(kEPSILON_SECURITY)), R(4.5));
  return fmax(R(0.0001), r);
}

// psi_h and psi_m, mo_pbl.F90:382-433
template <class R>
__device__ __forceinline__ R sfc_psi_h(R eff, R l) {
  const R ll = fabs(l) < R(kEPSILON_SECURITY) ? R(kEPSILON_SECURITY) : l;
  if (ll < R(0)) {
    const R x = pow(R(1) - R(15.0) * eff / ll, R(0.25));
    return R(2.0) * log((R(1) + x * x) / R(2.0));
  }
  return R(-4.0) * eff / ll;
}
template <class R>
__device__ __forceinline__ R sfc_psi_m(R eff, R l) {
  const R ll = fabs(l) < R(kEPSILON_SECURITY) ? R(kEPSILON_SECURITY) : l;
  if (ll < R(0)) {
    const R x = pow(R(1) - R(15.0) * eff / ll, R(0.25));
    return R(2.0) * log((R(1) + x) / R(2.0)) + log((R(1) + x * x) / R(2.0)) - R(2.0) * atan(x) + R(kPI) / R(2.0);
  }
  return R(-4.7) * eff / ll;
}

// roughness_velocity, mo_pbl.F90:358-380
template <class R>
__device__ __forceinline__ R sfc_rough_vel(const SfcPar& P, R wind_speed, R z_agl, R rl) {
  R den = log(z_agl / rl);
  if (fabs(den) < R(kEPSILON_SECURITY)) den = R(kEPSILON_SECURITY);
  return fmax(R(kEPSILON_SECURITY), wind_speed * R(P.karman) / den);
}

// scalar_flux_resistance and momentum_flux_resistance, mo_pbl.F90:284-356
template <class R>
__device__ __forceinline__ R sfc_scalar_res(const SfcPar& P, R rv, R z_agl, R rl, R mol) {
  const R h = fmin(z_agl, R(P.h_prandtl));
  R r = R(1) / (R(P.karman) * rv) * (log(h / rl) - sfc_psi_h<R>(h, mol) + log(R(7.0)));
  if (r < R(P.dtime) / z_agl) r = R(P.dtime) / z_agl;
  return r;
}
template <class R>
__device__ __forceinline__ R sfc_mom_res(const SfcPar& P, R wind, R z_agl, R rl, R mol) {
  const R h = fmin(z_agl, R(P.h_prandtl));
  R r = R(1) / (R(P.karman) * sfc_rough_vel<R>(P, wind, z_agl, rl)) * (log(h / rl) - sfc_psi_m<R>(h, mol));
  if (r < R(P.dtime) / z_agl) r = R(P.dtime) / z_agl;
  return r;
}

// update_sfc_turb_quantities, mo_pbl.F90:19-108, one thread per column; vsq is the v_squared
// the previous step's second substep left (zero before the first step)
template <class R>
__global__ void k_sfc_turb(Dims D, Grid<double> G, State S, const double* __restrict__ vsq, SfcBuf B, SfcPar P) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const int nl = D.nl;
  const long long c = IX(D, ji, jk, 1), iN = IX(D, ji, jk, nl), iN1 = IX(D, ji, jk, nl - 1);
  const R agl = R(G.z_scalar[iN] - G.z_w[IX(D, ji, jk, D.NL)]);
  const R u_low = sqrt(R(vsq[iN]));  // v_squared**0.5_wp
  R rl = R(B.rl[c]);
  const R u10 = u_low * log(R(10.0) / rl) / log(agl / rl);
  const R land = R(B.land[c]);
  if (land < R(1)) rl = land * R(B.rl_grid[c]) + (R(1) - land) * sfc_rl_sea<R>(u10);
  B.rl[c] = rl;
  const R rv = sfc_rough_vel<R>(P, u_low, agl, rl);
  B.rv[c] = rv;
  const R tv1 = R(G.theta_v_bg[iN] + S.tp[iN]);
  const R tv2 = R(G.theta_v_bg[iN1] + S.tp[iN1]);
  const R dz = R(G.z_scalar[iN1] - G.z_scalar[iN]);
  const R dtvdz = (tv2 - tv1) / dz;
  const R w_pert = u10 * fmax(R(0.001), R(0.02) * (R(1) - dtvdz / R(0.01)));
  const R tv_pert = -(R(0.2) * R(P.dtime) * w_pert * dtvdz);
  R wt = R(0.2) * w_pert * tv_pert;
  if (fabs(wt) < R(kEPSILON_SECURITY)) wt = R(kEPSILON_SECURITY);
  const R mol = -(tv1 * ((rv * rv) * rv)) / (R(P.karman) * R(kGRAVITY) * wt);
  B.mol[c] = mol;
  if (P.prog_soil) B.sfr[c] = sfc_scalar_res<R>(P, rv, agl, rl, mol);
}

// the friction of one lowest-layer vector point between the columns (a1,b1) and (a2,b2),
// mo_pbl.F90:133-156: the acceleration that is subtracted
template <class R>
__device__ __forceinline__ R sfc_friction(const Dims& D, const Grid<double>& G, const double* vsq, const SfcBuf& B,
                                          const SfcPar& P, double z_vec, double wind, int a1, int b1, int a2, int b2) {
  const int nl = D.nl, NL = D.NL;
  const R ws = R(0.5) * (sqrt(R(vsq[IX(D, a1, b1, nl)])) + sqrt(R(vsq[IX(D, a2, b2, nl)])));
  const double zs1 = G.z_w[IX(D, a1, b1, NL)], zs2 = G.z_w[IX(D, a2, b2, NL)];
  const R z_agl = R(z_vec - 0.5 * (zs1 + zs2));
  const R lt = R(0.5 * (G.z_w[IX(D, a1, b1, nl)] + G.z_w[IX(D, a2, b2, nl)]) - 0.5 * (zs1 + zs2));
  const long long c1 = IX(D, a1, b1, 1), c2 = IX(D, a2, b2, 1);
  const R rl = R(0.5 * (B.rl[c1] + B.rl[c2]));
  const R mol = R(0.5 * (B.mol[c1] + B.mol[c2]));
  const R fr = sfc_mom_res<R>(P, ws, z_agl, rl, mol);
  R wrf = R(1);
  if (z_agl > R(P.h_prandtl)) wrf = log(R(P.h_prandtl) / rl) / log(z_agl / rl);
  return wrf * R(wind) / fr / lt;
}

// pbl_wind_tendency, mo_pbl.F90:110-251: one thread per lowest-layer u point (ji <= ny) and v
// point (jk <= nx).  With periodic boundaries the thread of the first column (row) forms the
// wrap point and writes its copy at nx+1 (ny+1), as the reference copies it.
template <class R, class T>
__global__ void k_pbl(Dims D, Grid<double> G, State S, const double* __restrict__ vsq, SfcBuf B, SfcPar P,
                      T* __restrict__ mdtx, T* __restrict__ mdty) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  const int ny = D.ny, nx = D.nx, nl = D.nl;
  if (ji <= ny && jk <= nx) {
    const long long i = IX(D, ji, jk, nl);
    if (jk >= 2) {
      const R f = sfc_friction<R>(D, G, vsq, B, P, G.z_u[i], S.u[i], ji, jk - 1, ji, jk);
      mdtx[i] = cvt<T>(cvt<R>(mdtx[i]) - f);
    } else if (D.periodic) {
      const R f = sfc_friction<R>(D, G, vsq, B, P, G.z_u[i], S.u[i], ji, nx, ji, 1);
      const T v = cvt<T>(cvt<R>(mdtx[i]) - f);
      mdtx[i] = v;
      mdtx[IX(D, ji, nx + 1, nl)] = v;
    }
    if (ji >= 2) {
      const R f = sfc_friction<R>(D, G, vsq, B, P, G.z_v[i], S.v[i], ji - 1, jk, ji, jk);
      mdty[i] = cvt<T>(cvt<R>(mdty[i]) - f);
    } else if (D.periodic) {
      const R f = sfc_friction<R>(D, G, vsq, B, P, G.z_v[i], S.v[i], ny, jk, 1, jk);
      const T v = cvt<T>(cvt<R>(mdty[i]) - f);
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
  auto zi = [&](int k) { return P.zi[k - 1]; };  // z_soil_interface, 1-based like the reference
  auto zc = [&](int k) { return P.zc[k - 1]; };  // z_soil_center, 1-based
#pragma unroll 1
  for (int jl = 1; jl <= ns - 1; ++jl)
    h[jl] = -(rc * tc * (ts_o[c + (jl - 1) * pl] - ts_o[c + jl * pl]) / (zc(jl) - zc(jl + 1)));
  h[ns] = -(rc * tc * (ts_o[c + (ns - 1) * pl] - B.tconst[c]) / (2.0 * (zc(ns) - P.z_t_const)));
  // the latent heat flux over lakes is formed only by the phase transitions, which the
  // reference's step never calls (its initial zero then; with lphase_trans, their value)
  const double lat_lake = B.lat_lake[c];
  rv[1] = ts_o[c] + (B.sens_soil[c] + lat_lake + B.sw_in[c] - B.lw_out[c] + 0.5 * h[1]) / ((zi(1) - zi(2)) * rc) * dt;
#pragma unroll 1
  for (int jl = 2; jl <= ns; ++jl)
    rv[jl] = ts_o[c + (jl - 1) * pl] + 0.5 * (-h[jl - 1] + h[jl]) / ((zi(jl) - zi(jl + 1)) * rc) * dt;
#pragma unroll 1
  for (int jl = 1; jl <= ns; ++jl) {
    const double q = 0.5 * dt * rc * tc / ((zi(jl) - zi(jl + 1)) * rc);
    if (jl == 1) dv[jl] = 1.0 + q * 1.0 / (zc(jl) - zc(jl + 1));
    else if (jl == ns) dv[jl] = 1.0 + q * 1.0 / (zc(jl - 1) - zc(jl));
    else dv[jl] = 1.0 + q * (1.0 / (zc(jl - 1) - zc(jl)) + 1.0 / (zc(jl) - zc(jl + 1)));
  }
#pragma unroll 1
  for (int jl = 1; jl <= ns - 1; ++jl) {
    cv[jl] = -(0.5 * dt * rc * tc / ((zi(jl + 1) - zi(jl + 2)) * rc) / (zc(jl) - zc(jl + 1)));
    ev[jl] = -(0.5 * dt * rc * tc / ((zi(jl) - zi(jl + 1)) * rc) / (zc(jl) - zc(jl + 1)));
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

// The split step's form of k_sfc_column: the same sensible heat flux, and the soil rows with the
// soil grid's spacings as host-formed reciprocals and the heat capacity cancelled where the
// reference multiplies and divides by it (rho_c*tc/(dz*rho_c) = tc/dz), the Thomas sweep with
// one reciprocal per row: six FP64 divisions per column where k_sfc_column has about fifty-five
// (each a sequence of FP64-pipe instructions, which bound this two-dimensional kernel).  FP64
// still, as the split step's other column solve: a step changes the soil temperature by far
// less than FP32's resolution of it.
template <class T>
__global__ void k_sfc_column_split(Dims D, Grid<double> G, State So, State Snu, T* __restrict__ trt, SfcBuf B,
                                   SfcPar P, const double* __restrict__ ts_o, const double* ts_nu, double* ts_n) {
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
    const double isfr = 1.0 / B.sfr[c], land = B.land[c], lake = B.lake[c], sst = B.sst[c];
    const double ss = (land + lake) * 0.5 * kC_D_V * (rg_n * (t_old - ts_o[c]) + rg_o * (t_new - ts_nu[c])) * isfr;
    const double se = (1.0 - land - lake) * 0.5 * kC_D_V * (rg_n * (t_old - sst) + rg_o * (t_new - sst)) * isfr;
    B.sens_soil[c] = ss;
    B.sens_sea[c] = se;
    trt[i] = cvt<T>(cvt<double>(trt[i]) - G.area_z[IX(D, ji, jk, D.NL)] * (ss + se) /
                                                ((G.exner_bg[i] + Snu.ep[i]) * kC_D_P * G.volume[i]));
  }
  if (!P.prog_soil) return;
  const int ns = P.ns;
  const double dt = P.dtime, rc = B.rhoc[c], tc = B.tcond[c], irc_dt = dt / rc, htc = 0.5 * dt * tc;
  double h[LGAME_MAX_SOIL_LAYERS + 1], cv[LGAME_MAX_SOIL_LAYERS + 1], dv[LGAME_MAX_SOIL_LAYERS + 1];
  double ev[LGAME_MAX_SOIL_LAYERS + 1], rv[LGAME_MAX_SOIL_LAYERS + 1];
  auto idzi = [&](int k) { return P.idzi[k - 1]; };  // 1-based
  auto idzc = [&](int k) { return P.idzc[k - 1]; };
  const double rct = rc * tc;
#pragma unroll 1
  for (int jl = 1; jl <= ns - 1; ++jl) h[jl] = -(rct * (ts_o[c + (jl - 1) * pl] - ts_o[c + jl * pl]) * idzc(jl));
  h[ns] = -(rct * (ts_o[c + (ns - 1) * pl] - B.tconst[c]) * P.i2dzt);
  rv[1] = ts_o[c] + (B.sens_soil[c] + B.lat_lake[c] + B.sw_in[c] - B.lw_out[c] + 0.5 * h[1]) * idzi(1) * irc_dt;
#pragma unroll 1
  for (int jl = 2; jl <= ns; ++jl)
    rv[jl] = ts_o[c + (jl - 1) * pl] + 0.5 * (h[jl] - h[jl - 1]) * idzi(jl) * irc_dt;
#pragma unroll 1
  for (int jl = 1; jl <= ns; ++jl) {
    const double q = htc * idzi(jl);
    const double above = (jl >= 2) ? idzc(jl - 1) : 0.0, below = (jl <= ns - 1) ? idzc(jl) : 0.0;
    dv[jl] = 1.0 + q * (above + below);
  }
#pragma unroll 1
  for (int jl = 1; jl <= ns - 1; ++jl) {
    cv[jl] = -(htc * idzi(jl + 1) * idzc(jl));
    ev[jl] = -(htc * idzi(jl) * idzc(jl));
  }
  // Thomas sweep, one reciprocal per row
  double inv = 1.0 / dv[1];
  ev[1] = ev[1] * inv;
  rv[1] = rv[1] * inv;
#pragma unroll 1
  for (int jl = 2; jl <= ns; ++jl) {
    inv = 1.0 / (dv[jl] - ev[jl - 1] * cv[jl - 1]);
    if (jl <= ns - 1) ev[jl] = ev[jl] * inv;
    rv[jl] = (rv[jl] - rv[jl - 1] * cv[jl - 1]) * inv;
  }
  double x = rv[ns];
  ts_n[c + (ns - 1) * pl] = x;
#pragma unroll 1
  for (int jl = ns - 1; jl >= 1; --jl) {
    x = rv[jl] - ev[jl] * x;
    ts_n[c + (jl - 1) * pl] = x;
  }
}

}  // namespace lg
