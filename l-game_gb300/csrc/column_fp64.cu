// column_fp64.cu -- the vertically implicit part of the HEVI step, FP64, one thread per
// column (compiled with -fmad=false).
//
// A warp owns 32 adjacent columns of one x-row, so every level load of every field is
// one coalesced 256-byte access.  Each thread runs the Thomas algorithm of its column
// (mo_column_solvers.F90:606-640); the forward sweep and the back substitution are
// sequential in the level index, which is why the work is spread over the ~10^6
// columns of the domain instead of over the levels (parallel cyclic reduction would
// multiply the FP64 divisions by log2(n_layers), and FP64 throughput is the scarce
// resource of this GPU).
#include "kernels.cuh"

namespace lg {

constexpr int kMaxLayers = 128;

// the Thomas algorithm of mo_column_solvers.F90:606-640 (arrays 1-based)
__device__ __forceinline__ void thomas(const double* c, const double* d, const double* e, const double* r,
                                       double* sol, double* ep, double* rp, int n) {
  ep[1] = e[1] / d[1];
  rp[1] = r[1] / d[1];
  for (int jl = 2; jl <= n; ++jl) {
    const double den = d[jl] - ep[jl - 1] * c[jl - 1];
    if (jl <= n - 1) ep[jl] = e[jl] / den;
    rp[jl] = (r[jl] - rp[jl - 1] * c[jl - 1]) / den;
  }
  sol[n] = rp[n];
  for (int jl = n - 1; jl >= 1; --jl) sol[jl] = rp[jl] - ep[jl] * sol[jl + 1];
}

// three_band_solver_ver, mo_column_solvers.F90:21-351, plus the array-wide update of
// theta_v_pert (:346-349) and w_free_slip (mo_inner_product.F90:52-75) of this column,
// both of which only touch the column itself.
__global__ void k_column_ver(Dims D, Grid<double> G, State So, State Sn, Tend<double> Tn, int rk_step) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const int nl = D.nl;
  const double dtime = D.dtime;
  const long long goff = (long long)(D.g - 1) * D.fstride;
  const State& Su = (rk_step == 1) ? So : Sn;  // state_new_used
  const double* rho_o = So.rho + goff;
  const double* rho_u = Su.rho + goff;
  double* rho_n = Sn.rho + goff;
  const double* t_rho = Tn.rho + goff;
  const double pdw = 0.5;

  double alpha[kMaxLayers + 1], beta[kMaxLayers + 1], gammaa[kMaxLayers + 1];
  double rho_expl[kMaxLayers + 1], rt_expl[kMaxLayers + 1], ep_expl[kMaxLayers + 1], tp_expl[kMaxLayers + 1];
  double rio[kMaxLayers + 1], rie[kMaxLayers + 1], ti[kMaxLayers + 1];
  double cv[kMaxLayers + 1], dv[kMaxLayers + 1], evec[kMaxLayers + 1], rv[kMaxLayers + 1];
  double sol[kMaxLayers + 1], epr[kMaxLayers + 1], rpr[kMaxLayers + 1];

  for (int jl = 1; jl <= nl; ++jl) {
    const long long i = IX(D, ji, jk, jl);
    const double V = G.volume[i];
    rho_expl[jl] = rho_o[i] + dtime * t_rho[i];
    rt_expl[jl] = So.rt[i] + dtime * Tn.rt[i];
    if (rk_step == 1) {
      alpha[jl] = -So.rt[i] / (rho_o[i] * rho_o[i]) / V;
      beta[jl] = 1.0 / rho_o[i] / V;
      gammaa[jl] = kR_D / (kC_D_V * So.rt[i]) * (G.exner_bg[i] + So.ep[i]) / V;
    } else {
      const double alpha_old = -So.rt[i] / (rho_o[i] * rho_o[i]);
      const double beta_old = 1.0 / rho_o[i];
      const double gamma_old = kR_D / (kC_D_V * So.rt[i]) * (G.exner_bg[i] + So.ep[i]);
      const double alpha_new = -Su.rt[i] / (rho_u[i] * rho_u[i]);
      const double beta_new = 1.0 / rho_u[i];
      const double gamma_new = kR_D / (kC_D_V * Su.rt[i]) * (G.exner_bg[i] + Su.ep[i]);
      alpha[jl] = ((1.0 - pdw) * alpha_old + pdw * alpha_new) / V;
      beta[jl] = ((1.0 - pdw) * beta_old + pdw * beta_new) / V;
      gammaa[jl] = ((1.0 - pdw) * gamma_old + pdw * gamma_new) / V;
    }
    tp_expl[jl] = So.tp[i] + dtime * V * (alpha[jl] * t_rho[i] + beta[jl] * Tn.rt[i]);
    ep_expl[jl] = So.ep[i] + dtime * V * gammaa[jl] * Tn.rt[i];
  }
  for (int jl = 1; jl <= nl - 1; ++jl) {
    const long long a = IX(D, ji, jk, jl), b = IX(D, ji, jk, jl + 1);
    rio[jl] = 0.5 * (rho_o[a] + rho_o[b]);
    rie[jl] = 0.5 * (rho_expl[jl] + rho_expl[jl + 1]);
    ti[jl] = 0.5 * (Su.rt[a] / rho_u[a] + Su.rt[b] / rho_u[b]);
  }
  const double c_imp2 = kIMPL_THERMO_WEIGHT * (dtime * dtime) * kC_D_P;
  const double c_imp1 = kIMPL_THERMO_WEIGHT * dtime * kC_D_P;
  for (int jl = 1; jl <= nl - 1; ++jl) {
    const long long a = IX(D, ji, jk, jl), b = IX(D, ji, jk, jl + 1);
    const double zs0 = G.z_scalar[a], zs1 = G.z_scalar[b];
    const double eb0 = G.exner_bg[a], eb1 = G.exner_bg[b];
    const double dp = G.damp[b];  // prefactor at level jl+1
    const double wo = So.w[b];
    const double t = ti[jl];
    dv[jl] = -(t * t) * (gammaa[jl] + gammaa[jl + 1])
           + 0.5 * (eb0 - eb1) * (alpha[jl + 1] - alpha[jl] + t * (beta[jl + 1] - beta[jl]))
           - (zs0 - zs1) / (c_imp2 * rio[jl])
           * (2.0 / G.area_z[b] + dtime * wo * 0.5 * (-1.0 / G.volume[a] + 1.0 / G.volume[b])) * dp;
    rv[jl] = -(wo + dtime * Tn.w[b]) * (zs0 - zs1) / c_imp2
           + t * (ep_expl[jl] - ep_expl[jl + 1]) / dtime
           + 0.5 / dtime * (tp_expl[jl] + tp_expl[jl + 1]) * (eb0 - eb1)
           - (zs0 - zs1) / c_imp2 * wo * rie[jl] / rio[jl];
  }
  for (int jl = 1; jl <= nl - 2; ++jl) {
    const long long a = IX(D, ji, jk, jl), b = IX(D, ji, jk, jl + 1), c = IX(D, ji, jk, jl + 2);
    cv[jl] = ti[jl + 1] * gammaa[jl + 1] * ti[jl]
           + 0.5 * (G.exner_bg[b] - G.exner_bg[c]) * (alpha[jl + 1] + beta[jl + 1] * ti[jl])
           - (G.z_scalar[b] - G.z_scalar[c]) / c_imp1 * 0.5 * So.w[c] / (G.volume[b] * rio[jl + 1]) * G.damp[c];
    evec[jl] = ti[jl] * gammaa[jl + 1] * ti[jl + 1]
             - 0.5 * (G.exner_bg[a] - G.exner_bg[b]) * (alpha[jl + 1] + beta[jl + 1] * ti[jl + 1])
             + (G.z_scalar[a] - G.z_scalar[b]) / c_imp1 * 0.5 * So.w[b] / (G.volume[b] * rio[jl]) * G.damp[b];
  }
  thomas(cv, dv, evec, rv, sol, epr, rpr, nl - 1);
  for (int jl = 2; jl <= nl - 1; ++jl) {
    const long long i = IX(D, ji, jk, jl);
    rho_n[i] = rho_expl[jl] + dtime * (-sol[jl - 1] + sol[jl]) / G.volume[i];
    Sn.rt[i] = rt_expl[jl] + dtime * (-(ti[jl - 1] * sol[jl - 1]) + ti[jl] * sol[jl]) / G.volume[i];
  }
  {
    const long long i1 = IX(D, ji, jk, 1), iN = IX(D, ji, jk, nl);
    rho_n[i1] = rho_expl[1] + dtime * sol[1] / G.volume[i1];
    Sn.rt[i1] = rt_expl[1] + dtime * ti[1] * sol[1] / G.volume[i1];
    rho_n[iN] = rho_expl[nl] - dtime * sol[nl - 1] / G.volume[iN];
    Sn.rt[iN] = rt_expl[nl] - dtime * ti[nl - 1] * sol[nl - 1] / G.volume[iN];
  }
  for (int jl = 2; jl <= nl; ++jl) {
    const long long i = IX(D, ji, jk, jl);
    const double rin = 0.5 * (rho_n[IX(D, ji, jk, jl - 1)] + rho_n[i]);
    Sn.w[i] = (2.0 * sol[jl - 1] / G.area_z[i] - rin * So.w[i]) / rio[jl - 1];
  }
  for (int jl = 1; jl <= nl; ++jl) {
    const long long i = IX(D, ji, jk, jl);
    Sn.ep[i] = So.ep[i] + G.volume[i] * gammaa[jl] * (Sn.rt[i] - So.rt[i]);
    Sn.tp[i] = Sn.rt[i] / rho_n[i] - G.theta_v_bg[i];
  }
  if (D.freeslip) {
    const int n = nl;
    Sn.w[IX(D, ji, jk, n + 1)] =
        W_(1, ji, jk, n) * Sn.u[IX(D, ji, jk + 1, n)] * G.slope_x[IX(D, ji, jk + 1, n)]
      + W_(2, ji, jk, n) * Sn.v[IX(D, ji, jk, n)] * G.slope_y[IX(D, ji, jk, n)]
      + W_(3, ji, jk, n) * Sn.u[IX(D, ji, jk, n)] * G.slope_x[IX(D, ji, jk, n)]
      + W_(4, ji, jk, n) * Sn.v[IX(D, ji + 1, jk, n)] * G.slope_y[IX(D, ji + 1, jk, n)];
  }
}

// v_fall_liquid, mo_derived.F90:218-263 (state_old, diag%temperature)
__device__ __forceinline__ double v_fall_liquid(const Dims& D, const Grid<double>& G, const double* rho_g,
                                                const double* T, double radius, int ji, int jk, int jl) {
  double g;
  if (jl == 1) g = G.gm[IX(D, ji, jk, jl + 1)];
  else if (jl == D.nl) g = G.gm[IX(D, ji, jk, jl)];
  else g = W_(5, ji, jk, jl) * G.gm[IX(D, ji, jk, jl)] + W_(6, ji, jk, jl) * G.gm[IX(D, ji, jk, jl + 1)];
  const long long i = IX(D, ji, jk, jl);
  const double rg = rho_g[i];
  const double nu = calc_diff_coeff(T[i], rg);
  double v = 2.0 * (radius * radius) * (kRHO_H2O - rg) * g / (9.0 * rg * nu);
  const double re = v * radius / nu;
  if (re > 10.0) v = sqrt(8.0 * radius * kRHO_H2O * g / (3.0 * rg * 0.8));
  return v;
}

// v_fall_solid, mo_derived.F90:265-283 (threshold is the default-real literal 250.e-6)
__device__ __forceinline__ double v_fall_solid(double radius) {
  return (radius > (double)250.e-6f) ? 1.0 : 0.001;
}

// three_band_solver_gen_densities, mo_column_solvers.F90:353-604, all tracers of one column.
// Quantities that the reference evaluates with the same operands for several tracers or
// twice per level are evaluated once and reused (identical bits): itw*dtime/volume, the
// cloud-droplet fall speed of a level, c_p of ice and water at the interface temperature.
// Rain and graupel use the radius diag%a_rain, which the reference never sets (zero), so
// their fall speed is exactly 0 (v_fall_liquid with radius 0 returns 0 for finite states).
__global__ void k_column_tracers(Dims D, Grid<double> G, State So, State Sn, const double* t_rho_all,
                                 const double* T, double* csh, int rk_step) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const int nl = D.nl, NL = D.NL, nc = D.nc;
  const double dtime = D.dtime;
  const double itw = 0.5, expl_weight = 1.0 - itw;
  const double* rho_g_o = So.rho + (long long)(D.g - 1) * D.fstride;
  const double snow_r = 500.e-6, ice_r = 95.e-6, cloud_r = 12.e-6;  // mo_dictionary.F90:276-318
  double vfi[kMaxLayers + 1], vfr[kMaxLayers + 1], vefv[kMaxLayers + 1], v_fall[kMaxLayers + 1];
  double cv[kMaxLayers + 1], dv[kMaxLayers + 1], evec[kMaxLayers + 1], rv[kMaxLayers + 1];
  double sol[kMaxLayers + 1], epr[kMaxLayers + 1], rpr[kMaxLayers + 1];
  double itwdtv[kMaxLayers + 1], vcloud[kMaxLayers + 1], cpi[kMaxLayers + 2], cpw[kMaxLayers + 2];
  for (int jl = 1; jl <= nl; ++jl) {
    const long long i = IX(D, ji, jk, jl);
    itwdtv[jl] = itw * dtime / G.volume[i];
    vcloud[jl] = v_fall_liquid(D, G, rho_g_o, T, cloud_r, ji, jk, jl);
    if (jl >= 2) { cpi[jl] = c_p_ice(T[i]); cpw[jl] = c_p_water(T[i]); }
  }
  for (int jc = 1; jc <= D.ncons; ++jc) {
    if (jc == D.g) continue;
    const double* rho_o = So.rho + (long long)(jc - 1) * D.fstride;
    double* rho_n = Sn.rho + (long long)(jc - 1) * D.fstride;
    const double* t_rho = t_rho_all + (long long)(jc - 1) * D.fstride;
    const bool ice = (jc - 1) % 2 == 0;
    for (int jl = 1; jl <= nl - 1; ++jl) {
      const long long a = IX(D, ji, jk, jl), b = IX(D, ji, jk, jl + 1);
      if (rk_step == 1 && jc == 1) csh[a] = 0.0;
      vfi[jl] = So.w[b];
      vfr[jl] = Sn.w[b];
      double vf;
      if (jc == 1) vf = 0.5 * (v_fall_solid(snow_r) + v_fall_solid(snow_r));
      else if (jc == 2 || jc == 5) vf = 0.0;
      else if (jc == 3) vf = 0.5 * (v_fall_solid(ice_r) + v_fall_solid(ice_r));
      else if (jc == 4) vf = 0.5 * (vcloud[jl] + vcloud[jl + 1]);
      else vf = 0.0;
      v_fall[jl] = vf;
      vfi[jl] = vfi[jl] - vf;
      vfr[jl] = vfr[jl] - vf;
      vfi[jl] = G.area_z[b] * vfi[jl];
      vfr[jl] = G.area_z[b] * vfr[jl];
      const double doi = (vfr[jl] >= 0.0) ? rho_o[b] : rho_o[a];
      const double toi = T[b];
      vfr[jl] = doi * vfr[jl];
      vefv[jl] = (jc <= nc) ? (ice ? cpi[jl + 1] : cpw[jl + 1]) * toi * vfr[jl] : 0.0;
    }
    if (rk_step == 1 && jc == 1) csh[IX(D, ji, jk, nl)] = 0.0;
    if (jc == 1) v_fall[nl] = v_fall_solid(snow_r);
    else if (jc == 2 || jc == 5) v_fall[nl] = 0.0;
    else if (jc == 3) v_fall[nl] = v_fall_solid(ice_r);
    else if (jc == 4) v_fall[nl] = vcloud[nl];
    else v_fall[nl] = 0.0;
    for (int jl = 1; jl <= nl - 1; ++jl) {
      if (vfi[jl] >= 0.0) {
        cv[jl] = 0.0;
        evec[jl] = -(itwdtv[jl] * vfi[jl]);
      } else {
        cv[jl] = itwdtv[jl + 1] * vfi[jl];
        evec[jl] = 0.0;
      }
    }
    for (int jl = 1; jl <= nl; ++jl) {
      const long long i = IX(D, ji, jk, jl);
      const double V = G.volume[i];
      if (jl == 1) {
        dv[jl] = (vfi[1] >= 0.0) ? 1.0 : 1.0 - itwdtv[jl] * vfi[1];
      } else if (jl == nl) {
        dv[jl] = (vfi[jl - 1] >= 0.0) ? 1.0 + itwdtv[jl] * vfi[jl - 1] : 1.0;
        if (jc <= nc) dv[jl] = dv[jl] + itw * v_fall[jl] * dtime * G.area_z[IX(D, ji, jk, jl + 1)] / V;
      } else {
        double d = 1.0;
        if (vfi[jl - 1] >= 0.0) d = d + itwdtv[jl] * vfi[jl - 1];
        if (vfi[jl] < 0.0) d = d - itwdtv[jl] * vfi[jl];
        dv[jl] = d;
      }
      double r = rho_o[i] + dtime * t_rho[i];
      if (jl == 1) {
        r = r + expl_weight * dtime * vfr[jl] / V;
        if (rk_step == 1 && jc <= nc) csh[i] = csh[i] + vefv[jl] / V;
      } else if (jl == nl) {
        r = r - expl_weight * dtime * vfr[jl - 1] / V;
        if (rk_step == 1 && jc <= nc) csh[i] = csh[i] - vefv[jl - 1] / V;
        if (jc <= nc) {
          r = r - expl_weight * v_fall[jl] * dtime * rho_o[i] * G.area_z[IX(D, ji, jk, jl + 1)] / V;
          if (jc > nc / 4 && rk_step == 1) {  // rain branch and cloud branch, not snow
            const double Tn = T[IX(D, ji, jk, nl)];
            csh[i] = csh[i] - v_fall[jl] * Tn * (ice ? cpi[nl] : cpw[nl]) * rho_o[IX(D, ji, jk, nl)] *
                              G.area_z[IX(D, ji, jk, NL)] / V;
          }
        }
      } else {
        r = r + expl_weight * dtime * (-vfr[jl - 1] + vfr[jl]) / V;
        if (rk_step == 1 && jc <= nc) csh[i] = csh[i] + (-vefv[jl - 1] + vefv[jl]) / V;
      }
      rv[jl] = r;
    }
    thomas(cv, dv, evec, rv, sol, epr, rpr, nl);
    for (int jl = 1; jl <= nl; ++jl) {
      double s = sol[jl];
      if (s < 0.0) s = 0.0;
      rho_n[IX(D, ji, jk, jl)] = s;
    }
  }
}

}  // namespace lg
