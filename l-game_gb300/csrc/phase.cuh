// phase.cuh -- the phase transitions of the water constituents (calc_h2otracers_source_rates,
// src/constituents/mo_phase_trans.F90:22-330, with the thermodynamic functions of
// mo_dictionary.F90:88-476), behind the lphase_trans extension switch: the reference compiles
// the routine but never calls it, so its rates are zero in the reference's step.  With the
// switch on, k_phase_trans forms them at the first substep from state_old and its diagnosed
// temperature, one thread per cell, in FP64 in both precision modes (TO: the type of the rate
// arrays the scalar tendencies read, double in the FP64 step, float in the split step).
//
// Integer powers are the multiplication chains x*x, (x*x)*x, (x*x)*(x*x), x^3*x^2, x^3*x^3;
// x**0.5 is a correctly rounded square root; pow, exp and log are CUDA's.
#pragma once

#include "dev.cuh"
#include "surface.cuh"

namespace lg {

// saturation_pressure_over_water, mo_dictionary.F90:256-291 (Huang above 0 C, the
// Pruppacher-Klett polynomial below, in its own units, as the reference has it)
__device__ __forceinline__ double pt_sat_water(double temperature) {
  double tc = temperature - kT_0;
  if (tc > 100.0) tc = 100.0;
  if (tc > 0.0) return exp(34.494 - 4924.99 / (tc + 237.1)) / pow(tc + 105.0, 1.57);
  if (tc < -50.0) tc = -50.0;
  const double t2 = tc * tc, t3 = t2 * tc, t4 = t2 * t2;
  return 6.107799961 + 4.436518521e-1 * tc + 1.428945805e-2 * t2 + 2.650648471e-4 * t3 + 3.031240396e-6 * t4 +
         2.034080948e-8 * (t3 * t2) + 6.136820929e-11 * (t3 * t3);
}

// dsaturation_pressure_over_water_dT, mo_dictionary.F90:293-316
__device__ __forceinline__ double pt_dsat_water(double temperature) {
  const double tc = temperature - kT_0;
  if (tc > 100.0 || tc < 0.0) return 0.0;
  const double d = tc + 237.1;
  return pt_sat_water(temperature) * (4924.99 / (d * d) - 1.57 / (tc + 105.0));
}

// dsaturation_pressure_over_ice_dT with the Huang and Murphy derivatives, mo_dictionary.F90:
// 355-388, 444-476 (the blend written "+ (1-w) +")
__device__ __forceinline__ double pt_dsat_ice_huang(double temperature) {
  const double tc = temperature - kT_0;
  const double d = tc + 278.0;
  return sat_ice_huang(temperature) * (6545.8 / (d * d) - 2.0 / (tc + 868.0));
}
__device__ __forceinline__ double pt_dsat_ice_murphy(double temperature) {
  return sat_ice_murphy(temperature) * (5723.265 / (temperature * temperature) + 3.53068 / temperature - 0.00728332);
}
__device__ __forceinline__ double pt_dsat_ice(double temperature) {
  const double tc = temperature - kT_0;
  if (tc > 0.0) return 0.0;
  if (tc >= -80.0) return pt_dsat_ice_huang(temperature);
  if (tc >= -100.0) {
    const double w = (tc + 100.0) / 20.0;
    return w * pt_dsat_ice_huang(temperature) + (1.0 - w) + pt_dsat_ice_murphy(temperature);
  }
  if (temperature >= 110.0) return pt_dsat_ice_murphy(temperature);
  return 0.0;
}

// enhancement_factor_over_water / _over_ice, mo_dictionary.F90:390-412
__device__ __forceinline__ double pt_enh_water(double p) { return 1.00071 * exp(0.000000045 * p); }
__device__ __forceinline__ double pt_enh_ice(double p) { return 0.99882 * exp(0.00000008 * p); }

// enthalpy_evaporation, enthalpy_sublimation and phase_trans_heat, mo_dictionary.F90:88-110,
// 191-254 (direction 1 gas to liquid, 2 gas to solid, 3 liquid to solid)
__device__ __forceinline__ double pt_evaporation(double temperature) {
  double tl = temperature;
  if (tl < kT_0) {
    if (tl < 30.0) tl = 30.0;
    return (56579.0 - 42.212 * tl + exp(0.1149 * (281.6 - tl))) / kM_V;
  }
  if (tl > kT_0 + 100.0) tl = kT_0 + 100.0;
  return 3151378.0 - 2386.0 * tl;
}
__device__ __forceinline__ double pt_sublimation(double temperature) {
  double tl = temperature;
  if (tl < 30.0) tl = 30.0;
  if (tl > kT_0) tl = kT_0;
  const double q = tl / 123.75;
  return (46782.5 + 35.8925 * tl - 0.07414 * (tl * tl) + 541.5 * exp(-(q * q))) / kM_V;
}
__device__ __forceinline__ double pt_heat(int direction, double temperature) {
  if (direction == 1) return pt_evaporation(temperature);
  if (direction == 2) return pt_sublimation(temperature);
  return pt_sublimation(temperature) - pt_evaporation(temperature);
}

// calc_h2otracers_source_rates, one thread per cell: the rates of snow (1), rain (2), cloud ice
// (3), cloud water (4) and water vapour (nc+1) into `rates` (nc+1 fields of fstride; graupel's
// rate 5 is never written, as in the reference), the heating rate into `heat`, and with `sfc`
// (lsfc_phase_trans) at the lowest layer the evaporation from the sea and lakes and the latent
// heat flux densities into them (B.lat_lake, B.lat_sea).  Tm: the temperature diagnosed from S
// at the start of the step; ts: S's soil temperature.
template <class TM, class TO>
__global__ void k_phase_trans(Dims D, Grid<double> G, State S, const TM* __restrict__ Tm, SfcBuf B,
                              const double* __restrict__ ts, int sfc, double dtime, TO* __restrict__ rates,
                              TO* __restrict__ heat_out) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl), F = D.fstride;
  const int nc = D.nc;
  auto rho = [&](int jc) { return S.rho[q + (long long)(jc - 1) * F]; };
  const double Tc = cvt<double>(Tm[q]);
  const bool warm = Tc >= kT_0;
  const double rv = rho(nc + 2), rg = rho(nc + 1);
  const double wvp = rv * kR_V * Tc;
  const double air = (rg - rv) * kR_D * Tc + wvp;
  const double ef = warm ? pt_enh_water(air) : pt_enh_ice(air);
  const double sp = ef * (warm ? pt_sat_water(Tc) : sat_ice(Tc));
  // c_v_mass_weighted_air, mo_derived.F90:157-187
  double cv = 0.0;
  for (int jc = 1; jc <= nc; ++jc) cv = cv + rho(jc) * c_p_cond(jc, Tc);
  cv = cv + (rg - rv) * kC_D_V;
  cv = cv + rv * kC_V_V;
  // the density that changes phase: the root of a quadratic (mo_phase_trans.F90:100-112)
  const double h = pt_heat(warm ? 1 : 2, Tc);
  const double a = -kR_V * h / cv;
  const double b = kR_V * Tc - kR_V * rv * h / cv + ef * (warm ? pt_dsat_water(Tc) : pt_dsat_ice(Tc)) * h / cv;
  const double p = b / a, qq = (wvp - sp) / a;
  const double diff_density = -0.5 * p - sqrt(0.25 * (p * p) - qq);
  const double h3 = pt_heat(3, Tc);
  double r1, r2, r3, r4, rvap, heat;
  if (sp >= wvp) {  // not over-saturated: evaporation / sublimation, at most what is there
    if (warm) {
      r3 = -rho(3) / dtime;
      const double ptd = fmin(rho(4), diff_density);
      rvap = ptd / dtime;
      r4 = rho(3) / dtime - ptd / dtime;
      heat = r3 * h3 - ptd * h / dtime;
    } else {
      r4 = -rho(4) / dtime;
      const double ptd = fmin(rho(3), diff_density);
      rvap = ptd / dtime;
      r3 = rho(4) / dtime - ptd / dtime;
      heat = -r4 * h3 - ptd * h / dtime;
    }
  } else {  // over-saturated: condensation / resublimation
    if (warm) {
      r3 = -rho(3) / dtime;
      rvap = diff_density / dtime;
      r4 = rho(3) / dtime - diff_density / dtime;
      heat = r3 * h3 - diff_density * h / dtime;
    } else {
      r4 = -rho(4) / dtime;
      rvap = diff_density / dtime;
      r3 = rho(4) / dtime - diff_density / dtime;
      heat = -r4 * h3 - diff_density * h / dtime;
    }
  }
  // precipitation (:226-263)
  const double mcwc = 0.2e-3;  // maximum cloud water content
  r1 = 0.0;
  r2 = 0.0;
  if (!warm) {
    r1 = fmax(rho(3) - mcwc * rg, 0.0) / 1000.0;
    r3 = r3 - r1;
  } else {
    r2 = fmax(rho(4) - mcwc * rg, 0.0) / 1000.0;
    r4 = r4 - r2;
  }
  if (warm && rho(1) > 0.0) {
    r1 = -rho(1) / dtime;
    r2 = r2 - r1;
    heat = heat + r1 * h3;
  }
  if (!warm && rho(2) > 0.0) {
    r2 = -rho(2) / dtime;
    r1 = r1 - r2;
    heat = heat - r2 * h3;
  }
  // surface evaporation and the latent heat flux densities (:266-324)
  if (sfc && jl == D.nl) {
    const long long c = IX(D, ji, jk, 1);
    const double land = B.land[c];
    if (land < 1.0) {
      const double lake = B.lake[c], sea_fraction = 1.0 - land - lake;
      const double t1 = ts[c], sst = B.sst[c];
      const double sp_lake = (t1 >= kT_0) ? pt_enh_water(air) * pt_sat_water(t1) : pt_enh_ice(air) * sat_ice(t1);
      const double sp_sea = (sst >= kT_0) ? pt_enh_water(air) * pt_sat_water(sst) : pt_enh_ice(air) * sat_ice(sst);
      const double dd_sea = sea_fraction * (sp_sea / (kR_V * sst) - rv);
      const double dd_lake = lake * (sp_lake / (kR_V * t1) - rv);
      const double sfr = B.sfr[c], lt = G.layer_thickness[q];
      const double e_sea = fmax(0.0, dd_sea / sfr), e_lake = fmax(0.0, dd_lake / sfr);
      rvap = rvap + e_sea / lt + e_lake / lt;
      B.lat_lake[c] = -pt_heat(t1 >= kT_0 ? 1 : 2, t1) * e_lake;
      B.lat_sea[c] = -pt_heat(sst >= kT_0 ? 1 : 2, sst) * e_sea;
    }
  }
  rates[q] = cvt<TO>(r1);
  rates[q + F] = cvt<TO>(r2);
  rates[q + 2 * F] = cvt<TO>(r3);
  rates[q + 3 * F] = cvt<TO>(r4);
  rates[q + (long long)nc * F] = cvt<TO>(rvap);
  heat_out[q] = cvt<TO>(heat);
}

}  // namespace lg
