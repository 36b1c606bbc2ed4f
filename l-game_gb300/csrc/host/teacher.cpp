// teacher.cpp -- stand-in radiation scheme (CPU) that produces the training targets of the
// radiation emulator and serves as the check of its error and its fallback.
//
// The reference computes radiation with RTE+RRTMGP (src/radiation/mo_rterrtmgp_coupler.F90),
// an external package that is not part of the reference tree and cannot be built here.  In
// its place this file implements a small scheme from published methods, as a deterministic
// function of exactly the emulator's 4*nlev+2 input features (one column, layer 1 = top):
//
//   T[nlev] (K), p[nlev] dry-air pressure r_d*rho_dry*T (Pa, mo_rterrtmgp_coupler.F90:166),
//   rho_v[nlev] water vapour density, rho_o3[nlev] ozone density (kg m^-3),
//   surface albedo, cosine of the solar zenith angle mu0.
//
// Shortwave: Lacis and Hansen (1974, J. Atmos. Sci. 31, 118-133) absorptivities of water
// vapour, A_w(y) = 2.9 y / ((1 + 141.5 y)^0.635 + 5.925 y) with y the precipitable water (cm)
// along the slant path, and of ozone, A_o(x) = 0.02118 x / (1 + 0.042 x + 0.000323 x^2)
// + 1.082 x / (1 + 138.6 x)^0.805 + 0.0658 x / (1 + (103.6 x)^3) with x the ozone path
// (cm STP); magnification M = 35 / sqrt(1224 mu0^2 + 1) for the direct beam and 1.66 for
// the beam reflected at the surface.  Heating of a layer = the difference of the absorbed
// fluxes at its two interfaces.  No Rayleigh scattering, no clouds.
//
// Longwave: semi-gray two-stream Schwarzschild equations (as in gray-radiation GCMs, e.g.
// Frierson, Held and Zurita-Gotor 2006, J. Atmos. Sci. 63, 2548-2566), diffusivity 1.66,
// layer optical depth 1.66 * (kappa_v * water vapour path + kappa_d * dry air mass), layers
// isothermal at their temperature, no downward flux at the top, black surface at the
// temperature of the lowest layer.
//
// Heating rates are returned in K/day as Q / (rho c_p) with the dry-air mass of the layer
// (pressure thickness / g) and c_p of dry air.
#include "lgame_emulator.h"
#include "common.h"

#include <cmath>
#include <cstdio>
#include <vector>

namespace {

constexpr double kG = 9.80665;
constexpr double kCP = 1005.0;             // c_d_p, mo_constants.F90
constexpr double kSIGMA = 5.670374419e-8;  // Stefan-Boltzmann
constexpr double kS0 = 1361.0;             // total solar irradiance, W m^-2
constexpr double kRD = 287.057811;         // r_d, mo_constants.F90
constexpr double kKAPPA_V = 0.12;          // gray LW absorption by water vapour, m^2 kg^-1
constexpr double kKAPPA_D = 2.0e-4;        // gray LW absorption by the well-mixed gases, m^2 kg^-1
constexpr double kDIFF = 1.66;             // diffusivity factor
constexpr double kO3_CM_STP = 0.021415;    // kg m^-2 of ozone in a 1 cm STP column

double a_water(double y_cm) { return 2.9 * y_cm / (std::pow(1.0 + 141.5 * y_cm, 0.635) + 5.925 * y_cm); }
double a_ozone(double x) {
  return 0.02118 * x / (1.0 + 0.042 * x + 0.000323 * x * x) + 1.082 * x / std::pow(1.0 + 138.6 * x, 0.805) +
         0.0658 * x / (1.0 + std::pow(103.6 * x, 3.0));
}

void column(const float* f, int nl, float* hr) {
  const float* T = f;
  const float* p = f + nl;
  const float* rv = f + 2 * nl;
  const float* ro = f + 3 * nl;
  const double albedo = f[4 * nl];
  const double mu0 = f[4 * nl + 1];
  // interface pressures: midpoints, extrapolated at the top (not below 0) and at the bottom
  std::vector<double> pi(nl + 1), m(nl), uv(nl), uo(nl);
  for (int l = 1; l < nl; ++l) pi[l] = 0.5 * ((double)p[l - 1] + (double)p[l]);
  pi[0] = std::fmax(0.0, (double)p[0] - 0.5 * ((double)p[1] - (double)p[0]));
  pi[nl] = (double)p[nl - 1] + 0.5 * ((double)p[nl - 1] - (double)p[nl - 2]);
  for (int l = 0; l < nl; ++l) {
    m[l] = std::fmax(pi[l + 1] - pi[l], 1e-3) / kG;            // dry air mass, kg m^-2
    const double rho_d = (double)p[l] / (kRD * (double)T[l]);
    uv[l] = m[l] * (double)rv[l] / rho_d;                      // water vapour path, kg m^-2
    uo[l] = m[l] * (double)ro[l] / rho_d;                      // ozone path, kg m^-2
  }
  // shortwave
  std::vector<double> sw(nl, 0.0);
  if (mu0 > 0.0) {
    const double M = 35.0 / std::sqrt(1224.0 * mu0 * mu0 + 1.0);
    const double s = kS0 * mu0;
    // downward: absorbed fraction above each interface
    std::vector<double> yd(nl + 1, 0.0), xd(nl + 1, 0.0);
    for (int l = 0; l < nl; ++l) {
      yd[l + 1] = yd[l] + uv[l] * 0.1 * M;  // kg m^-2 -> cm of precipitable water
      xd[l + 1] = xd[l] + uo[l] / kO3_CM_STP * M;
    }
    auto absd = [&](int i) { return a_water(yd[i]) + a_ozone(xd[i]); };
    // after reflection at the surface: the whole slant path down plus the diffuse path from
    // the surface up to each interface (Lacis and Hansen's effective path for the reflected beam)
    std::vector<double> yu(nl + 1, 0.0), xu(nl + 1, 0.0);
    for (int l = nl - 1; l >= 0; --l) {
      yu[l] = yu[l + 1] + uv[l] * 0.1 * kDIFF;
      xu[l] = xu[l + 1] + uo[l] / kO3_CM_STP * kDIFF;
    }
    auto absu = [&](int i) { return a_water(yd[nl] + yu[i]) + a_ozone(xd[nl] + xu[i]); };
    for (int l = 0; l < nl; ++l) sw[l] = s * (absd(l + 1) - absd(l)) + s * albedo * (absu(l) - absu(l + 1));
  }
  // longwave
  std::vector<double> tr(nl), B(nl), D(nl + 1, 0.0), U(nl + 1, 0.0);
  for (int l = 0; l < nl; ++l) {
    tr[l] = std::exp(-kDIFF * (kKAPPA_V * uv[l] + kKAPPA_D * m[l]));
    const double t = T[l];
    B[l] = kSIGMA * (t * t) * (t * t);
  }
  for (int l = 0; l < nl; ++l) D[l + 1] = D[l] * tr[l] + B[l] * (1.0 - tr[l]);
  U[nl] = B[nl - 1];
  for (int l = nl - 1; l >= 0; --l) U[l] = U[l + 1] * tr[l] + B[l] * (1.0 - tr[l]);
  for (int l = 0; l < nl; ++l) {
    const double lw = (U[l + 1] - U[l]) + (D[l] - D[l + 1]);  // net flux into the layer
    const double k = 86400.0 / (m[l] * kCP);
    hr[l] = (float)(sw[l] * k);
    hr[nl + l] = (float)(lw * k);
  }
}

}  // namespace

extern "C" int lgame_rad_teacher(const float* features, long long ncol, int nlev, float* heating) {
  if (!features || !heating || ncol < 0 || nlev < 3) {
    lgame_set_error("lgame_rad_teacher: bad arguments");
    return LGAME_ERR_INVALID_ARG;
  }
  const int nf = 4 * nlev + 2;
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (long long c = 0; c < ncol; ++c) {
    const float* f = features + c * nf;
    bool ok = true;
    for (int l = 0; l < nlev; ++l) ok = ok && f[l] > 0.f && f[nlev + l] > 0.f;
    if (!ok) { bad |= 1; continue; }
    column(f, nlev, heating + c * 2 * nlev);
  }
  if (bad) {
    lgame_set_error("lgame_rad_teacher: a column has a non-positive temperature or pressure");
    return LGAME_ERR_INVALID_ARG;
  }
  return LGAME_OK;
}
