// setup.cpp -- grid, background state and idealised initial state on the host.
//
// Restates the set-up the reference runs once before its time loop:
//   grid_setup   src/io/mo_grid_generator.F90:29-1387 (idealised-orography branches)
//   bg_setup     src/io/mo_grid_generator.F90:1389-1457
//   ideal_init   src/io/mo_set_initial_state.F90:22-257, unessential_ideal_init :322-382
// Arrays use the reference's column-major layout and extents, so the result can be
// handed to lgame_gpu_set_grid / lgame_gpu_set_state unchanged.  Two generators have
// no reference counterpart and are documented where they are defined: orography_id 5
// (seeded Gaussian hills) and scenario "baroclinic_jet" (seeded moist jet).
#include "lgame_host.h"
#include "common.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

// physical constants, src/mo_constants.F90:12-44
constexpr double r_e = 6371000.789927;
constexpr double p_0 = 100000.0;
constexpr double omega = 7.292115e-5;
constexpr double gravity = 9.80616;
constexpr double r_d = 287.057811;
constexpr double c_d_p = 1005.0;
constexpr double M_PI_ = 3.14159265358979323846;
constexpr double lapse_rate = 0.0065;
constexpr double surface_temp = 288.15;
constexpr double tropo_height = 11000.0;
constexpr double inv_height = 20000.0;
constexpr double t_grad_inv = 0.001;
constexpr double p_0_standard = 101325.0;
constexpr double n_a = 6.02214076e23;
const double m_d = n_a * 0.004810e-23;
const double m_v = n_a * 0.002991e-23;

using Vec = std::vector<double>;

// Deterministic, platform-independent random numbers (splitmix64); the host setup
// runs on x86 and on the Arm GPU host and must give the same fields on both.
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double normal() {  // Box-Muller
    double u1 = uniform(), u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI_ * u2);
  }
};

}  // namespace

struct lgame_host_model {
  lgame_namelist nml;
  int ny, nx, nl, NL, nf, no;
  // grid
  Vec lat_scalar, lon_scalar, lat_geo_scalar, lon_geo_scalar, lat_geo_u, lon_geo_u, dir_geo_u;
  Vec lat_geo_v, lon_geo_v, dir_geo_v, dir_geo_u_scalar;
  Vec z_scalar, oro, oro_smoothed, dx, dy, dz, z_u, z_v, z_w, gravity_potential, gravity_m_v, volume;
  Vec area_x, area_y, area_z, slope_x, slope_y, ipw, area_dual_x, area_dual_y, area_dual_z, z_area_dual_z;
  Vec fvec_x, fvec_y, fvec_z, trsk_u, trsk_v, exner_bg_grad_u, exner_bg_grad_v, exner_bg_grad_w;
  Vec theta_v_bg, exner_bg, sfc_albedo, dx_dual, dy_dual, layer_thickness;
  // surface and soil (grid%roughness_length is `roughness_length`)
  Vec land_fraction, lake_fraction, roughness_length, sfc_rho_c, t_conduc_soil, t_const_soil;
  Vec z_soil_interface, z_soil_center, z_t_const;
  // state
  Vec rho, rhotheta_v, theta_v_pert, exner_pert, wind_u, wind_v, wind_w, temperature_soil;
  // carried diagnostics (only the ones the set-up writes; the rest start at zero)
  Vec diag[LGAME_DIAG_NFIELDS];

  size_t IS(int i, int j, int k) const { return (size_t)(i - 1) + (size_t)ny * ((size_t)(j - 1) + (size_t)nx * (size_t)(k - 1)); }
  size_t IU(int i, int j, int k) const { return (size_t)(i - 1) + (size_t)ny * ((size_t)(j - 1) + (size_t)(nx + 1) * (size_t)(k - 1)); }
  size_t IV(int i, int j, int k) const { return (size_t)(i - 1) + (size_t)(ny + 1) * ((size_t)(j - 1) + (size_t)nx * (size_t)(k - 1)); }
  size_t IZ(int i, int j, int k) const { return (size_t)(i - 1) + (size_t)(ny + 1) * ((size_t)(j - 1) + (size_t)(nx + 1) * (size_t)(k - 1)); }
  size_t I2(int i, int j) const { return (size_t)(i - 1) + (size_t)ny * (size_t)(j - 1); }
  double& W(int n, int i, int j, int k) { return ipw[(size_t)(n - 1) + 6 * IS(i, j, k)]; }
};

namespace {

using M = lgame_host_model;

// ---- geometry helpers, mo_grid_generator.F90:1598-1706 ----------------------
double patch_area(const M& m, double center_lat, double dx_as_angle, double dy_as_angle) {
  double a = (r_e * r_e) * dx_as_angle * (std::sin(center_lat + 0.5 * dy_as_angle) - std::sin(center_lat - 0.5 * dy_as_angle));
  if (m.nml.lplane) a = (r_e * r_e) * dx_as_angle * dy_as_angle;
  return a;
}
double vertical_face_area(const M& m, double lower_z, double upper_z, double lower_length) {
  double a = 0.5 * lower_length * (r_e + upper_z + r_e + lower_z) / (r_e + lower_z) * (upper_z - lower_z);
  if (m.nml.lplane) a = lower_length * (upper_z - lower_z);
  return a;
}
void find_global_normal(double lat, double lon, double r[3]) {
  r[0] = std::cos(lat) * std::cos(lon);
  r[1] = std::cos(lat) * std::sin(lon);
  r[2] = std::sin(lat);
}
void find_geos(const double r[3], double* lat, double* lon) {
  *lat = std::asin(r[2] / std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]));
  *lon = std::atan2(r[1], r[0]);
}
void calc_local_i(double lon, double v[3]) { v[0] = -std::sin(lon); v[1] = std::cos(lon); v[2] = 0.0; }
void calc_local_j(double lat, double lon, double v[3]) {
  v[0] = -std::sin(lat) * std::cos(lon); v[1] = -std::sin(lat) * std::sin(lon); v[2] = std::cos(lat);
}
void matvec(const double a[3][3], const double x[3], double y[3]) {
  for (int i = 0; i < 3; ++i) y[i] = a[i][0] * x[0] + a[i][1] * x[1] + a[i][2] * x[2];
}
double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// ---- background profiles, mo_set_initial_state.F90:384-438 -------------------
double bg_temp(double h) {
  if (h < tropo_height) return surface_temp - lapse_rate * h;
  if (h < inv_height) return surface_temp - lapse_rate * tropo_height;
  return surface_temp - lapse_rate * tropo_height + t_grad_inv * (h - inv_height);
}
bool bg_pres(double h, double* p) {
  if (h < inv_height) {
    *p = p_0_standard * std::pow(1.0 - lapse_rate * h / surface_temp, gravity / (r_d * lapse_rate));
    return true;
  }
  return false;  // "Argument of bg_pres is above the inversion height." (:416-420)
}
double geopot(const M& m, double h) {
  double g = -gravity * (r_e * r_e) / (r_e + h) + gravity * r_e;
  if (m.nml.lplane) g = gravity * h;
  return g;
}

// ---- host operators used by the set-up (mo_gradient_operators.F90) -----------
void grad_hor_cov(M& m, const Vec& s, Vec& rx, Vec& ry) {
  const int ny = m.ny, nx = m.nx, nl = m.nl;
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 2; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji)
        rx[m.IU(ji, jk, jl)] = (s[m.IS(ji, jk, jl)] - s[m.IS(ji, jk - 1, jl)]) / m.dx[m.IU(ji, jk, jl)];
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 2; ji <= ny; ++ji)
        ry[m.IV(ji, jk, jl)] = (s[m.IS(ji - 1, jk, jl)] - s[m.IS(ji, jk, jl)]) / m.dy[m.IV(ji, jk, jl)];
  if (m.nml.lperiodic) {
    for (int jl = 1; jl <= nl; ++jl)
      for (int ji = 1; ji <= ny; ++ji) {
        rx[m.IU(ji, 1, jl)] = (s[m.IS(ji, 1, jl)] - s[m.IS(ji, nx, jl)]) / m.dx[m.IU(ji, 1, jl)];
        rx[m.IU(ji, nx + 1, jl)] = rx[m.IU(ji, 1, jl)];
      }
    for (int jl = 1; jl <= nl; ++jl)
      for (int jk = 1; jk <= nx; ++jk) {
        ry[m.IV(1, jk, jl)] = (s[m.IS(ny, jk, jl)] - s[m.IS(1, jk, jl)]) / m.dy[m.IV(1, jk, jl)];
        ry[m.IV(ny + 1, jk, jl)] = ry[m.IV(1, jk, jl)];
      }
  }
}
void grad_vert(M& m, const Vec& s, Vec& rz) {
#pragma omp parallel for schedule(static)
  for (int jl = 2; jl <= m.nl; ++jl)
    for (int jk = 1; jk <= m.nx; ++jk)
      for (int ji = 1; ji <= m.ny; ++ji)
        rz[m.IS(ji, jk, jl)] = (s[m.IS(ji, jk, jl - 1)] - s[m.IS(ji, jk, jl)]) / m.dz[m.IS(ji, jk, jl)];
}
double remap_x(M& m, const Vec& vc, int ji, int jk, int jl) {  // mo_averaging.F90:56-95
  const int nx = m.nx, nl = m.nl;
  double r = 0.0;
  if (jk == 1 || jk == nx + 1) {
    if (!m.nml.lperiodic) return r;
    r = r + m.W(5, ji, nx, jl) * vc[m.IS(ji, nx, jl)];
    r = r + m.W(5, ji, 1, jl) * vc[m.IS(ji, 1, jl)];
    if (jl < nl || m.nml.lfreeslip) {
      r = r + m.W(6, ji, nx, jl) * vc[m.IS(ji, nx, jl + 1)];
      r = r + m.W(6, ji, 1, jl) * vc[m.IS(ji, 1, jl + 1)];
    }
  } else {
    r = r + m.W(5, ji, jk - 1, jl) * vc[m.IS(ji, jk - 1, jl)];
    r = r + m.W(5, ji, jk, jl) * vc[m.IS(ji, jk, jl)];
    if (jl < nl || m.nml.lfreeslip) {
      r = r + m.W(6, ji, jk - 1, jl) * vc[m.IS(ji, jk - 1, jl + 1)];
      r = r + m.W(6, ji, jk, jl) * vc[m.IS(ji, jk, jl + 1)];
    }
  }
  return 0.5 * r;
}
double remap_y(M& m, const Vec& vc, int ji, int jk, int jl) {  // mo_averaging.F90:97-136
  const int ny = m.ny, nl = m.nl;
  double r = 0.0;
  if (ji == 1 || ji == ny + 1) {
    if (!m.nml.lperiodic) return r;
    r = r + m.W(5, ny, jk, jl) * vc[m.IS(ny, jk, jl)];
    r = r + m.W(5, 1, jk, jl) * vc[m.IS(1, jk, jl)];
    if (jl < nl || m.nml.lfreeslip) {
      r = r + m.W(6, ny, jk, jl) * vc[m.IS(ny, jk, jl + 1)];
      r = r + m.W(6, 1, jk, jl) * vc[m.IS(1, jk, jl + 1)];
    }
  } else {
    r = r + m.W(5, ji - 1, jk, jl) * vc[m.IS(ji - 1, jk, jl)];
    r = r + m.W(5, ji, jk, jl) * vc[m.IS(ji, jk, jl)];
    if (jl < nl || m.nml.lfreeslip) {
      r = r + m.W(6, ji - 1, jk, jl) * vc[m.IS(ji - 1, jk, jl + 1)];
      r = r + m.W(6, ji, jk, jl) * vc[m.IS(ji, jk, jl + 1)];
    }
  }
  return 0.5 * r;
}
void grad_hor(M& m, const Vec& s, Vec& rx, Vec& ry, const Vec& rz) {
  grad_hor_cov(m, s, rx, ry);
#pragma omp parallel for schedule(static)
  for (int jl = m.nf + 1; jl <= m.nl; ++jl)
    for (int jk = 1; jk <= m.nx + 1; ++jk)
      for (int ji = 1; ji <= m.ny; ++ji)
        rx[m.IU(ji, jk, jl)] = rx[m.IU(ji, jk, jl)] - m.slope_x[m.IU(ji, jk, jl)] * remap_x(m, rz, ji, jk, jl);
#pragma omp parallel for schedule(static)
  for (int jl = m.nf + 1; jl <= m.nl; ++jl)
    for (int jk = 1; jk <= m.nx; ++jk)
      for (int ji = 1; ji <= m.ny + 1; ++ji)
        ry[m.IV(ji, jk, jl)] = ry[m.IV(ji, jk, jl)] - m.slope_y[m.IV(ji, jk, jl)] * remap_y(m, rz, ji, jk, jl);
}

int fail(int code, const std::string& msg) {
  lgame_set_error(msg.c_str());
  return code;
}

// x coordinate of the idealised mountains, mo_grid_generator.F90:707
double x_coord_of(const M& m, int jk) { return m.nml.dx * jk - (m.nml.nx / 2 + 1) * m.nml.dx; }

// ---- grid_setup, mo_grid_generator.F90:29-1387 ------------------------------
int grid_setup(M& m) {
  const lgame_namelist& n = m.nml;
  const int ny = m.ny, nx = m.nx, nl = m.nl, NL = m.NL, nf = m.nf;
  const double dlat = n.dy / r_e, dlon = n.dx / r_e;
  const double lat_left_upper = (ny - 1.0) / 2.0 * dlat;
  const double lon_left_upper = -((nx - 1.0) / 2.0 * dlon);
  for (int ji = 1; ji <= ny; ++ji) {
    m.lat_scalar[ji - 1] = lat_left_upper - dlat * (ji - 1.0);
    for (int jk = 1; jk <= nx; ++jk) m.lat_geo_scalar[m.I2(ji, jk)] = m.lat_scalar[ji - 1];
  }
  for (int jk = 1; jk <= nx; ++jk) {
    m.lon_scalar[jk - 1] = lon_left_upper + dlon * (jk - 1.0);
    for (int ji = 1; ji <= ny; ++ji) m.lon_geo_scalar[m.I2(ji, jk)] = m.lon_scalar[jk - 1];
  }
  for (int jk = 1; jk <= nx + 1; ++jk)
    for (int ji = 1; ji <= ny; ++ji) {
      m.lat_geo_u[m.IU(ji, jk, 1)] = m.lat_scalar[ji - 1];
      m.lon_geo_u[m.IU(ji, jk, 1)] = (jk == nx + 1) ? m.lon_scalar[jk - 2] + 0.5 * dlon : m.lon_scalar[jk - 1] - 0.5 * dlon;
    }
  for (int jk = 1; jk <= nx; ++jk)
    for (int ji = 1; ji <= ny + 1; ++ji) {
      m.lat_geo_v[m.IV(ji, jk, 1)] = (ji == ny + 1) ? m.lat_scalar[ji - 2] - 0.5 * dlat : m.lat_scalar[ji - 1] + 0.5 * dlat;
      m.lon_geo_v[m.IV(ji, jk, 1)] = m.lon_scalar[jk - 1];
    }
  // rotation, :192-210
  double rot_y[3][3] = {{std::cos(n.lat_center), 0.0, -std::sin(n.lat_center)},
                        {0.0, 1.0, 0.0},
                        {std::sin(n.lat_center), 0.0, std::cos(n.lat_center)}};
  double rot_z[3][3] = {{std::cos(n.lon_center), -std::sin(n.lon_center), 0.0},
                        {std::sin(n.lon_center), std::cos(n.lon_center), 0.0},
                        {0.0, 0.0, 1.0}};
  double rot[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) rot[i][j] = rot_z[i][0] * rot_y[0][j] + rot_z[i][1] * rot_y[1][j] + rot_z[i][2] * rot_y[2][j];
  double r_old[3], r_new[3], b_old[3], b_new[3], li[3], lj[3];
  for (int jk = 1; jk <= nx; ++jk)
    for (int ji = 1; ji <= ny; ++ji) {
      double& lat = m.lat_geo_scalar[m.I2(ji, jk)];
      double& lon = m.lon_geo_scalar[m.I2(ji, jk)];
      calc_local_i(lon, b_old);
      find_global_normal(lat, lon, r_old);
      matvec(rot, r_old, r_new);
      find_geos(r_new, &lat, &lon);
      calc_local_i(lon, li); calc_local_j(lat, lon, lj);
      matvec(rot, b_old, b_new);
      m.dir_geo_u_scalar[m.I2(ji, jk)] = std::atan2(dot3(lj, b_new), dot3(li, b_new));
    }
  for (int jk = 1; jk <= nx + 1; ++jk)
    for (int ji = 1; ji <= ny; ++ji) {
      double& lat = m.lat_geo_u[m.IU(ji, jk, 1)];
      double& lon = m.lon_geo_u[m.IU(ji, jk, 1)];
      calc_local_i(lon, b_old);
      find_global_normal(lat, lon, r_old);
      matvec(rot, r_old, r_new);
      find_geos(r_new, &lat, &lon);
      calc_local_i(lon, li); calc_local_j(lat, lon, lj);
      matvec(rot, b_old, b_new);
      m.dir_geo_u[m.IU(ji, jk, 1)] = std::atan2(dot3(lj, b_new), dot3(li, b_new));
    }
  for (int jk = 1; jk <= nx; ++jk)
    for (int ji = 1; ji <= ny + 1; ++ji) {
      double& lat = m.lat_geo_v[m.IV(ji, jk, 1)];
      double& lon = m.lon_geo_v[m.IV(ji, jk, 1)];
      calc_local_j(lat, lon, b_old);
      find_global_normal(lat, lon, r_old);
      matvec(rot, r_old, r_new);
      find_geos(r_new, &lat, &lon);
      calc_local_i(lon, li); calc_local_j(lat, lon, lj);
      matvec(rot, b_old, b_new);
      m.dir_geo_v[m.IV(ji, jk, 1)] = std::atan2(dot3(lj, b_new), dot3(li, b_new));
    }
  // Coriolis vector, :284-320
  for (int jk = 1; jk <= nx; ++jk)
    for (int ji = 1; ji <= ny + 1; ++ji) {
      const double yb = std::sin(m.dir_geo_v[m.IV(ji, jk, 1)] - 0.5 * M_PI_);
      m.fvec_x[m.IV(ji, jk, 1)] = 2.0 * omega * std::cos(m.lat_geo_v[m.IV(ji, jk, 1)]) * yb;
    }
  for (int jk = 1; jk <= nx + 1; ++jk)
    for (int ji = 1; ji <= ny; ++ji) {
      const double yb = std::sin(m.dir_geo_u[m.IU(ji, jk, 1)] + 0.5 * M_PI_);
      m.fvec_y[m.IU(ji, jk, 1)] = 2.0 * omega * std::cos(m.lat_geo_u[m.IU(ji, jk, 1)]) * yb;
    }
  for (int jk = 1; jk <= nx + 1; ++jk)
    for (int ji = 1; ji <= ny + 1; ++ji) {
      double lat = (ji == ny + 1) ? m.lat_scalar[ji - 2] - 0.5 * dlat : m.lat_scalar[ji - 1] + 0.5 * dlat;
      double lon = (jk == nx + 1) ? m.lon_scalar[jk - 2] + 0.5 * dlon : m.lon_scalar[jk - 1] - 0.5 * dlon;
      find_global_normal(lat, lon, r_old);
      matvec(rot, r_old, r_new);
      find_geos(r_new, &lat, &lon);
      m.fvec_z[m.IZ(ji, jk, 1)] = 2.0 * omega * std::sin(lat);
    }
  // orography, :325-737
  switch (n.orography_id) {
    case 0:  // mean surface temperature of an Earth without orography, :333
      for (size_t p = 0; p < m.t_const_soil.size(); ++p) m.t_const_soil[p] = 273.15 + 25.0 * std::cos(2.0 * m.lat_geo_scalar[p]);
      break;
    case 2: {  // Schaer wave test, :703-711
      const double h = 250.0;
      for (int jk = 1; jk <= nx; ++jk) {
        const double x = x_coord_of(m, jk);
        const double c = std::cos(M_PI_ * x / 4000.0);
        const double o = h * std::exp(-(x * x) / (5000.0 * 5000.0)) * (c * c);
        const double os = 0.5 * h * std::exp(-(x * x) / (5000.0 * 5000.0));
        for (int ji = 1; ji <= ny; ++ji) { m.oro[m.I2(ji, jk)] = o; m.oro_smoothed[m.I2(ji, jk)] = os; }
      }
      break;
    }
    case 3: {  // Schaer advection test, :714-725
      const double h = 3000.0;
      for (int jk = 1; jk <= nx; ++jk) {
        const double x = x_coord_of(m, jk);
        double o = 0.0;
        if (std::fabs(x) <= 25e3) {
          const double c1 = std::cos(0.5 * M_PI_ * x / 25000.0), c2 = std::cos(M_PI_ * x / 8000.0);
          o = h * (c1 * c1) * (c2 * c2);
        }
        for (int ji = 1; ji <= ny; ++ji) m.oro[m.I2(ji, jk)] = o;
      }
      break;
    }
    case 4: {  // Gaussian mountain, :728-735
      const double h = 500.0;
      for (int jk = 1; jk <= nx; ++jk) {
        const double x = x_coord_of(m, jk);
        const double e = std::exp(-(x * x) / (4.0 * (5000.0 * 5000.0)));
        for (int ji = 1; ji <= ny; ++ji) m.oro[m.I2(ji, jk)] = h * (e * e);
      }
      break;
    }
    case 5: {
      // No reference counterpart: the sum of n_hills Gaussian hills with heights
      // U[hill_height_min,hill_height_max], half-widths U[hill_width_min,hill_width_max]
      // and centres uniform over the domain, drawn from a splitmix64 stream seeded by
      // &gpu seed.  On a periodic domain the distance to each centre is the shortest
      // periodic distance, so the orography is periodic too.  oro_smoothed = 0.5*oro.  The
      // soil's constant deep temperature is that of orography_id 0.
      for (size_t p = 0; p < m.t_const_soil.size(); ++p) m.t_const_soil[p] = 273.15 + 25.0 * std::cos(2.0 * m.lat_geo_scalar[p]);
      Rng rng((uint64_t)n.seed);
      const double Lx = nx * n.dx, Ly = ny * n.dy;
      std::vector<double> hh(n.n_hills), ww(n.n_hills), xc(n.n_hills), yc(n.n_hills);
      for (int h = 0; h < n.n_hills; ++h) {
        hh[h] = n.hill_height_min + (n.hill_height_max - n.hill_height_min) * rng.uniform();
        ww[h] = n.hill_width_min + (n.hill_width_max - n.hill_width_min) * rng.uniform();
        xc[h] = Lx * rng.uniform();
        yc[h] = Ly * rng.uniform();
      }
      for (int jk = 1; jk <= nx; ++jk)
        for (int ji = 1; ji <= ny; ++ji) {
          const double x = (jk - 0.5) * n.dx, y = (ji - 0.5) * n.dy;
          double o = 0.0;
          for (int h = 0; h < n.n_hills; ++h) {
            double ddx = std::fabs(x - xc[h]), ddy = std::fabs(y - yc[h]);
            if (n.lperiodic) { ddx = std::fmin(ddx, Lx - ddx); ddy = std::fmin(ddy, Ly - ddy); }
            // half-width w: the hill falls to half its height at distance w
            const double q = (ddx * ddx + ddy * ddy) / (ww[h] * ww[h]);
            o += hh[h] * std::exp(-std::log(2.0) * q);
          }
          m.oro[m.I2(ji, jk)] = o;
          m.oro_smoothed[m.I2(ji, jk)] = 0.5 * o;
        }
      break;
    }
    default:
      return fail(LGAME_ERR_UNSUPPORTED, "orography_id " + std::to_string(n.orography_id) +
                  " needs external data (netCDF) that this host does not read; use 0, 2, 3, 4 or 5");
  }
  for (int jk = 1; jk <= nx; ++jk)
    for (int ji = 1; ji <= ny; ++ji) m.z_w[m.IS(ji, jk, NL)] = m.oro[m.I2(ji, jk)];
  // physical surface properties (lread_geo=.false. branch, :746-813): water everywhere, land
  // for the seabreeze mask, no lakes; albedo, roughness length (of an idealised vegetation
  // height, :1636-1652), volumetric heat capacity and temperature conductivity
  for (int jk = 1; jk <= nx; ++jk)
    for (int ji = 1; ji <= ny; ++ji) {
      const size_t p = m.I2(ji, jk);
      if (std::string(n.scenario) == "seabreeze" && jk >= nx / 4 && jk <= 3 * nx / 4) m.land_fraction[p] = 1.0;
      const double land = m.land_fraction[p], lake = m.lake_fraction[p];
      m.sfc_albedo[p] = 0.06;
      m.roughness_length[p] = 0.08;
      m.sfc_rho_c[p] = 1024.0 * 4184.0;
      m.t_conduc_soil[p] = 1.4e-7;
      if (land > 1e-10) {
        m.t_conduc_soil[p] = (land * 7.5e-7 + lake * 1.4e-7) / (land + lake);
        m.sfc_rho_c[p] = (land * 1442.0 * 830.0 + lake * 1024.0 * 4184.0) / (land + lake);
        if (std::fabs(360.0 / (2.0 * M_PI_) * m.lat_geo_scalar[p]) > 70.0) m.sfc_albedo[p] = land * 0.8 + (1.0 - land) * 0.06;
        else m.sfc_albedo[p] = land * 0.12 + (1.0 - land) * 0.06;
        const double vegetation_height = 20.0 * std::cos(m.lat_geo_scalar[p]) * std::exp(-m.z_w[m.IS(ji, jk, NL)] / 1500.0);
        m.roughness_length[p] = vegetation_height / 8.0;
      }
      m.roughness_length[p] = std::fmax(0.0001, m.roughness_length[p]);
    }
  // soil grid, :1360-1378: interfaces spaced by powers of sigma_soil, rescaled to reach
  // z_t_const at the bottom (the integer powers by repeated squaring, as Fortran's real**integer)
  if (n.nsoillays >= 1) {
    const int ns = n.nsoillays;
    const double sigma_soil = 0.352;
    auto powi = [](double x, int e) {
      unsigned k = e < 0 ? 0u - (unsigned)e : (unsigned)e;
      double y = (k & 1u) ? x : 1.0;
      while (k >>= 1) {
        x = x * x;
        if (k & 1u) y = y * x;
      }
      return e < 0 ? 1.0 / y : y;
    };
    m.z_t_const[0] = -10.0;
    m.z_soil_interface[0] = 0.0;
    for (int jl = 2; jl <= ns + 1; ++jl) m.z_soil_interface[jl - 1] = m.z_soil_interface[jl - 2] + powi(sigma_soil, ns - jl);
    const double rescale_factor = m.z_t_const[0] / m.z_soil_interface[ns];
    for (int jl = 2; jl <= ns + 1; ++jl) m.z_soil_interface[jl - 1] = rescale_factor * m.z_soil_interface[jl - 1];
    for (int jl = 1; jl <= ns; ++jl) m.z_soil_center[jl - 1] = 0.5 * (m.z_soil_interface[jl - 1] + m.z_soil_interface[jl]);
  }
  // vertical grid, :894-951
  double max_oro = -1e300;
  for (double v : m.oro) max_oro = std::fmax(max_oro, v);
  int vgrid_err = 0;
#pragma omp parallel for schedule(static) reduction(|:vgrid_err)
  for (int jk = 1; jk <= nx; ++jk)
    for (int ji = 1; ji <= ny; ++ji) {
      std::vector<double> vvp(NL + 1);
      const double zsurf = m.z_w[m.IS(ji, jk, NL)];
      const double os = m.oro_smoothed[m.I2(ji, jk)];
      for (int jl = 1; jl <= NL; ++jl) {
        const double z_rel = 1.0 - (jl - 1.0) / nl;
        const double sigma_z = std::pow(z_rel, n.stretching_parameter);
        const double A = sigma_z * n.toa;
        if (jl > nf + 1) {
          if (n.lsleve) {
            const double toa_oro = vvp[nf + 1];
            if (n.orography_id == 2) {
              vvp[jl] = A + std::sinh((toa_oro - A) / 5.e3) / std::sinh(toa_oro / 5.e3) * os
                        + std::sinh((toa_oro - A) / 2.e3) / std::sinh(toa_oro / 2.e3) * (zsurf - os);
            } else {
              vvp[jl] = A + std::sinh((toa_oro - A) / (0.5 * toa_oro)) / std::sinh(toa_oro / (0.5 * toa_oro)) * os
                        + std::sinh((toa_oro - A) / (0.25 * toa_oro)) / std::sinh(toa_oro / (0.25 * toa_oro)) * (zsurf - os);
            }
          } else {
            const double B = (jl - (nf + 1.0)) / m.no;
            vvp[jl] = A + B * zsurf;
          }
        } else {
          vvp[jl] = A;
        }
        if (jl > 1 && vvp[jl] >= vvp[jl - 1]) vgrid_err |= 1;
      }
      if (ji == 1 && jk == 1 && max_oro >= vvp[nf + 1]) vgrid_err |= 2;
      for (int jl = 1; jl <= nl; ++jl) m.z_scalar[m.IS(ji, jk, jl)] = 0.5 * (vvp[jl] + vvp[jl + 1]);
    }
  if (vgrid_err & 1)
    return fail(LGAME_ERR_BAD_CONFIG, "Problem in vertical grid generation. You might have to change SLEVE parameters.");
  if (vgrid_err & 2)
    return fail(LGAME_ERR_BAD_CONFIG, "Maximum of orography larger or equal to the height of the lowest flat level.");
  // z_u, z_v, :953-991
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int ji = 1; ji <= ny; ++ji) {
      for (int jk = 2; jk <= nx; ++jk)
        m.z_u[m.IU(ji, jk, jl)] = 0.5 * (m.z_scalar[m.IS(ji, jk - 1, jl)] + m.z_scalar[m.IS(ji, jk, jl)]);
      if (n.lperiodic) {
        m.z_u[m.IU(ji, 1, jl)] = 0.5 * (m.z_scalar[m.IS(ji, 1, jl)] + m.z_scalar[m.IS(ji, nx, jl)]);
        m.z_u[m.IU(ji, nx + 1, jl)] = m.z_u[m.IU(ji, 1, jl)];
      } else {
        m.z_u[m.IU(ji, 1, jl)] = m.z_scalar[m.IS(ji, 1, jl)] + 0.5 * (m.z_scalar[m.IS(ji, 1, jl)] - m.z_scalar[m.IS(ji, 2, jl)]);
        m.z_u[m.IU(ji, nx + 1, jl)] = m.z_scalar[m.IS(ji, nx, jl)] + 0.5 * (m.z_scalar[m.IS(ji, nx, jl)] - m.z_scalar[m.IS(ji, nx - 1, jl)]);
      }
    }
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx; ++jk) {
      for (int ji = 2; ji <= ny; ++ji)
        m.z_v[m.IV(ji, jk, jl)] = 0.5 * (m.z_scalar[m.IS(ji - 1, jk, jl)] + m.z_scalar[m.IS(ji, jk, jl)]);
      if (n.lperiodic) {
        m.z_v[m.IV(1, jk, jl)] = 0.5 * (m.z_scalar[m.IS(1, jk, jl)] + m.z_scalar[m.IS(ny, jk, jl)]);
        m.z_v[m.IV(ny + 1, jk, jl)] = m.z_v[m.IV(1, jk, jl)];
      } else {
        m.z_v[m.IV(1, jk, jl)] = m.z_scalar[m.IS(1, jk, jl)] + 0.5 * (m.z_scalar[m.IS(1, jk, jl)] - m.z_scalar[m.IS(2, jk, jl)]);
        m.z_v[m.IV(ny + 1, jk, jl)] = m.z_scalar[m.IS(ny, jk, jl)] + 0.5 * (m.z_scalar[m.IS(ny, jk, jl)] - m.z_scalar[m.IS(ny - 1, jk, jl)]);
      }
    }
  // dx, dy, :993-1010
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx + 1; ++jk)
      for (int ji = 1; ji <= ny; ++ji)
        m.dx[m.IU(ji, jk, jl)] = n.lplane ? n.dx : n.dx * std::cos(m.lat_scalar[ji - 1]) * (r_e + m.z_u[m.IU(ji, jk, jl)]) / r_e;
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny + 1; ++ji)
        m.dy[m.IV(ji, jk, jl)] = n.lplane ? n.dy : n.dy * (r_e + m.z_v[m.IV(ji, jk, jl)]) / r_e;
  // dx_dual, dy_dual, :1012-1032
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny + 1; ++ji) {
        const double lat = (ji == ny + 1) ? m.lat_scalar[ji - 2] - 0.5 * dlat : m.lat_scalar[ji - 1] + 0.5 * dlat;
        m.dx_dual[m.IV(ji, jk, jl)] = n.lplane ? n.dx : n.dx * std::cos(lat) * (r_e + m.z_v[m.IV(ji, jk, jl)]) / r_e;
      }
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx + 1; ++jk)
      for (int ji = 1; ji <= ny; ++ji)
        m.dy_dual[m.IU(ji, jk, jl)] = n.lplane ? n.dy : n.dy * (r_e + m.z_u[m.IU(ji, jk, jl)]) / r_e;
  // slopes, :1036
  grad_hor_cov(m, m.z_scalar, m.slope_x, m.slope_y);
  // z_w, :1039-1047
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji)
        m.z_w[m.IS(ji, jk, jl)] = (jl == 1) ? n.toa : 0.5 * (m.z_scalar[m.IS(ji, jk, jl - 1)] + m.z_scalar[m.IS(ji, jk, jl)]);
  // layer thicknesses, :1060-1064
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji)
        m.layer_thickness[m.IS(ji, jk, jl)] = m.z_w[m.IS(ji, jk, jl)] - m.z_w[m.IS(ji, jk, jl + 1)];
  // dz, :1068-1078
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= NL; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji) {
        double d;
        if (jl == 1) d = 2.0 * (n.toa - m.z_scalar[m.IS(ji, jk, jl)]);
        else if (jl == NL) d = 2.0 * (m.z_scalar[m.IS(ji, jk, jl - 1)] - m.z_w[m.IS(ji, jk, jl)]);
        else d = m.z_scalar[m.IS(ji, jk, jl - 1)] - m.z_scalar[m.IS(ji, jk, jl)];
        m.dz[m.IS(ji, jk, jl)] = d;
      }
  // horizontal areas, :1081-1102
  for (int jk = 1; jk <= nx; ++jk)
    for (int ji = 1; ji <= ny; ++ji) {
      const double s = r_e + m.z_w[m.IS(ji, jk, NL)];
      m.area_z[m.IS(ji, jk, NL)] = patch_area(m, m.lat_scalar[ji - 1], dlon, dlat) * (s * s) / (r_e * r_e);
    }
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji) {
        const double a = r_e + m.z_w[m.IS(ji, jk, jl)], b = r_e + m.z_w[m.IS(ji, jk, NL)];
        m.area_z[m.IS(ji, jk, jl)] = m.area_z[m.IS(ji, jk, NL)] * (a * a) / (b * b);
      }
  if (n.lplane)
    for (auto& v : m.area_z) v = n.dx * n.dy;
  // vertical areas in x-direction, :1114-1140
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx + 1; ++jk)
      for (int ji = 1; ji <= ny; ++ji) {
        double lz, uz;
        if (jk == 1) {
          lz = m.z_w[m.IS(ji, 1, jl + 1)] + 0.5 * (m.z_w[m.IS(ji, 1, jl + 1)] - m.z_w[m.IS(ji, 2, jl + 1)]);
          uz = m.z_w[m.IS(ji, 1, jl)] + 0.5 * (m.z_w[m.IS(ji, 1, jl)] - m.z_w[m.IS(ji, 2, jl)]);
        } else if (jk == nx + 1) {
          lz = m.z_w[m.IS(ji, nx, jl + 1)] + 0.5 * (m.z_w[m.IS(ji, nx, jl + 1)] - m.z_w[m.IS(ji, nx - 1, jl + 1)]);
          uz = m.z_w[m.IS(ji, nx, jl)] + 0.5 * (m.z_w[m.IS(ji, nx, jl)] - m.z_w[m.IS(ji, nx - 1, jl)]);
        } else {
          lz = 0.5 * (m.z_w[m.IS(ji, jk - 1, jl + 1)] + m.z_w[m.IS(ji, jk, jl + 1)]);
          uz = 0.5 * (m.z_w[m.IS(ji, jk - 1, jl)] + m.z_w[m.IS(ji, jk, jl)]);
        }
        double ll = n.dy * (r_e + lz) / r_e;
        if (n.lplane) ll = n.dy;
        m.area_x[m.IU(ji, jk, jl)] = vertical_face_area(m, lz, uz, ll);
      }
  // vertical areas in y-direction, :1143-1173
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny + 1; ++ji) {
        double lz, uz;
        if (ji == 1) {
          lz = m.z_w[m.IS(1, jk, jl + 1)] + 0.5 * (m.z_w[m.IS(1, jk, jl + 1)] - m.z_w[m.IS(2, jk, jl + 1)]);
          uz = m.z_w[m.IS(1, jk, jl)] + 0.5 * (m.z_w[m.IS(1, jk, jl)] - m.z_w[m.IS(2, jk, jl)]);
        } else if (ji == ny + 1) {
          lz = m.z_w[m.IS(ny, jk, jl + 1)] + 0.5 * (m.z_w[m.IS(ny, jk, jl + 1)] - m.z_w[m.IS(ny - 1, jk, jl + 1)]);
          uz = m.z_w[m.IS(ny, jk, jl)] + 0.5 * (m.z_w[m.IS(ny, jk, jl)] - m.z_w[m.IS(ny - 1, jk, jl)]);
        } else {
          lz = 0.5 * (m.z_w[m.IS(ji - 1, jk, jl + 1)] + m.z_w[m.IS(ji, jk, jl + 1)]);
          uz = 0.5 * (m.z_w[m.IS(ji - 1, jk, jl)] + m.z_w[m.IS(ji, jk, jl)]);
        }
        double ll;
        if (ji == ny + 1) ll = n.dx * std::cos(m.lat_scalar[ji - 2] - 0.5 * dlat) * (r_e + lz) / r_e;
        else ll = n.dx * std::cos(m.lat_scalar[ji - 1] + 0.5 * dlat) * (r_e + lz) / r_e;
        if (n.lplane) ll = n.dx;
        m.area_y[m.IV(ji, jk, jl)] = vertical_face_area(m, lz, uz, ll);
      }
  // horizontal dual areas, :1176-1206
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx + 1; ++jk)
      for (int ji = 1; ji <= ny + 1; ++ji) {
        double zd;
        if (jk == 1) zd = m.z_v[m.IV(ji, 1, jl)] + 0.5 * (m.z_v[m.IV(ji, 1, jl)] - m.z_v[m.IV(ji, 2, jl)]);
        else if (jk == nx + 1) zd = m.z_v[m.IV(ji, nx, jl)] + 0.5 * (m.z_v[m.IV(ji, nx, jl)] - m.z_v[m.IV(ji, nx - 1, jl)]);
        else zd = 0.5 * (m.z_v[m.IV(ji, jk - 1, jl)] + m.z_v[m.IV(ji, jk, jl)]);
        m.z_area_dual_z[m.IZ(ji, jk, jl)] = zd;
        const double s = r_e + zd;
        double a;
        if (ji == ny + 1) a = patch_area(m, m.lat_scalar[ji - 2] - 0.5 * dlat, dlon, dlat) * (s * s) / (r_e * r_e);
        else a = patch_area(m, m.lat_scalar[ji - 1] + 0.5 * dlat, dlon, dlat) * (s * s) / (r_e * r_e);
        if (n.lplane) a = n.dx * n.dy;
        m.area_dual_z[m.IZ(ji, jk, jl)] = a;
      }
  // vertical dual areas in x-direction, :1209-1245 (extents (ny+1,nx,nl+1))
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= NL; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny + 1; ++ji) {
        double lz, ll, uz;
        if (jl == NL) {
          if (ji == 1) lz = m.z_w[m.IS(1, jk, jl)] + 0.5 * (m.z_w[m.IS(1, jk, jl)] - m.z_w[m.IS(2, jk, jl)]);
          else if (ji == ny + 1) lz = m.z_w[m.IS(ny, jk, jl)] + 0.5 * (m.z_w[m.IS(ny, jk, jl)] - m.z_w[m.IS(ny - 1, jk, jl)]);
          else lz = 0.5 * (m.z_w[m.IS(ji - 1, jk, jl)] + m.z_w[m.IS(ji, jk, jl)]);
          ll = m.dy[m.IV(ji, jk, nl)] * (r_e + lz) / (r_e + m.z_v[m.IV(ji, jk, nl)]);
        } else {
          lz = m.z_v[m.IV(ji, jk, jl)];
          ll = m.dy[m.IV(ji, jk, jl)];
        }
        if (jl == 1) {
          if (ji == 1) uz = m.z_w[m.IS(1, jk, jl)] + 0.5 * (m.z_w[m.IS(1, jk, jl)] - m.z_w[m.IS(2, jk, jl)]);
          else if (ji == ny + 1) uz = m.z_w[m.IS(ny, jk, jl)] + 0.5 * (m.z_w[m.IS(ny, jk, jl)] - m.z_w[m.IS(ny - 1, jk, jl)]);
          else uz = 0.5 * (m.z_w[m.IS(ji - 1, jk, jl)] + m.z_w[m.IS(ji, jk, jl)]);
        } else {
          uz = m.z_v[m.IV(ji, jk, jl - 1)];
        }
        if (n.lplane) ll = n.dy;
        m.area_dual_x[m.IV(ji, jk, jl)] = vertical_face_area(m, lz, uz, ll);
      }
  // vertical dual areas in y-direction, :1248-1284 (extents (ny,nx+1,nl+1))
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= NL; ++jl)
    for (int jk = 1; jk <= nx + 1; ++jk)
      for (int ji = 1; ji <= ny; ++ji) {
        double lz, ll, uz;
        if (jl == NL) {
          if (jk == 1) lz = m.z_w[m.IS(ji, 1, jl)] + 0.5 * (m.z_w[m.IS(ji, 1, jl)] - m.z_w[m.IS(ji, 2, jl)]);
          else if (jk == nx + 1) lz = m.z_w[m.IS(ji, nx, jl)] + 0.5 * (m.z_w[m.IS(ji, nx, jl)] - m.z_w[m.IS(ji, nx - 1, jl)]);
          else lz = 0.5 * (m.z_w[m.IS(ji, jk - 1, jl)] + m.z_w[m.IS(ji, jk, jl)]);
          ll = m.dx[m.IU(ji, jk, nl)] * (r_e + lz) / (r_e + m.z_u[m.IU(ji, jk, nl)]);
        } else {
          lz = m.z_u[m.IU(ji, jk, jl)];
          ll = m.dx[m.IU(ji, jk, jl)];
        }
        if (jl == 1) {
          if (jk == 1) uz = m.z_w[m.IS(ji, 1, jl)] + 0.5 * (m.z_w[m.IS(ji, 1, jl)] - m.z_w[m.IS(ji, 2, jl)]);
          else if (jk == nx + 1) uz = m.z_w[m.IS(ji, nx, jl)] + 0.5 * (m.z_w[m.IS(ji, nx, jl)] - m.z_w[m.IS(ji, nx - 1, jl)]);
          else uz = 0.5 * (m.z_w[m.IS(ji, jk - 1, jl)] + m.z_w[m.IS(ji, jk, jl)]);
        } else {
          uz = m.z_u[m.IU(ji, jk, jl - 1)];
        }
        if (n.lplane) ll = n.dx;
        m.area_dual_y[m.IU(ji, jk, jl)] = vertical_face_area(m, lz, uz, ll);
      }
  // volumes, :1287-1296
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji) {
        const double a = r_e + m.z_w[m.IS(ji, jk, jl)], b = r_e + m.z_w[m.IS(ji, jk, jl + 1)];
        double v = 1.0 / 3.0 * ((a * a) * a - (b * b) * b) / (b * b) * m.area_z[m.IS(ji, jk, jl + 1)];
        if (n.lplane) v = m.area_z[m.IS(ji, jk, jl + 1)] * (m.z_w[m.IS(ji, jk, jl)] - m.z_w[m.IS(ji, jk, jl + 1)]);
        m.volume[m.IS(ji, jk, jl)] = v;
      }
  // inner product weights, :1302-1315
#pragma omp parallel for schedule(static)
  for (int jl = 1; jl <= nl; ++jl)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji) {
        const double v2 = 2.0 * m.volume[m.IS(ji, jk, jl)];
        m.W(1, ji, jk, jl) = m.area_x[m.IU(ji, jk + 1, jl)] * m.dx[m.IU(ji, jk + 1, jl)] / v2;
        m.W(2, ji, jk, jl) = m.area_y[m.IV(ji, jk, jl)] * m.dy[m.IV(ji, jk, jl)] / v2;
        m.W(3, ji, jk, jl) = m.area_x[m.IU(ji, jk, jl)] * m.dx[m.IU(ji, jk, jl)] / v2;
        m.W(4, ji, jk, jl) = m.area_y[m.IV(ji + 1, jk, jl)] * m.dy[m.IV(ji + 1, jk, jl)] / v2;
        m.W(5, ji, jk, jl) = m.area_z[m.IS(ji, jk, jl)] * m.dz[m.IS(ji, jk, jl)] / v2;
        m.W(6, ji, jk, jl) = m.area_z[m.IS(ji, jk, jl + 1)] * m.dz[m.IS(ji, jk, jl + 1)] / v2;
      }
  // TRSK weights, :1317-1357
  for (int ji = 1; ji <= ny; ++ji) {
    const double lat = m.lat_scalar[ji - 1];
    const double base_area = patch_area(m, lat, dlon, dlat);
    double w1 = 0.5 - patch_area(m, lat + 0.25 * dlat, 0.5 * dlon, 0.5 * dlat) / base_area;
    w1 = n.lplane ? w1 * n.dx / n.dx : w1 * n.dx * std::cos(lat + 0.5 * dlat) / (n.dx * std::cos(lat));
    double w2 = -(0.5 - patch_area(m, lat + 0.25 * dlat, dlon, 0.5 * dlat) / base_area);
    w2 = n.lplane ? w2 * n.dy / n.dx : w2 * n.dy / (n.dx * std::cos(lat));
    double w3 = -(0.5 - (patch_area(m, lat + 0.25 * dlat, dlon, 0.5 * dlat) + patch_area(m, lat - 0.25 * dlat, 0.5 * dlon, 0.5 * dlat)) / base_area);
    w3 = n.lplane ? w3 * n.dx / n.dx : w3 * n.dx * std::cos(lat - 0.5 * dlat) / (n.dx * std::cos(lat));
    m.trsk_u[3 * (ji - 1) + 0] = w1; m.trsk_u[3 * (ji - 1) + 1] = w2; m.trsk_u[3 * (ji - 1) + 2] = w3;
  }
  for (int ji = 1; ji <= ny + 1; ++ji) {
    const double llc = (ji == ny + 1) ? m.lat_scalar[ny - 1] - dlat : m.lat_scalar[ji - 1];
    double base_area = patch_area(m, llc, dlon, dlat);
    m.trsk_v[2 * (ji - 1) + 0] = -(0.5 - patch_area(m, llc + 0.25 * dlat, 0.5 * dlon, 0.5 * dlat) / base_area);
    const double luc = (ji == 1) ? m.lat_scalar[0] + dlat : m.lat_scalar[ji - 2];
    base_area = patch_area(m, luc, dlon, dlat);
    m.trsk_v[2 * (ji - 1) + 1] = -(0.5 - patch_area(m, luc - 0.25 * dlat, 0.5 * dlon, 0.5 * dlat) / base_area);
  }
  return LGAME_OK;
}

// ---- bg_setup, mo_grid_generator.F90:1389-1457 --------------------------------
int bg_setup(M& m) {
  const int ny = m.ny, nx = m.nx, nl = m.nl;
  int pres_err = 0;
#pragma omp parallel for schedule(static) reduction(|:pres_err)
  for (int jk = 1; jk <= nx; ++jk)
    for (int ji = 1; ji <= ny; ++ji)
      for (int jl = nl; jl >= 1; --jl) {
        const size_t i = m.IS(ji, jk, jl);
        m.gravity_potential[i] = geopot(m, m.z_scalar[i]);
        if (jl == nl) {
          double p = p_0;
          if (!bg_pres(m.z_scalar[i], &p)) pres_err = 1;
          m.exner_bg[i] = std::pow(p / p_0, r_d / c_d_p);
        } else {
          const size_t ib = m.IS(ji, jk, jl + 1);
          const double T0 = bg_temp(m.z_scalar[i]), T1 = bg_temp(m.z_scalar[ib]);
          const double b = -0.5 * m.exner_bg[ib] / T1 * (T0 - T1 + 2.0 / c_d_p * (m.gravity_potential[i] - m.gravity_potential[ib]));
          const double c = m.exner_bg[ib] * m.exner_bg[ib] * T0 / T1;
          m.exner_bg[i] = b + std::sqrt(b * b + c);
        }
        m.theta_v_bg[i] = bg_temp(m.z_scalar[i]) / m.exner_bg[i];
      }
  if (pres_err)
    return fail(LGAME_ERR_BAD_CONFIG, "Argument of bg_pres is above the inversion height. This is unrealistic in the lowest layer.");
  grad_vert(m, m.exner_bg, m.exner_bg_grad_w);
  grad_hor(m, m.exner_bg, m.exner_bg_grad_u, m.exner_bg_grad_v, m.exner_bg_grad_w);
  if (!m.nml.luse_bg_state) {
    std::fill(m.theta_v_bg.begin(), m.theta_v_bg.end(), 0.0);
    std::fill(m.exner_bg.begin(), m.exner_bg.end(), 0.0);
  }
  grad_vert(m, m.gravity_potential, m.gravity_m_v);
  if (!m.nml.luse_bg_state) {
    grad_hor_cov(m, m.gravity_potential, m.diag[LGAME_DIAG_P_GRAD_ACC_NEG_L_U], m.diag[LGAME_DIAG_P_GRAD_ACC_NEG_L_V]);
    m.diag[LGAME_DIAG_P_GRAD_ACC_NEG_L_W] = m.gravity_m_v;
  }
  return LGAME_OK;
}

// w_free_slip, mo_inner_product.F90:52-75
void w_free_slip(M& m) {
  const int ny = m.ny, nx = m.nx, nl = m.nl;
  for (int jk = 1; jk <= nx; ++jk)
    for (int ji = 1; ji <= ny; ++ji)
      m.wind_w[m.IS(ji, jk, nl + 1)] =
          m.W(1, ji, jk, nl) * m.wind_u[m.IU(ji, jk + 1, nl)] * m.slope_x[m.IU(ji, jk + 1, nl)]
        + m.W(2, ji, jk, nl) * m.wind_v[m.IV(ji, jk, nl)] * m.slope_y[m.IV(ji, jk, nl)]
        + m.W(3, ji, jk, nl) * m.wind_u[m.IU(ji, jk, nl)] * m.slope_x[m.IU(ji, jk, nl)]
        + m.W(4, ji, jk, nl) * m.wind_v[m.IV(ji + 1, jk, nl)] * m.slope_y[m.IV(ji + 1, jk, nl)];
}

// unessential_ideal_init, mo_set_initial_state.F90:322-382.  sp = virtual temperature.
void unessential_ideal_init(M& m, const Vec& sp, const Vec& pres_lowest) {
  const int ny = m.ny, nx = m.nx, nl = m.nl, g = m.nml.n_condensed_constituents + 1;
  const size_t nS = (size_t)ny * nx * nl;
#pragma omp parallel for schedule(static)
  for (int jk = 1; jk <= nx; ++jk)
    for (int ji = 1; ji <= ny; ++ji)
      for (int jl = nl; jl >= 1; --jl) {
        const size_t i = m.IS(ji, jk, jl);
        if (jl == nl) {
          m.exner_pert[i] = std::pow(pres_lowest[m.I2(ji, jk)] / p_0, r_d / c_d_p);
        } else {
          const size_t ib = m.IS(ji, jk, jl + 1);
          const double b = -0.5 * m.exner_pert[ib] / sp[ib] *
                           (sp[i] - sp[ib] + 2.0 / c_d_p * (geopot(m, m.z_scalar[i]) - geopot(m, m.z_scalar[ib])));
          const double c = m.exner_pert[ib] * m.exner_pert[ib] * sp[i] / sp[ib];
          m.exner_pert[i] = b + std::sqrt(b * b + c);
        }
        m.theta_v_pert[i] = sp[i] / m.exner_pert[i];
      }
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < nS; ++i) {
    m.rho[i + nS * (size_t)(g - 1)] = p_0 * std::pow(m.exner_pert[i], c_d_p / r_d) / (r_d * sp[i]);
    m.rhotheta_v[i] = m.rho[i + nS * (size_t)(g - 1)] * m.theta_v_pert[i];
    m.theta_v_pert[i] = m.theta_v_pert[i] - m.theta_v_bg[i];
    m.exner_pert[i] = m.exner_pert[i] - m.exner_bg[i];
  }
  std::fill(m.wind_w.begin(), m.wind_w.end(), 0.0);
}

// Saturation vapour pressure over water (Magnus form, Alduchov & Eskridge 1996),
// used only to build the seeded moist initial state.
double e_sat(double T) {
  const double tc = T - 273.15;
  return 610.94 * std::exp(17.625 * tc / (tc + 243.04));
}

// ---- ideal_init, mo_set_initial_state.F90:22-257 ------------------------------
int ideal_init(M& m) {
  const lgame_namelist& n = m.nml;
  const int ny = m.ny, nx = m.nx, nl = m.nl, nc = n.n_condensed_constituents;
  const size_t nS = (size_t)ny * nx * nl;
  Vec sp(nS, 0.0), pres_lowest((size_t)ny * nx, 0.0);
  const std::string sc = n.scenario;
  std::fill(m.rho.begin(), m.rho.end(), 0.0);
  if (sc == "standard" || sc == "seabreeze") {
    std::fill(m.wind_u.begin(), m.wind_u.end(), 0.0);
    std::fill(m.wind_v.begin(), m.wind_v.end(), 0.0);
    for (size_t i = 0; i < nS; ++i) sp[i] = bg_temp(m.z_scalar[i]);
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji)
        if (!bg_pres(m.z_scalar[m.IS(ji, jk, nl)], &pres_lowest[m.I2(ji, jk)]))
          return fail(LGAME_ERR_BAD_CONFIG, "Argument of bg_pres is above the inversion height.");
  } else if (sc == "advection") {
    const double u_0 = 10.0, z_1 = 4e3, z_2 = 5e3, A_x = 25e3, A_z = 3e3, x_0 = -50e3, z_0 = 9e3, rho_0 = 1e-3;
    for (int jl = 1; jl <= nl; ++jl)
      for (int jk = 1; jk <= nx + 1; ++jk)
        for (int ji = 1; ji <= ny; ++ji) {
          const double z = m.z_u[m.IU(ji, jk, jl)];
          double u = 0.0;
          if (z >= z_2) u = u_0;
          else if (z_1 <= z && z <= z_2) { const double s = std::sin(0.5 * M_PI_ * (z - z_1) / (z_2 - z_1)); u = u_0 * (s * s); }
          m.wind_u[m.IU(ji, jk, jl)] = u;
        }
    std::fill(m.wind_v.begin(), m.wind_v.end(), 0.0);
    for (size_t i = 0; i < nS; ++i) sp[i] = bg_temp(m.z_scalar[i]);
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji)
        if (!bg_pres(m.z_scalar[m.IS(ji, jk, nl)], &pres_lowest[m.I2(ji, jk)]))
          return fail(LGAME_ERR_BAD_CONFIG, "Argument of bg_pres is above the inversion height.");
    if (n.lmoist) {
      for (int jl = 1; jl <= nl; ++jl)
        for (int jk = 1; jk <= nx; ++jk)
          for (int ji = 1; ji <= ny; ++ji) {
            const double x = x_coord_of(m, jk);
            const double a = (x - x_0) / A_x, b = (m.z_scalar[m.IS(ji, jk, jl)] - z_0) / A_z;
            const double r = std::pow(a * a + b * b, 0.5);
            double v = 0.0;
            if (r <= 1.0) { const double c = std::cos(0.5 * M_PI_ * r); v = rho_0 * (c * c); }
            m.rho[m.IS(ji, jk, jl) + nS * (size_t)(nc + 1)] = v;
          }
    }
  } else if (sc == "schaer" || sc == "mountain_rest") {
    if (sc == "schaer") std::fill(m.wind_u.begin(), m.wind_u.end(), 10.0);
    const double n_squared = 0.01 * 0.01, T_0 = 288.0;
    Vec th(nl + 1), ex(nl + 1);
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji) {
        double dz = m.z_scalar[m.IS(ji, jk, nl)];
        double gl = geopot(m, m.z_scalar[m.IS(ji, jk, nl)]) / dz;
        th[nl] = T_0 * (1.0 + n_squared * dz / (2.0 * gl)) / (1.0 - n_squared * dz / (2.0 * gl));
        ex[nl] = 1.0 - 2.0 * geopot(m, m.z_scalar[m.IS(ji, jk, nl)]) / (c_d_p * (th[nl] + T_0));
        for (int jl = nl - 1; jl >= 1; --jl) {
          dz = m.z_scalar[m.IS(ji, jk, jl)] - m.z_scalar[m.IS(ji, jk, jl + 1)];
          gl = (geopot(m, m.z_scalar[m.IS(ji, jk, jl)]) - geopot(m, m.z_scalar[m.IS(ji, jk, jl + 1)])) / dz;
          th[jl] = th[jl + 1] * (1.0 + n_squared * dz / (2.0 * gl)) / (1.0 - n_squared * dz / (2.0 * gl));
        }
        for (int jl = nl - 1; jl >= 1; --jl)
          ex[jl] = ex[jl + 1] - 2.0 * (geopot(m, m.z_scalar[m.IS(ji, jk, jl)]) - geopot(m, m.z_scalar[m.IS(ji, jk, jl + 1)]))
                   / (c_d_p * (th[jl] + th[jl + 1]));
        for (int jl = 1; jl <= nl; ++jl) sp[m.IS(ji, jk, jl)] = ex[jl] * th[jl];
        pres_lowest[m.I2(ji, jk)] = p_0 * std::pow(ex[nl], c_d_p / r_d);
      }
  } else if (sc == "baroclinic_jet") {
    // No reference counterpart.  A zonal jet u(z) = jet_speed*sin^2(pi/2*z/z_j) for
    // z <= 2*z_j (zero above), z_j the ICAO height of jet_pressure; the ICAO
    // temperature plus a random-phase perturbation (8 periodic Fourier modes, seeded,
    // scaled to standard deviation t_pert_sigma, vanishing at the surface and the top);
    // water vapour at a lognormal relative humidity around rh_mean below 12 km; sparse
    // cloud water (4-8 km), cloud ice (8-11 km), rain (< 4 km) and snow (5-9 km) where a
    // second seeded field exceeds a threshold; graupel zero.  The virtual temperature
    // then goes through the reference's hydrostatic integration.
    if (!n.lmoist) return fail(LGAME_ERR_BAD_CONFIG, "scenario baroclinic_jet needs lmoist=.true.");
    Rng rng((uint64_t)n.seed + 17);
    const double z_j = surface_temp / lapse_rate * (1.0 - std::pow(n.jet_pressure / p_0_standard, r_d * lapse_rate / gravity));
    for (int jl = 1; jl <= nl; ++jl)
      for (int jk = 1; jk <= nx + 1; ++jk)
        for (int ji = 1; ji <= ny; ++ji) {
          const double z = m.z_u[m.IU(ji, jk, jl)];
          double u = 0.0;
          if (z <= 2.0 * z_j) { const double s = std::sin(0.5 * M_PI_ * z / z_j); u = n.jet_speed * s * s; }
          m.wind_u[m.IU(ji, jk, jl)] = u;
        }
    std::fill(m.wind_v.begin(), m.wind_v.end(), 0.0);
    const int nmodes = 8;
    int kx[nmodes], ky[nmodes];
    double ph[nmodes];
    for (int q = 0; q < nmodes; ++q) {
      kx[q] = 1 + (int)(rng.uniform() * 6.0);
      ky[q] = 1 + (int)(rng.uniform() * 6.0);
      ph[q] = 2.0 * M_PI_ * rng.uniform();
    }
    const double amp = n.t_pert_sigma * std::sqrt(2.0 / nmodes);  // each cos mode has variance amp^2/2
    Vec qv(nS, 0.0);
    // horizontal structure of the perturbation, one value per column
    Vec tcol((size_t)ny * nx, 0.0);
#pragma omp parallel for schedule(static)
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji) {
        double tp = 0.0;
        for (int q = 0; q < nmodes; ++q)
          tp += std::cos(2.0 * M_PI_ * (kx[q] * (jk - 0.5) / nx + ky[q] * (ji - 0.5) / ny) + ph[q]);
        tcol[m.I2(ji, jk)] = tp;
      }
    const uint64_t seed_h = (uint64_t)n.seed * 0x2545F4914F6CDD1Dull + 0x1234567ull;
#pragma omp parallel for schedule(static)
    for (int jl = 1; jl <= nl; ++jl)
      for (int jk = 1; jk <= nx; ++jk)
        for (int ji = 1; ji <= ny; ++ji) {
          const size_t i = m.IS(ji, jk, jl);
          const double z = m.z_scalar[i];
          const double tp = tcol[m.I2(ji, jk)];
          const double env = std::sin(M_PI_ * z / n.toa);
          const double T = bg_temp(z) + amp * tp * env;
          // relative humidity (lognormal, a counter-based random number per cell) and
          // specific humidity (vapour mass / gas mass)
          double rh = 0.0;
          Rng cell(seed_h ^ (uint64_t)i);
          if (z < 12000.0) rh = std::fmin(0.98, n.rh_mean * std::exp(0.15 * cell.normal() - 0.5 * 0.15 * 0.15)) * (1.0 - z / 12000.0 * 0.7);
          double pz = 0.0;
          if (!bg_pres(std::fmin(z, inv_height - 1.0), &pz)) pz = 5000.0;
          const double e = rh * e_sat(T);
          const double q = 0.622 * e / std::fmax(pz - 0.378 * e, 1.0);
          qv[i] = q;
          sp[i] = T * (1.0 + q * (m_d / m_v - 1.0));
        }
    for (int jk = 1; jk <= nx; ++jk)
      for (int ji = 1; ji <= ny; ++ji)
        if (!bg_pres(m.z_scalar[m.IS(ji, jk, nl)], &pres_lowest[m.I2(ji, jk)]))
          return fail(LGAME_ERR_BAD_CONFIG, "Argument of bg_pres is above the inversion height.");
    unessential_ideal_init(m, sp, pres_lowest);
    const size_t g = (size_t)nc;  // gas index - 1
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < nS; ++i) {
      const double rg = m.rho[i + nS * g];
      m.rho[i + nS * (g + 1)] = qv[i] * rg;
      const double z = m.z_scalar[i];
      Rng cell((seed_h + 0x9E37ull) ^ (uint64_t)i);
      const double r = cell.uniform();
      if (r > 0.85) {
        if (z > 4000.0 && z < 8000.0) m.rho[i + nS * 3] = 2e-4 * rg * (r - 0.85) / 0.15;  // cloud water
        if (z > 8000.0 && z < 11000.0) m.rho[i + nS * 2] = 5e-5 * rg * (r - 0.85) / 0.15;  // cloud ice
        if (z < 4000.0) m.rho[i + nS * 1] = 1e-4 * rg * (r - 0.85) / 0.15;  // rain
        if (z > 5000.0 && z < 9000.0) m.rho[i + nS * 0] = 5e-5 * rg * (r - 0.85) / 0.15;  // snow
      }
    }
    if (n.lfreeslip) w_free_slip(m);
    return LGAME_OK;
  } else {
    return fail(LGAME_ERR_BAD_CONFIG, std::string("unknown scenario ") + sc);
  }
  // humidity and condensates stay zero (:84-86, :160-162, :228-233) except the
  // advection tracer set above
  unessential_ideal_init(m, sp, pres_lowest);
  if (n.lfreeslip) w_free_slip(m);
  return LGAME_OK;
}

}  // namespace

extern "C" int lgame_host_setup(const lgame_namelist* nml, lgame_host_model** out) {
  if (!nml || !out) return fail(LGAME_ERR_INVALID_ARG, "lgame_host_setup: null argument");
  auto* m = new lgame_host_model();
  m->nml = *nml;
  m->ny = nml->ny; m->nx = nml->nx; m->nl = nml->n_layers; m->NL = nml->n_layers + 1;
  m->nf = nml->n_layers - nml->n_oro_layers; m->no = nml->n_oro_layers;
  const size_t ny = m->ny, nx = m->nx, nl = m->nl;
  const size_t nS = ny * nx * nl, nU = ny * (nx + 1) * nl, nV = (ny + 1) * nx * nl, nW = ny * nx * (nl + 1);
  const size_t nZ = (ny + 1) * (nx + 1) * nl;
  m->lat_scalar.assign(ny, 0); m->lon_scalar.assign(nx, 0);
  m->lat_geo_scalar.assign(ny * nx, 0); m->lon_geo_scalar.assign(ny * nx, 0);
  m->lat_geo_u.assign(ny * (nx + 1), 0); m->lon_geo_u.assign(ny * (nx + 1), 0); m->dir_geo_u.assign(ny * (nx + 1), 0);
  m->lat_geo_v.assign((ny + 1) * nx, 0); m->lon_geo_v.assign((ny + 1) * nx, 0);
  m->dir_geo_v.assign((ny + 1) * nx, 0.5 * M_PI_); m->dir_geo_u_scalar.assign(ny * nx, 0);
  m->z_scalar.assign(nS, 0); m->oro.assign(ny * nx, 0); m->oro_smoothed.assign(ny * nx, 0);
  m->dx.assign(nU, 0); m->dy.assign(nV, 0); m->dz.assign(nW, 0); m->z_u.assign(nU, 0); m->z_v.assign(nV, 0);
  m->z_w.assign(nW, 0); m->gravity_potential.assign(nS, 0); m->gravity_m_v.assign(nW, 0);
  m->volume.assign(nS, 0); m->area_x.assign(nU, 0); m->area_y.assign(nV, 0); m->area_z.assign(nW, 0);
  m->slope_x.assign(nU, 0); m->slope_y.assign(nV, 0); m->ipw.assign(6 * nS, 0);
  m->area_dual_x.assign((ny + 1) * nx * (nl + 1), 0); m->area_dual_y.assign(ny * (nx + 1) * (nl + 1), 0);
  m->area_dual_z.assign(nZ, 0); m->z_area_dual_z.assign(nZ, 0);
  m->fvec_x.assign((ny + 1) * nx, 0); m->fvec_y.assign(ny * (nx + 1), 0); m->fvec_z.assign((ny + 1) * (nx + 1), 0);
  m->trsk_u.assign(3 * ny, 0); m->trsk_v.assign(2 * (ny + 1), 0);
  m->exner_bg_grad_u.assign(nU, 0); m->exner_bg_grad_v.assign(nV, 0); m->exner_bg_grad_w.assign(nW, 0);
  m->theta_v_bg.assign(nS, 0); m->exner_bg.assign(nS, 0); m->sfc_albedo.assign(ny * nx, 0);
  m->dx_dual.assign(nV, 0); m->dy_dual.assign(nU, 0); m->layer_thickness.assign(nS, 0);
  if (nml->nsoillays < 0 || nml->nsoillays > LGAME_MAX_SOIL_LAYERS) {
    delete m;
    return fail(LGAME_ERR_BAD_CONFIG, "nsoillays must lie in 0.." + std::to_string(LGAME_MAX_SOIL_LAYERS));
  }
  const size_t n2 = ny * nx, ns = (size_t)nml->nsoillays;
  for (Vec* v : {&m->land_fraction, &m->lake_fraction, &m->roughness_length, &m->sfc_rho_c, &m->t_conduc_soil,
                 &m->t_const_soil})
    v->assign(n2, 0);
  m->z_soil_interface.assign(ns + 1, 0); m->z_soil_center.assign(ns, 0); m->z_t_const.assign(1, 0);
  const int ncons = nml->n_constituents;
  m->rho.assign(nS * ncons, 0); m->rhotheta_v.assign(nS, 0); m->theta_v_pert.assign(nS, 0);
  m->exner_pert.assign(nS, 0); m->wind_u.assign(nU, 0); m->wind_v.assign(nV, 0); m->wind_w.assign(nW, 0);
  m->temperature_soil.assign(n2 * ns, 0);
  const size_t dsz[LGAME_DIAG_NFIELDS] = {nU, nV, nW, nU, nV, nW, nU, nV, nU, nV, nW, nU, nV, nW, nS, nS, nS,
                                          nS * ncons, nS, nU, nV, nW, nS, nS, nS, nU, nV, nW,
                                          nS, n2, n2, n2, n2, n2, n2, n2, n2, n2,
                                          nS * (size_t)(nml->n_condensed_constituents + 1), nS, n2, n2,
                                          nS, nS * ncons};
  for (int f = 0; f < LGAME_DIAG_NFIELDS; ++f) m->diag[f].assign(dsz[f], 0.0);
  int rc = grid_setup(*m);
  if (rc == LGAME_OK) rc = bg_setup(*m);
  if (rc == LGAME_OK) rc = ideal_init(*m);
  if (rc != LGAME_OK) { delete m; return rc; }
  // soil temperature and sea surface temperature, mo_set_initial_state.F90:237-247; the
  // carried roughness length starts at the grid's, control.F90:458
  std::fill(m->temperature_soil.begin(), m->temperature_soil.end(), 280.0);
  if (ns > 0) std::copy(m->temperature_soil.begin(), m->temperature_soil.begin() + n2, m->diag[LGAME_DIAG_SST].begin());
  m->diag[LGAME_DIAG_ROUGHNESS_LENGTH] = m->roughness_length;
  *out = m;
  return LGAME_OK;
}

extern "C" void lgame_host_destroy(lgame_host_model* m) { delete m; }

extern "C" double* lgame_host_grid_field(lgame_host_model* m, int f, size_t* n) {
  if (!m) return nullptr;
  Vec* v = nullptr;
  switch (f) {
    case LGAME_GRID_Z_SCALAR: v = &m->z_scalar; break;
    case LGAME_GRID_Z_U: v = &m->z_u; break;
    case LGAME_GRID_Z_V: v = &m->z_v; break;
    case LGAME_GRID_Z_W: v = &m->z_w; break;
    case LGAME_GRID_DX: v = &m->dx; break;
    case LGAME_GRID_DY: v = &m->dy; break;
    case LGAME_GRID_DZ: v = &m->dz; break;
    case LGAME_GRID_VOLUME: v = &m->volume; break;
    case LGAME_GRID_AREA_X: v = &m->area_x; break;
    case LGAME_GRID_AREA_Y: v = &m->area_y; break;
    case LGAME_GRID_AREA_Z: v = &m->area_z; break;
    case LGAME_GRID_AREA_DUAL_X: v = &m->area_dual_x; break;
    case LGAME_GRID_AREA_DUAL_Y: v = &m->area_dual_y; break;
    case LGAME_GRID_AREA_DUAL_Z: v = &m->area_dual_z; break;
    case LGAME_GRID_Z_AREA_DUAL_Z: v = &m->z_area_dual_z; break;
    case LGAME_GRID_SLOPE_X: v = &m->slope_x; break;
    case LGAME_GRID_SLOPE_Y: v = &m->slope_y; break;
    case LGAME_GRID_INNER_PRODUCT_WEIGHTS: v = &m->ipw; break;
    case LGAME_GRID_THETA_V_BG: v = &m->theta_v_bg; break;
    case LGAME_GRID_EXNER_BG: v = &m->exner_bg; break;
    case LGAME_GRID_EXNER_BG_GRAD_U: v = &m->exner_bg_grad_u; break;
    case LGAME_GRID_EXNER_BG_GRAD_V: v = &m->exner_bg_grad_v; break;
    case LGAME_GRID_EXNER_BG_GRAD_W: v = &m->exner_bg_grad_w; break;
    case LGAME_GRID_GRAVITY_M_V: v = &m->gravity_m_v; break;
    case LGAME_GRID_GRAVITY_POTENTIAL: v = &m->gravity_potential; break;
    case LGAME_GRID_FVEC_X: v = &m->fvec_x; break;
    case LGAME_GRID_FVEC_Y: v = &m->fvec_y; break;
    case LGAME_GRID_FVEC_Z: v = &m->fvec_z; break;
    case LGAME_GRID_TRSK_WEIGHTS_U: v = &m->trsk_u; break;
    case LGAME_GRID_TRSK_WEIGHTS_V: v = &m->trsk_v; break;
    case LGAME_GRID_DX_DUAL: v = &m->dx_dual; break;
    case LGAME_GRID_DY_DUAL: v = &m->dy_dual; break;
    case LGAME_GRID_LAYER_THICKNESS: v = &m->layer_thickness; break;
    case LGAME_GRID_LAND_FRACTION: v = &m->land_fraction; break;
    case LGAME_GRID_LAKE_FRACTION: v = &m->lake_fraction; break;
    case LGAME_GRID_ROUGHNESS_LENGTH: v = &m->roughness_length; break;
    case LGAME_GRID_SFC_RHO_C: v = &m->sfc_rho_c; break;
    case LGAME_GRID_T_CONDUC_SOIL: v = &m->t_conduc_soil; break;
    case LGAME_GRID_T_CONST_SOIL: v = &m->t_const_soil; break;
    case LGAME_GRID_Z_SOIL_INTERFACE: v = &m->z_soil_interface; break;
    case LGAME_GRID_Z_SOIL_CENTER: v = &m->z_soil_center; break;
    case LGAME_GRID_Z_T_CONST: v = &m->z_t_const; break;
    default: return nullptr;
  }
  if (n) *n = v->size();
  return v->data();
}

extern "C" double* lgame_host_state_field(lgame_host_model* m, int f, size_t* n) {
  if (!m) return nullptr;
  Vec* v = nullptr;
  switch (f) {
    case LGAME_STATE_RHO: v = &m->rho; break;
    case LGAME_STATE_RHOTHETA_V: v = &m->rhotheta_v; break;
    case LGAME_STATE_THETA_V_PERT: v = &m->theta_v_pert; break;
    case LGAME_STATE_EXNER_PERT: v = &m->exner_pert; break;
    case LGAME_STATE_WIND_U: v = &m->wind_u; break;
    case LGAME_STATE_WIND_V: v = &m->wind_v; break;
    case LGAME_STATE_WIND_W: v = &m->wind_w; break;
    case LGAME_STATE_TEMPERATURE_SOIL: v = &m->temperature_soil; break;
    default: return nullptr;
  }
  if (n) *n = v->size();
  return v->data();
}

extern "C" double* lgame_host_diag_field(lgame_host_model* m, int f, size_t* n) {
  if (!m || f < 0 || f >= LGAME_DIAG_NFIELDS) return nullptr;
  if (n) *n = m->diag[f].size();
  return m->diag[f].data();
}

extern "C" double* lgame_host_surface_field(lgame_host_model* m, int f, size_t* n) {
  if (!m) return nullptr;
  Vec* v = nullptr;
  switch (f) {
    case 0: v = &m->oro; break;
    case 1: v = &m->sfc_albedo; break;
    case 2: v = &m->lat_geo_scalar; break;
    case 3: v = &m->lon_geo_scalar; break;
    default: return nullptr;
  }
  if (n) *n = v->size();
  return v->data();
}
