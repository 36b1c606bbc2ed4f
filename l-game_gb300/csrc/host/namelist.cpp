// namelist.cpp -- Fortran namelist reader with the reference's defaults and checks.
//
// The reference reads one group per module from ./namelist.nml
// (src/namelists/mo_run_nml.F90:50-143 and the six sibling modules).  This reader
// accepts the same text: groups "&name ... /", "key=value" items separated by
// blanks, commas or newlines, "!" comments, logicals .true./.false./T/F, integers,
// reals with e/d exponents and quoted strings.  Unknown groups are skipped (a
// Fortran read of one group ignores the others); an unknown key inside a known group
// is an error, as a Fortran namelist read would abort on it.
#include "lgame_host.h"
#include "common.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace {

std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

enum class Kind { Int, Real, Logical, Str };
struct Item {
  const char* group;
  const char* key;
  Kind kind;
  void* ptr;
  size_t cap;  // string capacity
};

std::vector<Item> items_of(lgame_namelist* n) {
  std::vector<Item> v;
  auto I = [&](const char* g, const char* k, int* p) { v.push_back({g, k, Kind::Int, p, 0}); };
  auto R = [&](const char* g, const char* k, double* p) { v.push_back({g, k, Kind::Real, p, 0}); };
  auto L = [&](const char* g, const char* k, int* p) { v.push_back({g, k, Kind::Logical, p, 0}); };
  auto S = [&](const char* g, const char* k, char* p, size_t c) { v.push_back({g, k, Kind::Str, p, c}); };
  // &run, mo_run_nml.F90:44-46
  I("run", "ny", &n->ny); I("run", "nx", &n->nx); I("run", "n_layers", &n->n_layers);
  R("run", "dy", &n->dy); R("run", "dx", &n->dx); I("run", "run_span_min", &n->run_span_min);
  R("run", "stretching_parameter", &n->stretching_parameter);
  I("run", "theta_adv_order", &n->theta_adv_order); R("run", "toa", &n->toa);
  S("run", "scenario", n->scenario, sizeof n->scenario); L("run", "llinear", &n->llinear);
  S("run", "run_id", n->run_id, sizeof n->run_id); L("run", "lcorio", &n->lcorio);
  I("run", "n_oro_layers", &n->n_oro_layers); R("run", "lat_center", &n->lat_center);
  R("run", "lon_center", &n->lon_center); I("run", "start_year", &n->start_year);
  I("run", "start_month", &n->start_month); I("run", "start_day", &n->start_day);
  I("run", "start_hour", &n->start_hour); I("run", "start_minute", &n->start_minute);
  L("run", "lplane", &n->lplane); L("run", "luse_bg_state", &n->luse_bg_state);
  // &io, mo_io_nml.F90:242
  I("io", "dt_write_min", &n->dt_write_min); L("io", "lread_geo", &n->lread_geo);
  L("io", "lwrite_grid", &n->lwrite_grid);
  S("io", "grid_filename", n->grid_filename, sizeof n->grid_filename);
  S("io", "restart_filename", n->restart_filename, sizeof n->restart_filename);
  L("io", "lwrite_integrals", &n->lwrite_integrals);
  // &constituents, mo_constituents_nml.F90:227
  L("constituents", "lmoist", &n->lmoist);
  // &diff, mo_diff_nml.F90:28-29
  L("diff", "lmom_diff_h", &n->lmom_diff_h); L("diff", "lmom_diff_v", &n->lmom_diff_v);
  L("diff", "ltemp_diff_h", &n->ltemp_diff_h); L("diff", "ltemp_diff_v", &n->ltemp_diff_v);
  L("diff", "lmass_diff_h", &n->lmass_diff_h); L("diff", "lmass_diff_v", &n->lmass_diff_v);
  R("diff", "h_prandtl", &n->h_prandtl); R("diff", "karman", &n->karman);
  L("diff", "lklemp", &n->lklemp); R("diff", "klemp_damp_max", &n->klemp_damp_max);
  R("diff", "klemp_begin_rel", &n->klemp_begin_rel);
  S("diff", "diff_coeff_scheme_h", n->diff_coeff_scheme_h, 9);
  S("diff", "diff_coeff_scheme_v", n->diff_coeff_scheme_v, 9);
  R("diff", "bg_shear", &n->bg_shear); R("diff", "c_s", &n->c_s);
  // &surface, mo_surface_nml.F90:138
  I("surface", "orography_id", &n->orography_id); L("surface", "lprog_soil_temp", &n->lprog_soil_temp);
  I("surface", "nsoillays", &n->nsoillays);
  L("surface", "lsfc_sensible_heat_flux", &n->lsfc_sensible_heat_flux);
  L("surface", "lsfc_phase_trans", &n->lsfc_phase_trans); L("surface", "lpbl", &n->lpbl);
  L("surface", "lsleve", &n->lsleve);
  // &bc, mo_bc_nml.F90:283
  I("bc", "n_swamp", &n->n_swamp); L("bc", "lperiodic", &n->lperiodic);
  L("bc", "lfreeslip", &n->lfreeslip); I("bc", "dtime_bc", &n->dtime_bc);
  S("bc", "bc_root_filename", n->bc_root_filename, sizeof n->bc_root_filename);
  // &rad, mo_rad_nml.F90:195-196
  L("rad", "lrad", &n->lrad); R("rad", "dtime_rad", &n->dtime_rad);
  S("rad", "rrtmgp_coefficients_file_sw", n->rrtmgp_coefficients_file_sw, sizeof n->rrtmgp_coefficients_file_sw);
  S("rad", "rrtmgp_coefficients_file_lw", n->rrtmgp_coefficients_file_lw, sizeof n->rrtmgp_coefficients_file_lw);
  S("rad", "cloud_coefficients_file_sw", n->cloud_coefficients_file_sw, sizeof n->cloud_coefficients_file_sw);
  S("rad", "cloud_coefficients_file_lw", n->cloud_coefficients_file_lw, sizeof n->cloud_coefficients_file_lw);
  // &gpu (extension)
  I("gpu", "precision", &n->precision); R("gpu", "dtime_override", &n->dtime_override);
  L("gpu", "strict_reference", &n->strict_reference);
  v.push_back({"gpu", "seed", Kind::Int, &n->seed, 8});
  I("gpu", "n_hills", &n->n_hills);
  R("gpu", "hill_height_min", &n->hill_height_min); R("gpu", "hill_height_max", &n->hill_height_max);
  R("gpu", "hill_width_min", &n->hill_width_min); R("gpu", "hill_width_max", &n->hill_width_max);
  R("gpu", "jet_speed", &n->jet_speed); R("gpu", "jet_pressure", &n->jet_pressure);
  R("gpu", "t_pert_sigma", &n->t_pert_sigma); R("gpu", "rh_mean", &n->rh_mean);
  L("gpu", "check_finite", &n->check_finite);
  L("gpu", "lphase_trans", &n->lphase_trans);
  return v;
}

bool parse_logical(const std::string& t, int* out) {
  std::string s = lower(trim(t));
  if (!s.empty() && s[0] == '.') s = s.substr(1);
  if (s.empty()) return false;
  if (s[0] == 't') { *out = 1; return true; }
  if (s[0] == 'f') { *out = 0; return true; }
  return false;
}

bool parse_real(const std::string& t, double* out) {
  std::string s = lower(trim(t));
  for (auto& c : s) if (c == 'd') c = 'e';
  // Fortran kind suffix, e.g. 1.0_wp, is not valid in a namelist file; reject it.
  char* end = nullptr;
  double v = std::strtod(s.c_str(), &end);
  if (end == s.c_str() || *end != '\0') return false;
  *out = v;
  return true;
}

bool parse_int(const std::string& t, long long* out) {
  std::string s = trim(t);
  char* end = nullptr;
  long long v = std::strtoll(s.c_str(), &end, 10);
  if (end == s.c_str() || *end != '\0') return false;
  *out = v;
  return true;
}

// Splits the body of one group into key=value pairs (values may be quoted strings).
bool split_items(const std::string& body, std::vector<std::pair<std::string, std::string>>& kv,
                 std::string& err) {
  size_t i = 0, n = body.size();
  while (i < n) {
    while (i < n && (std::isspace((unsigned char)body[i]) || body[i] == ',')) ++i;
    if (i >= n) break;
    size_t k0 = i;
    while (i < n && body[i] != '=' && !std::isspace((unsigned char)body[i])) ++i;
    std::string key = lower(body.substr(k0, i - k0));
    while (i < n && std::isspace((unsigned char)body[i])) ++i;
    if (i >= n || body[i] != '=') { err = "expected '=' after '" + key + "'"; return false; }
    ++i;
    while (i < n && std::isspace((unsigned char)body[i])) ++i;
    std::string val;
    if (i < n && (body[i] == '"' || body[i] == '\'')) {
      char q = body[i++];
      while (i < n) {
        if (body[i] == q) {
          if (i + 1 < n && body[i + 1] == q) { val += q; i += 2; continue; }  // doubled quote
          ++i;
          break;
        }
        val += body[i++];
      }
      val = "\x01" + val;  // marks a quoted string
    } else {
      size_t v0 = i;
      while (i < n && !std::isspace((unsigned char)body[i]) && body[i] != ',') ++i;
      val = body.substr(v0, i - v0);
    }
    kv.emplace_back(key, val);
  }
  return true;
}

}  // namespace

extern "C" void lgame_namelist_defaults(lgame_namelist* n) {
  std::memset(n, 0, sizeof *n);
  // mo_run_nml.F90:55-80
  n->ny = 35; n->nx = 37; n->n_layers = 50; n->n_oro_layers = 40;
  n->dy = 25e3; n->dx = 25e3; n->run_span_min = 1440;
  n->start_year = 2000; n->start_month = 1; n->start_day = 1; n->start_hour = 0; n->start_minute = 0;
  n->toa = 40000.0; n->stretching_parameter = 1.3;
  n->lplane = 0; std::strcpy(n->scenario, "standard"); std::strcpy(n->run_id, "ideal");
  n->llinear = 0; n->lcorio = 1; n->lat_center = 0.0; n->lon_center = 0.0;
  n->theta_adv_order = 2; n->luse_bg_state = 1;
  // mo_io_nml.F90:251-257
  n->dt_write_min = 60; n->lread_geo = 1; n->lwrite_grid = 0;
  std::strcpy(n->grid_filename, "grid.nc"); std::strcpy(n->restart_filename, "init.nc");
  n->lwrite_integrals = 0;
  // mo_constituents_nml.F90:236
  n->lmoist = 1;
  // mo_diff_nml.F90:39-53
  n->h_prandtl = 100.0; n->lmom_diff_h = 1; n->lmom_diff_v = 1; n->ltemp_diff_h = 1;
  n->ltemp_diff_v = 1; n->lmass_diff_h = 1; n->lmass_diff_v = 1; n->karman = 0.4;
  n->lklemp = 1; n->klemp_damp_max = 0.25; n->klemp_begin_rel = 0.53;
  std::strcpy(n->diff_coeff_scheme_h, "smag"); std::strcpy(n->diff_coeff_scheme_v, "tke");
  n->bg_shear = 1.5e-5; n->c_s = 0.2;
  // mo_surface_nml.F90:148-154
  n->orography_id = 1; n->lprog_soil_temp = 1; n->nsoillays = 5; n->lsfc_sensible_heat_flux = 1;
  n->lsfc_phase_trans = 1; n->lpbl = 1; n->lsleve = 0;
  // mo_bc_nml.F90:293-297
  n->n_swamp = 5; n->lperiodic = 0; n->lfreeslip = 0; n->dtime_bc = 10800;
  std::strcpy(n->bc_root_filename, "bc");
  // mo_rad_nml.F90:206-211 (dtime_rad depends on dy and is derived after reading)
  n->lrad = 1; n->dtime_rad = -1.0;
  std::strcpy(n->rrtmgp_coefficients_file_sw, "rrtmgp-data-sw-g112-210809.nc");
  std::strcpy(n->rrtmgp_coefficients_file_lw, "rrtmgp-data-lw-g128-210809.nc");
  std::strcpy(n->cloud_coefficients_file_sw, "rrtmgp-cloud-optics-coeffs-reordered-sw.nc");
  std::strcpy(n->cloud_coefficients_file_lw, "rrtmgp-cloud-optics-coeffs-lw.nc");
  // &gpu
  n->precision = 0; n->dtime_override = 0.0; n->strict_reference = 1; n->seed = 1;
  n->n_hills = 32; n->hill_height_min = 200.0; n->hill_height_max = 2000.0;
  n->hill_width_min = 5e3; n->hill_width_max = 30e3;
  n->jet_speed = 30.0; n->jet_pressure = 25000.0; n->t_pert_sigma = 0.5; n->rh_mean = 0.8;
  n->check_finite = 0;
}

namespace {

int leap_year_correction(int year) {  // mo_run_nml.F90:145-158
  int c = (year - 1969) / 4;
  if (year > 2000) c = c - 1;
  return c;
}

int month_day_vector(int month, int year) {  // mo_run_nml.F90:160-196
  int md[12] = {31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31};
  if (year / 4 == 0 && year != 2000 && month > 2) md[1] = 29;
  int s = 0;
  for (int m = 1; m < month; ++m) s += md[m - 1];
  return s;
}

int fail(int code, const std::string& msg) {
  lgame_set_error(msg.c_str());
  return code;
}

}  // namespace

extern "C" int lgame_namelist_parse(const char* text, lgame_namelist* n) {
  if (!text || !n) return fail(LGAME_ERR_INVALID_ARG, "lgame_namelist_parse: null argument");
  // strip comments outside quotes
  std::string src;
  {
    bool inq = false; char q = 0;
    for (const char* p = text; *p; ++p) {
      char c = *p;
      if (inq) { src += c; if (c == q) inq = false; continue; }
      if (c == '"' || c == '\'') { inq = true; q = c; src += c; continue; }
      if (c == '!') { while (*p && *p != '\n') ++p; if (!*p) break; src += '\n'; continue; }
      src += c;
    }
  }
  auto items = items_of(n);
  size_t pos = 0;
  while (true) {
    size_t amp = src.find('&', pos);
    if (amp == std::string::npos) break;
    size_t g0 = amp + 1, g1 = g0;
    while (g1 < src.size() && (std::isalnum((unsigned char)src[g1]) || src[g1] == '_')) ++g1;
    std::string group = lower(src.substr(g0, g1 - g0));
    // find the terminating '/' outside quotes
    size_t i = g1; bool inq = false; char q = 0;
    for (; i < src.size(); ++i) {
      char c = src[i];
      if (inq) { if (c == q) inq = false; continue; }
      if (c == '"' || c == '\'') { inq = true; q = c; continue; }
      if (c == '/') break;
    }
    if (i >= src.size()) return fail(LGAME_ERR_BAD_CONFIG, "namelist group &" + group + " has no terminating '/'");
    std::string body = src.substr(g1, i - g1);
    pos = i + 1;
    bool known = false;
    for (auto& it : items) if (group == it.group) { known = true; break; }
    if (!known) continue;
    std::vector<std::pair<std::string, std::string>> kv;
    std::string err;
    if (!split_items(body, kv, err)) return fail(LGAME_ERR_BAD_CONFIG, "&" + group + ": " + err);
    for (auto& p : kv) {
      const Item* it = nullptr;
      for (auto& c : items) if (group == c.group && p.first == c.key) { it = &c; break; }
      if (!it) return fail(LGAME_ERR_BAD_CONFIG, "&" + group + ": unknown variable '" + p.first + "'");
      const bool quoted = !p.second.empty() && p.second[0] == '\x01';
      std::string val = quoted ? p.second.substr(1) : p.second;
      bool ok = true;
      switch (it->kind) {
        case Kind::Int: {
          long long v;
          ok = !quoted && parse_int(val, &v);
          if (ok) {
            if (it->cap == 8) *(long long*)it->ptr = v; else *(int*)it->ptr = (int)v;
          }
          break;
        }
        case Kind::Real: { double v; ok = !quoted && parse_real(val, &v); if (ok) *(double*)it->ptr = v; break; }
        case Kind::Logical: { int v; ok = !quoted && parse_logical(val, &v); if (ok) *(int*)it->ptr = v; break; }
        case Kind::Str: {
          if (val.size() >= it->cap) val = val.substr(0, it->cap - 1);  // Fortran truncates
          std::strcpy((char*)it->ptr, val.c_str());
          break;
        }
      }
      if (!ok) return fail(LGAME_ERR_BAD_CONFIG, "&" + group + ": bad value '" + val + "' for " + p.first);
    }
  }
  // derived quantities, mo_run_nml.F90:89-101, mo_constituents_nml.F90:246-253,
  // mo_io_nml.F90:266, mo_rad_nml.F90:207
  n->n_levels = n->n_layers + 1;
  n->n_flat_layers = n->n_layers - n->n_oro_layers;
  n->eff_hor_res = std::sqrt(n->dx * n->dy);
  n->dtime = 1.61 * n->eff_hor_res / 1000.0;
  if (n->dtime_override > 0.0) n->dtime = n->dtime_override;
  n->t_init = (double)((n->start_year - 1970) * 365 * 24 * 3600 + leap_year_correction(n->start_year) * 24 * 3600 +
                       month_day_vector(n->start_month, n->start_year) * 24 * 3600 +
                       (n->start_day - 1) * 24 * 3600 + n->start_hour * 3600 + n->start_minute * 60 + 27);
  n->n_condensed_constituents = n->lmoist ? 5 : 0;
  n->n_constituents = n->n_condensed_constituents + (n->lmoist ? 2 : 1);
  n->dt_write = 60.0 * n->dt_write_min;
  if (n->dtime_rad < 0.0) n->dtime_rad = 60.0 * n->dy / 1000.0;
  // sanity checks, mo_run_nml.F90:103-141
  if (n->ny < 3) return fail(LGAME_ERR_BAD_DIMS, "Error: ny must be larger or equal than three.");
  if (n->nx < 3) return fail(LGAME_ERR_BAD_DIMS, "Error: nx must be larger or equal than three.");
  if (n->strict_reference && n->ny % 2 == 0) return fail(LGAME_ERR_BAD_DIMS, "Error: ny must be odd.");
  if (n->strict_reference && n->nx % 2 == 0) return fail(LGAME_ERR_BAD_DIMS, "Error: nx must be odd.");
  if (n->toa <= 0) return fail(LGAME_ERR_BAD_CONFIG, "Error: TOA must be positive.");
  const double pi = 3.14159265358979323846;
  if (n->lat_center < -0.5 * pi || n->lat_center > 0.5 * pi)
    return fail(LGAME_ERR_BAD_CONFIG, "Error: lat_center must be between -90 and 90.");
  if (n->lon_center < -pi || n->lon_center > pi)
    return fail(LGAME_ERR_BAD_CONFIG, "Error: lon_center must be between -180 and 180.");
  if (n->n_oro_layers >= n->n_layers) return fail(LGAME_ERR_BAD_DIMS, "Error: it must be n_oro_layers<n_layers.");
  if (n->n_oro_layers < 1) return fail(LGAME_ERR_BAD_DIMS, "Error: it must be n_oro_layers>=1.");
  if (n->theta_adv_order != 2 && n->theta_adv_order != 3)
    return fail(LGAME_ERR_BAD_CONFIG, "Error: it must be theta_adv_order=2 or theta_adv_order=3.");
  // mo_diff_nml.F90:91-98
  std::string sh = trim(n->diff_coeff_scheme_h), sv = trim(n->diff_coeff_scheme_v);
  if (sh != "smag" && sh != "tke") return fail(LGAME_ERR_BAD_CONFIG, "diff_coeff_scheme_h must be either smag or tke.");
  if (sv != "tke") return fail(LGAME_ERR_BAD_CONFIG, "diff_coeff_scheme_v must be tke.");
  // mo_surface_nml.F90:163-166
  if (n->lpbl && !n->lmom_diff_h) return fail(LGAME_ERR_BAD_CONFIG, "Error: lmom_diff_h must be true is lpbl is true.");
  // control.F90:94-97
  if (n->dtime > n->dt_write) return fail(LGAME_ERR_BAD_CONFIG, "Error: It must be dtime <= dt_write.");
  if (n->precision != LGAME_PRECISION_FP64 && n->precision != LGAME_PRECISION_SPLIT &&
      n->precision != LGAME_PRECISION_SPLIT_FP64_COLUMN)
    return fail(LGAME_ERR_BAD_CONFIG, "&gpu: precision must be 0 (fp64), 1 (split) or 2 (split, fp64 column solve).");
  return LGAME_OK;
}

extern "C" int lgame_namelist_read_file(const char* path, lgame_namelist* n) {
  if (!path || !n) return fail(LGAME_ERR_INVALID_ARG, "lgame_namelist_read_file: null argument");
  std::ifstream f(path);
  if (!f) return fail(LGAME_ERR_INVALID_ARG, std::string("cannot open namelist file ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  lgame_namelist_defaults(n);
  return lgame_namelist_parse(ss.str().c_str(), n);
}

extern "C" int lgame_config_from_namelist(const lgame_namelist* n, lgame_config* c) {
  if (!n || !c) return fail(LGAME_ERR_INVALID_ARG, "lgame_config_from_namelist: null argument");
  std::memset(c, 0, sizeof *c);
  c->ny = n->ny; c->nx = n->nx; c->n_layers = n->n_layers; c->n_oro_layers = n->n_oro_layers;
  c->dx = n->dx; c->dy = n->dy; c->toa = n->toa; c->dtime = n->dtime;
  c->theta_adv_order = n->theta_adv_order; c->llinear = n->llinear; c->lcorio = n->lcorio;
  c->luse_bg_state = n->luse_bg_state; c->lplane = n->lplane; c->lmoist = n->lmoist;
  c->lklemp = n->lklemp; c->klemp_damp_max = n->klemp_damp_max; c->klemp_begin_rel = n->klemp_begin_rel;
  c->lmom_diff_h = n->lmom_diff_h; c->lmom_diff_v = n->lmom_diff_v; c->ltemp_diff_h = n->ltemp_diff_h;
  c->ltemp_diff_v = n->ltemp_diff_v; c->lmass_diff_h = n->lmass_diff_h; c->lmass_diff_v = n->lmass_diff_v;
  c->lprog_soil_temp = n->lprog_soil_temp; c->lsfc_sensible_heat_flux = n->lsfc_sensible_heat_flux;
  c->lsfc_phase_trans = n->lsfc_phase_trans; c->lpbl = n->lpbl;
  c->lperiodic = n->lperiodic; c->lfreeslip = n->lfreeslip;
  c->precision = n->precision; c->check_finite = n->check_finite;
  c->diff_coeff_scheme_h = (trim(n->diff_coeff_scheme_h) == "tke") ? LGAME_DIFF_COEFF_TKE : LGAME_DIFF_COEFF_SMAG;
  c->bg_shear = n->bg_shear; c->c_s = n->c_s;
  c->nsoillays = n->nsoillays; c->h_prandtl = n->h_prandtl; c->karman = n->karman;
  c->lphase_trans = n->lphase_trans;
  return LGAME_OK;
}
