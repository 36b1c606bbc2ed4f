// files.cpp -- raw binary files of the host side, where the reference uses netCDF (absent here):
// restart snapshots and lateral boundary levels.
//
// Every file is a 64-byte header followed by FP64 arrays in the reference's layout
// (column-major, reference extents), all little-endian:
//   bytes 0-7    magic, "LGAMESNP" (snapshot) or "LGAMEBCL" (boundary level)
//   bytes 8-11   int32 format version (3: the soil temperature and the surface diagnostics)
//   bytes 12-27  int32 ny, nx, n_layers, n_constituents
//   bytes 28-35  int64 step counter (snapshot) or the valid time in seconds as FP64 (level)
//   bytes 36-39  int32 nsoillays (snapshot; 0 in a boundary level)
//   bytes 40-63  zero
// Snapshot arrays: the LGAME_STATE_NFIELDS state fields of slot 0, then of slot 1 (enum
// lgame_state_field order, the soil temperature last), then the LGAME_DIAG_NFIELDS carried
// diagnostics (enum lgame_diag_field order): what
// resuming a run bit for bit needs (the reference's restart, mo_set_initial_state.F90:259-320,
// reads rho, rhotheta_v and the winds of one state from netCDF, and its output is FP32).
// Boundary level arrays: rho, rhotheta_v, wind_u, wind_v, wind_w of one time index of t_bc
// (mo_definitions.F90:117-131), as read_boundaries fills them (mo_boundaries.F90:99-123).
#include "common.h"
#include "lgame_gpu.h"
#include "lgame_host.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr int kVersion = 4;

struct Header {
  char magic[8];
  int32_t version, ny, nx, nl, ncons;
  unsigned char tag[8];  // int64 step or FP64 valid time
  int32_t nsoil;
  unsigned char pad[24];
};
static_assert(sizeof(Header) == 64, "header is 64 bytes");

int fail(int code, const std::string& msg) {
  lgame_set_error(msg.c_str());
  return code;
}

bool dims_ok(int ny, int nx, int nl, int ncons) {
  return ny >= 1 && nx >= 1 && nl >= 1 && (ncons == 1 || ncons == 7);
}

// element counts of the state and diagnostic fields (reference extents)
size_t state_n(int f, int ny, int nx, int nl, int ncons, int ns) {
  const size_t s = (size_t)ny * nx * nl;
  switch (f) {
    case LGAME_STATE_RHO: return s * ncons;
    case LGAME_STATE_TEMPERATURE_SOIL: return (size_t)ny * nx * (size_t)ns;
    case LGAME_STATE_WIND_U: return (size_t)ny * (nx + 1) * nl;
    case LGAME_STATE_WIND_V: return (size_t)(ny + 1) * nx * nl;
    case LGAME_STATE_WIND_W: return (size_t)ny * nx * (nl + 1);
    default: return s;
  }
}
size_t diag_n(int f, int ny, int nx, int nl, int ncons) {
  const size_t s = (size_t)ny * nx * nl, u = (size_t)ny * (nx + 1) * nl, v = (size_t)(ny + 1) * nx * nl,
               w = (size_t)ny * nx * (nl + 1);
  switch (f) {
    case LGAME_DIAG_P_GRAD_ACC_NEG_NL_U: case LGAME_DIAG_P_GRAD_ACC_NEG_L_U: case LGAME_DIAG_P_GRAD_ACC_OLD_U:
    case LGAME_DIAG_POT_VORT_TEND_X: case LGAME_DIAG_V_SQUARED_GRAD_X: case LGAME_DIAG_TEND_WIND_U:
    case LGAME_DIAG_MOM_DIFF_TEND_X: return u;
    case LGAME_DIAG_P_GRAD_ACC_NEG_NL_V: case LGAME_DIAG_P_GRAD_ACC_NEG_L_V: case LGAME_DIAG_P_GRAD_ACC_OLD_V:
    case LGAME_DIAG_POT_VORT_TEND_Y: case LGAME_DIAG_V_SQUARED_GRAD_Y: case LGAME_DIAG_TEND_WIND_V:
    case LGAME_DIAG_MOM_DIFF_TEND_Y: return v;
    case LGAME_DIAG_P_GRAD_ACC_NEG_NL_W: case LGAME_DIAG_P_GRAD_ACC_NEG_L_W: case LGAME_DIAG_POT_VORT_TEND_Z:
    case LGAME_DIAG_V_SQUARED_GRAD_Z: case LGAME_DIAG_TEND_WIND_W: case LGAME_DIAG_MOM_DIFF_TEND_Z: return w;
    case LGAME_DIAG_TEND_RHO: case LGAME_DIAG_MASS_DIFF_TENDENCY: return s * ncons;
    case LGAME_DIAG_ROUGHNESS_LENGTH: case LGAME_DIAG_ROUGHNESS_VELOCITY: case LGAME_DIAG_MONIN_OBUKHOV_LENGTH:
    case LGAME_DIAG_SCALAR_FLUX_RESISTANCE: case LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SOIL:
    case LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SEA: case LGAME_DIAG_SST: case LGAME_DIAG_SFC_SW_IN:
    case LGAME_DIAG_SFC_LW_OUT: case LGAME_DIAG_POWER_FLUX_DENSITY_LAT_LAKE:
    case LGAME_DIAG_POWER_FLUX_DENSITY_LAT_SEA: return (size_t)ny * nx;
    case LGAME_DIAG_PHASE_TRANS_RATES: return s * (ncons == 7 ? 6 : 1);
    default: return s;
  }
}

// FP64 arrays are written and read as little-endian bytes whatever the host's byte order
bool little_endian() {
  const uint16_t x = 1;
  unsigned char b[2];
  std::memcpy(b, &x, 2);
  return b[0] == 1;
}
void swap8(unsigned char* p, size_t n) {
  for (size_t i = 0; i < n; ++i, p += 8)
    for (int k = 0; k < 4; ++k) std::swap(p[k], p[7 - k]);
}

class File {
 public:
  File(const char* path, const char* mode) : f_(path ? std::fopen(path, mode) : nullptr) {}
  ~File() {
    if (f_) std::fclose(f_);
  }
  bool ok() const { return f_ != nullptr; }
  bool write(const void* p, size_t bytes) { return std::fwrite(p, 1, bytes, f_) == bytes; }
  bool read(void* p, size_t bytes) { return std::fread(p, 1, bytes, f_) == bytes; }
  bool write_doubles(const double* a, size_t n) {
    if (little_endian()) return write(a, n * 8);
    std::vector<unsigned char> b(n * 8);
    std::memcpy(b.data(), a, n * 8);
    swap8(b.data(), n);
    return write(b.data(), b.size());
  }
  bool read_doubles(double* a, size_t n) {
    if (!read(a, n * 8)) return false;
    if (!little_endian()) swap8(reinterpret_cast<unsigned char*>(a), n);
    return true;
  }
  bool close() {
    const bool ok = f_ && std::fclose(f_) == 0;
    f_ = nullptr;
    return ok;
  }
  bool at_end() { return f_ && std::fgetc(f_) == EOF; }

 private:
  std::FILE* f_;
};

Header make_header(const char* magic, int ny, int nx, int nl, int ncons, int ns, const void* tag8) {
  Header h;
  std::memset(&h, 0, sizeof h);
  std::memcpy(h.magic, magic, 8);
  h.version = kVersion;
  h.ny = ny;
  h.nx = nx;
  h.nl = nl;
  h.ncons = ncons;
  h.nsoil = ns;
  std::memcpy(h.tag, tag8, 8);
  if (!little_endian()) {  // the header's integers little-endian too
    for (int32_t* v : {&h.version, &h.ny, &h.nx, &h.nl, &h.ncons, &h.nsoil}) {
      unsigned char* b = reinterpret_cast<unsigned char*>(v);
      std::swap(b[0], b[3]);
      std::swap(b[1], b[2]);
    }
    swap8(h.tag, 1);
  }
  return h;
}

int check_header(Header h, const char* magic, const char* path, int ny, int nx, int nl, int ncons, int ns, void* tag8) {
  if (!little_endian()) {
    for (int32_t* v : {&h.version, &h.ny, &h.nx, &h.nl, &h.ncons, &h.nsoil}) {
      unsigned char* b = reinterpret_cast<unsigned char*>(v);
      std::swap(b[0], b[3]);
      std::swap(b[1], b[2]);
    }
    swap8(h.tag, 1);
  }
  if (std::memcmp(h.magic, magic, 8) != 0)
    return fail(LGAME_ERR_INVALID_ARG, std::string(path) + ": not a file of this kind (magic)");
  if (h.version != kVersion) return fail(LGAME_ERR_INVALID_ARG, std::string(path) + ": unknown format version");
  if (h.ny != ny || h.nx != nx || h.nl != nl || h.ncons != ncons || h.nsoil != ns)
    return fail(LGAME_ERR_BAD_DIMS, std::string(path) + ": written for other dimensions");
  std::memcpy(tag8, h.tag, 8);
  return LGAME_OK;
}

}  // namespace

extern "C" int lgame_host_write_snapshot(const char* path, int ny, int nx, int n_layers, int n_constituents,
                                         int nsoillays, long long step, const double* const* slot0,
                                         const double* const* slot1, const double* const* diag) {
  if (!path || !slot0 || !slot1 || !diag || !dims_ok(ny, nx, n_layers, n_constituents) || step < 0 ||
      nsoillays < 0 || nsoillays > LGAME_MAX_SOIL_LAYERS)
    return fail(LGAME_ERR_INVALID_ARG, "lgame_host_write_snapshot: bad arguments");
  for (int f = 0; f < LGAME_STATE_NFIELDS; ++f)
    if ((!slot0[f] || !slot1[f]) && state_n(f, ny, nx, n_layers, n_constituents, nsoillays) > 0)
      return fail(LGAME_ERR_INVALID_ARG, "lgame_host_write_snapshot: a state array is null");
  for (int f = 0; f < LGAME_DIAG_NFIELDS; ++f)
    if (!diag[f]) return fail(LGAME_ERR_INVALID_ARG, "lgame_host_write_snapshot: a diagnostic array is null");
  File out(path, "wb");
  if (!out.ok()) return fail(LGAME_ERR_INVALID_ARG, std::string("lgame_host_write_snapshot: cannot open ") + path);
  const int64_t s = step;
  const Header h = make_header("LGAMESNP", ny, nx, n_layers, n_constituents, nsoillays, &s);
  bool ok = out.write(&h, sizeof h);
  for (const double* const* slot : {slot0, slot1})
    for (int f = 0; f < LGAME_STATE_NFIELDS && ok; ++f)
      ok = out.write_doubles(slot[f], state_n(f, ny, nx, n_layers, n_constituents, nsoillays));
  for (int f = 0; f < LGAME_DIAG_NFIELDS && ok; ++f)
    ok = out.write_doubles(diag[f], diag_n(f, ny, nx, n_layers, n_constituents));
  if (!out.close() || !ok) return fail(LGAME_ERR_INVALID_ARG, std::string("lgame_host_write_snapshot: write failed: ") + path);
  return LGAME_OK;
}

extern "C" int lgame_host_read_snapshot(const char* path, int ny, int nx, int n_layers, int n_constituents,
                                        int nsoillays, long long* step, double* const* slot0, double* const* slot1,
                                        double* const* diag) {
  if (!path || !slot0 || !slot1 || !diag || !dims_ok(ny, nx, n_layers, n_constituents) || nsoillays < 0 ||
      nsoillays > LGAME_MAX_SOIL_LAYERS)
    return fail(LGAME_ERR_INVALID_ARG, "lgame_host_read_snapshot: bad arguments");
  for (int f = 0; f < LGAME_STATE_NFIELDS; ++f)
    if ((!slot0[f] || !slot1[f]) && state_n(f, ny, nx, n_layers, n_constituents, nsoillays) > 0)
      return fail(LGAME_ERR_INVALID_ARG, "lgame_host_read_snapshot: a state array is null");
  for (int f = 0; f < LGAME_DIAG_NFIELDS; ++f)
    if (!diag[f]) return fail(LGAME_ERR_INVALID_ARG, "lgame_host_read_snapshot: a diagnostic array is null");
  File in(path, "rb");
  if (!in.ok()) return fail(LGAME_ERR_INVALID_ARG, std::string("lgame_host_read_snapshot: cannot open ") + path);
  Header h;
  if (!in.read(&h, sizeof h)) return fail(LGAME_ERR_INVALID_ARG, std::string(path) + ": truncated header");
  int64_t s = 0;
  int rc = check_header(h, "LGAMESNP", path, ny, nx, n_layers, n_constituents, nsoillays, &s);
  if (rc) return rc;
  bool ok = true;
  for (double* const* slot : {slot0, slot1})
    for (int f = 0; f < LGAME_STATE_NFIELDS && ok; ++f)
      ok = in.read_doubles(slot[f], state_n(f, ny, nx, n_layers, n_constituents, nsoillays));
  for (int f = 0; f < LGAME_DIAG_NFIELDS && ok; ++f)
    ok = in.read_doubles(diag[f], diag_n(f, ny, nx, n_layers, n_constituents));
  if (!ok) return fail(LGAME_ERR_INVALID_ARG, std::string(path) + ": truncated");
  if (!in.at_end()) return fail(LGAME_ERR_INVALID_ARG, std::string(path) + ": longer than its header says");
  if (step) *step = (long long)s;
  return LGAME_OK;
}

extern "C" int lgame_host_write_bc_level(const char* path, int ny, int nx, int n_layers, int n_constituents,
                                         double t_valid, const double* rho, const double* rhotheta_v,
                                         const double* wind_u, const double* wind_v, const double* wind_w) {
  if (!path || !rho || !rhotheta_v || !wind_u || !wind_v || !wind_w || !dims_ok(ny, nx, n_layers, n_constituents))
    return fail(LGAME_ERR_INVALID_ARG, "lgame_host_write_bc_level: bad arguments");
  File out(path, "wb");
  if (!out.ok()) return fail(LGAME_ERR_INVALID_ARG, std::string("lgame_host_write_bc_level: cannot open ") + path);
  const Header h = make_header("LGAMEBCL", ny, nx, n_layers, n_constituents, 0, &t_valid);
  const double* a[5] = {rho, rhotheta_v, wind_u, wind_v, wind_w};
  const int f[5] = {LGAME_STATE_RHO, LGAME_STATE_RHOTHETA_V, LGAME_STATE_WIND_U, LGAME_STATE_WIND_V, LGAME_STATE_WIND_W};
  bool ok = out.write(&h, sizeof h);
  for (int k = 0; k < 5 && ok; ++k) ok = out.write_doubles(a[k], state_n(f[k], ny, nx, n_layers, n_constituents, 0));
  if (!out.close() || !ok) return fail(LGAME_ERR_INVALID_ARG, std::string("lgame_host_write_bc_level: write failed: ") + path);
  return LGAME_OK;
}

extern "C" int lgame_host_read_bc_level(const char* path, int ny, int nx, int n_layers, int n_constituents,
                                        double* t_valid, double* rho, double* rhotheta_v, double* wind_u,
                                        double* wind_v, double* wind_w) {
  if (!path || !rho || !rhotheta_v || !wind_u || !wind_v || !wind_w || !dims_ok(ny, nx, n_layers, n_constituents))
    return fail(LGAME_ERR_INVALID_ARG, "lgame_host_read_bc_level: bad arguments");
  File in(path, "rb");
  if (!in.ok()) return fail(LGAME_ERR_INVALID_ARG, std::string("lgame_host_read_bc_level: cannot open ") + path);
  Header h;
  if (!in.read(&h, sizeof h)) return fail(LGAME_ERR_INVALID_ARG, std::string(path) + ": truncated header");
  double t = 0.0;
  int rc = check_header(h, "LGAMEBCL", path, ny, nx, n_layers, n_constituents, 0, &t);
  if (rc) return rc;
  double* a[5] = {rho, rhotheta_v, wind_u, wind_v, wind_w};
  const int f[5] = {LGAME_STATE_RHO, LGAME_STATE_RHOTHETA_V, LGAME_STATE_WIND_U, LGAME_STATE_WIND_V, LGAME_STATE_WIND_W};
  bool ok = true;
  for (int k = 0; k < 5 && ok; ++k) ok = in.read_doubles(a[k], state_n(f[k], ny, nx, n_layers, n_constituents, 0));
  if (!ok) return fail(LGAME_ERR_INVALID_ARG, std::string(path) + ": truncated");
  if (!in.at_end()) return fail(LGAME_ERR_INVALID_ARG, std::string(path) + ": longer than its header says");
  if (t_valid) *t_valid = t;
  return LGAME_OK;
}

extern "C" int lgame_host_bc_filename(const char* root, double t_update, double t_init, char* out, int n) {
  if (!root || !out || n < 1) return fail(LGAME_ERR_INVALID_ARG, "lgame_host_bc_filename: bad arguments");
  // int2string(int(t_update - t_init)) of mo_boundaries.F90:112-113, truncation toward zero
  const double d = t_update - t_init;
  if (!(std::fabs(d) < 2147483647.0)) return fail(LGAME_ERR_INVALID_ARG, "lgame_host_bc_filename: time out of range");
  const int secs = (int)d;
  const int len = std::snprintf(out, (size_t)n, "%s+%ds.bin", root, secs);
  if (len < 0 || len >= n) return fail(LGAME_ERR_INVALID_ARG, "lgame_host_bc_filename: buffer too small");
  return LGAME_OK;
}

extern "C" int lgame_bc_file_loader(void* user, double t_update, int time_index) {
  auto* u = static_cast<lgame_bc_files*>(user);
  if (!u || !u->ctx || !u->root) return fail(LGAME_ERR_INVALID_ARG, "lgame_bc_file_loader: bad user data");
  char name[4096];
  int rc = lgame_host_bc_filename(u->root, t_update, u->t_init, name, (int)sizeof name);
  if (rc) return rc;
  const int ny = u->ny, nx = u->nx, nl = u->n_layers, nc = u->n_constituents;
  std::vector<double> rho(state_n(LGAME_STATE_RHO, ny, nx, nl, nc, 0)), rt(state_n(LGAME_STATE_RHOTHETA_V, ny, nx, nl, nc, 0)),
      wu(state_n(LGAME_STATE_WIND_U, ny, nx, nl, nc, 0)), wv(state_n(LGAME_STATE_WIND_V, ny, nx, nl, nc, 0)),
      ww(state_n(LGAME_STATE_WIND_W, ny, nx, nl, nc, 0));
  double t = 0.0;
  rc = lgame_host_read_bc_level(name, ny, nx, nl, nc, &t, rho.data(), rt.data(), wu.data(), wv.data(), ww.data());
  if (rc) return rc;
  return lgame_gpu_set_bc(u->ctx, time_index, rho.data(), rt.data(), wu.data(), wv.data(), ww.data());
}
