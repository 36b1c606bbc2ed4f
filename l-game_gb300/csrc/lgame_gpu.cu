// lgame_gpu.cu -- C ABI of the GB300 HEVI step: device memory, host<->device copies and
// the order of the kernels of one pchevi call (src/time_stepping/mo_manage_pchevi.F90).
#include "lgame_gpu.h"
#include "lgame_emulator.h"
#include "common.h"
#include "emulator.cuh"
#include "diffusion.cuh"
#include "kernels.cuh"
#include "phase.cuh"
#include "split.cuh"
#include "surface.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

using namespace lg;

namespace {

int set_err(int code, const std::string& msg) {
  lgame_set_error(msg.c_str());
  return code;
}

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return set_err(LGAME_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

}  // namespace

// device buffers of the radiation coupling (lgame_emulator.h): surface albedo, latitude and
// longitude per column, the feature rows and the heating rates of every column
struct RadBuffers {
  double *albedo = nullptr, *lat = nullptr, *lon = nullptr;
  float *features = nullptr, *heating = nullptr;
  long long ncol = 0;
  int nlev = 0;
};

struct lgame_gpu {
  lgame_config cfg;
  Dims D;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocations;
  long long bytes = 0;
  bool grid_set = false;
  int kernels_last_step = 0;
  // device fields (FP64)
  double* grid[LGAME_GRID_NFIELDS + 8] = {};
  double* ipw[6] = {};
  double* trsk_u[3] = {};
  double* trsk_v[2] = {};
  double* damp = nullptr;
  State st[2];
  Tend<double> tend;
  double *pg_nl_u, *pg_nl_v, *pg_nl_w, *pg_l_u, *pg_l_v, *pg_l_w, *pg_old_u, *pg_old_v, *pgcw;
  double *vsg_x, *vsg_y, *vsg_z, *pvt_x, *pvt_y, *pvt_z, *csh, *rad, *temperature;
  double* hdiss;  // heating_diss: dissipative heating, formed at each step's first substep
  // diffusion closure (&diff): which parts run, their buffers (tke, viscosity and the momentum
  // diffusion accelerations are carried diagnostics, allocated always) and constants
  bool diff_mom_h = false, diff_mom_v = false, diff_temp_h = false, diff_temp_v = false;
  bool diff_mass_h = false, diff_mass_v = false;
  DiffBuf<double> dbuf{};
  DiffPar dpar{};
  // surface layer, PBL and soil (&surface): which parts run, the surface grid planes and
  // diagnostics, the soil temperature of the two slots (nsoillays planes each)
  bool sfc_turb = false, sfc_pbl = false, sfc_sens = false, sfc_soil = false;
  SfcBuf sbuf{};
  SfcPar spar{};
  double* sfc_grid[6] = {};  // land, lake, roughness length, rho_c, conductivity, constant temperature
  double* tsoil[2] = {};
  // the phase transitions (lphase_trans extension): rates (nc+1 fields) and heating rate
  bool phase = false;
  double *ptr = nullptr, *pth = nullptr;
  // scratch
  double *theta, *gz, *gx, *gy, *divf, *tvu, *tvv, *tpu, *tpv, *ex, *ey, *ez, *uph, *vph, *wph, *vsq;
  double* staging = nullptr;
  size_t staging_elems = 0;
  double* reduce_buf = nullptr;
  int* flag = nullptr;
  Grid<double> G{};
  SplitCtx* split = nullptr;
  bool mirror_valid[2] = {false, false};  // split mode: FP32 mirror of the slot matches its FP64 state
  // the step as a CUDA graph, one per (old, new) slot pair, captured at its first use after
  // step 0 (every later step launches the same kernels with the same arguments)
  bool use_graphs = true;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  int graph_kernels[2] = {0, 0};
  // lateral boundary relaxation (t_bc, mo_definitions.F90:117-131): two levels in the
  // state's padded layout, the rescale factors on the padded plane, the bookkeeping
  bool bc_on = false;
  int bc_index_old = 1, bc_index_new = 2, dtime_bc = 0;
  double t_latest_bc = 0.0;
  lgame_bc_loader bc_loader = nullptr;
  void* bc_user = nullptr;
  State bc_lev[2]{};
  double *bcf_s = nullptr, *bcf_u = nullptr, *bcf_v = nullptr;
  int* bc_rim = nullptr;  // plane indices of the swamp layer (any factor nonzero), split path
  int bc_nrim = 0;
  // output fields (compact FP32, rho then T, RH, u, v, w), allocated at the first output
  float* out_buf = nullptr;
  // radiation emulator attached with lgame_gpu_rad_attach: run by lgame_gpu_pchevi when its
  // lrad_update is set (update_rad_fluxes, mo_manage_pchevi.F90:56-58), with the zenith angle
  // at t_0 + dtime_rad/2 (mo_manage_radiation_calls.F90:46-51); the report of the last update
  RadBuffers radbuf;
  lgame_emu* rad_emu = nullptr;
  double rad_dtime = 0.0, rad_bound = 0.0;
  int rad_stride = 0;
  double rad_report[4] = {0.0, 0.0, 0.0, 0.0};
  int rad_updates = 0;
  // lgame_gpu_pchevi_host: a second stream that copies the fields of the new state out while
  // the step still runs, and the two events the step records when they are final
  cudaStream_t side = nullptr;
  cudaEvent_t ev_mark[2] = {nullptr, nullptr};
  bool mark_on = false;
  int marks[2] = {0, 0};
  // per-kernel tracing
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<const char*, int>> ev_used;  // (kernel name, index of its start event)
  std::vector<std::pair<std::string, std::pair<int, double>>> prof_acc;
};

namespace lg {
// start/stop events around one launch when tracing is on (called from the step code)
int trace_begin(lgame_gpu* c, const char* name);
void trace_end(lgame_gpu* c, int slot);
}

namespace {

int dalloc(lgame_gpu* c, double** p, size_t n) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, n * sizeof(double));
  if (e != cudaSuccess) return set_err(LGAME_ERR_ALLOC, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  e = cudaMemset(q, 0, n * sizeof(double));
  if (e != cudaSuccess) return set_err(LGAME_ERR_CUDA, cudaGetErrorString(e));
  c->allocations.push_back(q);
  c->bytes += (long long)(n * sizeof(double));
  *p = (double*)q;
  return LGAME_OK;
}

// host array extents of the reference layout
struct Ext { size_t n1, n2, n3; };
Ext ext_s(const Dims& d) { return {(size_t)d.ny, (size_t)d.nx, (size_t)d.nl}; }
Ext ext_u(const Dims& d) { return {(size_t)d.ny, (size_t)d.nx + 1, (size_t)d.nl}; }
Ext ext_v(const Dims& d) { return {(size_t)d.ny + 1, (size_t)d.nx, (size_t)d.nl}; }
Ext ext_w(const Dims& d) { return {(size_t)d.ny, (size_t)d.nx, (size_t)d.nl + 1}; }
Ext ext_z(const Dims& d) { return {(size_t)d.ny + 1, (size_t)d.nx + 1, (size_t)d.nl}; }
Ext ext_ex(const Dims& d) { return {(size_t)d.ny + 1, (size_t)d.nx, (size_t)d.nl + 1}; }
Ext ext_ey(const Dims& d) { return {(size_t)d.ny, (size_t)d.nx + 1, (size_t)d.nl + 1}; }

Ext grid_ext(const Dims& d, int f) {
  switch (f) {
    case LGAME_GRID_Z_SCALAR: case LGAME_GRID_VOLUME: case LGAME_GRID_THETA_V_BG:
    case LGAME_GRID_EXNER_BG: case LGAME_GRID_GRAVITY_POTENTIAL: return ext_s(d);
    case LGAME_GRID_Z_U: case LGAME_GRID_DX: case LGAME_GRID_AREA_X: case LGAME_GRID_SLOPE_X:
    case LGAME_GRID_EXNER_BG_GRAD_U: return ext_u(d);
    case LGAME_GRID_Z_V: case LGAME_GRID_DY: case LGAME_GRID_AREA_Y: case LGAME_GRID_SLOPE_Y:
    case LGAME_GRID_EXNER_BG_GRAD_V: return ext_v(d);
    case LGAME_GRID_Z_W: case LGAME_GRID_DZ: case LGAME_GRID_AREA_Z: case LGAME_GRID_EXNER_BG_GRAD_W:
    case LGAME_GRID_GRAVITY_M_V: return ext_w(d);
    case LGAME_GRID_AREA_DUAL_X: return ext_ex(d);
    case LGAME_GRID_AREA_DUAL_Y: return ext_ey(d);
    case LGAME_GRID_AREA_DUAL_Z: case LGAME_GRID_Z_AREA_DUAL_Z: return ext_z(d);
    case LGAME_GRID_FVEC_X: return {(size_t)d.ny + 1, (size_t)d.nx, 1};
    case LGAME_GRID_FVEC_Y: return {(size_t)d.ny, (size_t)d.nx + 1, 1};
    case LGAME_GRID_FVEC_Z: return {(size_t)d.ny + 1, (size_t)d.nx + 1, 1};
    case LGAME_GRID_DX_DUAL: return ext_v(d);
    case LGAME_GRID_DY_DUAL: return ext_u(d);
    case LGAME_GRID_LAYER_THICKNESS: return ext_s(d);
    case LGAME_GRID_LAND_FRACTION: case LGAME_GRID_LAKE_FRACTION: case LGAME_GRID_ROUGHNESS_LENGTH:
    case LGAME_GRID_SFC_RHO_C: case LGAME_GRID_T_CONDUC_SOIL: case LGAME_GRID_T_CONST_SOIL:
      return {(size_t)d.ny, (size_t)d.nx, 1};
  }
  return {0, 0, 0};
}

Ext diag_ext(const Dims& d, int f) {
  switch (f) {
    case LGAME_DIAG_P_GRAD_ACC_NEG_NL_U: case LGAME_DIAG_P_GRAD_ACC_NEG_L_U: case LGAME_DIAG_P_GRAD_ACC_OLD_U:
    case LGAME_DIAG_POT_VORT_TEND_X: case LGAME_DIAG_V_SQUARED_GRAD_X: case LGAME_DIAG_TEND_WIND_U: return ext_u(d);
    case LGAME_DIAG_P_GRAD_ACC_NEG_NL_V: case LGAME_DIAG_P_GRAD_ACC_NEG_L_V: case LGAME_DIAG_P_GRAD_ACC_OLD_V:
    case LGAME_DIAG_POT_VORT_TEND_Y: case LGAME_DIAG_V_SQUARED_GRAD_Y: case LGAME_DIAG_TEND_WIND_V: return ext_v(d);
    case LGAME_DIAG_P_GRAD_ACC_NEG_NL_W: case LGAME_DIAG_P_GRAD_ACC_NEG_L_W: case LGAME_DIAG_POT_VORT_TEND_Z:
    case LGAME_DIAG_V_SQUARED_GRAD_Z: case LGAME_DIAG_TEND_WIND_W: return ext_w(d);
    case LGAME_DIAG_MOM_DIFF_TEND_X: return ext_u(d);
    case LGAME_DIAG_MOM_DIFF_TEND_Y: return ext_v(d);
    case LGAME_DIAG_MOM_DIFF_TEND_Z: return ext_w(d);
    case LGAME_DIAG_ROUGHNESS_LENGTH: case LGAME_DIAG_ROUGHNESS_VELOCITY: case LGAME_DIAG_MONIN_OBUKHOV_LENGTH:
    case LGAME_DIAG_SCALAR_FLUX_RESISTANCE: case LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SOIL:
    case LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SEA: case LGAME_DIAG_SST: case LGAME_DIAG_SFC_SW_IN:
    case LGAME_DIAG_SFC_LW_OUT: case LGAME_DIAG_POWER_FLUX_DENSITY_LAT_LAKE: case LGAME_DIAG_POWER_FLUX_DENSITY_LAT_SEA:
      return {(size_t)d.ny, (size_t)d.nx, 1};
    default: return ext_s(d);
  }
}

// host (column-major, extents e) <-> device (padded), one pitched 3-D copy
int copy_h2d(lgame_gpu* c, double* dev, const double* host, Ext e) {
  cudaMemcpy3DParms p = {};
  p.srcPtr = make_cudaPitchedPtr((void*)host, e.n1 * sizeof(double), e.n1, e.n2);
  p.dstPtr = make_cudaPitchedPtr(dev, (size_t)c->D.P * sizeof(double), (size_t)c->D.P, (size_t)c->D.NX1);
  p.extent = make_cudaExtent(e.n1 * sizeof(double), e.n2, e.n3);
  p.kind = cudaMemcpyHostToDevice;
  CK(cudaMemcpy3DAsync(&p, c->stream));
  return LGAME_OK;
}
int copy_d2h(lgame_gpu* c, double* host, const double* dev, Ext e, cudaStream_t stream = nullptr) {
  cudaMemcpy3DParms p = {};
  p.srcPtr = make_cudaPitchedPtr((void*)dev, (size_t)c->D.P * sizeof(double), (size_t)c->D.P, (size_t)c->D.NX1);
  p.dstPtr = make_cudaPitchedPtr(host, e.n1 * sizeof(double), e.n1, e.n2);
  p.extent = make_cudaExtent(e.n1 * sizeof(double), e.n2, e.n3);
  p.kind = cudaMemcpyDeviceToHost;
  CK(cudaMemcpy3DAsync(&p, stream ? stream : c->stream));
  return LGAME_OK;
}

// State transfer by the GPU itself over the coherent CPU-GPU link, for host arrays the GPU can
// address (page-locked and mapped: cudaPointerGetAttributes gives a device pointer).  One
// thread per element of a column-major host array of extent n1 x n2 x (n3*nrep) (nrep
// constituents back to back), coalesced along n1 on both sides.  k_state_in writes the padded
// FP64 field of both state slots and, with m0/m1 given, the FP32 mirror of both (rounded to
// nearest, as the mirror refresh does); k_state_out writes a slot's field back to the host.
__global__ void k_state_in(Dims D, const double* src, int n1, int n2, int n3, double* d0, double* d1, float* m0,
                           float* m1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n1) return;
  const int j = blockIdx.y, z = blockIdx.z, c = z / n3, k = z % n3;
  const long long h = i + (long long)n1 * (j + (long long)n2 * z);
  const long long q = (long long)c * D.fstride + i + (long long)D.P * (j + (long long)D.NX1 * k);
  const double v = src[h];
  d0[q] = v;
  d1[q] = v;
  if (m0) {
    const float f = narrow(v);
    m0[q] = f;
    m1[q] = f;
  }
}
__global__ void k_state_out(Dims D, const double* s, int n1, int n2, int n3, double* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n1) return;
  const int j = blockIdx.y, z = blockIdx.z, c = z / n3, k = z % n3;
  dst[i + (long long)n1 * (j + (long long)n2 * z)] =
      s[(long long)c * D.fstride + i + (long long)D.P * (j + (long long)D.NX1 * k)];
}

// the device address of a host array the GPU can read and write directly, or null
const double* device_view(const double* host) {
  if (!host) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();  // an unregistered pointer may leave an error behind
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return (const double*)a.devicePointer;
}

__global__ void k_split_ipw(Dims D, const double* src, double* w1, double* w2, double* w3, double* w4,
                            double* w5, double* w6) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const size_t h = 6 * ((size_t)(ji - 1) + (size_t)D.ny * ((size_t)(jk - 1) + (size_t)D.nx * (size_t)(jl - 1)));
  const long long q = IX(D, ji, jk, jl);
  w1[q] = src[h]; w2[q] = src[h + 1]; w3[q] = src[h + 2]; w4[q] = src[h + 3]; w5[q] = src[h + 4]; w6[q] = src[h + 5];
}

__global__ void k_check_finite(Dims D, State S, int* flag) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.y + 1;
  bool bad = false;
  if (ji <= D.ny && jk <= D.nx && jl <= D.nl) {
    const long long q = IX(D, ji, jk, jl);
    for (int jc = 0; jc < D.ncons; ++jc) bad |= !isfinite(S.rho[q + (long long)jc * D.fstride]);
    bad |= !isfinite(S.rt[q]) || !isfinite(S.ep[q]) || !isfinite(S.tp[q]);
  }
  if (ji <= D.ny && jk <= D.nx + 1 && jl <= D.nl) bad |= !isfinite(S.u[IX(D, ji, jk, jl)]);
  if (ji <= D.ny + 1 && jk <= D.nx && jl <= D.nl) bad |= !isfinite(S.v[IX(D, ji, jk, jl)]);
  if (ji <= D.ny && jk <= D.nx && jl <= D.NL) bad |= !isfinite(S.w[IX(D, ji, jk, jl)]);
  if (bad) atomicExch(flag, 1);
}

// update_boundaries, mo_boundaries.F90:19-97, one thread per point of the padded grid:
// x = factor*(w_old*x_old + w_new*x_new) + (1 - factor)*x for rho (every constituent),
// rhotheta_v and w at scalar columns, u and v at their points (the factors on the padded
// plane), then theta_v_pert and exner_pert from the relaxed rho and rhotheta_v (:92-95).
// With an FP32 mirror (split precision) every changed value is also written rounded.
__global__ void k_bc_update(Dims D, State S, StateF M, State B0, State B1, const double* fs, const double* fu,
                            const double* fv, double ow, double nw, const double* theta_v_bg, const double* exner_bg) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.y + 1;
  const long long p = (long long)(ji - 1) + (long long)D.P * (jk - 1);
  const bool mir = M.rho != nullptr;
  auto relax = [&](double f, const double* b0, const double* b1, double* x, float* xm, long long q) {
    const double r = f * (ow * b0[q] + nw * b1[q]) + (1.0 - f) * x[q];
    x[q] = r;
    if (mir) xm[q] = narrow(r);
    return r;
  };
  if (ji <= D.ny && jk <= D.nx) {
    const double f = fs[p];
    if (jl <= D.nl) {
      const long long q = IX(D, ji, jk, jl);
      double rho_g = 0.0;
      for (int jc = 0; jc < D.ncons; ++jc) {
        const long long qc = q + (long long)jc * D.fstride;
        const double r = relax(f, B0.rho, B1.rho, S.rho, M.rho, qc);
        if (jc == D.g - 1) rho_g = r;
      }
      const double rt = relax(f, B0.rt, B1.rt, S.rt, M.rt, q);
      const double tp = rt / rho_g - theta_v_bg[q];
      const double ep = pow(kR_D * rt / kP_0, kR_D / kC_D_V) - exner_bg[q];
      S.tp[q] = tp;
      S.ep[q] = ep;
      if (mir) {
        M.tp[q] = narrow(tp);
        M.ep[q] = narrow(ep);
      }
    }
    if (jl <= D.NL) relax(f, B0.w, B1.w, S.w, M.w, IX(D, ji, jk, jl));
  }
  if (ji <= D.ny && jk <= D.nx + 1 && jl <= D.nl) relax(fu[p], B0.u, B1.u, S.u, M.u, IX(D, ji, jk, jl));
  if (ji <= D.ny + 1 && jk <= D.nx && jl <= D.nl) relax(fv[p], B0.v, B1.v, S.v, M.v, IX(D, ji, jk, jl));
}

// rel_humidity of mo_derived.F90:131-155 with the quotient by the saturation pressure folded
// into one exponential: Huang's formulas are exp(a)/d^1.57 over water and exp(a)/d^2 over
// ice, so vp/sat = vp*exp(1.57*log(d) - a) and vp*d*d*exp(-a), the same values to a few FP64
// ulps with two transcendental calls fewer per point (the kernel below is bound by the FP64
// pipe); below -80 C (Murphy's formula and the blend) the reference's form is kept.
__device__ __forceinline__ double rel_humidity_out(double abs_humidity, double temperature) {
  const double vp = abs_humidity * kR_V * temperature;
  const double tc = temperature - kT_0;
  if (temperature > kT_0) {
    const double tw = tc > 100.0 ? 100.0 : tc;
    return vp * exp(1.57 * log(tw + 105.0) - (34.494 - 4924.99 / (tw + 237.1)));
  }
  if (tc >= -80.0) {  // min(T, t_0) = T here
    const double d = tc + 868.0;
    return vp * (d * d) * exp(-(43.494 - 6545.8 / (tc + 278.0)));
  }
  return vp / sat_ice(temperature);
}
// FP64 -> float rounded to nearest, zeros included, in integer operations (narrow)
__device__ __forceinline__ float to_f32(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  if (((hi & 0x7FFFFFFFu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
  return narrow(x);
}

// The output of the time loop: linear_combine_two_states (mo_linear_combination.F90:26-35)
// of states A and B, then the fields of write_output (mo_write_out.F90:167-217), one thread per
// scalar point, in the reference's order of operations (this file is compiled without fused
// multiply-adds; the relative humidity as rel_humidity_out), rounded to float as the file
// stores them.  out: compact column-major fields
// of ny*nx*nl floats, rho (ncons of them), T, RH, u, v, w.  *nan_flag = 1 if a combined
// exner_pert is NaN (mo_write_out.F90:60-67).
__global__ void k_output(Dims D, Grid<double> G, State A, State B, double c1, double c2, float* out, int* nan_flag) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl);
  const long long nS = (long long)D.ny * D.nx * D.nl;
  const long long o = (long long)(ji - 1) + (long long)D.ny * ((long long)(jk - 1) + (long long)D.nx * (jl - 1));
  double rho_g = 0.0, rho_v = 0.0;
  for (int jc = 0; jc < D.ncons; ++jc) {
    const long long qc = q + (long long)jc * D.fstride;
    const double r = c1 * A.rho[qc] + c2 * B.rho[qc];
    out[jc * nS + o] = to_f32(r);
    if (jc == D.g - 1) rho_g = r;
    if (jc == D.g) rho_v = r;  // water vapour follows the gas
  }
  const double rt = c1 * A.rt[q] + c2 * B.rt[q];
  const double tp = rt / rho_g - G.theta_v_bg[q];
  const double ep = c1 * A.ep[q] + c2 * B.ep[q];
  if (isnan(ep)) atomicExch(nan_flag, 1);
  float* f = out + (long long)D.ncons * nS;
  const double temperature = (G.theta_v_bg[q] + tp) * (G.exner_bg[q] + ep);
  f[o] = to_f32(temperature);
  if (D.ncons > 1) f[nS + o] = to_f32(rel_humidity_out(rho_v, temperature));
  const long long qu = IX(D, ji, jk + 1, jl), qv = IX(D, ji + 1, jk, jl), qw = IX(D, ji, jk, jl + 1);
  const double u0 = c1 * A.u[q] + c2 * B.u[q], u1 = c1 * A.u[qu] + c2 * B.u[qu];
  const double v0 = c1 * A.v[q] + c2 * B.v[q], v1 = c1 * A.v[qv] + c2 * B.v[qv];
  const double w0 = c1 * A.w[q] + c2 * B.w[q], w1 = c1 * A.w[qw] + c2 * B.w[qw];
  f[2 * nS + o] = to_f32(0.5 * (u0 + u1));
  f[3 * nS + o] = to_f32(0.5 * (v0 + v1));
  const double upper_weight = (G.z_scalar[q] - G.z_w[qw]) / (G.z_w[q] - G.z_w[qw]);
  f[4 * nS + o] = to_f32(upper_weight * w0 + (1.0 - upper_weight) * w1);
}

// simple_dissipation_rate, mo_momentum_diff_diss.F90:333-389, with the diffusion accelerations
// zero (diffusion is not in the step): the Klemp swamp layer's deceleration of w,
// (w/damping_prefactor - w)/dtime at w levels 2..n_damping_levels, its inner product with the
// wind (only the two vertical terms are nonzero) times -sum(rho(1:nc+1)).  damping_prefactor =
// 1 + dtime*damping_coeff is the column solver's prefactor G.damp (the same bits); it is 1 at the
// top level and wherever z_w lies below the layer, where the deceleration is then 0 as in the
// reference's loop bounds.  One thread per scalar point of layers 1..min(nl, n_damping_levels);
// the deeper layers stay 0.
__global__ void k_heating_diss(Dims D, Grid<double> G, State S, double* hd) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx || jl > D.nl) return;
  const long long q = IX(D, ji, jk, jl), b = q + D.plane;
  auto decel = [&](long long p, int lev) -> double {
    if (lev < 2 || lev > D.ndamp) return 0.0;
    const double w = S.w[p];
    return 0.0 + (w / G.damp[p] - w) / D.dtime;  // mom_diff_tend_z (0) plus the swamp layer's part
  };
  const double ip = G.ipw[4][q] * S.w[q] * decel(q, jl) + G.ipw[5][q] * S.w[b] * decel(b, jl + 1);
  hd[q] = -rho_sum_cond_gas<double, double>(D, S.rho, q) * ip;
}

// deterministic FP64 sums: every block sums a fixed strided subset in a fixed order;
// the partial sums are then added by one thread in block order.
constexpr int kRedBlocks = 1024, kRedThreads = 256;
__global__ void k_budget_partial(Dims D, Grid<double> G, State S, const double* T, double* part, int nq) {
  __shared__ double sh[kRedThreads];
  const long long n = (long long)D.ny * D.nx * D.nl;
  for (int k = 0; k < nq; ++k) {
    double acc = 0.0;
    for (long long e = (long long)blockIdx.x * kRedThreads + threadIdx.x; e < n; e += (long long)kRedBlocks * kRedThreads) {
      const int ji = (int)(e % D.ny) + 1;
      const int jk = (int)((e / D.ny) % D.nx) + 1;
      const int jl = (int)(e / ((long long)D.ny * D.nx)) + 1;
      const long long q = IX(D, ji, jk, jl);
      const double V = G.volume[q];
      const double rg = S.rho[q + (long long)(D.g - 1) * D.fstride];
      double x;
      if (k < D.ncons) x = S.rho[q + (long long)k * D.fstride] * V;
      else if (k == D.ncons) x = S.rt[q] * V;
      else if (k == D.ncons + 1) x = (rg * inner_product_at(D, G, S.u, S.v, S.w, ji, jk, jl)) * V;
      else if (k == D.ncons + 2) x = (rg * G.gp[q]) * V;
      else x = (kC_D_V * rg * T[q]) * V;
      acc = acc + x;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = kRedThreads / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[(long long)k * kRedBlocks + blockIdx.x] = sh[0];
    __syncthreads();
  }
}
__global__ void k_budget_final(const double* part, double* out, int nq) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int k = 0; k < nq; ++k) {
    double s = 0.0;
    for (int b = 0; b < kRedBlocks; ++b) s = s + part[(long long)k * kRedBlocks + b];
    out[k] = s;
  }
}

// Scratch of lgame_gpu_budgets_static: kRedBlocks partial sums for each of at most
// LGAME_BUDGETS_MAX budget quantities, plus the LGAME_BUDGETS_MAX results, (1024 * 11 + 11)
// doubles = 90,200 bytes per device, part of the loaded module (no cudaMalloc).  Nothing in it
// has to start at zero: k_budget_partial writes every partial sum before k_budget_final reads
// it, and k_budget_final writes every result before it is copied out.
constexpr int kStaticBudgetDoubles = kRedBlocks * LGAME_BUDGETS_MAX + LGAME_BUDGETS_MAX;
static __device__ __align__(256) double g_budget_scratch[kStaticBudgetDoubles];

// Loads, on the current device, the module that holds g_budget_scratch and the two reduction
// kernels (under CUDA's lazy loading a module or a kernel is loaded, and its memory taken, at
// its first use).  lgame_gpu_create calls this, so that lgame_gpu_budgets_static itself never
// triggers a load inside a host's time loop.
int preload_budget_scratch() {
  void* p = nullptr;
  cudaFuncAttributes fa;
  if (cudaGetSymbolAddress(&p, g_budget_scratch) != cudaSuccess || !p ||
      cudaFuncGetAttributes(&fa, k_budget_partial) != cudaSuccess ||
      cudaFuncGetAttributes(&fa, k_budget_final) != cudaSuccess)
    return set_err(LGAME_ERR_CUDA, std::string("loading the budget reduction module: ") +
                                       cudaGetErrorString(cudaGetLastError()));
  return LGAME_OK;
}

// FP64 instantiations of the kernel templates of kernels.cuh (this file is compiled with
// -fmad=false like the rest of the FP64 step)
namespace kd {
const auto k_temperature = lg::k_temperature<double>;
const auto k_theta = lg::k_theta<double>;
const auto k_grad_vert = lg::k_grad_vert<double, double>;
const auto k_grad_hor = lg::k_grad_hor<double, double>;
const auto k_div_h = lg::k_div_h<double>;
const auto k_theta_edges = lg::k_theta_edges<double>;
const auto k_eta_xy = lg::k_eta_xy<double>;
const auto k_eta_z = lg::k_eta_z<double>;
const auto k_mass_flux = lg::k_mass_flux<double>;
const auto k_vort_flux = lg::k_vort_flux<double>;
const auto k_ke = lg::k_ke<double>;
const auto k_tend_wind = lg::k_tend_wind<double>;
const auto k_tracers = lg::k_tracers<double>;
const auto k_gas_theta = lg::k_gas_theta<double>;
const auto k_pgrad = lg::k_pgrad;
const auto k_column_ver = lg::k_column_ver;
const auto k_column_tracers = lg::k_column_tracers;
const auto k_diff_tke = lg::k_diff_tke<double, double>;
const auto k_diff_visc = lg::k_diff_visc<double, double>;
const auto k_diff_zeta = lg::k_diff_zeta<double, double>;
const auto k_diff_vz = lg::k_diff_vz<double, double>;
const auto k_mom_diff_h = lg::k_mom_diff_h<double, double>;
const auto k_mom_diff_v = lg::k_mom_diff_v<double, double>;
const auto k_diss_rate = lg::k_diss_rate<double, double>;
const auto k_diff_fluxes1 = lg::k_diff_fluxes<double, double, double, 1>;
const auto k_diff_fluxes7 = lg::k_diff_fluxes<double, double, double, 7>;
const auto k_diff_divs1 = lg::k_diff_divs<double, 1>;
const auto k_diff_divs7 = lg::k_diff_divs<double, 7>;
const auto k_sfc_turb = lg::k_sfc_turb<double>;
const auto k_pbl = lg::k_pbl<double, double>;
const auto k_sfc_column = lg::k_sfc_column<double>;
const auto k_phase_trans = lg::k_phase_trans<double, double>;
}  // namespace kd

dim3 blk() { return dim3(32, 8, 1); }
// x: row tiles, y: levels, z: column tiles (see LG_IDX3)
dim3 grd(const Dims& D, int rows, int cols, int levs) {
  return dim3((unsigned)((rows + 31) / 32), (unsigned)levs, (unsigned)((cols + 7) / 8));
}

int klaunch_check(lgame_gpu* c, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_err(LGAME_ERR_CUDA, std::string("launch of ") + what + ": " + cudaGetErrorString(e));
  ++c->kernels_last_step;
  return LGAME_OK;
}
#define LAUNCH(kernel, grid_, ...)                                             \
  do {                                                                         \
    const int tr_ = c->profiling ? lg::trace_begin(c, #kernel) : -1;           \
    kernel<<<grid_, blk(), 0, c->stream>>>(__VA_ARGS__);                       \
    if (tr_ >= 0) lg::trace_end(c, tr_);                                       \
    int rc_ = klaunch_check(c, #kernel);                                       \
    if (rc_ != LGAME_OK) return rc_;                                           \
  } while (0)

// theta_v_adv_3rd_order (mo_multiplications.F90:116-204) of theta = theta_v_bg + tp
// (mode 0) or tp (mode 1): gradient, divergence, edge values into (ou, ov)
int theta3(lgame_gpu* c, const double* tp, int mode, const double* u, const double* v, double* ou, double* ov) {
  const Dims& D = c->D;
  LAUNCH(kd::k_theta, grd(D, D.ny, D.nx, D.nl), D, c->G, tp, c->theta, mode);
  LAUNCH(kd::k_grad_vert, grd(D, D.ny, D.nx, D.nl - 1), D, c->G, c->theta, c->gz);
  LAUNCH(kd::k_grad_hor, grd(D, D.ny + 1, D.nx + 1, D.nl), D, c->G, c->theta, c->gz, c->gx, c->gy);
  LAUNCH(kd::k_div_h, grd(D, D.ny, D.nx, D.nl), D, c->G, c->gx, c->gy, c->divf);
  LAUNCH(kd::k_theta_edges, grd(D, D.ny + 1, D.nx + 1, D.nl), D, c->G, c->theta, c->divf, u, v, ou, ov);
  return LGAME_OK;
}

// momentum advection of vector_tend_expl, mo_vector_tend_expl.F90:188-229
int advection(lgame_gpu* c, const State& S) {
  const Dims& D = c->D;
  if (!(!D.llinear || D.lcorio)) return LGAME_OK;
  LAUNCH(kd::k_eta_xy, grd(D, D.ny + 1, D.nx + 1, D.NL), D, c->G, S, c->ex, c->ey);
  LAUNCH(kd::k_eta_z, grd(D, D.ny + 1, D.nx + 1, D.nl), D, c->G, S, c->ez);
  LAUNCH(kd::k_mass_flux, grd(D, D.ny + 1, D.nx + 1, D.nl), D, c->G, S, c->uph, c->vph, c->wph);
  LAUNCH(kd::k_vort_flux, grd(D, D.ny + 1, D.nx + 1, D.nl), D, c->G, S, c->ex, c->ey, c->ez, c->uph, c->vph, c->wph,
         c->pvt_x, c->pvt_y, c->pvt_z);
  if (!D.llinear) {
    LAUNCH(kd::k_ke, grd(D, D.ny, D.nx, D.nl), D, c->G, S, c->vsq);
    LAUNCH(kd::k_grad_vert, grd(D, D.ny, D.nx, D.nl - 1), D, c->G, c->vsq, c->vsg_z);
    LAUNCH(kd::k_grad_hor, grd(D, D.ny + 1, D.nx + 1, D.nl), D, c->G, c->vsq, c->vsg_z, c->vsg_x, c->vsg_y);
  }
  return LGAME_OK;
}

// momentum diffusion and dissipation at the first substep, mo_vector_tend_expl.F90:100-126:
// n_squared and the TKE (the vertical coefficient scheme is always tke), the viscosity,
// mom_diff_h, mom_diff_v, then the dissipation rate (with the Klemp layer alone, its part)
int diffusion_vector(lgame_gpu* c, const State& So) {
  const Dims& D = c->D;
  const Grid<double>& G = c->G;
  const DiffBuf<double>& B = c->dbuf;
  if (c->diff_mom_h) {
    LAUNCH(kd::k_diff_tke, grd(D, D.ny, D.nx, D.nl), D, G, So, B, c->dpar);
    LAUNCH(kd::k_diff_zeta, grd(D, D.ny + 1, D.nx + 1, D.nl), D, G, So, B);
    LAUNCH(kd::k_diff_visc, grd(D, D.ny, D.nx, D.nl), D, G, So, c->temperature, B, c->dpar);
    LAUNCH(kd::k_diff_vz, grd(D, D.ny + 1, D.nx + 1, D.nl), D, G, So, B);
    LAUNCH(kd::k_mom_diff_h, grd(D, D.ny, D.nx, D.nl), D, G, So, B);
    if (c->diff_mom_v) LAUNCH(kd::k_mom_diff_v, grd(D, D.ny, D.nx, D.nl - 1), D, G, So, B);
    // pbl_wind_tendency (mo_vector_tend_expl.F90:119-121), before the dissipation reads the
    // momentum diffusion acceleration
    if (c->sfc_pbl) LAUNCH(kd::k_pbl, grd(D, D.ny, D.nx, 1), D, G, So, c->vsq, c->sbuf, c->spar, B.mdtx, B.mdty);
    LAUNCH(kd::k_diss_rate, grd(D, D.ny, D.nx, D.nl), D, G, So, B, G.damp, (const double*)nullptr);
  } else if (D.lklemp && D.ndamp > 0) {
    LAUNCH(k_heating_diss, grd(D, D.ny, D.nx, std::min(D.nl, D.ndamp)), D, G, So, c->hdiss);
  }
  return LGAME_OK;
}

// temperature and mass diffusion of scalar_tend_expl's first substep, mo_scalar_tend_expl.F90:
// 60-101 (the second substep's temperature diffusion repeats the first's: same temperature,
// same coefficients, so its result is reused)
int diffusion_scalar(lgame_gpu* c, const State& So) {
  const Dims& D = c->D;
  const Grid<double>& G = c->G;
  const DiffBuf<double>& B = c->dbuf;
  const dim3 gs = grd(D, D.ny, D.nx, D.nl), ge = grd(D, D.ny + 1, D.nx + 1, D.nl);
  if (c->diff_temp_h) {
    const int vert = c->diff_temp_v ? 1 : 0;
    LAUNCH(kd::k_diff_fluxes1, ge, D, G, So, B, (const double*)c->temperature, 1, vert, B.flx, B.fly, B.flw);
    LAUNCH(kd::k_diff_divs1, gs, D, G, B.flx, B.fly, B.flw, vert, B.tdh);
  }
  if (c->diff_mass_h) {  // every constituent in one launch each (1 dry, 7 moist)
    const int vert = c->diff_mass_v ? 1 : 0;
    if (D.ncons == 7) {
      LAUNCH(kd::k_diff_fluxes7, ge, D, G, So, B, (const double*)So.rho, 0, vert, B.flx, B.fly, B.flw);
      LAUNCH(kd::k_diff_divs7, gs, D, G, B.flx, B.fly, B.flw, vert, B.mdt);
    } else {
      LAUNCH(kd::k_diff_fluxes1, ge, D, G, So, B, (const double*)So.rho, 0, vert, B.flx, B.fly, B.flw);
      LAUNCH(kd::k_diff_divs1, gs, D, G, B.flx, B.fly, B.flw, vert, B.mdt);
    }
  }
  return LGAME_OK;
}

int step_fp64(lgame_gpu* c, int so, int sn, int step) {
  const Dims& D = c->D;
  const State& So = c->st[so];
  const State& Sn = c->st[sn];
  const Grid<double>& G = c->G;
  LAUNCH(kd::k_temperature, grd(D, D.ny, D.nx, D.nl), D, G, So, c->temperature);
  // update_sfc_turb_quantities (mo_manage_pchevi.F90:51-53)
  if (c->sfc_turb) LAUNCH(kd::k_sfc_turb, grd(D, D.ny, D.nx, 1), D, G, So, c->vsq, c->sbuf, c->spar);
  PGrad<double> P{c->pg_nl_u, c->pg_nl_v, c->pg_nl_w, c->pg_l_u, c->pg_l_v, c->pg_l_w, c->pg_old_u, c->pg_old_v, c->pgcw};
  Carried<double> C{c->pg_nl_u, c->pg_nl_v, c->pg_nl_w, c->pg_l_u, c->pg_l_v, c->pg_l_w, c->pg_old_u, c->pg_old_v, c->pgcw,
            c->vsg_x, c->vsg_y, c->vsg_z, c->pvt_x, c->pvt_y, c->pvt_z};
  for (int rk = 1; rk <= 2; ++rk) {
    const State& Sv = (rk == 1) ? So : Sn;   // state of vector_tend_expl
    if (rk == 1) {
      // manage_p_grad (mo_p_grad.F90:20-104) and calc_p_grad_condensates_v (:106-120):
      // theta edge values first (they use gx/gy/gz as scratch), then grad(exner_pert)
      if (D.theta_order == 3) {
        int rc = theta3(c, So.tp, 0, So.u, So.v, c->tvu, c->tvv);
        if (rc != LGAME_OK) return rc;
        if (D.luse_bg) { rc = theta3(c, So.tp, 1, So.u, So.v, c->tpu, c->tpv); if (rc != LGAME_OK) return rc; }
      }
      LAUNCH(kd::k_grad_vert, grd(D, D.ny, D.nx, D.nl - 1), D, G, So.ep, c->gz);
      LAUNCH(kd::k_grad_hor, grd(D, D.ny + 1, D.nx + 1, D.nl), D, G, So.ep, c->gz, c->gx, c->gy);
      LAUNCH(kd::k_pgrad, grd(D, D.ny + 1, D.nx + 1, D.nl), D, G, So, c->gx, c->gy, c->gz, c->tvu, c->tvv, c->tpu, c->tpv,
             P, step == 0 ? 1 : 0);
    }
    if (rk == 2 || step == 0) {
      int rc = advection(c, Sv);
      if (rc != LGAME_OK) return rc;
    }
    // momentum diffusion and dissipation at the first substep (mo_vector_tend_expl.F90:100-126)
    if (rk == 1) {
      const int rc = diffusion_vector(c, So);
      if (rc != LGAME_OK) return rc;
    }
    Tend<double> T = c->tend;
    if (c->diff_mom_h) { C.mdt_x = c->dbuf.mdtx; C.mdt_y = c->dbuf.mdty; C.mdt_z = c->dbuf.mdtz; }
    LAUNCH(kd::k_tend_wind, grd(D, D.ny + 1, D.nx + 1, D.NL), D, So, Sn, T, C, rk, (float*)nullptr, (float*)nullptr);
    // scalar_tend_expl (mo_scalar_tend_expl.F90:24-181)
    const State& Ss = (rk == 1) ? So : Sn;
    if (rk == 1) {
      const int rc = diffusion_scalar(c, So);
      if (rc != LGAME_OK) return rc;
    }
    const double* mdt = c->diff_mass_h ? c->dbuf.mdt : nullptr;
    const double* tdh = c->diff_temp_h ? c->dbuf.tdh : nullptr;
    // the phase transitions (extension; the reference never calls them) at the first substep,
    // from state_old and the temperature diagnosed from it; both substeps read the rates
    if (rk == 1 && c->phase)
      LAUNCH(kd::k_phase_trans, grd(D, D.ny, D.nx, D.nl), D, G, So, (const double*)c->temperature, c->sbuf,
             (const double*)c->tsoil[so], c->cfg.lsfc_phase_trans, D.dtime, c->ptr, c->pth);
    const double* ptr = c->phase ? c->ptr : nullptr;
    const double* pth = c->phase ? c->pth : nullptr;
    if (D.ncons > 1) LAUNCH(kd::k_tracers, grd(D, D.ny, D.nx, D.nl), D, G, Ss, Sn.u, Sn.v, T.rho, rk, mdt, ptr);
    // theta_v_adv_3rd_order of the state used here: in the first substep that is state_old,
    // whose edges manage_p_grad's call above already left in tvu/tvv (nothing in between
    // writes state_old or tvu/tvv), so only the second substep recomputes them -- the same
    // values the reference recomputes
    if (D.theta_order == 3 && rk == 2) {
      int rc = theta3(c, Ss.tp, 0, Ss.u, Ss.v, c->tvu, c->tvv);
      if (rc != LGAME_OK) return rc;
    }
    LAUNCH(kd::k_gas_theta, grd(D, D.ny, D.nx, D.nl), D, G, Ss, Sn.u, Sn.v, c->tvu, c->tvv, c->temperature, c->hdiss,
           c->rad, c->csh, T.rho, T.rt, mdt, tdh, ptr, pth);
    // three_band_solver_ver (+ w_free_slip), three_band_solver_gen_densities
    {
      // the sensible heat flux and the soil rows of three_band_solver_ver (mo_column_solvers.F90:
      // 80-120, 228-300), ahead of its atmospheric rows, which read the heated tendency
      if (c->sfc_sens || c->sfc_soil)
        LAUNCH(kd::k_sfc_column, grd(D, D.ny, D.nx, 1), D, G, So, rk == 1 ? So : Sn, T.rt, c->sbuf, c->spar,
               c->tsoil[so], c->tsoil[rk == 1 ? so : sn], c->tsoil[sn]);
      dim3 g2((unsigned)((D.ny + 31) / 32), (unsigned)((D.nx + 7) / 8), 1);
      LAUNCH(kd::k_column_ver, g2, D, G, So, Sn, T, rk);
      if (D.ncons > 1) LAUNCH(kd::k_column_tracers, g2, D, G, So, Sn, T.rho, c->temperature, c->csh, rk);
    }
  }
  return LGAME_OK;
}

// split mode keeps the diagnostics that the FP32 stencils produce in FP32 buffers; they
// are converted to/from the FP64 arrays of the C ABI on set_diag (to_split) and get_diag
int split_sync_carried(lgame_gpu* c, bool to_split) {
  const SplitCarriedF F = split_carried(c->split);
  const long long n = c->D.fstride;
  struct Pair { double* d; float* f; long long n; };
  const Pair pairs[] = {{c->pgcw, F.pgcw, n}, {c->vsg_x, F.vsg_x, n}, {c->vsg_y, F.vsg_y, n}, {c->vsg_z, F.vsg_z, n},
                        {c->pvt_x, F.pvt_x, n}, {c->pvt_y, F.pvt_y, n}, {c->pvt_z, F.pvt_z, n}, {c->csh, F.csh, n},
                        {c->rad, F.rad, n}, {c->temperature, F.temperature, n}, {c->tend.rho, F.tend.rho, n * c->D.ncons},
                        {c->tend.rt, F.tend.rt, n}, {c->tend.u, F.tend.u, n}, {c->tend.v, F.tend.v, n},
                        {c->tend.w, F.tend.w, n}, {c->hdiss, F.hdiss, n},
                        {c->dbuf.tke, F.tke, n}, {c->dbuf.visc, F.visc, n}, {c->dbuf.mdtx, F.mdtx, n},
                        {c->dbuf.mdty, F.mdty, n}, {c->dbuf.mdtz, F.mdtz, n},
                        {c->ptr, F.ptr, n * (c->D.nc + 1)}, {c->pth, F.pth, n},
                        {c->dbuf.tdh, F.tdh, n}, {c->dbuf.mdt, F.mdt, n * c->D.ncons}};
  for (const Pair& p : pairs) {
    if (!p.f || !p.d) continue;  // the part is off: no FP32 copy, or no FP64 array
    const int rc = to_split ? split_convert(p.d, p.f, p.n, c->stream) : split_convert_back(p.f, p.d, p.n, c->stream);
    if (rc != LGAME_OK) return set_err(rc, "conversion of the split-mode diagnostics failed");
  }
  // with a background state the split step keeps the pressure-gradient terms the wind update
  // uses in FP32 (net nl + l, previous -(nl + l)); p_grad_acc_old lives only in that form
  if (c->D.luse_bg) {
    int rc = LGAME_OK;
    if (to_split) {
      if (!rc) rc = split_net(c->pg_nl_u, c->pg_l_u, F.pnet_u, n, c->stream);
      if (!rc) rc = split_net(c->pg_nl_v, c->pg_l_v, F.pnet_v, n, c->stream);
      if (!rc) rc = split_net(c->pg_nl_w, c->pg_l_w, F.pnet_w, n, c->stream);
      if (!rc) rc = split_convert(c->pg_old_u, F.pold_u, n, c->stream);
      if (!rc) rc = split_convert(c->pg_old_v, F.pold_v, n, c->stream);
    } else {
      if (!rc) rc = split_convert_back(F.pold_u, c->pg_old_u, n, c->stream);
      if (!rc) rc = split_convert_back(F.pold_v, c->pg_old_v, n, c->stream);
    }
    if (rc != LGAME_OK) return set_err(rc, "conversion of the split-mode pressure-gradient terms failed");
  }
  return LGAME_OK;
}

int trace_begin_cb(void* c, const char* name) { return lg::trace_begin((lgame_gpu*)c, name); }
void trace_end_cb(void* c, int slot) { lg::trace_end((lgame_gpu*)c, slot); }
// marks of the split step for lgame_gpu_pchevi_host: event 0 after the second substep's wind
// update (u and v final), event 1 after its vertical solve (rhotheta_v, theta_v_pert,
// exner_pert, w and the gas density final; the tracer solver writes only the other densities)
int mark_begin_cb(void* p, const char* name) {
  auto* c = (lgame_gpu*)p;
  if (std::strcmp(name, "ks_tend_wind") == 0 && ++c->marks[0] == 2) return 0;
  if (std::strcmp(name, "ks_column_ver") == 0 && ++c->marks[1] == 2) return 1;
  return -1;
}
void mark_end_cb(void* p, int k) {
  auto* c = (lgame_gpu*)p;
  if (cudaEventRecord(c->ev_mark[k], c->stream) != cudaSuccess) c->marks[k] = -1;  // no early copy
}

int check_cfg(const lgame_config* cfg) {
  if (cfg->ny < 3 || cfg->nx < 3) return set_err(LGAME_ERR_BAD_DIMS, "ny and nx must be >= 3");
  if (cfg->n_layers < 3 || cfg->n_layers > 128) return set_err(LGAME_ERR_BAD_DIMS, "n_layers must be in 3..128");
  {  // one field's padded extent must stay below 2^31 points (32-bit offsets within a field)
    const long long P = ((long long)cfg->ny + 1 + 31) / 32 * 32;
    if (P * ((long long)cfg->nx + 1) * ((long long)cfg->n_layers + 1) >= (1LL << 31))
      return set_err(LGAME_ERR_BAD_DIMS, "the grid is too large: (ny+1 rounded up to 32)*(nx+1)*(n_layers+1) must be < 2^31");
  }
  if (cfg->n_oro_layers < 1 || cfg->n_oro_layers >= cfg->n_layers)
    return set_err(LGAME_ERR_BAD_DIMS, "it must be 1 <= n_oro_layers < n_layers");
  if (cfg->theta_adv_order != 2 && cfg->theta_adv_order != 3)
    return set_err(LGAME_ERR_BAD_CONFIG, "theta_adv_order must be 2 or 3");
  if (!(cfg->dtime > 0.0) || !(cfg->toa > 0.0) || !(cfg->dx > 0.0) || !(cfg->dy > 0.0))
    return set_err(LGAME_ERR_BAD_CONFIG, "dtime, toa, dx and dy must be positive");
  if (cfg->precision != LGAME_PRECISION_FP64 && cfg->precision != LGAME_PRECISION_SPLIT &&
      cfg->precision != LGAME_PRECISION_SPLIT_FP64_COLUMN)
    return set_err(LGAME_ERR_BAD_CONFIG,
                   "precision must be LGAME_PRECISION_FP64, LGAME_PRECISION_SPLIT or LGAME_PRECISION_SPLIT_FP64_COLUMN");
  if (cfg->diff_coeff_scheme_h != LGAME_DIFF_COEFF_SMAG && cfg->diff_coeff_scheme_h != LGAME_DIFF_COEFF_TKE)
    return set_err(LGAME_ERR_BAD_CONFIG, "diff_coeff_scheme_h must be LGAME_DIFF_COEFF_SMAG or LGAME_DIFF_COEFF_TKE");
  // the reference's diffusion reads coefficients and TKE values only horizontal momentum
  // diffusion forms in the same step (mo_eff_diff_coeffs.F90:541-596, mo_momentum_diff_diss.F90:
  // 286, mo_vector_tend_expl.F90:104-117): without it they are those of earlier calls
  if ((cfg->ltemp_diff_h || cfg->lmass_diff_h || cfg->lmom_diff_v) && !cfg->lmom_diff_h)
    return set_err(LGAME_ERR_UNSUPPORTED, "temperature, mass or vertical momentum diffusion without horizontal momentum "
                                          "diffusion (lmom_diff_h) is not part of the GPU step");
  // non-periodic: tke_update's inner product reads grad(tke) at the boundary edges, which the
  // reference leaves at the zero of mom_diff_v's or the third-order theta advection's last
  // whole-array write only in these configurations
  if (cfg->lmom_diff_h && !cfg->lperiodic && !cfg->lmom_diff_v && cfg->theta_adv_order != 3)
    return set_err(LGAME_ERR_UNSUPPORTED, "non-periodic horizontal momentum diffusion without lmom_diff_v needs "
                                          "theta_adv_order 3 in the GPU step");

  // &surface: the reference stops when lpbl is on without lmom_diff_h (mo_surface_nml.F90:46-49);
  // its sensible heat flux divides by the scalar flux resistance, which only the prognostic
  // soil's branch of update_sfc_turb_quantities forms (mo_pbl.F90:96-106), so without it the
  // flux is x/0
  if (cfg->lpbl && !cfg->lmom_diff_h)
    return set_err(LGAME_ERR_BAD_CONFIG, "lpbl needs lmom_diff_h (mo_surface_nml.F90:46-49)");
  if (cfg->lsfc_sensible_heat_flux && !cfg->lprog_soil_temp)
    return set_err(LGAME_ERR_UNSUPPORTED, "lsfc_sensible_heat_flux without lprog_soil_temp divides by a zero scalar flux "
                                          "resistance in the reference");
  if ((cfg->lprog_soil_temp || cfg->lsfc_sensible_heat_flux) &&
      (cfg->nsoillays < 2 || cfg->nsoillays > LGAME_MAX_SOIL_LAYERS))
    return set_err(LGAME_ERR_BAD_CONFIG, "nsoillays must lie in 2.." + std::to_string(LGAME_MAX_SOIL_LAYERS) +
                                         " with the prognostic soil");
  if (cfg->nsoillays < 0 || cfg->nsoillays > LGAME_MAX_SOIL_LAYERS)
    return set_err(LGAME_ERR_BAD_CONFIG, "nsoillays out of range");
  if ((cfg->lsfc_sensible_heat_flux || cfg->lsfc_phase_trans || cfg->lpbl) && !(cfg->karman > 0.0 && cfg->h_prandtl > 0.0))
    return set_err(LGAME_ERR_BAD_CONFIG, "karman and h_prandtl must be positive with the surface layer on");
  // the phase transitions (extension) act on the water constituents; their surface evaporation
  // divides by the scalar flux resistance, which only the prognostic soil forms
  if (cfg->lphase_trans && !cfg->lmoist)
    return set_err(LGAME_ERR_BAD_CONFIG, "lphase_trans needs lmoist");
  if (cfg->lphase_trans && cfg->lsfc_phase_trans && !cfg->lprog_soil_temp)
    return set_err(LGAME_ERR_UNSUPPORTED, "the surface phase transitions without lprog_soil_temp divide by a zero scalar "
                                          "flux resistance");
  return LGAME_OK;
}

}  // namespace

extern "C" int lgame_gpu_create(const lgame_config* cfg, lgame_gpu** out) {
  if (!cfg || !out) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_create: null argument");
  *out = nullptr;
  int rc = check_cfg(cfg);
  if (rc != LGAME_OK) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_err(LGAME_ERR_NO_DEVICE, "no CUDA device is visible");
  }
  const int dev = cfg->device;
  if (dev < 0 || dev >= ndev) return set_err(LGAME_ERR_NO_DEVICE, "lgame_config.device is not a visible device");
  CK(cudaSetDevice(dev));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, dev));
  if (prop.major != 10 || prop.minor != 3)
    return set_err(LGAME_ERR_NO_DEVICE, std::string("this library is built for sm_103 (GB300); device is ") + prop.name);
  auto* c = new lgame_gpu();
  c->cfg = *cfg;
  Dims& D = c->D;
  D.ny = cfg->ny; D.nx = cfg->nx; D.nl = cfg->n_layers; D.NL = cfg->n_layers + 1;
  D.nf = cfg->n_layers - cfg->n_oro_layers;
  D.P = ((D.ny + 1) + 31) / 32 * 32;
  D.NX1 = D.nx + 1;
  D.plane = (long long)D.P * D.NX1;
  D.fstride = D.plane * (D.nl + 1);
  D.nc = cfg->lmoist ? 5 : 0;
  D.ncons = D.nc + (cfg->lmoist ? 2 : 1);
  D.g = D.nc + 1;
  D.periodic = cfg->lperiodic; D.freeslip = cfg->lfreeslip; D.lcorio = cfg->lcorio; D.llinear = cfg->llinear;
  D.luse_bg = cfg->luse_bg_state; D.lmoist = cfg->lmoist; D.theta_order = cfg->theta_adv_order; D.lklemp = cfg->lklemp;
  D.dtime = cfg->dtime; D.toa = cfg->toa; D.dxn = cfg->dx; D.dyn = cfg->dy;
  D.theta_edge_c = 1.0 / 8.0 * D.dyn * D.dxn;  // the device expression, evaluated once
  D.ndamp = 0;                                  // set with the grid
  auto fail = [&](int code) { lgame_gpu_destroy(c); return code; };
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(set_err(LGAME_ERR_CUDA, "cudaStreamCreate failed"));
  if ((rc = preload_budget_scratch()) != LGAME_OK) return fail(rc);
  const size_t F = (size_t)D.fstride;
  // grid
  for (int f = 0; f < LGAME_GRID_LAND_FRACTION; ++f) {
    if (f == LGAME_GRID_INNER_PRODUCT_WEIGHTS || f == LGAME_GRID_TRSK_WEIGHTS_U || f == LGAME_GRID_TRSK_WEIGHTS_V) continue;
    size_t n = (f == LGAME_GRID_FVEC_X || f == LGAME_GRID_FVEC_Y || f == LGAME_GRID_FVEC_Z) ? (size_t)D.plane : F;
    if ((rc = dalloc(c, &c->grid[f], n)) != LGAME_OK) return fail(rc);
  }
  // surface layer and soil: one plane per surface field, nsoillays planes of soil temperature
  // per slot, the soil grid in the kernels' parameter block
  {
    c->sfc_soil = cfg->lprog_soil_temp;
    c->sfc_sens = cfg->lsfc_sensible_heat_flux;
    c->sfc_pbl = cfg->lpbl;
    c->sfc_turb = cfg->lsfc_sensible_heat_flux || cfg->lsfc_phase_trans || cfg->lpbl;
    for (double*& p : c->sfc_grid) if ((rc = dalloc(c, &p, (size_t)D.plane)) != LGAME_OK) return fail(rc);
    SfcBuf& B = c->sbuf;
    double** diag[] = {&B.rl, &B.rv, &B.mol, &B.sfr, &B.sens_soil, &B.sens_sea, &B.sst, &B.sw_in, &B.lw_out,
                       &B.lat_lake, &B.lat_sea};
    for (double** p : diag) if ((rc = dalloc(c, p, (size_t)D.plane)) != LGAME_OK) return fail(rc);
    B.land = c->sfc_grid[0]; B.lake = c->sfc_grid[1]; B.rl_grid = c->sfc_grid[2];
    B.rhoc = c->sfc_grid[3]; B.tcond = c->sfc_grid[4]; B.tconst = c->sfc_grid[5];
    const int ns = cfg->nsoillays;
    if (ns > 0)
      for (double*& p : c->tsoil) if ((rc = dalloc(c, &p, (size_t)D.plane * ns)) != LGAME_OK) return fail(rc);
    SfcPar& P = c->spar;
    P.h_prandtl = cfg->h_prandtl; P.karman = cfg->karman; P.dtime = cfg->dtime; P.z_t_const = 0.0;
    P.ns = ns; P.prog_soil = cfg->lprog_soil_temp; P.sens = cfg->lsfc_sensible_heat_flux;
    c->phase = cfg->lphase_trans;
    if (c->phase && ((rc = dalloc(c, &c->ptr, F * (size_t)(D.nc + 1))) || (rc = dalloc(c, &c->pth, F)))) return fail(rc);
  }
  for (int k = 0; k < 6; ++k) if ((rc = dalloc(c, &c->ipw[k], F)) != LGAME_OK) return fail(rc);
  for (int k = 0; k < 3; ++k) if ((rc = dalloc(c, &c->trsk_u[k], (size_t)D.P)) != LGAME_OK) return fail(rc);
  for (int k = 0; k < 2; ++k) if ((rc = dalloc(c, &c->trsk_v[k], (size_t)D.P)) != LGAME_OK) return fail(rc);
  if ((rc = dalloc(c, &c->damp, F)) != LGAME_OK) return fail(rc);
  // states and tendencies
  for (int s = 0; s < 2; ++s) {
    State& S = c->st[s];
    if ((rc = dalloc(c, &S.rho, F * D.ncons)) || (rc = dalloc(c, &S.rt, F)) || (rc = dalloc(c, &S.tp, F)) ||
        (rc = dalloc(c, &S.ep, F)) || (rc = dalloc(c, &S.u, F)) || (rc = dalloc(c, &S.v, F)) || (rc = dalloc(c, &S.w, F)))
      return fail(rc);
  }
  if ((rc = dalloc(c, &c->tend.rho, F * D.ncons)) || (rc = dalloc(c, &c->tend.rt, F)) || (rc = dalloc(c, &c->tend.u, F)) ||
      (rc = dalloc(c, &c->tend.v, F)) || (rc = dalloc(c, &c->tend.w, F)))
    return fail(rc);
  double** carried[] = {&c->pg_nl_u, &c->pg_nl_v, &c->pg_nl_w, &c->pg_l_u, &c->pg_l_v, &c->pg_l_w, &c->pg_old_u,
                        &c->pg_old_v, &c->pgcw, &c->vsg_x, &c->vsg_y, &c->vsg_z, &c->pvt_x, &c->pvt_y, &c->pvt_z,
                        &c->csh, &c->rad, &c->temperature, &c->hdiss};
  for (double** p : carried) if ((rc = dalloc(c, p, F)) != LGAME_OK) return fail(rc);
  double** scratch[] = {&c->theta, &c->gz, &c->gx, &c->gy, &c->divf, &c->tvu, &c->tvv, &c->tpu, &c->tpv,
                        &c->ex, &c->ey, &c->ez, &c->uph, &c->vph, &c->wph, &c->vsq};
  for (double** p : scratch) if ((rc = dalloc(c, p, F)) != LGAME_OK) return fail(rc);
  // diffusion closure: the carried diagnostics always, the work arrays when a part is on
  {
    DiffBuf<double>& B = c->dbuf;
    double** carried_d[] = {&B.tke, &B.visc, &B.mdtx, &B.mdty, &B.mdtz};
    for (double** p : carried_d) if ((rc = dalloc(c, p, F)) != LGAME_OK) return fail(rc);
    B.hd = c->hdiss;
    c->diff_mom_h = cfg->lmom_diff_h; c->diff_mom_v = cfg->lmom_diff_v;
    c->diff_temp_h = cfg->ltemp_diff_h; c->diff_temp_v = cfg->ltemp_diff_v;
    c->diff_mass_h = cfg->lmass_diff_h; c->diff_mass_v = cfg->lmass_diff_v;
    if (c->diff_mom_h) {
      // temp_diff_heating and mass_diff_tendency in both modes (the C ABI's diagnostics), the work
      // arrays for the FP64 step only (the split step keeps FP32 ones)
      if (c->diff_temp_h && (rc = dalloc(c, &B.tdh, F)) != LGAME_OK) return fail(rc);
      if (c->diff_mass_h && (rc = dalloc(c, &B.mdt, F * D.ncons)) != LGAME_OK) return fail(rc);
    }
    if (c->diff_mom_h && cfg->precision == LGAME_PRECISION_FP64) {
      double** work[] = {&B.tke_new, &B.vmol, &B.nsq, &B.vz, &B.zz, &B.vdiv};
      for (double** p : work) if ((rc = dalloc(c, p, F)) != LGAME_OK) return fail(rc);
      if (c->diff_temp_h || c->diff_mass_h) {
        const size_t nf = c->diff_mass_h ? (size_t)D.ncons : 1;
        if ((rc = dalloc(c, &B.flx, F * nf)) || (rc = dalloc(c, &B.fly, F * nf)) || (rc = dalloc(c, &B.flw, F * nf)))
          return fail(rc);
      }
    }
    DiffPar& P = c->dpar;
    P.eff_hor_res = std::sqrt(cfg->dx * cfg->dy);
    P.c_s = cfg->c_s; P.bg_shear = cfg->bg_shear;
    P.tke_h = cfg->diff_coeff_scheme_h == LGAME_DIFF_COEFF_TKE;
    P.mom_v = cfg->lmom_diff_v;
    P.mva = 0.0;  // set with the grid
  }
  c->staging_elems = 6 * (size_t)D.ny * D.nx * D.nl;
  if ((rc = dalloc(c, &c->staging, c->staging_elems)) != LGAME_OK) return fail(rc);
  if ((rc = dalloc(c, &c->reduce_buf, (size_t)kRedBlocks * LGAME_BUDGETS_MAX + LGAME_BUDGETS_MAX)) != LGAME_OK) return fail(rc);
  {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(int)) != cudaSuccess) return fail(set_err(LGAME_ERR_ALLOC, "cudaMalloc(flag) failed"));
    c->allocations.push_back(q);
    c->flag = (int*)q;
  }
  Grid<double>& G = c->G;
  G.z_scalar = c->grid[LGAME_GRID_Z_SCALAR]; G.z_u = c->grid[LGAME_GRID_Z_U]; G.z_v = c->grid[LGAME_GRID_Z_V];
  G.z_w = c->grid[LGAME_GRID_Z_W]; G.dx = c->grid[LGAME_GRID_DX]; G.dy = c->grid[LGAME_GRID_DY];
  G.dz = c->grid[LGAME_GRID_DZ]; G.volume = c->grid[LGAME_GRID_VOLUME]; G.area_x = c->grid[LGAME_GRID_AREA_X];
  G.area_y = c->grid[LGAME_GRID_AREA_Y]; G.area_z = c->grid[LGAME_GRID_AREA_Z];
  G.area_dual_x = c->grid[LGAME_GRID_AREA_DUAL_X]; G.area_dual_y = c->grid[LGAME_GRID_AREA_DUAL_Y];
  G.area_dual_z = c->grid[LGAME_GRID_AREA_DUAL_Z]; G.z_area_dual_z = c->grid[LGAME_GRID_Z_AREA_DUAL_Z];
  G.slope_x = c->grid[LGAME_GRID_SLOPE_X]; G.slope_y = c->grid[LGAME_GRID_SLOPE_Y];
  for (int k = 0; k < 6; ++k) G.ipw[k] = c->ipw[k];
  G.theta_v_bg = c->grid[LGAME_GRID_THETA_V_BG]; G.exner_bg = c->grid[LGAME_GRID_EXNER_BG];
  G.egu = c->grid[LGAME_GRID_EXNER_BG_GRAD_U]; G.egv = c->grid[LGAME_GRID_EXNER_BG_GRAD_V];
  G.egw = c->grid[LGAME_GRID_EXNER_BG_GRAD_W]; G.gm = c->grid[LGAME_GRID_GRAVITY_M_V];
  G.gp = c->grid[LGAME_GRID_GRAVITY_POTENTIAL]; G.fvec_x = c->grid[LGAME_GRID_FVEC_X];
  G.fvec_y = c->grid[LGAME_GRID_FVEC_Y]; G.fvec_z = c->grid[LGAME_GRID_FVEC_Z];
  for (int k = 0; k < 3; ++k) G.trsk_u[k] = c->trsk_u[k];
  for (int k = 0; k < 2; ++k) G.trsk_v[k] = c->trsk_v[k];
  G.damp = c->damp;
  G.dx_dual = c->grid[LGAME_GRID_DX_DUAL]; G.dy_dual = c->grid[LGAME_GRID_DY_DUAL];
  G.layer_thickness = c->grid[LGAME_GRID_LAYER_THICKNESS];
  if (cfg->precision != LGAME_PRECISION_FP64) {
    SplitDiff sd;
    sd.mom_h = c->diff_mom_h; sd.mom_v = c->diff_mom_v; sd.temp_h = c->diff_temp_h; sd.temp_v = c->diff_temp_v;
    sd.mass_h = c->diff_mass_h; sd.mass_v = c->diff_mass_v; sd.par = c->dpar;
    SplitSfc sf;
    sf.turb = c->sfc_turb; sf.pbl = c->sfc_pbl; sf.sens = c->sfc_sens; sf.soil = c->sfc_soil;
    sf.phase = c->phase; sf.phase_sfc = c->phase && cfg->lsfc_phase_trans;
    sf.buf = c->sbuf; sf.par = c->spar; sf.vsq = c->vsq; sf.tsoil[0] = c->tsoil[0]; sf.tsoil[1] = c->tsoil[1];
    if ((rc = split_create(c->D, cfg->precision == LGAME_PRECISION_SPLIT_FP64_COLUMN, sd, sf, &c->split, &c->bytes)) !=
        LGAME_OK)
      return fail(rc);
  }
  *out = c;
  return LGAME_OK;
}

extern "C" int lgame_gpu_set_grid(lgame_gpu* c, const double* const* f, int nfields) {
  if (!c || !f || nfields != LGAME_GRID_NFIELDS) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_set_grid: bad arguments");
  const bool sfc_on = c->cfg.lprog_soil_temp || c->cfg.lsfc_sensible_heat_flux || c->cfg.lsfc_phase_trans || c->cfg.lpbl;
  for (int i = 0; i < nfields; ++i)
    if (!f[i] && (i < LGAME_GRID_LAND_FRACTION || sfc_on))
      return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_set_grid: null field");
  const Dims& D = c->D;
  int rc;
  for (int i = 0; i < LGAME_GRID_LAND_FRACTION; ++i) {
    if (i == LGAME_GRID_INNER_PRODUCT_WEIGHTS || i == LGAME_GRID_TRSK_WEIGHTS_U || i == LGAME_GRID_TRSK_WEIGHTS_V) continue;
    if ((rc = copy_h2d(c, c->grid[i], f[i], grid_ext(D, i))) != LGAME_OK) return rc;
  }
  // surface planes, the soil grid (parameters of the surface kernels), and the carried
  // roughness length set to the grid's (control.F90:458)
  for (int k = 0; k < 6; ++k) {
    const int i = LGAME_GRID_LAND_FRACTION + k;
    if (f[i] && (rc = copy_h2d(c, c->sfc_grid[k], f[i], grid_ext(D, i))) != LGAME_OK) return rc;
  }
  if (f[LGAME_GRID_ROUGHNESS_LENGTH])
    CK(cudaMemcpyAsync(c->sbuf.rl, c->sfc_grid[2], sizeof(double) * (size_t)D.plane, cudaMemcpyDeviceToDevice, c->stream));
  if (f[LGAME_GRID_Z_SOIL_INTERFACE] && f[LGAME_GRID_Z_SOIL_CENTER] && f[LGAME_GRID_Z_T_CONST]) {
    SfcPar& P = c->spar;
    for (int k = 0; k <= P.ns; ++k) P.zi[k] = f[LGAME_GRID_Z_SOIL_INTERFACE][k];
    for (int k = 0; k < P.ns; ++k) P.zc[k] = f[LGAME_GRID_Z_SOIL_CENTER][k];
    P.z_t_const = f[LGAME_GRID_Z_T_CONST][0];
    for (int k = 0; k < P.ns; ++k) P.idzi[k] = 1.0 / (P.zi[k] - P.zi[k + 1]);
    for (int k = 0; k + 1 < P.ns; ++k) P.idzc[k] = 1.0 / (P.zc[k] - P.zc[k + 1]);
    P.i2dzt = P.ns > 0 ? 1.0 / (2.0 * (P.zc[P.ns - 1] - P.z_t_const)) : 0.0;
    if (c->split) split_set_sfc_par(c->split, P);
  }
  // inner product weights: (6,ny,nx,nl) -> six padded fields
  CK(cudaMemcpyAsync(c->staging, f[LGAME_GRID_INNER_PRODUCT_WEIGHTS], 6 * sizeof(double) * (size_t)D.ny * D.nx * D.nl,
                     cudaMemcpyHostToDevice, c->stream));
  k_split_ipw<<<grd(D, D.ny, D.nx, D.nl), blk(), 0, c->stream>>>(D, c->staging, c->ipw[0], c->ipw[1], c->ipw[2],
                                                                  c->ipw[3], c->ipw[4], c->ipw[5]);
  CK(cudaGetLastError());
  // TRSK weights (3,ny) and (2,ny+1)
  std::vector<double> tmp((size_t)D.P, 0.0);
  for (int k = 0; k < 3; ++k) {
    for (int i = 0; i < D.ny; ++i) tmp[i] = f[LGAME_GRID_TRSK_WEIGHTS_U][3 * i + k];
    CK(cudaMemcpyAsync(c->trsk_u[k], tmp.data(), sizeof(double) * D.P, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  for (int k = 0; k < 2; ++k) {
    for (int i = 0; i < D.ny + 1; ++i) tmp[i] = f[LGAME_GRID_TRSK_WEIGHTS_V][2 * i + k];
    CK(cudaMemcpyAsync(c->trsk_v[k], tmp.data(), sizeof(double) * D.P, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  // Klemp damping prefactor at the w levels, mo_column_solvers.F90:187-196, evaluated on
  // the host with the same expression as the reference (a grid-only quantity)
  {
    const double* zw = f[LGAME_GRID_Z_W];
    const size_t ny = D.ny, nx = D.nx;
    std::vector<double> dp(ny * nx * (D.nl + 1), 1.0);
    const double dsh = c->cfg.klemp_begin_rel * c->cfg.toa;
    for (int jl = 1; jl <= D.nl - 1; ++jl)
      for (size_t jk = 0; jk < nx; ++jk)
        for (size_t ji = 0; ji < ny; ++ji) {
          const size_t i = ji + ny * (jk + nx * (size_t)jl);  // level jl+1 (0-based jl)
          const double above = zw[i] - dsh;
          double coeff;
          if (above < 0.0 || !c->cfg.lklemp) {
            coeff = 0.0;
          } else {
            const double s = std::sin(0.5 * 3.14159265358979323846 * above / (c->cfg.toa - dsh));
            coeff = c->cfg.klemp_damp_max * (s * s);
          }
          dp[i] = 1.0 + coeff * c->cfg.dtime;
        }
    if ((rc = copy_h2d(c, c->damp, dp.data(), ext_w(D))) != LGAME_OK) return rc;
    CK(cudaStreamSynchronize(c->stream));
    // n_damping_levels, mo_grid_generator.F90:1049-1058: the levels whose highest z_w lies above
    // the damping layer's lower boundary (the swamp layer's dissipation is formed there)
    int ndamp = 0;
    for (int jl = 0; jl <= D.nl; ++jl) {
      double max_z = -1e300;
      for (size_t p = 0; p < ny * nx; ++p) max_z = std::max(max_z, zw[p + ny * nx * (size_t)jl]);
      if (max_z > dsh) ++ndamp;
    }
    c->D.ndamp = ndamp;
    CK(cudaMemsetAsync(c->hdiss, 0, sizeof(double) * (size_t)D.fstride, c->stream));
  }
  // mean_velocity_area, mo_grid_generator.F90:1111: twice the surface areas' sum (array order)
  // over their number
  {
    const size_t n2 = (size_t)D.ny * D.nx;
    const double* az = f[LGAME_GRID_AREA_Z] + n2 * (size_t)D.nl;
    double sum = 0.0;
    for (size_t p = 0; p < n2; ++p) sum = sum + az[p];
    c->dpar.mva = 2.0 * sum / (double)n2;
    if (c->split) split_set_diff_par(c->split, c->dpar);
  }
  if (c->split) {
    if ((rc = split_set_grid(c->split, c->D, c->G, c->stream)) != LGAME_OK) return rc;
    // a new background for the boundary relaxation of a context already set up for it
    if (c->bc_on && (rc = split_bc_prepare(c->split, c->D, c->G, c->stream)) != LGAME_OK) return set_err(rc, "split_bc_prepare");
  }
  CK(cudaStreamSynchronize(c->stream));
  c->grid_set = true;
  return LGAME_OK;
}

namespace {
// the first nfields state fields (LGAME_STATE_NFIELDS_ATMOS or LGAME_STATE_NFIELDS) of a slot
int state_copy(lgame_gpu* c, int slot, double* const* hf, const double* const* cf, bool h2d,
               int nfields = LGAME_STATE_NFIELDS_ATMOS) {
  const Dims& D = c->D;
  const State& S = c->st[slot];
  double* dev[LGAME_STATE_NFIELDS] = {S.rho, S.rt, S.tp, S.ep, S.u, S.v, S.w, c->tsoil[slot]};
  const Ext ex[LGAME_STATE_NFIELDS] = {ext_s(D), ext_s(D), ext_s(D), ext_s(D), ext_u(D), ext_v(D), ext_w(D),
                                       {(size_t)D.ny, (size_t)D.nx, (size_t)c->spar.ns}};
  int rc;
  for (int f = 0; f < nfields; ++f) {
    if (f == LGAME_STATE_TEMPERATURE_SOIL && c->spar.ns == 0) continue;
    const int nrep = (f == LGAME_STATE_RHO) ? D.ncons : 1;
    const size_t hs = ex[f].n1 * ex[f].n2 * ex[f].n3;
    for (int r = 0; r < nrep; ++r) {
      double* d = dev[f] + (size_t)r * D.fstride;
      if (h2d) {
        if (!cf[f]) continue;
        rc = copy_h2d(c, d, cf[f] + r * hs, ex[f]);
      } else {
        if (!hf[f]) continue;
        rc = copy_d2h(c, hf[f] + r * hs, d, ex[f]);
      }
      if (rc != LGAME_OK) return rc;
    }
  }
  return LGAME_OK;
}
}  // namespace

extern "C" int lgame_gpu_set_state(lgame_gpu* c, int slot, const double* const* f, int nfields) {
  if (!c || !f || slot < 0 || slot > 1 || (nfields != LGAME_STATE_NFIELDS && nfields != LGAME_STATE_NFIELDS_ATMOS))
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_set_state: bad arguments");
  int rc = state_copy(c, slot, nullptr, f, true, nfields);
  if (rc != LGAME_OK) return rc;
  c->mirror_valid[slot] = false;
  CK(cudaStreamSynchronize(c->stream));
  return LGAME_OK;
}

extern "C" int lgame_gpu_get_state(lgame_gpu* c, int slot, double* const* f, int nfields) {
  if (!c || !f || slot < 0 || slot > 1 || (nfields != LGAME_STATE_NFIELDS && nfields != LGAME_STATE_NFIELDS_ATMOS))
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_get_state: bad arguments");
  int rc = state_copy(c, slot, f, nullptr, false, nfields);
  if (rc != LGAME_OK) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return LGAME_OK;
}

namespace {
// fields of one diagnostic: the constituents of the rho tendency, nc+1 phase transition rates
int diag_nrep(const Dims& D, int f) {
  if (f == LGAME_DIAG_TEND_RHO || f == LGAME_DIAG_MASS_DIFF_TENDENCY) return D.ncons;
  if (f == LGAME_DIAG_PHASE_TRANS_RATES) return D.nc + 1;
  return 1;
}
double* diag_dev(lgame_gpu* c, int f) {
  switch (f) {
    case LGAME_DIAG_P_GRAD_ACC_NEG_NL_U: return c->pg_nl_u;
    case LGAME_DIAG_P_GRAD_ACC_NEG_NL_V: return c->pg_nl_v;
    case LGAME_DIAG_P_GRAD_ACC_NEG_NL_W: return c->pg_nl_w;
    case LGAME_DIAG_P_GRAD_ACC_NEG_L_U: return c->pg_l_u;
    case LGAME_DIAG_P_GRAD_ACC_NEG_L_V: return c->pg_l_v;
    case LGAME_DIAG_P_GRAD_ACC_NEG_L_W: return c->pg_l_w;
    case LGAME_DIAG_P_GRAD_ACC_OLD_U: return c->pg_old_u;
    case LGAME_DIAG_P_GRAD_ACC_OLD_V: return c->pg_old_v;
    case LGAME_DIAG_POT_VORT_TEND_X: return c->pvt_x;
    case LGAME_DIAG_POT_VORT_TEND_Y: return c->pvt_y;
    case LGAME_DIAG_POT_VORT_TEND_Z: return c->pvt_z;
    case LGAME_DIAG_V_SQUARED_GRAD_X: return c->vsg_x;
    case LGAME_DIAG_V_SQUARED_GRAD_Y: return c->vsg_y;
    case LGAME_DIAG_V_SQUARED_GRAD_Z: return c->vsg_z;
    case LGAME_DIAG_CONDENSATES_SEDIMENT_HEAT: return c->csh;
    case LGAME_DIAG_RADIATION_TENDENCY: return c->rad;
    case LGAME_DIAG_TEMPERATURE: return c->temperature;
    case LGAME_DIAG_TEND_RHO: return c->tend.rho;
    case LGAME_DIAG_TEND_RHOTHETA_V: return c->tend.rt;
    case LGAME_DIAG_TEND_WIND_U: return c->tend.u;
    case LGAME_DIAG_TEND_WIND_V: return c->tend.v;
    case LGAME_DIAG_TEND_WIND_W: return c->tend.w;
    case LGAME_DIAG_TKE: return c->dbuf.tke;
    case LGAME_DIAG_VISCOSITY: return c->dbuf.visc;
    case LGAME_DIAG_HEATING_DISS: return c->hdiss;
    case LGAME_DIAG_MOM_DIFF_TEND_X: return c->dbuf.mdtx;
    case LGAME_DIAG_MOM_DIFF_TEND_Y: return c->dbuf.mdty;
    case LGAME_DIAG_MOM_DIFF_TEND_Z: return c->dbuf.mdtz;
    case LGAME_DIAG_V_SQUARED: return c->vsq;
    case LGAME_DIAG_ROUGHNESS_LENGTH: return c->sbuf.rl;
    case LGAME_DIAG_ROUGHNESS_VELOCITY: return c->sbuf.rv;
    case LGAME_DIAG_MONIN_OBUKHOV_LENGTH: return c->sbuf.mol;
    case LGAME_DIAG_SCALAR_FLUX_RESISTANCE: return c->sbuf.sfr;
    case LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SOIL: return c->sbuf.sens_soil;
    case LGAME_DIAG_POWER_FLUX_DENSITY_SENS_SEA: return c->sbuf.sens_sea;
    case LGAME_DIAG_SST: return c->sbuf.sst;
    case LGAME_DIAG_SFC_SW_IN: return c->sbuf.sw_in;
    case LGAME_DIAG_SFC_LW_OUT: return c->sbuf.lw_out;
    case LGAME_DIAG_PHASE_TRANS_RATES: return c->ptr;
    case LGAME_DIAG_PHASE_TRANS_HEATING_RATE: return c->pth;
    case LGAME_DIAG_POWER_FLUX_DENSITY_LAT_LAKE: return c->sbuf.lat_lake;
    case LGAME_DIAG_POWER_FLUX_DENSITY_LAT_SEA: return c->sbuf.lat_sea;
    case LGAME_DIAG_TEMP_DIFF_HEATING: return c->dbuf.tdh;
    case LGAME_DIAG_MASS_DIFF_TENDENCY: return c->dbuf.mdt;
  }
  return nullptr;
}
}  // namespace

extern "C" int lgame_gpu_set_diag(lgame_gpu* c, const double* const* f, int nfields) {
  if (!c || !f || nfields != LGAME_DIAG_NFIELDS) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_set_diag: bad arguments");
  const Dims& D = c->D;
  for (int i = 0; i < nfields; ++i) {
    if (!f[i] || !diag_dev(c, i)) continue;  // not given, or not formed in this run (phase transitions off)
    const Ext e = diag_ext(D, i);
    const int nrep = diag_nrep(D, i);
    for (int r = 0; r < nrep; ++r) {
      int rc = copy_h2d(c, diag_dev(c, i) + (size_t)r * D.fstride, f[i] + r * e.n1 * e.n2 * e.n3, e);
      if (rc != LGAME_OK) return rc;
    }
  }
  if (c->split) {
    int rc = split_sync_carried(c, true);
    if (rc != LGAME_OK) return rc;
  }
  CK(cudaStreamSynchronize(c->stream));
  return LGAME_OK;
}

extern "C" int lgame_gpu_get_diag(lgame_gpu* c, double* const* f, int nfields) {
  if (!c || !f || nfields != LGAME_DIAG_NFIELDS) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_get_diag: bad arguments");
  const Dims& D = c->D;
  if (c->split) {
    int rc = split_sync_carried(c, false);
    if (rc != LGAME_OK) return rc;
  }
  for (int i = 0; i < nfields; ++i) {
    if (!f[i]) continue;
    const Ext e = diag_ext(D, i);
    const int nrep = diag_nrep(D, i);
    if (!diag_dev(c, i)) {  // not formed in this run: the reference's zero
      std::memset(f[i], 0, sizeof(double) * e.n1 * e.n2 * e.n3 * (size_t)nrep);
      continue;
    }
    for (int r = 0; r < nrep; ++r) {
      int rc = copy_d2h(c, f[i] + r * e.n1 * e.n2 * e.n3, diag_dev(c, i) + (size_t)r * D.fstride, e);
      if (rc != LGAME_OK) return rc;
    }
  }
  CK(cudaStreamSynchronize(c->stream));
  return LGAME_OK;
}

extern "C" int lgame_gpu_pchevi(lgame_gpu* c, int old_slot, int new_slot, int total_step_counter, int lrad_update,
                                double t_0) {
  if (!c || old_slot < 0 || old_slot > 1 || new_slot < 0 || new_slot > 1 || old_slot == new_slot || total_step_counter < 0)
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_pchevi: bad arguments");
  if (!c->grid_set) return set_err(LGAME_ERR_STATE, "lgame_gpu_pchevi: lgame_gpu_set_grid has not been called");
  c->kernels_last_step = 0;
  int rc;
  // update_rad_fluxes(state_old, grid, diag, t_0) before the substeps (mo_manage_pchevi.F90:56-58)
  // when an emulator is attached; otherwise the radiation tendency is whatever the host set
  if (lrad_update && c->rad_emu) {
    if ((rc = lgame_gpu_rad_update(c, c->rad_emu, old_slot, t_0 + 0.5 * c->rad_dtime, c->rad_stride, c->rad_bound,
                                   c->rad_report)) != LGAME_OK)
      return rc;
    ++c->rad_updates;
  }
  if (c->split) {
    for (int slot : {old_slot, new_slot}) {
      if (c->mirror_valid[slot]) continue;
      if ((rc = split_refresh_mirror(c->split, c->D, slot, c->st[slot], c->stream)) != LGAME_OK)
        return set_err(rc, "lgame_gpu_pchevi: refresh of the FP32 state mirror failed");
      c->mirror_valid[slot] = true;
    }
  }
  // The split step's concurrent branches pay where its kernels are launched one by one (the
  // host-buffer step, whose copy-out then starts earlier: 132.5 against 137-139 ms end to end
  // at 1024x1024x80); a captured graph runs faster in the serial order (58.57 against 58.75 ms)
  auto launch_step = [&](bool serial) -> int {
    if (c->split) {
      PGrad<double> P{c->pg_nl_u, c->pg_nl_v, c->pg_nl_w, c->pg_l_u, c->pg_l_v, c->pg_l_w, c->pg_old_u, c->pg_old_v,
                      c->pgcw};
      return split_step(c->split, c->D, c->G, c->st[old_slot], c->st[new_slot], old_slot, new_slot, P,
                        total_step_counter, c->stream, &c->kernels_last_step,
                        c->profiling ? trace_begin_cb : (c->mark_on ? mark_begin_cb : nullptr),
                        c->profiling ? trace_end_cb : mark_end_cb, c, serial || c->profiling);
    }
    return step_fp64(c, old_slot, new_slot, total_step_counter);
  };
  // After step 0 a step is the same sequence of launches for a given slot pair, so it runs as
  // a CUDA graph (one launch from the host instead of ~30).  Not with per-kernel tracing,
  // whose events are recorded between the launches.
  if (c->use_graphs && !c->profiling && !c->mark_on && total_step_counter > 0) {
    cudaGraphExec_t& exec = c->graph[old_slot];
    if (!exec) {
      CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      rc = launch_step(true);
      cudaGraph_t graph = nullptr;
      const cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
      if (rc != LGAME_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
      }
      if (e != cudaSuccess) return set_err(LGAME_ERR_CUDA, std::string("capture of the step: ") + cudaGetErrorString(e));
      const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ei != cudaSuccess) {
        exec = nullptr;
        return set_err(LGAME_ERR_CUDA, std::string("instantiation of the step graph: ") + cudaGetErrorString(ei));
      }
      c->graph_kernels[old_slot] = c->kernels_last_step;
    }
    CK(cudaGraphLaunch(exec, c->stream));
    c->kernels_last_step = c->graph_kernels[old_slot];
    rc = LGAME_OK;
  } else {
    rc = launch_step(false);
  }
  if (rc != LGAME_OK) return rc;
  // mo_manage_pchevi.F90:114-116
  if (!c->cfg.lperiodic && c->bc_on) {
    if ((rc = lgame_gpu_update_boundaries(c, new_slot, (total_step_counter + 1) * c->D.dtime)) != LGAME_OK) return rc;
    c->kernels_last_step += (c->split && c->bc_nrim > 0) ? 2 : 1;
  }
  if (c->cfg.check_finite) {
    const Dims& D = c->D;
    CK(cudaMemsetAsync(c->flag, 0, sizeof(int), c->stream));
    k_check_finite<<<grd(D, D.ny + 1, D.nx + 1, D.NL), blk(), 0, c->stream>>>(D, c->st[new_slot], c->flag);
    CK(cudaGetLastError());
    int h = 0;
    CK(cudaMemcpyAsync(&h, c->flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (h) return set_err(LGAME_ERR_NONFINITE, "non-finite value in the new state");
  }
  return LGAME_OK;
}

extern "C" int lgame_gpu_pchevi_host(lgame_gpu* c, const double* const* state_old, double* const* state_new,
                                     int nfields, int total_step_counter, int lrad_update, double t_0) {
  if (!c || !state_old || !state_new || (nfields != LGAME_STATE_NFIELDS && nfields != LGAME_STATE_NFIELDS_ATMOS))
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_pchevi_host: bad arguments");
  const bool soil = nfields == LGAME_STATE_NFIELDS && c->spar.ns > 0;
  if (!soil && (c->sfc_soil || c->sfc_sens))
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_pchevi_host: the soil temperature is part of this run's state "
                                          "(pass LGAME_STATE_NFIELDS arrays)");
  if (soil && (!state_old[LGAME_STATE_TEMPERATURE_SOIL] || !state_new[LGAME_STATE_TEMPERATURE_SOIL]))
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_pchevi_host: null soil temperature");
  const Dims& D = c->D;
  const Ext ex[LGAME_STATE_NFIELDS_ATMOS] = {ext_s(D), ext_s(D), ext_s(D), ext_s(D), ext_u(D), ext_v(D), ext_w(D)};
  const Ext ex_soil{(size_t)D.ny, (size_t)D.nx, (size_t)c->spar.ns};
  const State& A = c->st[0];
  const State& B = c->st[1];
  double* da[LGAME_STATE_NFIELDS_ATMOS] = {A.rho, A.rt, A.tp, A.ep, A.u, A.v, A.w};
  double* db[LGAME_STATE_NFIELDS_ATMOS] = {B.rho, B.rt, B.tp, B.ep, B.u, B.v, B.w};
  const double* vin[LGAME_STATE_NFIELDS_ATMOS];
  double* vout[LGAME_STATE_NFIELDS_ATMOS];
  // the soil temperature (a few planes) takes the copy engines: into slots 0 and 1 (the new
  // state starts as a copy of the old one), out of slot 1 after the step
  if (soil) {
    int rc = copy_h2d(c, c->tsoil[0], state_old[LGAME_STATE_TEMPERATURE_SOIL], ex_soil);
    if (rc != LGAME_OK) return rc;
    CK(cudaMemcpyAsync(c->tsoil[1], c->tsoil[0], sizeof(double) * (size_t)D.plane * c->spar.ns,
                       cudaMemcpyDeviceToDevice, c->stream));
  }
  // the GPU moves the state itself when every array is one it can address; a null array (not
  // copied) or an unregistered one takes the copy engines, as before
  bool direct_in = true, direct_out = true;
  for (int f = 0; f < LGAME_STATE_NFIELDS_ATMOS; ++f) {
    direct_in = direct_in && (vin[f] = device_view(state_old[f])) != nullptr;
    direct_out = direct_out && (vout[f] = const_cast<double*>(device_view(state_new[f]))) != nullptr;
  }
  auto grid_of = [&](int f) {
    const int nrep = (f == LGAME_STATE_RHO) ? D.ncons : 1;
    return dim3((unsigned)((ex[f].n1 + 255) / 256), (unsigned)ex[f].n2, (unsigned)(ex[f].n3 * nrep));
  };
  if (direct_in) {
    // state_old into slot 0 and, as the reference's time loop starts state_new as a copy of
    // state_old, into slot 1, with the FP32 mirrors of both in split mode
    StateF m0{}, m1{};
    if (c->split) { m0 = split_mirror(c->split, 0); m1 = split_mirror(c->split, 1); }
    float* ma[LGAME_STATE_NFIELDS_ATMOS] = {m0.rho, m0.rt, m0.tp, m0.ep, m0.u, m0.v, m0.w};
    float* mb[LGAME_STATE_NFIELDS_ATMOS] = {m1.rho, m1.rt, m1.tp, m1.ep, m1.u, m1.v, m1.w};
    for (int f = 0; f < LGAME_STATE_NFIELDS_ATMOS; ++f) {
      k_state_in<<<grid_of(f), 256, 0, c->stream>>>(D, vin[f], (int)ex[f].n1, (int)ex[f].n2, (int)ex[f].n3, da[f],
                                                     db[f], ma[f], mb[f]);
      CK(cudaGetLastError());
    }
    c->mirror_valid[0] = c->mirror_valid[1] = c->split != nullptr;
  } else {
    int rc = state_copy(c, 0, nullptr, state_old, true);
    if (rc != LGAME_OK) return rc;
    c->mirror_valid[0] = c->mirror_valid[1] = false;
    // state_new starts as a copy of state_old, as in the reference's time loop
    const size_t F = (size_t)D.fstride * sizeof(double);
    CK(cudaMemcpyAsync(B.rho, A.rho, F * D.ncons, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(B.rt, A.rt, F, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(B.tp, A.tp, F, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(B.ep, A.ep, F, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(B.u, A.u, F, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(B.v, A.v, F, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(B.w, A.w, F, cudaMemcpyDeviceToDevice, c->stream));
  }
  // Split step without a boundary relaxation at its end: the copy engines move the fields that
  // are final before the step ends on a second stream while the step runs (u, v after the
  // second wind update; rhotheta_v, theta_v_pert, exner_pert, w and the gas density after the
  // second vertical solve); the step is then launched kernel by kernel, not as a graph, so that
  // it can record the two events.  The tracer densities follow the step.
  const bool overlap = direct_out && c->split && !c->profiling && !(c->bc_on && !c->cfg.lperiodic);
  if (overlap && !c->side) {
    CK(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    for (cudaEvent_t& e : c->ev_mark) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  c->mark_on = overlap;
  c->marks[0] = c->marks[1] = 0;
  int rc = lgame_gpu_pchevi(c, 0, 1, total_step_counter, lrad_update, t_0);
  c->mark_on = false;
  if (rc != LGAME_OK) return rc;
  const bool early = overlap && c->marks[0] == 2 && c->marks[1] == 2;
  if (direct_out && early) {
    const long long nS = (long long)D.ny * D.nx * D.nl;
    const int gi = D.g - 1;
    CK(cudaStreamWaitEvent(c->side, c->ev_mark[0], 0));
    for (int f : {LGAME_STATE_WIND_U, LGAME_STATE_WIND_V})
      if ((rc = copy_d2h(c, state_new[f], db[f], ex[f], c->side)) != LGAME_OK) return rc;
    CK(cudaStreamWaitEvent(c->side, c->ev_mark[1], 0));
    for (int f : {LGAME_STATE_RHOTHETA_V, LGAME_STATE_THETA_V_PERT, LGAME_STATE_EXNER_PERT, LGAME_STATE_WIND_W})
      if ((rc = copy_d2h(c, state_new[f], db[f], ex[f], c->side)) != LGAME_OK) return rc;
    if ((rc = copy_d2h(c, state_new[LGAME_STATE_RHO] + gi * nS, B.rho + (size_t)gi * D.fstride, ex[0], c->side)) != LGAME_OK)
      return rc;
    const dim3 g1((unsigned)((ex[0].n1 + 255) / 256), (unsigned)ex[0].n2, (unsigned)ex[0].n3);
    for (int jc = 0; jc < D.ncons; ++jc) {
      if (jc == gi) continue;
      k_state_out<<<g1, 256, 0, c->stream>>>(D, B.rho + (size_t)jc * D.fstride, (int)ex[0].n1, (int)ex[0].n2,
                                             (int)ex[0].n3, vout[LGAME_STATE_RHO] + jc * nS);
      CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(c->side));
  } else if (direct_out) {
    for (int f = 0; f < LGAME_STATE_NFIELDS_ATMOS; ++f) {
      k_state_out<<<grid_of(f), 256, 0, c->stream>>>(D, db[f], (int)ex[f].n1, (int)ex[f].n2, (int)ex[f].n3, vout[f]);
      CK(cudaGetLastError());
    }
  } else {
    rc = state_copy(c, 1, state_new, nullptr, false);
    if (rc != LGAME_OK) return rc;
  }
  if (soil && (rc = copy_d2h(c, state_new[LGAME_STATE_TEMPERATURE_SOIL], c->tsoil[1], ex_soil)) != LGAME_OK) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return LGAME_OK;
}

extern "C" int lgame_gpu_budgets(lgame_gpu* c, int slot, double* out, int nout) {
  if (!c || !out || slot < 0 || slot > 1) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_budgets: bad arguments");
  const Dims& D = c->D;
  const int nq = D.ncons + 4;
  if (nout < nq) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_budgets: output too small");
  k_budget_partial<<<kRedBlocks, kRedThreads, 0, c->stream>>>(D, c->G, c->st[slot], c->temperature, c->reduce_buf, nq);
  CK(cudaGetLastError());
  double* dout = c->reduce_buf + (size_t)kRedBlocks * LGAME_BUDGETS_MAX;
  k_budget_final<<<1, 32, 0, c->stream>>>(c->reduce_buf, dout, nq);
  CK(cudaGetLastError());
  std::vector<double> h(nq);
  CK(cudaMemcpyAsync(h.data(), dout, sizeof(double) * nq, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < nq; ++k) out[k] = h[k];
  out[D.ncons + 1] = 0.5 * out[D.ncons + 1];
  return LGAME_OK;
}

extern "C" int lgame_gpu_synchronize(lgame_gpu* c) {
  if (!c) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_synchronize: null context");
  CK(cudaStreamSynchronize(c->stream));
  return LGAME_OK;
}

extern "C" int lgame_gpu_kernels_per_step(const lgame_gpu* c) { return c ? c->kernels_last_step : 0; }

namespace lg {
int trace_begin(lgame_gpu* c, const char* name) {
  const int idx = (int)c->ev_used.size() * 2;
  while ((int)c->ev_pool.size() < idx + 2) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return -1;
    c->ev_pool.push_back(e);
  }
  cudaEventRecord(c->ev_pool[idx], c->stream);
  if (std::strncmp(name, "kd::", 4) == 0) name += 4;
  c->ev_used.push_back({name, idx});
  return idx;
}
void trace_end(lgame_gpu* c, int slot) { cudaEventRecord(c->ev_pool[slot + 1], c->stream); }
}  // namespace lg

extern "C" void* lgame_gpu_stream(const lgame_gpu* c) { return c ? (void*)c->stream : nullptr; }

extern "C" int lgame_gpu_output(lgame_gpu* c, int slot_1, int slot_2, double coeff_1, double coeff_2,
                                float* const* fields, int nfields, int* crashed) {
  if (!c || !fields || nfields != LGAME_OUTPUT_NFIELDS || slot_1 < 0 || slot_1 > 1 || slot_2 < 0 || slot_2 > 1)
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_output: bad arguments");
  if (!c->grid_set) return set_err(LGAME_ERR_STATE, "lgame_gpu_output: lgame_gpu_set_grid has not been called");
  const Dims& D = c->D;
  const size_t nS = (size_t)D.ny * D.nx * D.nl;
  if (!c->out_buf) {
    const size_t n = (size_t)(D.ncons + 5) * nS;
    CK(cudaMalloc(&c->out_buf, n * sizeof(float)));
    c->allocations.push_back(c->out_buf);
    c->bytes += (long long)(n * sizeof(float));
  }
  CK(cudaMemsetAsync(c->flag, 0, sizeof(int), c->stream));
  k_output<<<grd(D, D.ny, D.nx, D.nl), blk(), 0, c->stream>>>(D, c->G, c->st[slot_1], c->st[slot_2], coeff_1, coeff_2,
                                                              c->out_buf, c->flag);
  int rc = klaunch_check(c, "k_output");
  if (rc) return rc;
  if (fields[LGAME_OUTPUT_RHO])
    CK(cudaMemcpyAsync(fields[LGAME_OUTPUT_RHO], c->out_buf, sizeof(float) * nS * D.ncons, cudaMemcpyDeviceToHost,
                       c->stream));
  for (int k = LGAME_OUTPUT_TEMPERATURE; k < LGAME_OUTPUT_NFIELDS; ++k) {
    if (!fields[k] || (k == LGAME_OUTPUT_REL_HUMIDITY && D.ncons == 1)) continue;
    CK(cudaMemcpyAsync(fields[k], c->out_buf + (size_t)(D.ncons + k - 1) * nS, sizeof(float) * nS,
                       cudaMemcpyDeviceToHost, c->stream));
  }
  int h = 0;
  CK(cudaMemcpyAsync(&h, c->flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (crashed) *crashed = h;
  return LGAME_OK;
}

// ---- lateral boundary relaxation, src/io/mo_boundaries.F90 -----------------------------

namespace {
// setup_bc_factor, mo_boundaries.F90:125-170, into a padded plane (row pitch P): for the
// points ji = 1..n1, jk = 1..n2, sin^2(pi/2*max(1 - d/n_swamp, 0)) with d the index
// distance to the nearest edge of that staggering (converted to double before the division)
void bc_factors(int n_swamp, int n1, int n2, int P, std::vector<double>& out) {
  const double pi = 3.14159265358979323846;
  for (int jk = 1; jk <= n2; ++jk)
    for (int ji = 1; ji <= n1; ++ji) {
      const int d = std::min(std::min(ji - 1, jk - 1), std::min(n1 - ji, n2 - jk));
      double f = 1.0 - (double)d / n_swamp;
      if (f < 0.0) f = 0.0;
      const double sn = std::sin(0.5 * pi * f);
      out[(size_t)(ji - 1) + (size_t)P * (jk - 1)] = sn * sn;
    }
}
}  // namespace

extern "C" int lgame_gpu_bc_setup(lgame_gpu* c, int n_swamp, int dtime_bc, double t_latest_bc, lgame_bc_loader loader,
                                  void* user) {
  if (!c || n_swamp < 1 || dtime_bc < 1)
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_bc_setup: bad arguments (n_swamp >= 1, dtime_bc >= 1)");
  if (c->cfg.lperiodic) return set_err(LGAME_ERR_STATE, "lgame_gpu_bc_setup: the run is periodic (lperiodic = 1)");
  const Dims& D = c->D;
  if (!c->bcf_s) {
    for (State& L : c->bc_lev) {
      int rc = dalloc(c, &L.rho, (size_t)D.fstride * D.ncons);
      if (!rc) rc = dalloc(c, &L.rt, D.fstride);
      if (!rc) rc = dalloc(c, &L.u, D.fstride);
      if (!rc) rc = dalloc(c, &L.v, D.fstride);
      if (!rc) rc = dalloc(c, &L.w, D.fstride);
      if (rc) return rc;
    }
    int rc = dalloc(c, &c->bcf_s, D.plane);
    if (!rc) rc = dalloc(c, &c->bcf_u, D.plane);
    if (!rc) rc = dalloc(c, &c->bcf_v, D.plane);
    if (rc) return rc;
  }
  std::vector<double> h((size_t)D.plane);
  std::vector<char> any((size_t)D.plane, 0);
  double* dst[3] = {c->bcf_s, c->bcf_u, c->bcf_v};
  const int n1[3] = {D.ny, D.ny, D.ny + 1}, n2[3] = {D.nx, D.nx + 1, D.nx};
  for (int k = 0; k < 3; ++k) {
    std::fill(h.begin(), h.end(), 0.0);
    bc_factors(n_swamp, n1[k], n2[k], D.P, h);
    for (size_t i = 0; i < h.size(); ++i) any[i] |= (h[i] != 0.0);
    CK(cudaMemcpy(dst[k], h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
  }
  std::vector<int> rim;
  for (size_t i = 0; i < any.size(); ++i)
    if (any[i]) rim.push_back((int)i);
  if (c->bc_rim) cudaFree(c->bc_rim);
  c->bc_rim = nullptr;
  c->bc_nrim = (int)rim.size();
  if (!rim.empty()) {
    CK(cudaMalloc(&c->bc_rim, sizeof(int) * rim.size()));
    CK(cudaMemcpy(c->bc_rim, rim.data(), sizeof(int) * rim.size(), cudaMemcpyHostToDevice));
  }
  if (c->split) {
    if (!c->grid_set) return set_err(LGAME_ERR_STATE, "lgame_gpu_bc_setup: lgame_gpu_set_grid has not been called");
    const int rc = split_bc_prepare(c->split, D, c->G, c->stream);
    if (rc != LGAME_OK) return set_err(rc, "lgame_gpu_bc_setup: background rhotheta_v for the split path failed");
    CK(cudaStreamSynchronize(c->stream));
  }
  c->bc_index_old = 1;  // control.F90:358-359
  c->bc_index_new = 2;
  c->dtime_bc = dtime_bc;
  c->t_latest_bc = t_latest_bc;
  c->bc_loader = loader;
  c->bc_user = user;
  c->bc_on = true;
  return LGAME_OK;
}

extern "C" int lgame_gpu_set_bc(lgame_gpu* c, int time_index, const double* rho, const double* rhotheta_v,
                                const double* wind_u, const double* wind_v, const double* wind_w) {
  if (!c || time_index < 1 || time_index > 2 || !rho || !rhotheta_v || !wind_u || !wind_v || !wind_w)
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_set_bc: bad arguments");
  if (!c->bc_on) return set_err(LGAME_ERR_STATE, "lgame_gpu_set_bc: lgame_gpu_bc_setup has not been called");
  const Dims& D = c->D;
  const State& L = c->bc_lev[time_index - 1];
  const Ext es = ext_s(D);
  int rc = LGAME_OK;
  for (int r = 0; r < D.ncons && !rc; ++r) rc = copy_h2d(c, L.rho + (size_t)r * D.fstride, rho + r * es.n1 * es.n2 * es.n3, es);
  if (!rc) rc = copy_h2d(c, L.rt, rhotheta_v, es);
  if (!rc) rc = copy_h2d(c, L.u, wind_u, ext_u(D));
  if (!rc) rc = copy_h2d(c, L.v, wind_v, ext_v(D));
  if (!rc) rc = copy_h2d(c, L.w, wind_w, ext_w(D));
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));  // the host arrays may be reused on return
  return LGAME_OK;
}

extern "C" int lgame_gpu_update_boundaries(lgame_gpu* c, int slot, double t_now) {
  if (!c || slot < 0 || slot > 1) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_update_boundaries: bad arguments");
  if (!c->bc_on) return set_err(LGAME_ERR_STATE, "lgame_gpu_update_boundaries: lgame_gpu_bc_setup has not been called");
  const double old_weight = 1.0 - (t_now - c->t_latest_bc) / c->dtime_bc;
  if (old_weight < 0.0) {
    // read_boundaries(bc, t_latest_bc+dtime_bc, bc%index_old), then the index swap (:37-47)
    if (!c->bc_loader)
      return set_err(LGAME_ERR_STATE, "lgame_gpu_update_boundaries: a new boundary level is due and there is no loader");
    if (c->bc_loader(c->bc_user, c->t_latest_bc + c->dtime_bc, c->bc_index_old) != 0)
      return set_err(LGAME_ERR_STATE, "lgame_gpu_update_boundaries: the boundary loader failed");
    c->bc_index_old = c->bc_index_new;
    c->bc_index_new = (c->bc_index_old == 1) ? 2 : 1;
    c->t_latest_bc = c->t_latest_bc + c->dtime_bc;
  }
  const double new_weight = 1.0 - old_weight;
  const Dims& D = c->D;
  StateF M{};
  if (c->split && c->mirror_valid[slot]) M = split_mirror(c->split, slot);
  if (c->split) {
    const int rc = split_bc_update(c->split, D, c->G, c->st[slot], M, c->bc_lev[c->bc_index_old - 1],
                                   c->bc_lev[c->bc_index_new - 1], c->bc_rim, c->bc_nrim, c->bcf_s, c->bcf_u, c->bcf_v,
                                   old_weight, new_weight, c->stream);
    return rc == LGAME_OK ? LGAME_OK : set_err(rc, "lgame_gpu_update_boundaries: launch of the split kernels failed");
  }
  k_bc_update<<<grd(D, D.ny + 1, D.nx + 1, D.NL), blk(), 0, c->stream>>>(
      D, c->st[slot], M, c->bc_lev[c->bc_index_old - 1], c->bc_lev[c->bc_index_new - 1], c->bcf_s, c->bcf_u, c->bcf_v,
      old_weight, new_weight, c->G.theta_v_bg, c->G.exner_bg);
  return klaunch_check(c, "k_bc_update");
}

extern "C" int lgame_gpu_bc_state(lgame_gpu* c, int* index_old, int* index_new, double* t_latest_bc) {
  if (!c) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_bc_state: null context");
  if (!c->bc_on) return set_err(LGAME_ERR_STATE, "lgame_gpu_bc_state: lgame_gpu_bc_setup has not been called");
  if (index_old) *index_old = c->bc_index_old;
  if (index_new) *index_new = c->bc_index_new;
  if (t_latest_bc) *t_latest_bc = c->t_latest_bc;
  return LGAME_OK;
}

extern "C" int lgame_gpu_set_graphs(lgame_gpu* c, int enable) {
  if (!c) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_set_graphs: null context");
  c->use_graphs = enable != 0;
  return LGAME_OK;
}

extern "C" int lgame_gpu_set_profiling(lgame_gpu* c, int enable) {
  if (!c) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_set_profiling: null context");
  c->profiling = enable != 0;
  return LGAME_OK;
}

extern "C" int lgame_gpu_profile_report(lgame_gpu* c, char* buf, int len) {
  if (!c) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_profile_report: null context");
  CK(cudaStreamSynchronize(c->stream));
  for (auto& u : c->ev_used) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev_pool[u.second], c->ev_pool[u.second + 1]);
    bool found = false;
    for (auto& a : c->prof_acc)
      if (a.first == u.first) { a.second.first += 1; a.second.second += ms; found = true; break; }
    if (!found) c->prof_acc.push_back({u.first, {1, (double)ms}});
  }
  c->ev_used.clear();
  std::string js = "{";
  for (size_t i = 0; i < c->prof_acc.size(); ++i) {
    char tmp[256];
    std::snprintf(tmp, sizeof tmp, "%s\"%s\": {\"launches\": %d, \"ms\": %.6f}", i ? ", " : "",
                  c->prof_acc[i].first.c_str(), c->prof_acc[i].second.first, c->prof_acc[i].second.second);
    js += tmp;
  }
  js += "}";
  if (buf && len > (int)js.size()) {  // counts are reset only once they have been handed out
    std::memcpy(buf, js.c_str(), js.size() + 1);
    c->prof_acc.clear();
  }
  return (int)js.size();
}

extern "C" long long lgame_gpu_device_bytes(const lgame_gpu* c) { return c ? c->bytes : 0; }

extern "C" void lgame_gpu_destroy(lgame_gpu* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->side) cudaStreamSynchronize(c->side);  // copies of an lgame_gpu_pchevi_host that failed
  for (cudaGraphExec_t g : c->graph) if (g) cudaGraphExecDestroy(g);
  if (c->split) split_destroy(c->split);
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  for (void* p : c->allocations) cudaFree(p);
  if (c->bc_rim) cudaFree(c->bc_rim);
  for (cudaEvent_t e : c->ev_mark) if (e) cudaEventDestroy(e);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

// ---- lgame_gpu_budgets_static: the budget sums without any allocation -------------------
// The same two reduction kernels as lgame_gpu_budgets (so the same sums, bit for bit), with
// their scratch in the file-scope device array g_budget_scratch (defined beside the kernels)
// instead of the context's reduce_buf.  The array is part of the loaded module: one instance
// per device, no cudaMalloc, and the call allocates no host memory either (the result is
// copied straight into the caller's array).
namespace {
constexpr int kMaxDevices = 64;

// Device address of g_budget_scratch on device dev (which must be current).  It is looked up
// on every call and never cached: after a cudaDeviceReset the module is loaded again by the
// next context and the array may then sit at another address.  lgame_gpu_create has loaded
// the module, so the lookup allocates nothing.
int budget_scratch_address(int dev, double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_budget_scratch);
  if (e != cudaSuccess || !p) {
    char msg[256];
    std::snprintf(msg, sizeof msg, "lgame_gpu_budgets_static: cudaGetSymbolAddress of the scratch array on device %d: %s",
                  dev, cudaGetErrorString(e));
    lgame_set_error(msg);
    return LGAME_ERR_CUDA;
  }
  *out = static_cast<double*>(p);
  return LGAME_OK;
}

int budgets_static_on_device(lgame_gpu* c, int slot, double* out, int nq) {
  double* scratch = nullptr;
  int rc = budget_scratch_address(c->cfg.device, &scratch);
  if (rc != LGAME_OK) return rc;
  const Dims& D = c->D;
  double* dout = scratch + (size_t)kRedBlocks * LGAME_BUDGETS_MAX;
  k_budget_partial<<<kRedBlocks, kRedThreads, 0, c->stream>>>(D, c->G, c->st[slot], c->temperature, scratch, nq);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_budget_final<<<1, 32, 0, c->stream>>>(scratch, dout, nq);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, sizeof(double) * nq, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    char msg[256];
    std::snprintf(msg, sizeof msg, "lgame_gpu_budgets_static: %s", cudaGetErrorString(e));
    lgame_set_error(msg);
    return LGAME_ERR_CUDA;
  }
  out[D.ncons + 1] = 0.5 * out[D.ncons + 1];
  return LGAME_OK;
}
}  // namespace

extern "C" int lgame_gpu_budgets_static(lgame_gpu* c, int slot, double* out, int nout) {
  if (!c || !out || slot < 0 || slot > 1) {
    lgame_set_error("lgame_gpu_budgets_static: bad arguments");
    return LGAME_ERR_INVALID_ARG;
  }
  const int nq = c->D.ncons + 4;
  if (nq > LGAME_BUDGETS_MAX) {
    char msg[256];
    std::snprintf(msg, sizeof msg,
                  "lgame_gpu_budgets_static: %d budget quantities exceed the static scratch, which holds at most "
                  "LGAME_BUDGETS_MAX = %d (n_constituents <= 7)", nq, LGAME_BUDGETS_MAX);
    lgame_set_error(msg);
    return LGAME_ERR_INVALID_ARG;
  }
  if (nout < nq) {
    lgame_set_error("lgame_gpu_budgets_static: output array smaller than n_constituents+4");
    return LGAME_ERR_INVALID_ARG;
  }
  const int dev = c->cfg.device;
  if (dev < 0 || dev >= kMaxDevices) {
    lgame_set_error("lgame_gpu_budgets_static: device ordinal outside 0..63");
    return LGAME_ERR_INVALID_ARG;
  }
  // the context's device is made current for the call and the caller's device restored
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) {
    lgame_set_error("lgame_gpu_budgets_static: cudaGetDevice failed");
    return LGAME_ERR_CUDA;
  }
  if (prev != dev && cudaSetDevice(dev) != cudaSuccess) {
    lgame_set_error("lgame_gpu_budgets_static: cudaSetDevice failed");
    return LGAME_ERR_CUDA;
  }
  const int rc = budgets_static_on_device(c, slot, out, nq);
  if (prev != dev) cudaSetDevice(prev);
  return rc;
}

// ---- radiation: emulator features, heating rates -> power density, one emulator update ------
// (include/lgame_emulator.h; the reference's seam is update_rad_fluxes,
// src/radiation/mo_manage_radiation_calls.F90:17-59)
namespace {


// coszenith, mo_rterrtmgp_coupler.F90:550-629 (the sun's direction from the Earth's rotation
// and revolution relative to the winter solstice 2019-12-20 12:00 UTC), 0 at night
__device__ double coszenith(double lat, double lon, double t) {
  const double omega = 7.292115e-5, omega_rev = 1.99099e-7, obliquity = 0.409092592843564;
  const double tt = t - 1576843200.0;
  const double rot = omega * tt;
  const double n1 = cos(lat) * cos(lon), n2 = cos(lat) * sin(lon), n3 = sin(lat);
  const double s1 = -cos(rot) * cos(obliquity) * n1 + sin(rot) * cos(obliquity) * n2 + sin(obliquity) * n3;
  const double s2 = -sin(rot) * n1 - cos(rot) * n2;
  const double s3 = cos(rot) * sin(obliquity) * n1 - sin(rot) * sin(obliquity) * n2 + cos(obliquity) * n3;
  (void)s3;
  const double c = -(s1 * cos(omega_rev * tt) + s2 * sin(omega_rev * tt));
  return c < 0.0 ? 0.0 : c;
}

// one thread per column: T, dry-air pressure, vapour and ozone densities of every layer,
// albedo and cos(zenith); column index ji + ny*(jk-1), 4*nl+2 floats per column
__global__ void k_rad_features(Dims D, Grid<double> G, State S, const double* albedo, const double* lat,
                               const double* lon, double t, float* X) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const long long col = (ji - 1) + (long long)D.ny * (jk - 1);
  const int nl = D.nl, nf = 4 * nl + 2;
  float* x = X + col * nf;
  const double sigma = 20e3 / sqrt(8.0 * log(2.0));  // calc_o3_vmr: FWHM 20 km, maximum 8.5e-6 at 34 km
  const double m_o3 = 0.0479982;                       // kg/mol
  for (int jl = 1; jl <= nl; ++jl) {
    const long long i = IX(D, ji, jk, jl);
    const double rd = S.rho[i + (long long)(D.g - 1) * D.fstride];
    const double rv = D.lmoist ? S.rho[i + (long long)D.g * D.fstride] : 0.0;
    double T = (G.theta_v_bg[i] + S.tp[i]) * (G.exner_bg[i] + S.ep[i]);  // temperature_diagnostics
    if (D.lmoist) T = T / (1.0 + rv / rd * (kM_D / kM_V - 1.0));
    const double dz = G.z_scalar[i] - 34e3;
    const double vmr = 8.5e-6 * exp(-dz * dz / (2.0 * sigma * sigma));
    x[jl - 1] = (float)T;
    x[nl + jl - 1] = (float)(kR_D * rd * T);
    x[2 * nl + jl - 1] = (float)rv;
    x[3 * nl + jl - 1] = (float)(vmr * rd * m_o3 / kM_D);
  }
  x[4 * nl] = (float)albedo[col];
  x[4 * nl + 1] = (float)coszenith(lat[col], lon[col], t);
}

// radiation_tendency (W m^-3) = (shortwave + longwave heating rate)/86400 * rho_gas * c_d_p
__global__ void k_rad_apply(Dims D, State S, const float* heat, double* rad, float* rad_f) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx || jl > D.nl) return;
  const long long col = (ji - 1) + (long long)D.ny * (jk - 1);
  const long long i = IX(D, ji, jk, jl);
  const float hr = heat[col * 2 * D.nl + (jl - 1)] + heat[col * 2 * D.nl + D.nl + (jl - 1)];
  double rho = S.rho[i + (long long)(D.g - 1) * D.fstride];
  if (D.lmoist) rho += S.rho[i + (long long)D.g * D.fstride];
  const double q = (double)hr / 86400.0 * rho * kC_D_P;
  rad[i] = q;
  if (rad_f) rad_f[i] = (float)q;
}

// the context's radiation buffers, allocated at the first radiation call (they live and die
// with the context: its allocation list frees them)
int rad_buffers(lgame_gpu* c, RadBuffers** out) {
  RadBuffers* r = &c->radbuf;
  const Dims& D = c->D;
  if (!r->features) {
    r->ncol = (long long)D.ny * D.nx;
    r->nlev = D.nl;
    const size_t nf = 4 * (size_t)D.nl + 2;
    if (cudaMalloc(&r->albedo, sizeof(double) * r->ncol) != cudaSuccess ||
        cudaMalloc(&r->lat, sizeof(double) * r->ncol) != cudaSuccess ||
        cudaMalloc(&r->lon, sizeof(double) * r->ncol) != cudaSuccess ||
        cudaMalloc(&r->features, sizeof(float) * r->ncol * nf) != cudaSuccess ||
        cudaMalloc(&r->heating, sizeof(float) * r->ncol * 2 * D.nl) != cudaSuccess)
      return set_err(LGAME_ERR_ALLOC, "radiation buffers: cudaMalloc failed");
    c->allocations.push_back(r->albedo);
    c->allocations.push_back(r->lat);
    c->allocations.push_back(r->lon);
    c->allocations.push_back(r->features);
    c->allocations.push_back(r->heating);
    c->bytes += (long long)(sizeof(double) * 3 * r->ncol + sizeof(float) * r->ncol * (nf + 2 * D.nl));
    cudaMemset(r->albedo, 0, sizeof(double) * r->ncol);
    cudaMemset(r->lat, 0, sizeof(double) * r->ncol);
    cudaMemset(r->lon, 0, sizeof(double) * r->ncol);
  }
  *out = r;
  return LGAME_OK;
}

int rad_features_dev(lgame_gpu* c, RadBuffers* r, int slot, double t) {
  const Dims& D = c->D;
  k_rad_features<<<dim3((unsigned)((D.ny + 31) / 32), (unsigned)((D.nx + 3) / 4)), dim3(32, 4), 0, c->stream>>>(
      D, c->G, c->st[slot], r->albedo, r->lat, r->lon, t, r->features);
  CK(cudaGetLastError());
  return LGAME_OK;
}

int rad_apply_dev(lgame_gpu* c, RadBuffers* r, int slot) {
  const Dims& D = c->D;
  float* rad_f = c->split ? split_carried(c->split).rad : nullptr;
  k_rad_apply<<<grd(D, D.ny, D.nx, D.nl), blk(), 0, c->stream>>>(D, c->st[slot], r->heating, c->rad, rad_f);
  CK(cudaGetLastError());
  return LGAME_OK;
}
}  // namespace

extern "C" int lgame_gpu_rad_set_surface(lgame_gpu* c, const double* albedo, const double* lat, const double* lon) {
  if (!c || !albedo || !lat || !lon) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_rad_set_surface: bad arguments");
  RadBuffers* r = nullptr;
  int rc = rad_buffers(c, &r);
  if (rc) return rc;
  const size_t n = sizeof(double) * r->ncol;
  CK(cudaMemcpy(r->albedo, albedo, n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(r->lat, lat, n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(r->lon, lon, n, cudaMemcpyHostToDevice));
  return LGAME_OK;
}

extern "C" int lgame_gpu_rad_features(lgame_gpu* c, int slot, double t, float* features) {
  if (!c || slot < 0 || slot > 1) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_rad_features: bad arguments");
  if (!c->grid_set) return set_err(LGAME_ERR_STATE, "lgame_gpu_rad_features: lgame_gpu_set_grid has not been called");
  RadBuffers* r = nullptr;
  int rc = rad_buffers(c, &r);
  if (!rc) rc = rad_features_dev(c, r, slot, t);
  if (rc) return rc;
  if (features)
    CK(cudaMemcpyAsync(features, r->features, sizeof(float) * r->ncol * (4 * (size_t)r->nlev + 2), cudaMemcpyDeviceToHost,
                       c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return LGAME_OK;
}

extern "C" int lgame_gpu_rad_apply_heating(lgame_gpu* c, int slot, const float* heating) {
  if (!c || !heating || slot < 0 || slot > 1)
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_rad_apply_heating: bad arguments");
  RadBuffers* r = nullptr;
  int rc = rad_buffers(c, &r);
  if (rc) return rc;
  CK(cudaMemcpyAsync(r->heating, heating, sizeof(float) * r->ncol * 2 * r->nlev, cudaMemcpyHostToDevice, c->stream));
  rc = rad_apply_dev(c, r, slot);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return LGAME_OK;
}

extern "C" int lgame_gpu_rad_update(lgame_gpu* c, lgame_emu* emu, int slot, double t, int sample_stride,
                                    double bound, double* report) {
  if (!c || !emu || slot < 0 || slot > 1 || sample_stride < 0)
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_rad_update: bad arguments");
  if (emu::nlev_of(emu) != c->D.nl)
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_rad_update: the emulator's nlev differs from n_layers");
  const auto t0 = std::chrono::steady_clock::now();
  RadBuffers* r = nullptr;
  int rc = rad_buffers(c, &r);
  if (!rc) rc = rad_features_dev(c, r, slot, t);
  if (rc) return rc;
  rc = emu::infer_device(emu, r->features, r->ncol, r->heating, c->stream);
  if (rc) return rc;
  const int nl = r->nlev, nf = 4 * nl + 2, nh = 2 * nl;
  double rms = 0.0;
  long long nsample = 0;
  bool fallback = false;
  if (sample_stride > 0) {
    nsample = (r->ncol + sample_stride - 1) / sample_stride;
    std::vector<float> xs((size_t)nsample * nf), he((size_t)nsample * nh), ht((size_t)nsample * nh);
    CK(cudaMemcpy2DAsync(xs.data(), sizeof(float) * nf, r->features, sizeof(float) * nf * sample_stride,
                         sizeof(float) * nf, nsample, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpy2DAsync(he.data(), sizeof(float) * nh, r->heating, sizeof(float) * nh * sample_stride,
                         sizeof(float) * nh, nsample, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    rc = lgame_rad_teacher(xs.data(), nsample, nl, ht.data());
    if (rc) return rc;
    double s = 0.0;
    for (size_t k = 0; k < he.size(); ++k) s += (double)(he[k] - ht[k]) * (double)(he[k] - ht[k]);
    rms = std::sqrt(s / (double)he.size());
    if (rms > bound) {  // fallback: the teacher for every column
      fallback = true;
      std::vector<float> xa((size_t)r->ncol * nf), ha((size_t)r->ncol * nh);
      CK(cudaMemcpy(xa.data(), r->features, sizeof(float) * xa.size(), cudaMemcpyDeviceToHost));
      rc = lgame_rad_teacher(xa.data(), r->ncol, nl, ha.data());
      if (rc) return rc;
      CK(cudaMemcpy(r->heating, ha.data(), sizeof(float) * ha.size(), cudaMemcpyHostToDevice));
    }
  }
  rc = rad_apply_dev(c, r, slot);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  if (report) {
    report[0] = rms;
    report[1] = fallback ? 1.0 : 0.0;
    report[2] = (double)nsample;
    report[3] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  return LGAME_OK;
}

extern "C" int lgame_gpu_rad_attach(lgame_gpu* c, lgame_emu* emu, double dtime_rad, int sample_stride,
                                    double bound_k_per_day) {
  if (!c || sample_stride < 0 || (emu && dtime_rad < 0.0))
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_rad_attach: bad arguments");
  if (emu && emu::nlev_of(emu) != c->D.nl)
    return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_rad_attach: the emulator's nlev differs from n_layers");
  c->rad_emu = emu;
  c->rad_dtime = dtime_rad;
  c->rad_stride = sample_stride;
  c->rad_bound = bound_k_per_day;
  c->rad_updates = 0;
  for (double& r : c->rad_report) r = 0.0;
  return LGAME_OK;
}

extern "C" int lgame_gpu_rad_last_report(const lgame_gpu* c, double* report, int* updates) {
  if (!c || !report) return set_err(LGAME_ERR_INVALID_ARG, "lgame_gpu_rad_last_report: bad arguments");
  for (int k = 0; k < 4; ++k) report[k] = c->rad_report[k];
  if (updates) *updates = c->rad_updates;
  return LGAME_OK;
}
