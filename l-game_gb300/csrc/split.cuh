// split.cuh -- FP32/FP64 split-precision HEVI step (interface used by lgame_gpu.cu).
//
// FP32: explicit stencils (vorticity, Poisson-bracket flux, the kinetic-energy gradient's
//       division by the metric, third-order theta edges), scalar and tracer flux
//       divergences, tracer fall speeds and vertical fluxes, the coefficients of the
//       implicit systems, intermediate and tendency storage, and a mirror of the state
//       (each FP64 state value rounded once when it is written).
// FP64: the state, its accumulation state_old + dt*tendency, the gradient of the Exner
//       pressure perturbation and both pressure-gradient products (the hydrostatic
//       background subtraction), the kinetic energy and its differences (a vertical
//       difference over a thin layer cancels most of its digits), the right-hand side and
//       both substitution sweeps of the vertical acoustic solve (its coefficients and
//       elimination multipliers are FP32), the budget sums.  The tracer solve is FP32 for
//       the increment delta = rho_new - rho_old (coefficients, right-hand side, both sweeps),
//       so its rounding is relative to the flux terms; only rho_old + delta is FP64.
#pragma once

#include <cuda_runtime.h>

#include "diffusion.cuh"
#include "kernels.cuh"
#include "phase.cuh"
#include "surface.cuh"

namespace lg {

struct SplitCtx;

// diagnostic buffers of the split step that correspond to lgame_gpu.h's carried fields
struct SplitCarriedF {
  float *pgcw, *vsg_x, *vsg_y, *vsg_z, *pvt_x, *pvt_y, *pvt_z, *csh, *rad, *temperature;
  float* hdiss;  // dissipative heating, formed at each step's first substep
  // the carried diagnostics of the diffusion closure (null when horizontal momentum diffusion
  // is off): TKE, viscosity, momentum diffusion accelerations
  float *tke, *visc, *mdtx, *mdty, *mdtz;
  // temp_diff_heating and mass_diff_tendency (ncons fields), same condition
  float *tdh, *mdt;
  // the phase transitions' rates (nc+1 fields) and heating rate (null when lphase_trans is off)
  float *ptr, *pth;
  Tend<float> tend;
  // with a background state: the net pressure-gradient terms nl + l of u, v, w and the previous
  // substep's values -(nl + l) of u, v, rounded to FP32 (the only form the wind update uses)
  float *pnet_u, *pnet_v, *pnet_w, *pold_u, *pold_v;
};

// the diffusion closure of the split step: which parts run and their constants
struct SplitDiff {
  bool mom_h = false, mom_v = false, temp_h = false, temp_v = false, mass_h = false, mass_v = false;
  DiffPar par{};
};

// the surface layer, PBL and soil of the split step: which parts run and the FP64 buffers they
// share with the FP64 step (surface planes, soil temperature of the two slots, v_squared)
struct SplitSfc {
  bool turb = false, pbl = false, sens = false, soil = false;
  bool phase = false, phase_sfc = false;  // lphase_trans, and its surface part (lsfc_phase_trans)
  SfcBuf buf{};
  SfcPar par{};
  double* vsq = nullptr;
  double* tsoil[2] = {nullptr, nullptr};
};

// column_fp64: the vertical acoustic solve with FP64 coefficients and elimination; diff: the
// diffusion closure (its buffers are allocated when horizontal momentum diffusion is on);
// sfc: the surface parts, whose kinetic-energy array the split step uses as its own
int split_create(const Dims& D, bool column_fp64, const SplitDiff& diff, const SplitSfc& sfc, SplitCtx** out,
                 long long* bytes);
// the surface kernels' parameters once the soil grid is known
void split_set_sfc_par(SplitCtx* s, const SfcPar& par);
// the closure's constants once the grid is known (mean_velocity_area)
void split_set_diff_par(SplitCtx* s, const DiffPar& par);
void split_destroy(SplitCtx* s);
// builds the FP32 metric copies and the FP64 reciprocal metrics from the FP64 grid
int split_set_grid(SplitCtx* s, const Dims& D, const Grid<double>& G, cudaStream_t stream);
// the FP32 carried buffers of the split step, for conversion to and from FP64 arrays
SplitCarriedF split_carried(SplitCtx* s);
// net = narrow(a + b) for n elements (the net pressure-gradient buffers from the FP64 arrays)
int split_net(const double* a, const double* b, float* net, long long n, cudaStream_t stream);
// converts n elements FP64 <-> FP32 (field layout identical)
int split_convert(const double* src, float* dst, long long n, cudaStream_t stream);
int split_convert_back(const float* src, double* dst, long long n, cudaStream_t stream);
// the FP32 mirror of state slot `slot` (its arrays; for writers that fill it themselves)
StateF split_mirror(SplitCtx* s, int slot);
// lateral boundary relaxation: split_bc_prepare forms the background's rhotheta_v once (after
// the grid is set), split_bc_update relaxes state S (mirror M, may be empty) toward the levels
// B0 (weight ow) and B1 (weight nw) with the rescale factors fs, fu, fv on the padded plane, at
// the nrim plane points rim[] (plane indices where any factor is nonzero), and recomputes
// theta_v_pert and exner_pert (two launches)
int split_bc_prepare(SplitCtx* s, const Dims& D, const Grid<double>& G, cudaStream_t stream);
int split_bc_update(SplitCtx* s, const Dims& D, const Grid<double>& G, const State& S, const StateF& M, const State& B0,
                    const State& B1, const int* rim, int nrim, const double* fs, const double* fu, const double* fv,
                    double ow, double nw, cudaStream_t stream);
// FP32 mirror of state slot `slot` recomputed from the FP64 state S (after the host wrote S)
int split_refresh_mirror(SplitCtx* s, const Dims& D, int slot, const State& S, cudaStream_t stream);
// one step from slot so (state So) to slot sn (state Sn); pg holds the FP64 pressure-gradient
// arrays (shared with the FP64 path).  The mirrors of both slots must be current.
int split_step(SplitCtx* s, const Dims& D, const Grid<double>& G, const State& So, const State& Sn, int so, int sn,
               const PGrad<double>& pg, int step, cudaStream_t stream, int* nkernels,
               int (*trace_begin)(void*, const char*), void (*trace_end)(void*, int), void* tracer,
               bool serial);

}  // namespace lg
