// split.cu -- FP32/FP64 split-precision HEVI step (compiled with -fmad=true, -prec-div=false).
//
// The explicit stencils are the templates of kernels.cuh instantiated for float.  They read
// an FP32 mirror of the state: a rounded copy of every prognostic field, written by the
// kernels that update the FP64 state (k_tend_wind for u and v, the two column solvers for
// the rest) and refreshed from the FP64 state whenever the host replaces it.  On this GPU a
// conversion between FP64 and FP32 costs as much as an FP64 operation (both ~2 per clock
// per SM, against 128 FP32 operations), so converting each state value once when it is
// written, instead of at every stencil use, takes the FP32 stencils off the FP64 pipe.
//
// This file adds the parts that stay in FP64 in this mode -- the pressure gradient and the
// two column solvers -- written to spend as few FP64 operations per cell as the precision
// split allows: coefficients that only scale an increment (the partial derivatives of the
// implicit system, fall speeds, fluxes) come from the FP32 mirror; the right-hand sides,
// the substitution sweeps of the tridiagonal solves and the state updates are FP64.
#include "split.cuh"
#include "common.h"
#include "lgame_gpu.h"

#include <algorithm>
#include <string>
#include <vector>

namespace lg {

namespace {

constexpr int kMaxL = 128;

struct GridX {  // FP64 reciprocal metrics and FP32 metric differences of the FP64 parts
  const double *inv_dx, *inv_dy, *inv_dz, *inv_volume, *inv_area_z;
  // FP32: 1/volume, 1/area_z, and at w level jl (2..nl) z_scalar(jl-1)-z_scalar(jl) and
  // exner_bg(jl-1)-exner_bg(jl), differenced in FP64 before rounding (no cancellation)
  const float *inv_volume_f, *inv_area_z_f, *dzs_f, *deb_f;
  // FP32: the swamp layer's deceleration per unit w, (1/damping_prefactor - 1)/dtime, formed in
  // FP64 (w/p - w would cancel where the prefactor is near 1); 0 at the top level
  const float* kdamp_f;
};

// x / d to FP64 accuracy for an FP32 divisor d in the normal range.  r = 1/d correctly
// rounded in FP32; the residual 1 - d*r of a correctly rounded reciprocal is exact in FP32,
// so r + (1 - d*r)*r is 1/d to ~2^-48 as an unevaluated pair of FP32 numbers (the
// correction step of Markstein's division), and x*(r + r_lo) costs two FP64-pipe operations
// (relative error below 2^-47) instead of a conversion and an FP64 division.
__device__ __forceinline__ double div_f(double x, float d) {
  const float r = __frcp_rn(d);
  const float r_lo = __fmaf_rn(-d, r, 1.f) * r;
  return fma(x, wide(r_lo), x * wide(r));
}

}  // namespace

struct SplitCtx {
  std::vector<void*> allocs;
  Grid<float> GF{};
  GridX GX{};
  float *gf[40] = {};
  float *ipw[6] = {}, *trsk_u[3] = {}, *trsk_v[2] = {};
  double *inv_dx = nullptr, *inv_dy = nullptr, *inv_dz = nullptr, *inv_volume = nullptr, *inv_area_z = nullptr;
  // FP32 intermediates
  float *gx, *gy, *gz, *divf, *tvu, *tvv, *tpu, *tpv, *ex, *ey, *ez, *uph, *vph, *wph;
  // kinetic energy in FP64: its vertical differences over thin layers cancel most digits
  double* vsq = nullptr;
  // FP64 vertical gradient of exner' at w points (0 at the top and surface levels), and per
  // column and terrain-following layer l half its weighted sum 0.5*(W5*gz(l) + W6*gz(l+1))
  double* gzd = nullptr;
  double* rmz = nullptr;
  // sediment heating of each condensate (nc planes), summed into the carried csh
  float* csh_part = nullptr;
  // divergence of the gradient of theta_bg (the third-order theta chain of the background),
  // and the background's x and y edge averages as FP32 pairs
  float* dbg = nullptr;
  float2 *tbu = nullptr, *tbv = nullptr;
  // horizontal gas mass fluxes and theta_v fluxes of the scalar tendency
  float *fu = nullptr, *fv = nullptr, *gu = nullptr, *gv = nullptr;
  // FP32 mirrors of the two state slots
  StateF mir[2]{};
  SplitCarriedF C{};
  // rhotheta_v of the background state, p_0/r_d*exner_bg^(c_d_v/r_d) (boundary relaxation)
  double* rtbg = nullptr;
  // the vertical acoustic solve with FP64 coefficients and elimination (precision mode
  // LGAME_PRECISION_SPLIT_FP64_COLUMN)
  bool column_fp64 = false;
  // diffusion closure: configuration and FP32 buffers (the carried ones are in C)
  SplitDiff diff{};
  DiffBuf<float> db{};
  // surface layer, PBL and soil (FP64 buffers of the FP64 step)
  SplitSfc sfc{};
  // the step's concurrent branches: two side streams and the events of their forks and joins
  cudaStream_t br[2] = {nullptr, nullptr};
  cudaEvent_t ev[8] = {};
};

namespace {

template <class P>
int salloc(SplitCtx* s, P** p, size_t n, long long* bytes) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, n * sizeof(P));
  if (e != cudaSuccess) {
    lgame_set_error((std::string("cudaMalloc (split) failed: ") + cudaGetErrorString(e)).c_str());
    return LGAME_ERR_ALLOC;
  }
  if (cudaMemset(q, 0, n * sizeof(P)) != cudaSuccess) return LGAME_ERR_CUDA;
  s->allocs.push_back(q);
  *bytes += (long long)(n * sizeof(P));
  *p = (P*)q;
  return LGAME_OK;
}

__global__ void k_to_float(const double* a, float* b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}
__global__ void k_net(const double* a, const double* b, float* net, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    net[i] = narrow(a[i] + b[i]);
}
__global__ void k_to_double(const float* a, double* b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}
__global__ void k_recip(const double* a, double* b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (a[i] != 0.0) ? 1.0 / a[i] : 0.0;
}
// FP32 metric reciprocals and vertical differences of the column solver (set-up only)
__global__ void k_grid_extra(Dims D, Grid<double> G, float* ivol, float* iaz, float* dzs, float* deb, float* kd) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx || jl > D.NL) return;
  const long long q = IX(D, ji, jk, jl);
  iaz[q] = (G.area_z[q] != 0.0) ? float(1.0 / G.area_z[q]) : 0.f;
  kd[q] = (jl >= 2) ? float((1.0 / G.damp[q] - 1.0) / D.dtime) : 0.f;
  if (jl <= D.nl) ivol[q] = float(1.0 / G.volume[q]);
  if (jl >= 2 && jl <= D.nl) {
    const long long a = IX(D, ji, jk, jl - 1);
    dzs[q] = float(G.z_scalar[a] - G.z_scalar[q]);
    deb[q] = float(G.exner_bg[a] - G.exner_bg[q]);
  }
}

// ---- pressure gradient, mo_p_grad.F90:20-120, FP64 products ---------------------------
// gradient of the Exner pressure perturbation in FP64 (the small differences of a small
// field), theta edge values in FP32 (third order) or FP64 (second order), the background
// term theta'*grad(Pi_bg) in FP64, the condensate deceleration factor in FP32 from the
// mirror densities.  Six resident blocks of 256 threads per SM (40 registers) ran 12 % faster
// than five.
__global__ void __launch_bounds__(256, 6) ks_pgrad(Dims D, Grid<double> G, GridX X, State S, const double* gzd,
                                                  const double* rmz, const float* mrho, const float* tvu,
                                                  const float* tvv, const float* tpu, const float* tpv,
                                                  PGrad<double> P, SplitCarriedF PF, float* pgcw, int lfirst) {
  LG_IDX3;
  const double* ep = S.ep;
  auto theta = [&](int i, int j, int k) { const long long q = IX(D, i, j, k); return G.theta_v_bg[q] + S.tp[q]; };
  // condensate mass fraction sum(rho_cond)/sum(rho): the reference's rho_g/sum(rho) and
  // rho_g/sum(rho) - 1 (mo_p_grad.F90:86-87, :115-116) rewritten as 1 - f and -f, which
  // is exact for dry air and free of cancellation in FP32
  auto cond_frac = [&](long long q) -> float {
    if (D.nc == 0) return 0.f;
    float c = 0.f;
    for (int jc = 0; jc < D.nc; ++jc) c += mrho[q + (long long)jc * D.fstride];
    return c / (c + mrho[q + (long long)(D.g - 1) * D.fstride]);
  };
  auto decel = [&](int i, int j, int k) {
    return float(kC_D_P) - float(kC_D_P) * cond_frac(IX(D, i, j, k));
  };
  // vertical gradient of exner_pert at a w point of column (i,j) (ks_gzp), 0 at the boundary levels
  auto gzp = [&](int i, int j, int k) -> double { return gzd[IX(D, i, j, k)]; };
  // remap_ver2hor_x/_y (mo_averaging.F90:56-136) of gzp at a u or v face: the sum over the
  // face's two columns a and b of 0.5*(W5*gz(l) + W6*gz(l+1)), each column's term formed once
  // in ks_gzp (the reference adds the four products in the order W5a, W5b, W6a, W6b; here
  // the pairs of a column are added first, an FP64 rounding difference)
  auto remapx = [&](int ji_, int jk_, int jl_) -> double {
    const int a = (jk_ == 1 || jk_ == D.nx + 1) ? D.nx : jk_ - 1, b = (jk_ == 1 || jk_ == D.nx + 1) ? 1 : jk_;
    return rmz[IX(D, ji_, a, jl_)] + rmz[IX(D, ji_, b, jl_)];
  };
  auto remapy = [&](int ji_, int jk_, int jl_) -> double {
    const int a = (ji_ == 1 || ji_ == D.ny + 1) ? D.ny : ji_ - 1, b = (ji_ == 1 || ji_ == D.ny + 1) ? 1 : ji_;
    return rmz[IX(D, a, jk_, jl_)] + rmz[IX(D, b, jk_, jl_)];
  };
  // the products of the u face (jk) and the v face (ji) of layer jl: nl = decel*theta_edge*grad,
  // l = decel*theta'_edge*grad(Pi_bg) (with a background state); false at non-periodic edges.
  // decel and the edge theta are FP32 values; their product with the gradient is FP64 (an
  // extra FP32 rounding of either product would unbalance the two terms, which cancel in an
  // atmosphere at rest)
  auto face_u = [&](double* nlv, double* lv) -> bool {
    const bool inner = jk >= 2 && jk <= D.nx;
    if (!inner && !D.periodic) return false;
    const int kk = inner ? jk : 1, ka = inner ? jk - 1 : D.nx;
    const long long qr = IX(D, ji, kk, jl);
    double g = (ep[qr] - ep[IX(D, ji, ka, jl)]) * X.inv_dx[qr];
    if (jl > D.nf) g -= G.slope_x[qr] * remapx(ji, kk, jl);
    const double te = (D.theta_order == 2) ? 0.5 * (theta(ji, ka, jl) + theta(ji, kk, jl)) : wide(tvu[qr]);
    const double de = wide(0.5f * (decel(ji, ka, jl) + decel(ji, kk, jl)));
    *nlv = de * (te * g);
    if (D.luse_bg) {
      const double tp = (D.theta_order == 2) ? 0.5 * (S.tp[IX(D, ji, ka, jl)] + S.tp[qr]) : wide(tpu[qr]);
      *lv = de * (tp * G.egu[qr]);
    }
    return true;
  };
  auto face_v = [&](double* nlv, double* lv) -> bool {
    const bool inner = ji >= 2 && ji <= D.ny;
    if (!inner && !D.periodic) return false;
    const int ii = inner ? ji : 1, ia = inner ? ji - 1 : D.ny;
    const long long qr = IX(D, ii, jk, jl);
    double g = (ep[IX(D, ia, jk, jl)] - ep[qr]) * X.inv_dy[qr];
    if (jl > D.nf) g -= G.slope_y[qr] * remapy(ii, jk, jl);
    const double te = (D.theta_order == 2) ? 0.5 * (theta(ia, jk, jl) + theta(ii, jk, jl)) : wide(tvv[qr]);
    const double de = wide(0.5f * (decel(ia, jk, jl) + decel(ii, jk, jl)));
    *nlv = de * (te * g);
    if (D.luse_bg) {
      const double tp = (D.theta_order == 2) ? 0.5 * (S.tp[IX(D, ia, jk, jl)] + S.tp[qr]) : wide(tpv[qr]);
      *lv = de * (tp * G.egv[qr]);
    }
    return true;
  };
  // Both products are stored in FP64 (the reference's diagnostics).  With a background state
  // the wind update uses only the net nl + l and the previous substep's -(nl + l), both rounded
  // to FP32, so those are also kept in FP32 (net, old): the same values the update would round,
  // read at a third of the bytes.  p_grad_acc_old is updated in that form only.  Without a
  // background state nl alone carries the hydrostatic balance and the update reads the FP64
  // arrays.
  auto update = [&](const bool face, const double nlv, const double lv, double* nl, double* l, double* old,
                    float* net_f, float* old_f, long long q) {
    if (D.luse_bg) {
      const float net_prev = net_f[q];
      float o = -net_prev;
      if (face) {
        nl[q] = nlv;
        l[q] = lv;
        const float net = narrow(nlv + lv);
        net_f[q] = net;
        if (lfirst) o = -net;
      }
      old_f[q] = o;
    } else {
      const double nl_prev = nl[q];
      if (!lfirst) old[q] = -nl_prev;
      if (face) {
        nl[q] = nlv;
        if (lfirst) old[q] = -nlv;
      } else if (lfirst) {
        old[q] = -nl_prev;
      }
    }
  };
  if (jl <= D.nl && ji <= D.ny && jk <= D.nx + 1) {
    double nlv = 0.0, lv = 0.0;
    const bool face = face_u(&nlv, &lv);
    update(face, nlv, lv, P.nl_u, P.l_u, P.old_u, PF.pnet_u, PF.pold_u, IX(D, ji, jk, jl));
  }
  if (jl <= D.nl && ji <= D.ny + 1 && jk <= D.nx) {
    double nlv = 0.0, lv = 0.0;
    const bool face = face_v(&nlv, &lv);
    update(face, nlv, lv, P.nl_v, P.l_v, P.old_v, PF.pnet_v, PF.pold_v, IX(D, ji, jk, jl));
  }
  if (jl >= 2 && jl <= D.nl && ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl), qa = IX(D, ji, jk, jl - 1);
    const float fa = cond_frac(qa), fb = cond_frac(q);
    const double de = wide(0.5f * ((float(kC_D_P) - float(kC_D_P) * fa) + (float(kC_D_P) - float(kC_D_P) * fb)));
    const double nlw = de * (0.5 * (theta(ji, jk, jl - 1) + theta(ji, jk, jl)) * gzp(ji, jk, jl));
    P.nl_w[q] = nlw;
    if (D.luse_bg) {
      const double lw = de * (0.5 * (S.tp[qa] + S.tp[q]) * G.egw[q]);
      P.l_w[q] = lw;
      PF.pnet_w[q] = narrow(nlw + lw);
    }
    pgcw[q] = 0.5f * (-fa - fb) * float(G.gm[q]);
  }
}

// vertical gradient of exner_pert at the w levels 2..nl (grad_vert, mo_gradient_operators.F90:65-83),
// and in the terrain-following layers l > nf the column's half of the remap of that gradient
// to the horizontal faces, 0.5*(W5(l)*gz(l) + W6(l)*gz(l+1)) (mo_averaging.F90:56-136; the W6
// term only where l < nl or with a free-slip surface), gz being 0 at levels 1 and nl+1
__global__ void ks_gzp(Dims D, Grid<double> G, GridX X, const double* ep, double* gzd, double* rmz) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.y + 1;
  if (ji > D.ny || jk > D.nx || jl > D.nl) return;
  const long long q = IX(D, ji, jk, jl);
  double gz = 0.0;
  if (jl >= 2) {
    gz = (ep[IX(D, ji, jk, jl - 1)] - ep[q]) * X.inv_dz[q];
    gzd[q] = gz;
  }
  if (jl > D.nf) {
    double r = G.ipw[4][q] * gz;
    if (jl < D.nl || D.freeslip) {
      const double gz1 = (jl < D.nl) ? (ep[q] - ep[q + D.plane]) * X.inv_dz[q + D.plane] : 0.0;
      r += G.ipw[5][q] * gz1;
    }
    rmz[q] = 0.5 * r;
  }
}

// horizontal gas mass fluxes and theta_v fluxes of scalar_tend_expl, mo_scalar_tend_expl.F90:106-138:
// rho_g*u at u points, rho_g*v at v points (scalar_times_vector_h), times the theta_v edge
// values (third order: tvu, tvv; second order: the mean of the two cells).  Each face is
// computed once here and read by ks_gas_div; the reference's untouched boundary faces are 0.
__global__ void ks_gas_flux(Dims D, Grid<float> GF, StateF Ss, const float* u_new, const float* v_new,
                            const float* tvu, const float* tvv, float* fu, float* fv, float* gu, float* gv) {
  LG_IDX3;
  if (jl > D.nl) return;
  const float* rg = Ss.rho + (long long)(D.g - 1) * D.fstride;
  auto th = [&](int i, int j, int k) { const long long p = IX(D, i, j, k); return GF.theta_v_bg[p] + Ss.tp[p]; };
  if (ji <= D.ny && jk <= D.nx + 1) {
    const long long q = IX(D, ji, jk, jl);
    float f = 0.f, g = 0.f;
    if (stv_h_x<float>(D, rg, u_new, ji, jk, jl, &f)) {
      if (D.theta_order == 2) {
        const int ka = (jk >= 2 && jk <= D.nx) ? jk - 1 : D.nx, kb = (jk >= 2 && jk <= D.nx) ? jk : 1;
        g = 0.5f * (th(ji, ka, jl) + th(ji, kb, jl)) * f;
      } else {
        g = tvu[q] * f;
      }
    }
    fu[q] = f;
    gu[q] = g;
  }
  if (ji <= D.ny + 1 && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    float f = 0.f, g = 0.f;
    if (stv_h_y<float>(D, rg, v_new, ji, jk, jl, &f)) {
      if (D.theta_order == 2) {
        const int ia = (ji >= 2 && ji <= D.ny) ? ji - 1 : D.ny, ib = (ji >= 2 && ji <= D.ny) ? ji : 1;
        g = 0.5f * (th(ia, jk, jl) + th(ib, jk, jl)) * f;
      } else {
        g = tvv[q] * f;
      }
    }
    fv[q] = f;
    gv[q] = g;
  }
}

// theta_v_adv_3rd_order edge values, mo_multiplications.F90:134-202, from theta' and dv, the
// divergence of the gradient of theta'.  The chain theta -> gradient -> divergence is linear,
// so the full theta_v edge is the background's part plus theta''s: 0.5*(theta_bg,a +
// theta_bg,b) - c*dbg, with dbg the background's divergence and both formed once in FP64 at
// set-up (split_set_grid; the face average is kept as an FP32 pair hi + lo), plus
// 0.5*(theta'_a + theta'_b) - c*dv.  Adding the small parts first and hi last rounds the
// ~300 K edge value once, where theta_bg + theta' rounded per cell cost one to two units of
// the last place; the FP32 differences are taken of theta' rather than of theta_v.  With
// tpu/tpv given, the edges of theta' alone (the background-subtracted edges of the pressure
// gradient) come from the same pass.  The upwind cell of the correction follows the face
// velocity as in the reference.
__global__ void ks_theta_edges(Dims D, const float* tp, const float* dv, const float* dbg, const float2* tbu,
                               const float2* tbv, const float* u, const float* v, float* tvu, float* tvv, float* tpu,
                               float* tpv) {
  LG_IDX3;
  const float c = narrow(D.theta_edge_c);
  auto edge = [&](long long a, long long b, long long up, long long q, float2 bgf, float* ov, float* op) {
    const float d = dv[up];
    const float pe = 0.5f * (tp[a] + tp[b]);
    ov[q] = bgf.x + (bgf.y + ((pe - c * d) - c * dbg[up]));
    if (op) op[q] = pe - c * d;
  };
  if (ji <= D.ny && jk <= D.nx + 1) {  // x edges: cells west (a) and east (b) of the face
    const bool in = jk >= 2 && jk <= D.nx;
    if (in || D.periodic) {
      const int ka = in ? jk - 1 : D.nx, kb = in ? jk : 1;
      const long long a = IX(D, ji, ka, jl), b = IX(D, ji, kb, jl), q = IX(D, ji, jk, jl);
      edge(a, b, (u[IX(D, ji, kb, jl)] >= 0.f) ? a : b, q, tbu[q], tvu, tpu);
    }
  }
  if (ji <= D.ny + 1 && jk <= D.nx) {  // y edges: cells south (a, row ji) and north (b, row ji-1)
    const bool in = ji >= 2 && ji <= D.ny;
    if (in || D.periodic) {
      const int ia = in ? ji : 1, ib = in ? ji - 1 : D.ny;
      const long long a = IX(D, ia, jk, jl), b = IX(D, ib, jk, jl), q = IX(D, ji, jk, jl);
      edge(a, b, (v[IX(D, ia, jk, jl)] >= 0.f) ? a : b, q, tbv[q], tvv, tpv);
    }
  }
}

// the background's face averages 0.5*(theta_bg,a + theta_bg,b) at the x and y edges, in FP64,
// kept as FP32 pairs (hi = the rounded value, lo = the rounded remainder)
__global__ void k_bg_faces(Dims D, Grid<double> G, float2* tbu, float2* tbv) {
  LG_IDX3;
  auto pair = [](double x) {
    const float hi = narrow(x);
    return make_float2(hi, narrow(x - wide(hi)));
  };
  if (ji <= D.ny && jk <= D.nx + 1) {
    const bool in = jk >= 2 && jk <= D.nx;
    if (in || D.periodic) {
      const int ka = in ? jk - 1 : D.nx, kb = in ? jk : 1;
      tbu[IX(D, ji, jk, jl)] = pair(0.5 * (G.theta_v_bg[IX(D, ji, ka, jl)] + G.theta_v_bg[IX(D, ji, kb, jl)]));
    }
  }
  if (ji <= D.ny + 1 && jk <= D.nx) {
    const bool in = ji >= 2 && ji <= D.ny;
    if (in || D.periodic) {
      const int ia = in ? ji : 1, ib = in ? ji - 1 : D.ny;
      tbv[IX(D, ji, jk, jl)] = pair(0.5 * (G.theta_v_bg[IX(D, ia, jk, jl)] + G.theta_v_bg[IX(D, ib, jk, jl)]));
    }
  }
}

// simple_dissipation_rate, mo_momentum_diff_diss.F90:333-389, split step: the swamp layer's
// dissipative heating -sum(rho(1:nc+1))*(W5 w(jl) d(jl) + W6 w(jl+1) d(jl+1)), d = w*kdamp the
// deceleration at w levels 2..n_damping_levels, in FP32 from the mirror (a heating term, as
// the radiation and sediment heating it is added to)
__global__ void ks_heating_diss(Dims D, Grid<float> GF, GridX X, StateF M, float* hd) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx || jl > D.nl) return;
  const long long q = IX(D, ji, jk, jl), b = q + D.plane;
  const float wa = M.w[q], wb = M.w[b];
  const float da = (jl >= 2 && jl <= D.ndamp) ? wa * X.kdamp_f[q] : 0.f;
  const float db = (jl + 1 <= D.ndamp) ? wb * X.kdamp_f[b] : 0.f;
  const float ip = GF.ipw[4][q] * wa * da + GF.ipw[5][q] * wb * db;
  hd[q] = -rho_sum_cond_gas<float, float>(D, M.rho, q) * ip;
}

// ---- column-marching divergences -------------------------------------------------------
// div_h with the contravariant vertical correction (div_h_at above: div_h,
// mo_divergence_operators.F90:16-68, and vertical_contravariant_corr, mo_averaging.F90:16-54)
// evaluated by one thread per column walking down the levels.  The correction at the
// interface between layers l-1 and l is -(h(l-1) + h(l)), h(l) being half the slope-weighted
// sum of layer l's four face values (only h(l) at the top interface of the terrain-following
// layers, l = nf+1).  Each layer's faces are loaded once per column, each h once, and each
// interface's correction serves the cells on both sides of it; the next layer's loads are
// issued before the current layer's result is stored.

// the four face values of layer l of column (ji, jk) -- x at the east (jk+1) and west (jk)
// u points, y at the north (ji) and south (ji+1) v points -- and h(l)
struct LayerFaces { float xe, yn, xw, ys, h; };

// h(l) of a layer whose four face values are set
__device__ __forceinline__ void layer_h(const Dims& D, const Grid<float>& G, LayerFaces& f, int ji, int jk, int l) {
  f.h = 0.f;
  if (l >= D.nf + 1) {
    const long long p = IX(D, ji, jk, l);
    f.h = 0.5f * f.xe * G.slope_x[IX(D, ji, jk + 1, l)] * G.ipw[0][p] + 0.5f * f.yn * G.slope_y[p] * G.ipw[1][p]
        + 0.5f * f.xw * G.slope_x[p] * G.ipw[2][p] + 0.5f * f.ys * G.slope_y[IX(D, ji + 1, jk, l)] * G.ipw[3][p];
  }
}

template <class FX, class FY>
__device__ __forceinline__ LayerFaces layer_faces(const Dims& D, const Grid<float>& G, FX fx, FY fy, int ji, int jk,
                                                  int l) {
  LayerFaces f;
  f.xe = fx(ji, jk + 1, l);
  f.yn = fy(ji, jk, l);
  f.xw = fx(ji, jk, l);
  f.ys = fy(ji + 1, jk, l);
  layer_h(D, G, f, ji, jk, l);
  return f;
}

// contravariant corrections at the upper (cu, interface jl) and lower (cl, interface jl+1)
// face of cell jl, and which of them the reference's branches use (mo_divergence_operators.F90:
// the top terrain-following layer nf has only its lower face, the lowest layer only its upper
// one unless it is layer nf itself)
struct VertFaces { float cu, cl; bool up, lo; };
__device__ __forceinline__ VertFaces vert_faces(const Dims& D, float h_prev, float h_cur, float h_next, int jl) {
  VertFaces v;
  v.up = jl > D.nf;
  v.lo = jl == D.nf || (jl > D.nf && jl < D.nl);
  v.cu = (jl == D.nf + 1) ? -h_cur : -(h_prev + h_cur);
  v.cl = (jl + 1 == D.nf + 1) ? -h_next : -(h_cur + h_next);
  return v;
}

// the divergence of cell jl from its layer's faces and the corrections of its two interfaces
__device__ __forceinline__ float div_col(const Dims& D, const Grid<float>& G, const GridX& X, const LayerFaces& c,
                                         const VertFaces& v, int ji, int jk, int jl) {
  const long long q = IX(D, ji, jk, jl);
  const float comp_h = c.xe * G.area_x[IX(D, ji, jk + 1, jl)] + c.yn * G.area_y[q] - c.xw * G.area_x[q]
                     - c.ys * G.area_y[IX(D, ji + 1, jk, jl)];
  float comp_v = 0.f;
  if (v.up) comp_v += v.cu * G.area_z[q];
  if (v.lo) comp_v -= v.cl * G.area_z[IX(D, ji, jk, jl + 1)];
  return (comp_h + comp_v) * X.inv_volume_f[q];
}

// div_h of a stored horizontal vector field (the third-order theta chain)
__global__ void __launch_bounds__(128) ks_div_h(Dims D, Grid<float> GF, GridX X, const float* vx, const float* vy,
                                                float* out) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  auto fx = [&](int i, int j, int k) { return vx[IX(D, i, j, k)]; };
  auto fy = [&](int i, int j, int k) { return vy[IX(D, i, j, k)]; };
  LayerFaces cur = layer_faces(D, GF, fx, fy, ji, jk, 1), nxt{};
  float h_prev = 0.f;
  for (int jl = 1; jl <= D.nl; ++jl) {
    nxt.h = 0.f;
    if (jl < D.nl || jl == D.nf) nxt = layer_faces(D, GF, fx, fy, ji, jk, jl + 1);
    out[IX(D, ji, jk, jl)] = div_col(D, GF, X, cur, vert_faces(D, h_prev, cur.h, nxt.h, jl), ji, jk, jl);
    h_prev = cur.h;
    cur = nxt;
  }
}

// divergences of the gas and theta_v fluxes and the diabatic rho*theta_v term,
// mo_scalar_tend_expl.F90:106-177 (the gas has old_weight 0, new_weight 1), column-marching
__global__ void __launch_bounds__(128) ks_gas_div(Dims D, Grid<float> GF, GridX X, StateF Ss, const float* fu,
                                                  const float* fv, const float* gu, const float* gv, const float* Tm,
                                                  const float* hd, const float* rad, const float* csh, float* t_rho,
                                                  float* t_rt, const float* mdt, const float* tdh,
                                                  const float* ptr, const float* pth) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const long long goff = (long long)(D.g - 1) * D.fstride;
  auto fx = [&](int i, int j, int k) { return fu[IX(D, i, j, k)]; };
  auto fy = [&](int i, int j, int k) { return fv[IX(D, i, j, k)]; };
  auto gx = [&](int i, int j, int k) { return gu[IX(D, i, j, k)]; };
  auto gy = [&](int i, int j, int k) { return gv[IX(D, i, j, k)]; };
  LayerFaces mc = layer_faces(D, GF, fx, fy, ji, jk, 1), mn{};
  LayerFaces tc = layer_faces(D, GF, gx, gy, ji, jk, 1), tn{};
  float mh_prev = 0.f, th_prev = 0.f;
  for (int jl = 1; jl <= D.nl; ++jl) {
    const long long q = IX(D, ji, jk, jl);
    mn.h = 0.f;
    tn.h = 0.f;
    if (jl < D.nl || jl == D.nf) {
      mn = layer_faces(D, GF, fx, fy, ji, jk, jl + 1);
      tn = layer_faces(D, GF, gx, gy, ji, jk, jl + 1);
    }
    float heat = hd[q] + rad[q];           // dissipative, radiative heating
    if (pth) heat = heat + pth[q];         // phase transitions
    heat = heat + csh[q];                  // sediment heating
    if (tdh) heat = heat + tdh[q];         // temperature diffusion
    const float div_m = div_col(D, GF, X, mc, vert_faces(D, mh_prev, mc.h, mn.h, jl), ji, jk, jl);
    const float div_t = div_col(D, GF, X, tc, vert_faces(D, th_prev, tc.h, tn.h, jl), ji, jk, jl);
    float x = 0.f;
    if (heat != 0.f) {
      const float cv = c_v_mass_weighted_air<float>(D, Ss.rho, Tm, q);
      x = float(kC_D_V) * Ss.rho[q + goff] / cv * heat / (float(kC_D_P) * (GF.exner_bg[q] + Ss.ep[q]));
    }
    if (ptr) {  // phase transitions' vapour rate and mass diffusion of the gas
      const float mdg = mdt ? mdt[q + goff] : 0.f, ptg = ptr[q + goff];
      t_rho[q + goff] = -div_m + mdg + ptg;
      t_rt[q] = -div_t + x + (ptg + mdg) * (GF.theta_v_bg[q] + Ss.tp[q]);
    } else if (mdt) {  // mass diffusion of the gas, in its tendency and times theta_v in rho*theta_v's
      const float mdg = mdt[q + goff];
      t_rho[q + goff] = -div_m + mdg;
      t_rt[q] = -div_t + x + mdg * (GF.theta_v_bg[q] + Ss.tp[q]);
    } else {
      t_rho[q + goff] = -div_m;
      t_rt[q] = -div_t + x;
    }
    mh_prev = mc.h;
    th_prev = tc.h;
    mc = mn;
    tc = tn;
  }
}

// scalar_tend_expl for the tracers, mo_scalar_tend_expl.F90:24-104 (upstream fluxes,
// mo_scalar_tend_expl.F90:56-82; vertical upstream term with the contravariant correction,
// mo_averaging.F90:16-54), split step.  The velocity through each of the six faces of the
// cell, times the face area, and the index of the face's upwind cell are found once per
// cell; the tracer loop then only loads densities at known addresses, and every tracer's
// divergence is formed before the first tendency is stored, so no load waits on a velocity
// or on an earlier store.  The first substep (new weight 1) does not read the old tendency.
// Five resident blocks of 256 threads per SM (48 registers) ran 4 % faster than four.
constexpr int kTracers = 6;  // moist: five condensates and water vapour (the gas has its own kernel)
__global__ void __launch_bounds__(256, 5) ks_tracers(Dims D, Grid<float> GF, GridX X, StateF Ss, const float* u_new,
                                                     const float* v_new, float* t_rho, int rk_step,
                                                     const float* mdt, const float* ptr) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl);
  // horizontal faces: flux = rho(upwind cell) * velocity, 0 on a non-periodic boundary
  auto face_x = [&](int kf, float* a, long long* up) {
    int kk = kf, ka = kf - 1, kb = kf;
    if (kf < 2 || kf > D.nx) {
      if (!D.periodic) { *a = 0.f; *up = q; return; }
      kk = 1; ka = D.nx; kb = 1;
    }
    const float u = u_new[IX(D, ji, kk, jl)];
    *a = u * GF.area_x[IX(D, ji, kf, jl)];
    *up = IX(D, ji, (u >= 0.f) ? ka : kb, jl);
  };
  auto face_y = [&](int i_f, float* a, long long* up) {
    int ii = i_f, ia = i_f, ib = i_f - 1;
    if (i_f < 2 || i_f > D.ny) {
      if (!D.periodic) { *a = 0.f; *up = q; return; }
      ii = 1; ia = 1; ib = D.ny;
    }
    const float v = v_new[IX(D, ii, jk, jl)];
    *a = v * GF.area_y[IX(D, i_f, jk, jl)];
    *up = IX(D, (v >= 0.f) ? ia : ib, jk, jl);
  };
  float a_e, a_n, a_w, a_s, a_u = 0.f, a_l = 0.f;
  long long i_e, i_n, i_w, i_s, i_u = q, i_l = q;
  face_x(jk + 1, &a_e, &i_e);
  face_y(ji, &a_n, &i_n);
  face_x(jk, &a_w, &i_w);
  face_y(ji + 1, &a_s, &i_s);
  // vertical faces: the contravariant vertical velocity correction at the upper (jl) and
  // lower (jl+1) interface inside the terrain-following layers; the upwind cell by its sign
  auto wx = [&](int i, int j, int k) { return u_new[IX(D, i, j, k)]; };
  auto wy = [&](int i, int j, int k) { return v_new[IX(D, i, j, k)]; };
  // (the top terrain-following layer nf has only its lower face, the lowest layer nl only
  // its upper one, unless it is layer nf itself)
  if (jl > D.nf) {
    const float cu = vcc<float>(D, GF, wx, wy, ji, jk, jl);
    a_u = cu * GF.area_z[IX(D, ji, jk, jl)];
    i_u = (cu <= 0.f) ? IX(D, ji, jk, jl - 1) : q;
  }
  if (jl == D.nf || (jl > D.nf && jl < D.nl)) {
    const float cl = vcc<float>(D, GF, wx, wy, ji, jk, jl + 1);
    a_l = cl * GF.area_z[IX(D, ji, jk, jl + 1)];
    i_l = (cl <= 0.f) ? q : IX(D, ji, jk, jl + 1);
  }
  const float iv = X.inv_volume_f[q];
  float dv[kTracers];
#pragma unroll
  for (int t = 0; t < kTracers; ++t) {
    const int jc = t + 1 + (t + 1 >= D.g ? 1 : 0);
    const float* r = Ss.rho + (long long)(jc - 1) * D.fstride;
    const float comp = r[i_e] * a_e + r[i_n] * a_n - r[i_w] * a_w - r[i_s] * a_s + r[i_u] * a_u - r[i_l] * a_l;
    dv[t] = comp * iv;
  }
  if (mdt) {  // mass diffusion: -div + mass_diff_tendency
#pragma unroll
    for (int t = 0; t < kTracers; ++t) {
      const int jc = t + 1 + (t + 1 >= D.g ? 1 : 0);
      dv[t] = dv[t] - mdt[q + (long long)(jc - 1) * D.fstride];
    }
  }
  if (ptr) {  // phase transitions: the condensates' own rates, vapour's rate nc+1
#pragma unroll
    for (int t = 0; t < kTracers; ++t) {
      const int jc = t + 1 + (t + 1 >= D.g ? 1 : 0);
      dv[t] = dv[t] - ptr[q + (long long)((jc < D.g ? jc : D.g) - 1) * D.fstride];
    }
  }
  if (rk_step == 1) {
#pragma unroll
    for (int t = 0; t < kTracers; ++t) {
      const int jc = t + 1 + (t + 1 >= D.g ? 1 : 0);
      t_rho[q + (long long)(jc - 1) * D.fstride] = -dv[t];
    }
  } else {
    float o[kTracers];
#pragma unroll
    for (int t = 0; t < kTracers; ++t) {
      const int jc = t + 1 + (t + 1 >= D.g ? 1 : 0);
      o[t] = t_rho[q + (long long)(jc - 1) * D.fstride];
    }
#pragma unroll
    for (int t = 0; t < kTracers; ++t) {
      const int jc = t + 1 + (t + 1 >= D.g ? 1 : 0);
      t_rho[q + (long long)(jc - 1) * D.fstride] = 0.5f * o[t] - 0.5f * dv[t];
    }
  }
}

// the potential vorticity and its flux (calc_pot_vort, mo_vorticities.F90:189-421; vorticity
// flux, mo_vorticity_flux.F90:16-171) of the split step: the FP32 bodies of k_eta_xy, k_eta_z
// and k_vort_flux with register caps that keep six blocks of 256 threads resident
// eta_x, eta_y, eta_z and the mass flux densities (mo_vector_tend_expl.F90:64-66) in one
// launch: they read the same u, v, w and gas density around a point, which then come through
// the cache once
__global__ void __launch_bounds__(256, 6) ks_eta(Dims D, Grid<float> G, StateF S, float* ex, float* ey, float* ez,
                                                 float* uph, float* vph, float* wph) {
  LG_IDX3;
  if (jl > D.NL) return;
  if (ji <= D.ny + 1 && jk <= D.nx) ex[IX(D, ji, jk, jl)] = eta_x_at<float>(D, G, S, ji, jk, jl);
  if (ji <= D.ny && jk <= D.nx + 1) ey[IX(D, ji, jk, jl)] = eta_y_at<float>(D, G, S, ji, jk, jl);
  if (jl > D.nl) return;
  if (ji <= D.ny + 1 && jk <= D.nx + 1) ez[IX(D, ji, jk, jl)] = eta_z_at<float>(D, G, S, ji, jk, jl);
  const float* rg = S.rho + (long long)(D.g - 1) * D.fstride;
  if (ji <= D.ny && jk <= D.nx + 1) {
    float f;
    if (stv_h_x<float>(D, rg, S.u, ji, jk, jl, &f)) uph[IX(D, ji, jk, jl)] = f;
  }
  if (ji <= D.ny + 1 && jk <= D.nx) {
    float f;
    if (stv_h_y<float>(D, rg, S.v, ji, jk, jl, &f)) vph[IX(D, ji, jk, jl)] = f;
  }
  if (jl >= 2 && ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    wph[q] = 0.5f * (rg[IX(D, ji, jk, jl - 1)] + rg[q]) * S.w[q];
  }
}
__global__ void __launch_bounds__(256, 6) ks_vort_flux(Dims D, Grid<float> G, StateF S, const float* ex,
                                                       const float* ey, const float* ez, const float* uph,
                                                       const float* vph, const float* wph, float* px, float* py,
                                                       float* pz) {
  vort_flux_body<float, float>(D, G, S, ex, ey, ez, uph, vph, wph, px, py, pz);
}

// combination of the explicit wind tendencies, mo_vector_tend_expl.F90:258-310, and the
// forward step of the horizontal wind, mo_manage_pchevi.F90:86-89 (FP64 state), split step:
// the body of k_tend_wind<float> with the pressure-gradient terms of a background state read
// in the FP32 form ks_pgrad keeps for it (net nl + l and the previous substep's -(nl + l), the
// values k_tend_wind rounds to FP32 itself); without a background state the FP64 arrays.
// mu, mv: the FP32 mirrors of the new u, v.
__global__ void ks_tend_wind(Dims D, State So, State Sn, Tend<float> Tn, Carried<float> C, SplitCarriedF PF,
                             int rk_step, float* mu, float* mv) {
  LG_IDX3;
  const float new_weight = (rk_step == 2) ? 0.5f : 1.f;
  const float old_weight = 1.f - new_weight;
  const double chw_d = 0.5 + kIMPL_THERMO_WEIGHT, ohw_d = 1.0 - (0.5 + kIMPL_THERMO_WEIGHT);
  const double cvw_d = 1.0 - kIMPL_THERMO_WEIGHT, no_bg_d = D.luse_bg ? 0.0 : 1.0;
  auto pg_h = [&](const float* old_f, const float* net_f, const double* old, const double* nl, const double* l,
                  long long q) -> float {
    if (D.luse_bg) return float(ohw_d) * old_f[q] - float(chw_d) * net_f[q];
    return narrow(ohw_d * old[q] - chw_d * (nl[q] + l[q]));
  };
  if (jl <= D.nl && ji <= D.ny && jk <= D.nx + 1) {
    const long long q = IX(D, ji, jk, jl);
    float f = pg_h(PF.pold_u, PF.pnet_u, C.old_u, C.nl_u, C.l_u, q) - 0.5f * C.vsg_x[q] + C.pvt_x[q];
    if (C.mdt_x) f = f + C.mdt_x[q];
    const float t = old_weight * Tn.u[q] + new_weight * f;
    Tn.u[q] = t;
    const double un = So.u[q] + D.dtime * wide(t);
    Sn.u[q] = un;
    mu[q] = narrow(un);
  }
  if (jl <= D.nl && ji <= D.ny + 1 && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    float f = pg_h(PF.pold_v, PF.pnet_v, C.old_v, C.nl_v, C.l_v, q) - 0.5f * C.vsg_y[q] + C.pvt_y[q];
    if (C.mdt_y) f = f + C.mdt_y[q];
    const float t = old_weight * Tn.v[q] + new_weight * f;
    Tn.v[q] = t;
    const double vn = So.v[q] + D.dtime * wide(t);
    Sn.v[q] = vn;
    mv[q] = narrow(vn);
  }
  if (jl <= D.NL && ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    const float pg = D.luse_bg ? -(float(cvw_d) * PF.pnet_w[q])
                               : narrow(-(cvw_d * (C.nl_w[q] + C.l_w[q])) - no_bg_d * (1.0 - cvw_d) * C.l_w[q]);
    float f = pg - 0.5f * C.vsg_z[q] + C.pvt_z[q] + C.pgcw[q];
    if (C.mdt_z) f = f + C.mdt_z[q];
    Tn.w[q] = old_weight * Tn.w[q] + new_weight * f;
  }
}

// ---- three_band_solver_ver, mo_column_solvers.F90:21-351 --------------------------------
// The reference's implicit system for the vertical mass-flux increments at levels 2..nl,
// one thread per column, streamed top to bottom.  C = float (LGAME_PRECISION_SPLIT): from the
// FP32 mirror, the partial derivatives alpha, beta, gamma, the interface theta and density
// weights, the matrix and its elimination multipliers; FP64: the explicit predictions of theta'
// and exner', the right-hand side (where the pressure-gradient and buoyancy terms balance), the
// forward and back substitution, and the new rho_g, rho*theta_v, exner', w; theta' is formed as
// (rho*theta_v - theta_bg*rho)/rho with the small numerator in FP64.  C = double
// (LGAME_PRECISION_SPLIT_FP64_COLUMN): the same from the FP64 state, FP64 metric differences and
// reciprocals, with FP64 coefficients, multipliers and quotients -- the column solve wholly in
// FP64 (only the explicit tendencies it reads are FP32).
template <class C>
__global__ void __launch_bounds__(128, 6) ks_column_ver(Dims D, Grid<double> G, Grid<float> GF, GridX X, State So,
                                                     State Sn, StateF Mo, StateF Mn, Tend<float> Tn, int rk_step) {
  constexpr bool F64 = sizeof(C) == 8;
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const int nl = D.nl, n = nl - 1;
  const C dtf = C(D.dtime), idtf = C(1.0 / D.dtime);
  const double idtd = 1.0 / D.dtime;
  const long long goff = (long long)(D.g - 1) * D.fstride;
  const C rdcv = C(kR_D / kC_D_V);
  const C ic2 = C(1.0 / (kIMPL_THERMO_WEIGHT * (D.dtime * D.dtime) * kC_D_P));
  const C ic1 = C(1.0 / (kIMPL_THERMO_WEIGHT * D.dtime * kC_D_P));
  const StateF& Mu = (rk_step == 1) ? Mo : Mn;  // state_new_used, mo_column_solvers.F90:69-73
  const State& Su = (rk_step == 1) ? So : Sn;
  // the inputs of the coefficients, from the FP32 mirror or the FP64 state and metrics
  auto rho_o = [&](long long i) -> C { if constexpr (F64) return So.rho[goff + i]; else return Mo.rho[goff + i]; };
  auto rt_o = [&](long long i) -> C { if constexpr (F64) return So.rt[i]; else return Mo.rt[i]; };
  auto ep_o = [&](long long i) -> C { if constexpr (F64) return So.ep[i]; else return Mo.ep[i]; };
  auto rho_u = [&](long long i) -> C { if constexpr (F64) return Su.rho[goff + i]; else return Mu.rho[goff + i]; };
  auto rt_u = [&](long long i) -> C { if constexpr (F64) return Su.rt[i]; else return Mu.rt[i]; };
  auto ep_u = [&](long long i) -> C { if constexpr (F64) return Su.ep[i]; else return Mu.ep[i]; };
  auto w_o = [&](long long i) -> C { if constexpr (F64) return So.w[i]; else return Mo.w[i]; };
  auto ebg = [&](long long i) -> C { if constexpr (F64) return G.exner_bg[i]; else return GF.exner_bg[i]; };
  auto ivol = [&](long long i) -> C { if constexpr (F64) return X.inv_volume[i]; else return X.inv_volume_f[i]; };
  auto iarz = [&](long long i) -> C { if constexpr (F64) return X.inv_area_z[i]; else return X.inv_area_z_f[i]; };
  auto damp = [&](long long i) -> C { if constexpr (F64) return G.damp[i]; else return GF.damp[i]; };
  // at w level jl (2..nl): z_scalar(jl-1) - z_scalar(jl) and exner_bg(jl-1) - exner_bg(jl)
  auto dzs = [&](long long i) -> C {
    if constexpr (F64) return G.z_scalar[i - D.plane] - G.z_scalar[i]; else return X.dzs_f[i];
  };
  auto debg = [&](long long i) -> C {
    if constexpr (F64) return G.exner_bg[i - D.plane] - G.exner_bg[i]; else return X.deb_f[i];
  };
  auto W = [](C x) -> double { if constexpr (F64) return x; else return wide(x); };
  auto Nr = [](double x) -> float { return narrow(x); };
  auto quot = [](double x, C d) -> double { if constexpr (F64) return x / d; else return div_f(x, d); };

  // unscaled alpha, beta, gamma; theta of state_new_used (type C, and FP64 without a background
  // state, where theta * d(exner')/dz carries the whole hydrostatic balance)
  struct Lay { C a, b, g, th, ro, iv; double thd; };
  auto layer = [&](int jl) -> Lay {
    const long long i = IX(D, ji, jk, jl);
    Lay L;
    L.thd = D.luse_bg ? 0.0 : Su.rt[i] / Su.rho[goff + i];
    const C ro = rho_o(i), rto = rt_o(i);
    const C iro = C(1) / ro, irto = C(1) / rto;
    L.a = -rto * iro * iro;
    L.b = iro;
    L.g = rdcv * irto * (ebg(i) + ep_o(i));
    if (rk_step == 2) {
      const C ru = rho_u(i), rtu = rt_u(i);
      const C iru = C(1) / ru, irtu = C(1) / rtu;
      L.a = C(0.5) * (L.a - rtu * iru * iru);
      L.b = C(0.5) * (L.b + iru);
      L.g = C(0.5) * (L.g + rdcv * irtu * (ebg(i) + ep_u(i)));
      L.th = rtu * iru;
    } else {
      L.th = rto * iro;
    }
    L.ro = ro;
    L.iv = ivol(i);
    return L;
  };
  // explicit predictions of theta_v' and exner' (FP64 state plus increments) and of rho_g
  auto predict = [&](int jl, const Lay& L, double* tpe, double* epe, C* rhe) {
    const long long i = IX(D, ji, jk, jl);
    const C tr = C(Tn.rho[goff + i]), trt = C(Tn.rt[i]);
    *tpe = So.tp[i] + W(dtf * (L.a * tr + L.b * trt));
    *epe = So.ep[i] + W(dtf * L.g * trt);
    *rhe = L.ro + dtf * tr;
  };

  C epr[kMaxL + 1];       // elimination multipliers
  double rpr[kMaxL + 1];  // substituted right-hand side, then the solution (FP64)
  C tis[kMaxL + 1];       // interface theta
  C gs[kMaxL + 1];        // gamma of each layer
  Lay L0 = layer(1), L1 = layer(2), L2{};
  double tpe0, epe0, tpe1, epe1, tpe2 = 0.0, epe2 = 0.0;
  C rhe0, rhe1, rhe2 = C(0);
  predict(1, L0, &tpe0, &epe0, &rhe0);
  predict(2, L1, &tpe1, &epe1, &rhe1);
  gs[1] = L0.g;
  C cv_prev = C(0), epr_prev = C(0);
  double rpr_prev = 0.0;
  for (int jl = 1; jl <= n; ++jl) {  // row jl: level jl+1 between layers jl (a) and jl+1 (b)
    const long long ib = IX(D, ji, jk, jl + 1);
    gs[jl + 1] = L1.g;
    const C ti = C(0.5) * (L0.th + L1.th);
    tis[jl] = ti;
    const C irio = C(2) / (L0.ro + L1.ro);
    const C dz = dzs(ib), deb = debg(ib), dp = damp(ib);
    const double wo = So.w[ib];
    const C wof = w_o(ib);
    const C al0 = L0.a * L0.iv, al1 = L1.a * L1.iv, be0 = L0.b * L0.iv, be1 = L1.b * L1.iv;
    const C ga0 = L0.g * L0.iv, ga1 = L1.g * L1.iv;
    const C dv = -(ti * ti) * (ga0 + ga1) + C(0.5) * deb * (al1 - al0 + ti * (be1 - be0))
                 - dz * ic2 * irio * (C(2) * iarz(ib) + dtf * wof * C(0.5) * (L1.iv - L0.iv)) * dp;
    const C rie = C(0.5) * (rhe0 + rhe1);
    // The products of FP32 coefficients with FP64 values here and in the state update below
    // stay FP64 products of the FP32 factors: merging two FP32 factors into one rounded
    // coefficient (e.g. -dz*ic2*(1 + rie*irio) for w_old) saves two FP64 operations per cell
    // but lets an atmosphere at rest over hills drift about four times faster (1e-8 instead
    // of 3e-9 m/s of spurious wind after 3 h at 256 x 256 x 50).
    double rv = (wo + W(dtf * C(Tn.w[ib]))) * W(-dz * ic2);
    rv = fma(D.luse_bg ? W(ti * idtf) : 0.5 * (L0.thd + L1.thd) * idtd, epe0 - epe1, rv);
    rv = fma(W(C(0.5) * idtf * deb), tpe0 + tpe1, rv);
    rv = fma(W(-dz * ic2 * rie * irio), wo, rv);
    // couplings with row jl+1 (layer b's derivatives), which need layer jl+2
    C cv = C(0), ev = C(0);
    if (jl < n) {
      L2 = layer(jl + 2);
      predict(jl + 2, L2, &tpe2, &epe2, &rhe2);
      const long long ic = IX(D, ji, jk, jl + 2);
      const C ti_n = C(0.5) * (L1.th + L2.th);
      const C irio_n = C(2) / (L1.ro + L2.ro);
      cv = ti_n * ga1 * ti + C(0.5) * debg(ic) * (al1 + be1 * ti)
           - dzs(ic) * ic1 * C(0.5) * w_o(ic) * L1.iv * irio_n * damp(ic);
      ev = ti * ga1 * ti_n - C(0.5) * deb * (al1 + be1 * ti_n) + dz * ic1 * C(0.5) * wof * L1.iv * irio * dp;
    }
    const C piv = dv - epr_prev * cv_prev;
    const double x = (jl == 1) ? rv : fma(-W(cv_prev), rpr_prev, rv);
    rpr_prev = quot(x, piv);
    rpr[jl] = rpr_prev;
    epr_prev = ev / piv;
    epr[jl] = epr_prev;
    cv_prev = cv;
    L0 = L1; L1 = L2;
    tpe0 = tpe1; epe0 = epe1; rhe0 = rhe1;
    tpe1 = tpe2; epe1 = epe2; rhe1 = rhe2;
  }
  // back substitution fused with the new state, mo_column_solvers.F90:300-345, bottom to top:
  // layer jl needs the solutions of the rows above (w level jl) and below it (w level jl+1),
  // and w at level jl+1 the new densities of layers jl and jl+1, all known once the
  // substitution has reached row jl-1.  The inputs of the layer above are loaded before the
  // current layer's results are stored (a store may alias a later load, which stops the
  // compiler from moving the loads itself).
  struct StateIn { double rt, rho, ep, bg, w; C ivf, iaz, mro; float trho, trt; };
  auto state_in = [&](int m) {
    StateIn r;
    const long long p = IX(D, ji, jk, m);
    r.rt = So.rt[p];
    r.rho = So.rho[goff + p];
    r.ep = So.ep[p];
    r.bg = G.theta_v_bg[p];
    r.w = So.w[p];
    r.ivf = ivol(p);
    r.iaz = iarz(p);
    r.mro = rho_o(p);
    r.trho = Tn.rho[goff + p];
    r.trt = Tn.rt[p];
    return r;
  };
  StateIn in_cur = state_in(nl), in_up{}, in_below{};
  double s1 = 0.0;     // solution at the interface below the layer (w level jl+1)
  C rnf_below = C(0);  // new rho_g of the layer below (FP32: rounded)
  for (int jl = nl; jl >= 1; --jl) {
    if (jl > 1) in_up = state_in(jl - 1);
    const long long i = IX(D, ji, jk, jl);
    // solution of row jl-1 (w level jl), the interface above the layer
    double s0 = 0.0;
    if (jl >= 2) s0 = (jl - 1 == n) ? rpr[n] : fma(-W(epr[jl - 1]), s1, rpr[jl - 1]);
    const C t0 = (jl >= 2) ? tis[jl - 1] : C(0);
    const C t1 = (jl <= n) ? tis[jl] : C(0);
    const double dtv = W(dtf * in_cur.ivf);
    const double rto = in_cur.rt;
    const double rho_e = in_cur.rho + W(dtf * C(in_cur.trho));
    const double rt_e = rto + W(dtf * C(in_cur.trt));
    const double rn = fma(dtv, s1 - s0, rho_e);
    const double rtn = fma(dtv, fma(-W(t0), s0, W(t1) * s1), rt_e);
    const double epn = fma(W(gs[jl]), rtn - rto, in_cur.ep);
    const float rnf = Nr(rn);
    const C rnc = F64 ? C(rn) : C(rnf);
    if constexpr (F64) {
      const double tpn = fma(-in_cur.bg, rn, rtn) / rn;
      Sn.tp[i] = tpn;
      Mn.tp[i] = Nr(tpn);
    } else {
      const float tpf = narrow(fma(-in_cur.bg, rn, rtn)) / rnf;
      Sn.tp[i] = wide(tpf);
      Mn.tp[i] = tpf;
    }
    Sn.rho[goff + i] = rn;
    Sn.rt[i] = rtn;
    Sn.ep[i] = epn;
    Mn.rho[goff + i] = rnf;
    Mn.rt[i] = Nr(rtn);
    Mn.ep[i] = Nr(epn);
    if (jl <= n) {  // w at level jl+1 from the increment there, between this layer and the one below
      const long long ib = i + D.plane;
      const C rin = C(0.5) * (rnc + rnf_below);
      const C irio = C(2) / (in_cur.mro + in_below.mro);
      const double wn = fma(-W(rin), in_below.w, W(C(2) * in_below.iaz) * s1) * W(irio);
      Sn.w[ib] = wn;
      Mn.w[ib] = Nr(wn);
    }
    s1 = s0;
    rnf_below = rnc;
    in_below = in_cur;
    in_cur = in_up;
  }
  if (D.freeslip) {  // w_free_slip, mo_inner_product.F90:52-75, with the new u, v
    const int m = nl;
    const double wf =
        G.ipw[0][IX(D, ji, jk, m)] * Sn.u[IX(D, ji, jk + 1, m)] * G.slope_x[IX(D, ji, jk + 1, m)]
      + G.ipw[1][IX(D, ji, jk, m)] * Sn.v[IX(D, ji, jk, m)] * G.slope_y[IX(D, ji, jk, m)]
      + G.ipw[2][IX(D, ji, jk, m)] * Sn.u[IX(D, ji, jk, m)] * G.slope_x[IX(D, ji, jk, m)]
      + G.ipw[3][IX(D, ji, jk, m)] * Sn.v[IX(D, ji + 1, jk, m)] * G.slope_y[IX(D, ji + 1, jk, m)];
    Sn.w[IX(D, ji, jk, m + 1)] = wf;
    Mn.w[IX(D, ji, jk, m + 1)] = narrow(wf);
  }
}

// ---- three_band_solver_gen_densities, mo_column_solvers.F90:353-604 ----------------------
// The reference's system per (column, tracer)  d_l s_l + e_l s_{l+1} + c_{l-1} s_{l-1} = rho_l + inc_l
// (implicit-upwind vertical flux and sedimentation, inc = dt*tendency + explicit flux part) is
// solved for the increment delta = s - rho_old:
//   d_l delta_l + e_l delta_{l+1} + c_{l-1} delta_{l-1} = inc_l - (d_l - 1) rho_l - e_l rho_{l+1} - c_{l-1} rho_{l-1}
// in FP32 (coefficients from the mirror; the right-hand side's rounding is then relative to the
// flux terms, the size of delta, and not to the density), and the new density rho_old + delta
// is formed in FP64.  d - 1 is accumulated on its own, so the diagonal's rounding near 1 does
// not enter.  Each interface couples its two cells in one direction only (the upwind side:
// e_l = 0 or c_l = 0), so Thomas's pivots are the diagonal entries themselves and its sweeps
// are the affine recurrences
//   forward   r_l     = alpha_l r_{l-1} + beta_l,     alpha_l = -c_{l-1}/d_l, beta_l = rhs_l/d_l
//   backward  delta_l = r_l - e'_l delta_{l+1},        e'_l = e_l/d_l.
//
// A block owns 32 columns (a row tile, one per lane) and three tracers, in three phases:
//   1. the eight warps take contiguous chunks of levels (ten at 80 layers); a thread walks its
//      chunk top down and forms alpha, beta, e' of the three tracers into shared memory, and the
//      sediment heating.  What the three tracers share -- volume, area, old and new w,
//      temperature and heat capacities at each interface, the cloud droplets' fall speed -- is
//      loaded and formed once, the values of the interface below a level are carried to the next
//      level as the interface above it, and inputs are loaded two levels ahead;
//   2. three warps run the two sweeps of one tracer each, a lane per column, from shared memory
//      (no memory latency in the level chain), while the old FP64 densities of phase 3 arrive;
//   3. the chunks again: rho_old + delta in FP64, clipped (mo_column_solvers.F90:587-591), and
//      its rounded mirror.
// The elimination data never leave the chip: as a per-thread local stack (one thread per column
// and tracer walking all levels) they spilled through L2 to DRAM, 321 bytes per cell moved
// against 202.  The two blocks of a row tile are consecutive in the grid and read the tile's
// shared inputs once from DRAM.  A condensate's sediment heating goes to its own plane of
// csh_part (rk_step 1 only, FP32 heat capacities); ks_csh_sum adds the planes in order.
constexpr int kTrWarps = 8;   // level chunks in phases 1 and 3
constexpr int kTrSet = 3;     // tracers per block
constexpr int kTrPitch = 33;  // shared-memory row pitch (32 columns + 1)
constexpr int kTrPre = 10;    // levels per thread whose old densities are loaded before the sweeps
constexpr int kTrRow = 3 * kTrSet * kTrPitch;  // shared-memory floats per level

// inputs of one level m of a column for the three tracers of a block: the tracers' old mirror
// densities and tendencies, and at the interface above the level (w level m) area, old and
// new w; the level's 1/volume and temperature; for the cloud droplets' fall speed (second set
// only) the gas density, gravity at w levels m and m+1 and the two vertical weights
struct TrLevel { float ro[kTrSet], tr[kTrSet], az, wo, wn, iv, tm, rg, gm, gm1, w5, w6; };

// v_fall_liquid, mo_derived.F90:218-263, in FP32, at level m from its prefetched inputs
__device__ __forceinline__ float vfall_liquid_l(const TrLevel& L, float radius, int m, int nl) {
  const float g = (m == 1) ? L.gm1 : (m == nl) ? L.gm : L.w5 * L.gm + L.w6 * L.gm1;
  const float rg = L.rg;
  const float pm = float(kM_D / kN_A);
  const float tv = sqrtf(8.f * float(kK_B) / (float(kPI) * pm) * L.tm);
  const float mfp = 1.f / (1.41421356f * (rg / pm) * (4.f * float(kPI) * (130e-12f * 130e-12f)));
  const float nu = (1.f / 3.f) * tv * mfp;
  float v = 2.f * (radius * radius) * (float(kRHO_H2O) - rg) * g / (9.f * rg * nu);
  if (v * radius / nu > 10.f) v = sqrtf(8.f * radius * float(kRHO_H2O) * g / (3.f * rg * 0.8f));
  return v;
}

// properties of the block's tracers, fixed at compile time (the split path runs the moist
// constituent layout: 1 snow, 2 rain, 3 cloud ice, 4 cloud water, 5 graupel, 6 gas, 7 vapour):
// constituent index, condensate or not, ice or water heat capacity (odd constituents are ice,
// mo_dictionary.F90:175-189), fall speed (snow 1 m/s: radius 500 um above 250 um; cloud ice
// 0.001 m/s; cloud water v_fall_liquid at radius 12 um; rain, graupel and vapour 0, their
// radius never being set), and whether the surface sink's heat term applies (jc > nc/4)
template <int SET>
struct TrSet {
  __device__ static constexpr int jc(int q) { return SET == 0 ? q + 1 : (q == 2 ? 7 : q + 4); }
  __device__ static constexpr bool cond(int q) { return jc(q) <= 5; }
  __device__ static constexpr bool ice(int q) { return (jc(q) - 1) % 2 == 0; }
  __device__ static constexpr bool cloud(int q) { return jc(q) == 4; }
  __device__ static constexpr float vfix(int q) { return jc(q) == 1 ? 1.f : jc(q) == 3 ? 0.001f : 0.f; }
  __device__ static constexpr bool sfc_heat(int q) { return jc(q) > 1; }  // jc > nc/4 = 1
};

// One block: phases 1-3 above for tracer set SET; HEAT: the first substep, which also stores
// the sediment heating.  Shared memory [level-1][tracer q][alpha, beta, e'][33]: the nine values
// of a level sit at fixed offsets from one row address.
template <int SET, bool HEAT>
__device__ __forceinline__ void tracer_block(const Dims& D, const Grid<float>& GF, const GridX& X, const State& So,
                                             const State& Sn, const StateF& Mo, const StateF& Mn,
                                             const float* t_rho_all, const float* Tm, float* csh_part, float* sm) {
  using P = TrSet<SET>;
  const int nl = D.nl;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ji = blockIdx.y * 32 + lane + 1;
  const int jk = blockIdx.z + 1;
  const bool valid = ji <= D.ny;
  const float dt = float(D.dtime);
  const float itw = 0.5f, ew = 0.5f;
  const int pl = (int)D.plane;  // level stride; fstride*ncons < 2^31 for every supported grid
  // 32-bit element indices off the arrays' base addresses, which stay kernel parameters: level
  // jl of tracer q is at tq[q] + (jl-1)*pl
  const int c32 = (int)IX(D, valid ? ji : 1, jk, 1);
  int tq[kTrSet];
#pragma unroll
  for (int q = 0; q < kTrSet; ++q) tq[q] = (P::jc(q) - 1) * (int)D.fstride + c32;
  const int grg = (D.g - 1) * (int)D.fstride + c32;
  const int chunk = (nl + kTrWarps - 1) / kTrWarps;
  const int l0 = w * chunk + 1, l1 = min(nl, (w + 1) * chunk);
  auto load = [&](int m, TrLevel& L) {
    const int o = (m - 1) * pl;
#pragma unroll
    for (int q = 0; q < kTrSet; ++q) {
      L.ro[q] = Mo.rho[tq[q] + o];
      L.tr[q] = t_rho_all[tq[q] + o];
    }
    const int e = c32 + o;
    L.az = GF.area_z[e];
    L.wo = Mo.w[e];
    L.wn = Mn.w[e];
    L.iv = X.inv_volume_f[e];
    if (HEAT || SET == 1) L.tm = Tm[e];
    if (SET == 1) {
      L.rg = Mo.rho[grg + o];
      L.gm = GF.gm[e];
      L.gm1 = GF.gm[e + pl];
      L.w5 = GF.ipw[4][e];
      L.w6 = GF.ipw[5][e];
    }
  };
  auto vf_of = [&](int q, float vcl) -> float { return P::cloud(q) ? vcl : P::vfix(q); };
  auto cp_t = [&](int q, float tm) -> float { return (P::ice(q) ? c_p_ice(tm) : c_p_water(tm)) * tm; };
  // ---- phase 1: coefficients, a thread walking its chunk of levels ----------------------------
  // ring of level inputs: level jl in slot k, jl+1 in k+1, jl+2 and jl+3 loading (two levels of
  // look-ahead: the interface below level jl+1 needs level jl+2 in the next iteration)
  if (valid && l0 <= l1) {
    TrLevel ring[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) ring[k] = TrLevel{};
    load(l0, ring[0]);
    if (l0 + 1 <= nl) load(l0 + 1, ring[1]);
    if (l0 + 2 <= min(l1 + 1, nl)) load(l0 + 2, ring[2]);
    // carried from the interface above the current level: flux coefficient, flux, heat flux of
    // each tracer, the densities of the level above, and the cloud droplets' fall speed at the
    // current level
    float vfi_up[kTrSet], vfr_up[kTrSet], vefv_up[kTrSet], ro_up[kTrSet];
    float vcl_cur = (SET == 1) ? vfall_liquid_l(ring[0], 12.e-6f, l0, nl) : 0.f;
#pragma unroll
    for (int q = 0; q < kTrSet; ++q) vfi_up[q] = vfr_up[q] = vefv_up[q] = ro_up[q] = 0.f;
    if (l0 >= 2) {  // the interface above the chunk's first level, formed from scratch
      TrLevel up{};
      load(l0 - 1, up);
      const TrLevel& cur = ring[0];
      const float vcl_i = (SET == 1) ? 0.5f * (vfall_liquid_l(up, 12.e-6f, l0 - 1, nl) + vcl_cur) : 0.f;
#pragma unroll
      for (int q = 0; q < kTrSet; ++q) {
        const float vf = vf_of(q, vcl_i);
        vfi_up[q] = cur.az * (cur.wo - vf);
        float fr = cur.az * (cur.wn - vf);
        fr = ((fr >= 0.f) ? cur.ro[q] : up.ro[q]) * fr;
        vfr_up[q] = fr;
        if (HEAT && P::cond(q)) vefv_up[q] = cp_t(q, cur.tm) * fr;
        ro_up[q] = up.ro[q];
      }
    }
    for (int base = l0; base <= l1; base += 4) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int jl = base + k;
        if (jl > l1) break;
        if (jl + 3 <= min(l1 + 1, nl)) load(jl + 3, ring[(k + 3) % 4]);
        const TrLevel& cur = ring[k];
        const TrLevel& nxt = ring[(k + 1) % 4];
        const int o = (jl - 1) * pl;
        const float iv = cur.iv;
        const float itv_a = itw * dt * iv;
        const bool below = jl <= nl - 1;
        // shared parts of the interface below the level (w level jl+1)
        float vcl_b = 0.f, vcl_i = 0.f;
        if (SET == 1 && below) {
          vcl_b = vfall_liquid_l(nxt, 12.e-6f, jl + 1, nl);
          vcl_i = 0.5f * (vcl_cur + vcl_b);
        }
        const float az_sfc = (jl == nl) ? GF.area_z[c32 + o + pl] : 0.f;
        float* row = sm + (jl - 1) * kTrRow + lane;
#pragma unroll
        for (int q = 0; q < kTrSet; ++q) {
          const float ro = cur.ro[q];
          float vfi = 0.f, vfr = 0.f, vefv = 0.f, ro_dn = 0.f;
          if (below) {
            const float vf = vf_of(q, vcl_i);
            ro_dn = nxt.ro[q];
            vfi = nxt.az * (nxt.wo - vf);
            float fr = nxt.az * (nxt.wn - vf);
            fr = ((fr >= 0.f) ? ro_dn : ro) * fr;
            vfr = fr;
            if (HEAT && P::cond(q)) vefv = cp_t(q, nxt.tm) * fr;
          }
          // d - 1, explicit flux part and sediment heating of cell jl
          float dm1, fl, h = 0.f;
          if (jl == 1) {
            dm1 = (vfi >= 0.f) ? 0.f : -itv_a * vfi;
            fl = ew * dt * vfr * iv;
            h = vefv * iv;
          } else if (jl == nl) {
            dm1 = (vfi_up[q] >= 0.f) ? itv_a * vfi_up[q] : 0.f;
            fl = -ew * dt * vfr_up[q] * iv;
            h = -vefv_up[q] * iv;
            if (P::cond(q)) {
              const float vsurf = vf_of(q, vcl_cur);  // the lowest layer's own fall speed
              dm1 += itw * vsurf * dt * az_sfc * iv;
              fl -= ew * vsurf * dt * ro * az_sfc * iv;
              if (HEAT && P::sfc_heat(q)) {
                const float tn = cur.tm;
                h -= vsurf * tn * (P::ice(q) ? c_p_ice(tn) : c_p_water(tn)) * ro * az_sfc * iv;
              }
            }
          } else {
            dm1 = 0.f;
            if (vfi_up[q] >= 0.f) dm1 += itv_a * vfi_up[q];
            if (vfi < 0.f) dm1 -= itv_a * vfi;
            fl = ew * dt * (vfr - vfr_up[q]) * iv;
            h = (vefv - vefv_up[q]) * iv;
          }
          if (HEAT && P::cond(q)) csh_part[tq[q] + o] = h;
          // couplings: row jl to jl+1 (upward flux below), row jl to jl-1 (downward flux above);
          // the pivot is the diagonal 1 + (d - 1)
          const float ev = (below && vfi >= 0.f) ? -(itv_a * vfi) : 0.f;
          const float cv_up = (jl >= 2 && vfi_up[q] < 0.f) ? itv_a * vfi_up[q] : 0.f;
          const float rhs = (dt * cur.tr[q] + fl) - dm1 * ro - ev * ro_dn - cv_up * ro_up[q];
          const float ip = 1.f / (1.f + dm1);
          row[(3 * q + 0) * kTrPitch] = -cv_up * ip;
          row[(3 * q + 1) * kTrPitch] = rhs * ip;
          row[(3 * q + 2) * kTrPitch] = ev * ip;
          vfi_up[q] = vfi;
          vfr_up[q] = vfr;
          vefv_up[q] = vefv;
          ro_up[q] = ro;
        }
        vcl_cur = vcl_b;
      }
    }
  }
  // the old FP64 densities of phase 3, loaded before the sweeps so that they arrive meanwhile
  // (the registers of phase 1 are free by now); chunks longer than kTrPre levels load the rest
  // in phase 3
  double rq[kTrPre][kTrSet];
#pragma unroll
  for (int k = 0; k < kTrPre; ++k)
#pragma unroll
    for (int q = 0; q < kTrSet; ++q) rq[k][q] = (valid && l0 + k <= l1) ? So.rho[tq[q] + (l0 + k - 1) * pl] : 0.0;
  __syncthreads();
  // ---- phase 2: the sweeps, warp q for tracer q, a lane per column -----------------------------
  if (w < kTrSet) {
    float* row = sm + lane + 3 * w * kTrPitch;
    float r = 0.f;
#pragma unroll 4
    for (int jl = 1; jl <= nl; ++jl, row += kTrRow) {
      r = row[0] * r + row[kTrPitch];
      row[kTrPitch] = r;
    }
    float dl = 0.f;
#pragma unroll 4
    for (int jl = nl; jl >= 1; --jl) {
      row -= kTrRow;
      dl = row[kTrPitch] - row[2 * kTrPitch] * dl;
      row[kTrPitch] = dl;
    }
  }
  __syncthreads();
  // ---- phase 3: new densities rho_old + delta (FP64), clipped, and their mirror ---------------
  if (!valid || l0 > l1) return;
  // the mirror is rounded by the hardware conversion here (the bits of narrow() in one issue
  // slot): the FP64 pipe carries only this and the addition per value, against a dozen integer
  // operations for narrow()
  auto update = [&](int jl, int q, double ro_old) {
    const int e = tq[q] + (jl - 1) * pl;
    const double sn = ro_old + wide(sm[(jl - 1) * kTrRow + lane + (3 * q + 1) * kTrPitch]);
    const double v = __double2hiint(sn) < 0 ? 0.0 : sn;
    Sn.rho[e] = v;
    Mn.rho[e] = __double2float_rn(v);
  };
#pragma unroll
  for (int k = 0; k < kTrPre; ++k)
#pragma unroll
    for (int q = 0; q < kTrSet; ++q)
      if (l0 + k <= l1) update(l0 + k, q, rq[k][q]);
  for (int jl = l0 + kTrPre; jl <= l1; ++jl)
#pragma unroll
    for (int q = 0; q < kTrSet; ++q) update(jl, q, So.rho[tq[q] + (jl - 1) * pl]);
}

// grid (2 tracer sets, row tiles, nx), 256 threads, dynamic shared memory tracer_smem(D);
// HEAT: the first substep
template <bool HEAT>
__global__ void __launch_bounds__(kTrWarps * 32, 2) ks_column_tracers(Dims D, Grid<float> GF, GridX X, State So,
                                                                      State Sn, StateF Mo, StateF Mn,
                                                                      const float* t_rho_all, const float* Tm,
                                                                      float* csh_part) {
  extern __shared__ float sm[];
  if (blockIdx.x == 0) tracer_block<0, HEAT>(D, GF, X, So, Sn, Mo, Mn, t_rho_all, Tm, csh_part, sm);
  else tracer_block<1, HEAT>(D, GF, X, So, Sn, Mo, Mn, t_rho_all, Tm, csh_part, sm);
}

// sediment heating of all condensates: the per-condensate planes of ks_column_tracers added
// in condensate order (the order of the reference's accumulation over jc)
__global__ void ks_csh_sum(Dims D, const float* csh_part, float* csh) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl);
  float h = 0.f;
  for (int jc = 0; jc < D.nc; ++jc) h += csh_part[q + (long long)jc * D.fstride];
  csh[q] = h;
}

// dynamic shared memory of ks_column_tracers: alpha, beta and e' of three tracers, 32 columns
size_t tracer_smem(const Dims& D) { return (size_t)D.nl * kTrRow * sizeof(float); }

dim3 sblk() { return dim3(32, 8, 1); }
// x: row tiles, y: levels, z: column tiles (see LG_IDX3)
dim3 sgrd(int rows, int cols, int levs) {
  return dim3((unsigned)((rows + 31) / 32), (unsigned)levs, (unsigned)((cols + 7) / 8));
}
// column kernels: 128 threads, 32 rows x 4 columns
dim3 cblk() { return dim3(32, 4, 1); }
dim3 cgrd(int rows, int cols) { return dim3((unsigned)((rows + 31) / 32), (unsigned)((cols + 3) / 4), 1u); }

}  // namespace

int split_create(const Dims& D, bool column_fp64, const SplitDiff& diff, const SplitSfc& sfc, SplitCtx** out,
                 long long* bytes) {
  if (D.ncons > 1 && D.ncons != kTracers + 1) {
    lgame_set_error("split precision: the tracer kernel is built for five condensates and water vapour");
    return LGAME_ERR_UNSUPPORTED;
  }
  if (D.ncons > 1 &&
      (D.nl > 128 ||
       cudaFuncSetAttribute(ks_column_tracers<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)tracer_smem(D)) != cudaSuccess ||
       cudaFuncSetAttribute(ks_column_tracers<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)tracer_smem(D)) != cudaSuccess)) {
    lgame_set_error("split precision: the tracer solver supports at most 128 layers");
    return LGAME_ERR_UNSUPPORTED;
  }
  if (diff.mom_h &&
      (cudaFuncSetAttribute(k_diff_scalar_col<7, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)diff_scalar_smem(8)) != cudaSuccess ||
       cudaFuncSetAttribute(k_diff_scalar_col<7, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)diff_scalar_smem(7)) != cudaSuccess)) {
    lgame_set_error("split precision: shared memory of the scalar diffusion kernel refused");
    return LGAME_ERR_CUDA;
  }
  auto* s = new SplitCtx();
  s->column_fp64 = column_fp64;
  const size_t F = (size_t)D.fstride;
  int rc = LGAME_OK;
  auto fail = [&](int code) { split_destroy(s); *out = nullptr; return code; };
  for (int k = 0; k < 40; ++k) if ((rc = salloc(s, &s->gf[k], F, bytes))) return fail(rc);
  for (int k = 0; k < 6; ++k) if ((rc = salloc(s, &s->ipw[k], F, bytes))) return fail(rc);
  for (int k = 0; k < 3; ++k) if ((rc = salloc(s, &s->trsk_u[k], (size_t)D.P, bytes))) return fail(rc);
  for (int k = 0; k < 2; ++k) if ((rc = salloc(s, &s->trsk_v[k], (size_t)D.P, bytes))) return fail(rc);
  if ((rc = salloc(s, &s->inv_dx, F, bytes)) || (rc = salloc(s, &s->inv_dy, F, bytes)) ||
      (rc = salloc(s, &s->inv_dz, F, bytes)) || (rc = salloc(s, &s->inv_volume, F, bytes)) ||
      (rc = salloc(s, &s->inv_area_z, F, bytes)))
    return fail(rc);
  float** scratch[] = {&s->gx, &s->gy, &s->gz, &s->divf, &s->tvu, &s->tvv, &s->tpu, &s->tpv,
                       &s->ex, &s->ey, &s->ez, &s->uph, &s->vph, &s->wph};
  for (float** p : scratch) if ((rc = salloc(s, p, F, bytes))) return fail(rc);
  s->sfc = sfc;
  if (sfc.vsq) s->vsq = sfc.vsq;
  else if ((rc = salloc(s, &s->vsq, F, bytes))) return fail(rc);
  if ((rc = salloc(s, &s->gzd, F, bytes)) || (rc = salloc(s, &s->rmz, F, bytes))) return fail(rc);
  if (D.nc > 0 && (rc = salloc(s, &s->csh_part, F * D.nc, bytes))) return fail(rc);
  if ((rc = salloc(s, &s->dbg, F, bytes)) || (rc = salloc(s, &s->tbu, F, bytes)) || (rc = salloc(s, &s->tbv, F, bytes)))
    return fail(rc);
  float** fl[] = {&s->fu, &s->fv, &s->gu, &s->gv};
  for (float** p : fl) if ((rc = salloc(s, p, F, bytes))) return fail(rc);
  for (int k = 0; k < 2; ++k) {
    StateF& M = s->mir[k];
    if ((rc = salloc(s, &M.rho, F * D.ncons, bytes))) return fail(rc);
    float** mf[] = {&M.rt, &M.tp, &M.ep, &M.u, &M.v, &M.w};
    for (float** p : mf) if ((rc = salloc(s, p, F, bytes))) return fail(rc);
  }
  SplitCarriedF& C = s->C;
  float** car[] = {&C.pgcw, &C.vsg_x, &C.vsg_y, &C.vsg_z, &C.pvt_x, &C.pvt_y, &C.pvt_z, &C.csh, &C.rad, &C.temperature,
                   &C.hdiss,
                   &C.tend.rt, &C.tend.u, &C.tend.v, &C.tend.w, &C.pnet_u, &C.pnet_v, &C.pnet_w, &C.pold_u,
                   &C.pold_v};
  for (float** p : car) if ((rc = salloc(s, p, F, bytes))) return fail(rc);
  if ((rc = salloc(s, &C.tend.rho, F * D.ncons, bytes))) return fail(rc);
  s->diff = diff;
  if (diff.mom_h) {
    DiffBuf<float>& B = s->db;
    float** dfl[] = {&C.tke, &C.visc, &C.mdtx, &C.mdty, &C.mdtz, &B.tke_new, &B.vmol, &B.nsq, &B.vz, &B.tdh,
                     &B.zz, &B.vdiv};
    for (float** p : dfl) if ((rc = salloc(s, p, F, bytes))) return fail(rc);
    if ((rc = salloc(s, &B.mdt, F * D.ncons, bytes))) return fail(rc);
    // (no flux density arrays: the scalar diffusion forms its faces in shared memory)
    B.tke = C.tke; B.visc = C.visc; B.mdtx = C.mdtx; B.mdty = C.mdty; B.mdtz = C.mdtz; B.hd = C.hdiss;
    C.tdh = B.tdh; C.mdt = B.mdt;
  }
  if (sfc.phase) {  // the phase transitions' rates (graupel's is never written: stays zero) and heating
    if ((rc = salloc(s, &C.ptr, F * (size_t)(D.nc + 1), bytes)) || (rc = salloc(s, &C.pth, F, bytes))) return fail(rc);
  }
  for (cudaStream_t& b : s->br)
    if (cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking) != cudaSuccess) {
      lgame_set_error("split precision: cudaStreamCreate failed");
      return fail(LGAME_ERR_CUDA);
    }
  for (cudaEvent_t& e : s->ev)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      lgame_set_error("split precision: cudaEventCreate failed");
      return fail(LGAME_ERR_CUDA);
    }
  *out = s;
  return LGAME_OK;
}

void split_set_diff_par(SplitCtx* s, const DiffPar& par) { s->diff.par = par; }
void split_set_sfc_par(SplitCtx* s, const SfcPar& par) { s->sfc.par = par; }

void split_destroy(SplitCtx* s) {
  if (!s) return;
  for (void* p : s->allocs) cudaFree(p);
  for (cudaEvent_t e : s->ev) if (e) cudaEventDestroy(e);
  for (cudaStream_t b : s->br) if (b) cudaStreamDestroy(b);
  delete s;
}

SplitCarriedF split_carried(SplitCtx* s) { return s->C; }
StateF split_mirror(SplitCtx* s, int slot) { return s->mir[slot]; }

int split_net(const double* a, const double* b, float* net, long long n, cudaStream_t stream) {
  k_net<<<1216, 256, 0, stream>>>(a, b, net, n);
  return cudaGetLastError() == cudaSuccess ? LGAME_OK : LGAME_ERR_CUDA;
}

int split_convert(const double* src, float* dst, long long n, cudaStream_t stream) {
  k_to_float<<<1216, 256, 0, stream>>>(src, dst, n);
  return cudaGetLastError() == cudaSuccess ? LGAME_OK : LGAME_ERR_CUDA;
}
int split_convert_back(const float* src, double* dst, long long n, cudaStream_t stream) {
  k_to_double<<<1216, 256, 0, stream>>>(src, dst, n);
  return cudaGetLastError() == cudaSuccess ? LGAME_OK : LGAME_ERR_CUDA;
}

// ---- lateral boundary relaxation (mo_boundaries.F90:19-97) in split precision -------------
namespace {
__global__ void k_rtbg(const double* exner_bg, double* rtbg, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    rtbg[i] = kP_0 / kR_D * pow(exner_bg[i], kC_D_V / kR_D);
}

// Two kernels.  ks_bc_rim relaxes the swamp layer only: one thread per (listed plane point,
// level), the points being those where any of the three rescale factors is nonzero, with the
// FP64 blend x = f*(w_old*x_old + w_new*x_new) + (1 - f)*x of every field (FP32 mirror rounded
// from it).  Everywhere else the reference's 0*(...) + 1*x is x (for finite boundary data and
// a nonzero x), so nothing is written there.  ks_bc_thermo then recomputes theta_v_pert and
// exner_pert at every scalar point with one FP64 operation each:
//   theta_v_pert = (rhotheta_v - rho_gas*theta_v_bg)/rho_gas, the numerator in FP64 and
//                  the division in FP32 (relative error ~1e-7 of theta_v_pert),
//   exner_pert   = (r_d*rhotheta_v/p_0)^(r_d/c_d_v) - exner_bg
//                = exner_bg*((1 + d)^kappa - 1) = exner_bg*expm1(kappa*log1p(d)),
//                  d = (rhotheta_v - rt_bg)/rt_bg with rt_bg the background's rhotheta_v,
//                  in FP32 after the FP64 difference (relative error ~1e-7 of exner_pert).
// Keeping the blend out of the second kernel matters on this GPU: a warp covers 32 rows, so
// with one kernel every warp that touches the swamp layer issued the whole FP64 blend.

// (1 + d)^kappa - 1 in FP32 for |d| <= 0.25 from series with multiply-adds only:
// log1p(d) = 2 atanh(s) = 2 (s + s^3/3 + ... + s^13/13), s = d/(2 + d), |s| <= 1/7, and
// expm1(y) = y + y^2/2! + ... + y^8/8!, |y| = |kappa log1p(d)| <= 0.12 (truncation errors
// below 1e-11 relative); larger |d| goes through log1pf and expm1f.
__device__ __forceinline__ float pow1p_m1(float d, float kappa) {
  if (fabsf(d) > 0.25f) return expm1f(kappa * log1pf(d));
  const float sv = d / (2.f + d), s2 = sv * sv;
  float t = 1.f / 13.f;
  t = fmaf(t, s2, 1.f / 11.f);
  t = fmaf(t, s2, 1.f / 9.f);
  t = fmaf(t, s2, 1.f / 7.f);
  t = fmaf(t, s2, 1.f / 5.f);
  t = fmaf(t, s2, 1.f / 3.f);
  t = fmaf(t, s2, 1.f);
  const float y = kappa * (2.f * sv * t);
  float e = 1.f / 40320.f;
  e = fmaf(e, y, 1.f / 5040.f);
  e = fmaf(e, y, 1.f / 720.f);
  e = fmaf(e, y, 1.f / 120.f);
  e = fmaf(e, y, 1.f / 24.f);
  e = fmaf(e, y, 1.f / 6.f);
  e = fmaf(e, y, 0.5f);
  e = fmaf(e, y, 1.f);
  return y * e;
}
// the factors are +0 or positive: a bit test instead of an FP64 comparison
__device__ __forceinline__ bool nonzero(double f) { return __double_as_longlong(f) != 0; }

// grid (ceil(nrim/128), NL), 128 threads; rim[r] = plane index (ji-1) + P*(jk-1)
__global__ void __launch_bounds__(128) ks_bc_rim(Dims D, State S, StateF M, State B0, State B1, const int* rim, int nrim,
                                                 const double* fs, const double* fu, const double* fv, double ow,
                                                 double nw) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrim) return;
  const int p = rim[r], ji = p % D.P + 1, jk = p / D.P + 1, jl = blockIdx.y + 1;
  const bool mir = M.rho != nullptr;
  auto relax = [&](double f, const double* b0, const double* b1, double* x, float* xm, long long q) {
    const double v = f * (ow * b0[q] + nw * b1[q]) + (1.0 - f) * x[q];
    x[q] = v;
    if (mir) xm[q] = narrow(v);
  };
  const long long q = IX(D, ji, jk, jl);
  if (ji <= D.ny && jk <= D.nx && nonzero(fs[p])) {
    const double f = fs[p];
    if (jl <= D.nl) {
      for (int jc = 0; jc < D.ncons; ++jc) relax(f, B0.rho, B1.rho, S.rho, M.rho, q + (long long)jc * D.fstride);
      relax(f, B0.rt, B1.rt, S.rt, M.rt, q);
    }
    relax(f, B0.w, B1.w, S.w, M.w, q);
  }
  if (jl <= D.nl && ji <= D.ny && jk <= D.nx + 1 && nonzero(fu[p])) relax(fu[p], B0.u, B1.u, S.u, M.u, q);
  if (jl <= D.nl && ji <= D.ny + 1 && jk <= D.nx && nonzero(fv[p])) relax(fv[p], B0.v, B1.v, S.v, M.v, q);
}

__global__ void __launch_bounds__(256) ks_bc_thermo(Dims D, State S, StateF M, const double* theta_v_bg,
                                                    const double* exner_bg, const double* rtbg) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl);
  const double rho_g = S.rho[q + (long long)(D.g - 1) * D.fstride], rt = S.rt[q];
  const double tb = theta_v_bg[q], rb = rtbg[q], eb = exner_bg[q];
  const float tpf = narrow(fma(-rho_g, tb, rt)) / narrow(rho_g);
  const float d = narrow(rt - rb) / narrow(rb);
  const float epf = narrow(eb) * pow1p_m1(d, (float)(kR_D / kC_D_V));
  S.tp[q] = wide(tpf);
  S.ep[q] = wide(epf);
  if (M.tp) {
    M.tp[q] = tpf;
    M.ep[q] = epf;
  }
}
}  // namespace

int split_bc_prepare(SplitCtx* s, const Dims& D, const Grid<double>& G, cudaStream_t stream) {
  if (!s->rtbg) {
    long long bytes = 0;
    if (salloc(s, &s->rtbg, (size_t)D.fstride, &bytes)) return LGAME_ERR_ALLOC;
  }
  k_rtbg<<<1216, 256, 0, stream>>>(G.exner_bg, s->rtbg, D.fstride);
  return cudaGetLastError() == cudaSuccess ? LGAME_OK : LGAME_ERR_CUDA;
}

int split_bc_update(SplitCtx* s, const Dims& D, const Grid<double>& G, const State& S, const StateF& M, const State& B0,
                    const State& B1, const int* rim, int nrim, const double* fs, const double* fu, const double* fv,
                    double ow, double nw, cudaStream_t stream) {
  if (!s->rtbg) return LGAME_ERR_STATE;
  if (nrim > 0)
    ks_bc_rim<<<dim3((unsigned)((nrim + 127) / 128), (unsigned)D.NL), 128, 0, stream>>>(D, S, M, B0, B1, rim, nrim, fs, fu,
                                                                                        fv, ow, nw);
  ks_bc_thermo<<<sgrd(D.ny, D.nx, D.nl), dim3(32, 8), 0, stream>>>(D, S, M, G.theta_v_bg, G.exner_bg, s->rtbg);
  return cudaGetLastError() == cudaSuccess ? LGAME_OK : LGAME_ERR_CUDA;
}

int split_refresh_mirror(SplitCtx* s, const Dims& D, int slot, const State& S, cudaStream_t stream) {
  const long long F = D.fstride;
  const StateF& M = s->mir[slot];
  if (split_convert(S.rho, M.rho, F * D.ncons, stream)) return LGAME_ERR_CUDA;
  const double* src[] = {S.rt, S.tp, S.ep, S.u, S.v, S.w};
  float* dst[] = {M.rt, M.tp, M.ep, M.u, M.v, M.w};
  for (int k = 0; k < 6; ++k)
    if (split_convert(src[k], dst[k], F, stream)) return LGAME_ERR_CUDA;
  return LGAME_OK;
}

int split_set_grid(SplitCtx* s, const Dims& D, const Grid<double>& G, cudaStream_t stream) {
  const long long F = D.fstride;
  const double* src[] = {G.z_scalar, G.z_u, G.z_v, G.z_w, G.dx, G.dy, G.dz, G.volume, G.area_x, G.area_y, G.area_z,
                         G.area_dual_x, G.area_dual_y, G.area_dual_z, G.z_area_dual_z, G.slope_x, G.slope_y,
                         G.theta_v_bg, G.exner_bg, G.egu, G.egv, G.egw, G.gm, G.gp, G.fvec_x, G.fvec_y, G.fvec_z,
                         G.damp};
  const double* src2[] = {G.dx_dual, G.dy_dual, G.layer_thickness};  // -> gf[33..35]
  const int nsrc = sizeof(src) / sizeof(src[0]);
  for (int k = 0; k < nsrc; ++k) {
    const long long n = (src[k] == G.fvec_x || src[k] == G.fvec_y || src[k] == G.fvec_z) ? D.plane : F;
    if (split_convert(src[k], s->gf[k], n, stream)) return LGAME_ERR_CUDA;
  }
  for (int k = 0; k < 3; ++k) if (split_convert(src2[k], s->gf[33 + k], F, stream)) return LGAME_ERR_CUDA;
  for (int k = 0; k < 6; ++k) if (split_convert(G.ipw[k], s->ipw[k], F, stream)) return LGAME_ERR_CUDA;
  for (int k = 0; k < 3; ++k) if (split_convert(G.trsk_u[k], s->trsk_u[k], D.P, stream)) return LGAME_ERR_CUDA;
  for (int k = 0; k < 2; ++k) if (split_convert(G.trsk_v[k], s->trsk_v[k], D.P, stream)) return LGAME_ERR_CUDA;
  k_recip<<<1216, 256, 0, stream>>>(G.dx, s->inv_dx, F);
  k_recip<<<1216, 256, 0, stream>>>(G.dy, s->inv_dy, F);
  k_recip<<<1216, 256, 0, stream>>>(G.dz, s->inv_dz, F);
  k_recip<<<1216, 256, 0, stream>>>(G.volume, s->inv_volume, F);
  k_recip<<<1216, 256, 0, stream>>>(G.area_z, s->inv_area_z, F);
  float* ivol = s->gf[28];
  float* iaz = s->gf[29];
  float* dzs = s->gf[30];
  float* deb = s->gf[31];
  float* kd = s->gf[32];
  k_grid_extra<<<sgrd(D.ny, D.nx, D.NL), sblk(), 0, stream>>>(D, G, ivol, iaz, dzs, deb, kd);
  if (cudaGetLastError() != cudaSuccess) return LGAME_ERR_CUDA;
  Grid<float>& GF = s->GF;
  float** g = s->gf;
  GF.z_scalar = g[0]; GF.z_u = g[1]; GF.z_v = g[2]; GF.z_w = g[3]; GF.dx = g[4]; GF.dy = g[5]; GF.dz = g[6];
  GF.volume = g[7]; GF.area_x = g[8]; GF.area_y = g[9]; GF.area_z = g[10]; GF.area_dual_x = g[11];
  GF.area_dual_y = g[12]; GF.area_dual_z = g[13]; GF.z_area_dual_z = g[14]; GF.slope_x = g[15]; GF.slope_y = g[16];
  GF.theta_v_bg = g[17]; GF.exner_bg = g[18]; GF.egu = g[19]; GF.egv = g[20]; GF.egw = g[21]; GF.gm = g[22];
  GF.gp = g[23]; GF.fvec_x = g[24]; GF.fvec_y = g[25]; GF.fvec_z = g[26]; GF.damp = g[27];
  GF.dx_dual = g[33]; GF.dy_dual = g[34]; GF.layer_thickness = g[35];
  for (int k = 0; k < 6; ++k) GF.ipw[k] = s->ipw[k];
  for (int k = 0; k < 3; ++k) GF.trsk_u[k] = s->trsk_u[k];
  for (int k = 0; k < 2; ++k) GF.trsk_v[k] = s->trsk_v[k];
  s->GX = GridX{s->inv_dx, s->inv_dy, s->inv_dz, s->inv_volume, s->inv_area_z, ivol, iaz, dzs, deb, kd};
  // the third-order theta chain of the background, in FP64 on temporary arrays that start at 0
  // (the levels and boundary faces the chain does not write are read as 0)
  double* tmp[4] = {};
  bool ok = true;
  for (double*& t : tmp) {
    ok = ok && cudaMalloc(&t, (size_t)F * sizeof(double)) == cudaSuccess &&
         cudaMemsetAsync(t, 0, (size_t)F * sizeof(double), stream) == cudaSuccess;
  }
  if (ok) {
    const dim3 B = sblk();
    k_grad_vert<double, double><<<sgrd(D.ny, D.nx, D.nl - 1), B, 0, stream>>>(D, G, G.theta_v_bg, tmp[0]);
    k_grad_hor<double, double><<<sgrd(D.ny + 1, D.nx + 1, D.nl), B, 0, stream>>>(D, G, G.theta_v_bg, tmp[0], tmp[1],
                                                                                  tmp[2]);
    k_div_h<double><<<sgrd(D.ny, D.nx, D.nl), B, 0, stream>>>(D, G, tmp[1], tmp[2], tmp[3]);
    k_to_float<<<1216, 256, 0, stream>>>(tmp[3], s->dbg, F);
    k_bg_faces<<<sgrd(D.ny + 1, D.nx + 1, D.nl), B, 0, stream>>>(D, G, s->tbu, s->tbv);
    ok = cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(stream) == cudaSuccess;
  }
  for (double* t : tmp) if (t) cudaFree(t);
  if (!ok) {
    lgame_set_error("split set-up: theta chain of the background state failed");
    return LGAME_ERR_CUDA;
  }
  return LGAME_OK;
}

int split_step(SplitCtx* s, const Dims& D, const Grid<double>& G, const State& So, const State& Sn, int so, int sn,
               const PGrad<double>& pg, int step, cudaStream_t stream, int* nk,
               int (*tb)(void*, const char*), void (*te)(void*, int), void* tracer, bool serial) {
  const Grid<float>& GF = s->GF;
  const SplitCarriedF& C = s->C;
  const Tend<float> T = C.tend;
  const StateF& Mo = s->mir[so];
  const StateF& Mn = s->mir[sn];
  int launches = 0;
  // Kernels that do not depend on each other run on side streams, forked from and joined back
  // into `stream` by events:
  //   first substep:  the closure, swamp-layer heating and phase transitions (FP32 and
  //                   latency-bound) beside the theta edges and the FP64 pressure gradient;
  //   both substeps:  the tracer tendencies beside the gas fluxes, divergences and vertical solve;
  //   between them:   the first substep's tracer solver beside the second substep's vorticity,
  //                   kinetic energy (FP64, on a second side stream) and wind update.
  // Every pair was checked for the arrays one writes and the other reads (the comments at each
  // fork); with `serial` (per-kernel tracing, and the caller's graph capture, where the serial
  // order measured faster) everything runs on `stream` in the same order.
  const bool conc = !serial;
  cudaStream_t cur = stream;
  cudaStream_t side = conc ? s->br[0] : stream, side2 = conc ? s->br[1] : stream;
  enum { EV_A = 0, EV_JA, EV_B, EV_C, EV_CSH, EV_KE, EV_JKE, EV_END };
  // `to` starts after everything enqueued on `from` so far
  auto after = [&](cudaStream_t to, cudaStream_t from, int k) -> int {
    if (!conc || to == from) return LGAME_OK;
    if (cudaEventRecord(s->ev[k], from) != cudaSuccess || cudaStreamWaitEvent(to, s->ev[k], 0) != cudaSuccess) {
      lgame_set_error("split step: fork/join event failed");
      return LGAME_ERR_CUDA;
    }
    return LGAME_OK;
  };
#define SL(name, kernel, grid_, block_, ...) SLS(name, kernel, grid_, block_, 0, __VA_ARGS__)
#define SLS(name, kernel, grid_, block_, smem_, ...)                            \
  do {                                                                          \
    const int tr_ = tb ? tb(tracer, name) : -1;                                 \
    kernel<<<grid_, block_, smem_, cur>>>(__VA_ARGS__);                         \
    if (tr_ >= 0) te(tracer, tr_);                                              \
    cudaError_t e_ = cudaGetLastError();                                        \
    if (e_ != cudaSuccess) {                                                    \
      lgame_set_error((std::string("launch of ") + name + ": " + cudaGetErrorString(e_)).c_str()); \
      return LGAME_ERR_CUDA;                                                    \
    }                                                                           \
    ++launches;                                                                 \
  } while (0)
#define SYNC(call)                   \
  do {                               \
    const int rc_ = (call);          \
    if (rc_ != LGAME_OK) return rc_; \
  } while (0)
  const dim3 B = sblk();
  // third-order theta edges: the gradient of theta' (read from the mirror), its divergence and
  // the edges of theta_bg + theta' (and of theta' alone when pu/pv are given)
  auto theta3f = [&](const float* tp, const float* u, const float* v, float* ou, float* ov, float* pu,
                     float* pv) -> int {
    SL("ks_grad_vert", (k_grad_vert<float, float>), sgrd(D.ny, D.nx, D.nl - 1), B, D, GF, tp, s->gz);
    SL("ks_grad_hor", (k_grad_hor<float, float>), sgrd(D.ny + 1, D.nx + 1, D.nl), B, D, GF, tp, s->gz, s->gx, s->gy);
    SL("ks_div_h", ks_div_h, cgrd(D.ny, D.nx), cblk(), D, GF, s->GX, s->gx, s->gy, s->divf);
    SL("ks_theta_edges", ks_theta_edges, sgrd(D.ny + 1, D.nx + 1, D.nl), B, D, tp, s->divf, s->dbg, s->tbu, s->tbv, u,
       v, ou, ov, pu, pv);
    return LGAME_OK;
  };
  SL("ks_temperature", (k_temperature<float, float>), sgrd(D.ny, D.nx, D.nl), B, D, GF, Mo, C.temperature);
  // the surface parts in FP64 on the FP64 state (two-dimensional): update_sfc_turb_quantities
  // before the substeps (mo_manage_pchevi.F90:51-53)
  const SplitSfc& SF = s->sfc;
  if (SF.turb) SL("ks_sfc_turb", k_sfc_turb<float>, sgrd(D.ny, D.nx, 1), B, D, G, So, s->vsq, SF.buf, SF.par);
  Carried<float> CC{pg.nl_u, pg.nl_v, pg.nl_w, pg.l_u, pg.l_v, pg.l_w, pg.old_u, pg.old_v, C.pgcw,
                    C.vsg_x, C.vsg_y, C.vsg_z, C.pvt_x, C.pvt_y, C.pvt_z};
  const SplitDiff& SD = s->diff;
  const DiffBuf<float>& DB = s->db;
  const bool vort = !D.llinear || D.lcorio, tracers = D.ncons > 1;
  const float* mdt = (SD.mom_h && SD.mass_h) ? DB.mdt : nullptr;
  const float* tdh = (SD.mom_h && SD.temp_h) ? DB.tdh : nullptr;
  const float* ptr = SF.phase ? C.ptr : nullptr;
  const float* pth = SF.phase ? C.pth : nullptr;
  if (SD.mom_h) { CC.mdt_x = DB.mdtx; CC.mdt_y = DB.mdty; CC.mdt_z = DB.mdtz; }
  // the vorticity flux and the kinetic-energy gradient of state Sv (mirror Mv); with `branch`
  // the kinetic energy (FP64) runs on the second side stream beside the vorticity (FP32)
  auto vector_terms = [&](const State& Sv, const StateF& Mv, bool branch) -> int {
    if (!vort) return LGAME_OK;
    const bool ke = !D.llinear;
    if (ke && branch) {
      SYNC(after(side2, stream, EV_KE));
      cur = side2;
    }
    if (ke) {
      SL("ks_ke", (k_ke<double, double>), sgrd(D.ny, D.nx, D.nl), B, D, G, Sv, s->vsq);
      SL("ks_grad_vert", (k_grad_vert<float, double>), sgrd(D.ny, D.nx, D.nl - 1), B, D, GF, s->vsq, C.vsg_z);
      SL("ks_grad_hor", (k_grad_hor<float, double>), sgrd(D.ny + 1, D.nx + 1, D.nl), B, D, GF, s->vsq, C.vsg_z,
         C.vsg_x, C.vsg_y);
    }
    cur = stream;
    SL("ks_eta", ks_eta, sgrd(D.ny + 1, D.nx + 1, D.NL), B, D, GF, Mv, s->ex, s->ey, s->ez, s->uph, s->vph, s->wph);
    SL("ks_vort_flux", ks_vort_flux, sgrd(D.ny + 1, D.nx + 1, D.nl), B, D, GF, Mv, s->ex, s->ey,
       s->ez, s->uph, s->vph, s->wph, C.pvt_x, C.pvt_y, C.pvt_z);
    if (ke && branch) SYNC(after(stream, side2, EV_JKE));
    return LGAME_OK;
  };
  for (int rk = 1; rk <= 2; ++rk) {
    const StateF& Ms = (rk == 1) ? Mo : Mn;
    if (rk == 1) {
      // side: the closure (momentum diffusion, dissipation, scalar diffusion), or the swamp
      // layer's heating, and the phase transitions: they read the old mirror, its temperature
      // and the surface quantities, and write only their own buffers (DB, hdiss, ptr/pth, the
      // latent fluxes).  main: theta edges, gzp, pressure gradient (scratch gx..divf, tvu..tpv,
      // gzd, rmz, the pressure-gradient arrays).  Joined before the wind update.
      const bool side_work = SD.mom_h || (D.lklemp && D.ndamp > 0) || SF.phase;
      // step 0 forms the vector terms at the first substep too (mo_vector_tend_expl.F90:41-98),
      // before the closure: the PBL reads the kinetic energy they form
      if (step == 0) SYNC(vector_terms(So, Mo, false));
      if (side_work) {
        SYNC(after(side, stream, EV_A));
        cur = side;
      }
      if (SD.mom_h) {
        const dim3 gs = sgrd(D.ny, D.nx, D.nl);
        SL("ks_diff_tke", (k_diff_tke<float, float>), gs, B, D, GF, Mo, DB, SD.par);
        SL("ks_diff_zeta", (k_diff_zeta<float, float>), sgrd(D.ny + 1, D.nx + 1, D.nl), B, D, GF, Mo, DB);
        SL("ks_diff_visc", (k_diff_visc<float, float>), gs, B, D, GF, Mo, (const float*)C.temperature, DB, SD.par);
        SL("ks_diff_vz", (k_diff_vz<float, float>), sgrd(D.ny + 1, D.nx + 1, D.nl), B, D, GF, Mo, DB);
        SL("ks_mom_diff_h", (k_mom_diff_h<float, float>), gs, B, D, GF, Mo, DB);
        if (SD.mom_v) SL("ks_mom_diff_v", (k_mom_diff_v<float, float>), sgrd(D.ny, D.nx, D.nl - 1), B, D, GF, Mo, DB);
        if (SF.pbl)
          SL("ks_pbl", (k_pbl<float, float>), sgrd(D.ny, D.nx, 1), B, D, G, So, s->vsq, SF.buf, SF.par, DB.mdtx, DB.mdty);
        SL("ks_diss_rate", (k_diss_rate<float, float>), gs, B, D, GF, Mo, DB, GF.damp, s->GX.kdamp_f);
        // temperature and mass diffusion (mo_scalar_tend_expl.F90:60-101): fluxes and divergence of
        // every constituent and the temperature in one column-marching launch; the second
        // substep's temperature diffusion is the same (same temperature and coefficients)
        const dim3 gd((D.ny + DS_X - 1) / DS_X, (D.nx + DS_Y - 1) / DS_Y);
        if (SD.temp_h || SD.mass_h) {
          const float* tm = (const float*)C.temperature;
          const float* rm = (const float*)Mo.rho;
          const int vm = SD.mass_v ? 1 : 0, vt = SD.temp_v ? 1 : 0;
          const dim3 bd(DS_THREADS);
          if (SD.temp_h && SD.mass_h && D.ncons == 7)
            SLS("ks_diff_scalar", (k_diff_scalar_col<7, 1>), gd, bd, diff_scalar_smem(8), D, GF, Mo, DB, rm, vm, DB.mdt,
                tm, vt, DB.tdh);
          else if (SD.temp_h && SD.mass_h)
            SLS("ks_diff_scalar", (k_diff_scalar_col<1, 1>), gd, bd, diff_scalar_smem(2), D, GF, Mo, DB, rm, vm, DB.mdt,
                tm, vt, DB.tdh);
          else if (SD.temp_h)
            SLS("ks_diff_scalar", (k_diff_scalar_col<0, 1>), gd, bd, diff_scalar_smem(1), D, GF, Mo, DB, rm, 0,
                (float*)nullptr, tm, vt, DB.tdh);
          else if (D.ncons == 7)
            SLS("ks_diff_scalar", (k_diff_scalar_col<7, 0>), gd, bd, diff_scalar_smem(7), D, GF, Mo, DB, rm, vm, DB.mdt,
                tm, 0, (float*)nullptr);
          else
            SLS("ks_diff_scalar", (k_diff_scalar_col<1, 0>), gd, bd, diff_scalar_smem(1), D, GF, Mo, DB, rm, vm, DB.mdt,
                tm, 0, (float*)nullptr);
        }
      } else if (D.lklemp && D.ndamp > 0) {
        SL("ks_heating_diss", ks_heating_diss, sgrd(D.ny, D.nx, std::min(D.nl, D.ndamp)), B, D, GF, s->GX, Mo, C.hdiss);
      }
      // the phase transitions (extension) from state_old and its temperature, in FP64 on the FP64
      // state; both substeps read the rates
      if (SF.phase)
        SL("ks_phase_trans", (k_phase_trans<float, float>), sgrd(D.ny, D.nx, D.nl), B, D, G, So,
           (const float*)C.temperature, SF.buf, SF.tsoil[so], SF.phase_sfc ? 1 : 0, D.dtime, C.ptr, C.pth);
      cur = stream;
      if (D.theta_order == 3) {  // the edges of theta_v and, with a background state, of theta'
        const int rc = theta3f(Mo.tp, Mo.u, Mo.v, s->tvu, s->tvv, D.luse_bg ? s->tpu : nullptr,
                               D.luse_bg ? s->tpv : nullptr);
        if (rc) return rc;
      }
      SL("ks_gzp", ks_gzp, sgrd(D.ny, D.nx, D.nl), B, D, G, s->GX, So.ep, s->gzd, s->rmz);
      SL("ks_pgrad", ks_pgrad, sgrd(D.ny + 1, D.nx + 1, D.nl), B, D, G, s->GX, So, s->gzd, s->rmz, Mo.rho, s->tvu,
         s->tvv, s->tpu, s->tpv, pg, C, C.pgcw, step == 0 ? 1 : 0);
      if (side_work) SYNC(after(stream, side, EV_JA));
    } else {
      // main: vorticity of the new state; side 2: its kinetic energy (FP64); both read the state
      // of the first substep (u, v from its wind update, w and rho_g from its vertical solve),
      // which the tracer solver still running on the side stream does not write
      SYNC(vector_terms(Sn, Mn, true));
    }
    SL("ks_tend_wind", ks_tend_wind, sgrd(D.ny + 1, D.nx + 1, D.NL), B, D, So, Sn, T, CC, C, rk, Mn.u, Mn.v);
    // side: the tracer tendencies (read the tracer densities of Ms and the new u, v; write the
    // tracer fields of T.rho), beside the gas fluxes, divergence and vertical solve, which write
    // the gas field of T.rho, T.rt, the gas density, theta', exner', rhotheta_v and w
    if (tracers) {
      SYNC(after(side, stream, EV_B));
      cur = side;
      SL("ks_tracers", ks_tracers, sgrd(D.ny, D.nx, D.nl), B, D, GF, s->GX, Ms, Mn.u, Mn.v, T.rho, rk, mdt, ptr);
      cur = stream;
    }
    // third-order theta edges of the state used here; in the first substep that is the old
    // state, whose edges the pressure gradient's call above already left in tvu/tvv (nothing
    // in between writes the old mirror or tvu/tvv), so only the second substep recomputes them
    if (D.theta_order == 3 && rk == 2) {
      const int rc = theta3f(Ms.tp, Ms.u, Ms.v, s->tvu, s->tvv, nullptr, nullptr);
      if (rc) return rc;
    }
    SL("ks_gas_flux", ks_gas_flux, sgrd(D.ny + 1, D.nx + 1, D.nl), B, D, GF, Ms, Mn.u, Mn.v, s->tvu, s->tvv, s->fu,
       s->fv, s->gu, s->gv);
    // the second substep's gas divergence reads every density of the new mirror (the heat
    // capacity) and the sediment heating: it waits for the first substep's tracer solver
    if (rk == 2 && tracers && conc) {
      if (cudaStreamWaitEvent(stream, s->ev[EV_CSH], 0) != cudaSuccess) {
        lgame_set_error("split step: join event failed");
        return LGAME_ERR_CUDA;
      }
    }
    SL("ks_gas_div", ks_gas_div, cgrd(D.ny, D.nx), cblk(), D, GF, s->GX, Ms, s->fu, s->fv, s->gu, s->gv,
       C.temperature, C.hdiss, C.rad, C.csh, T.rho, T.rt, mdt, tdh, ptr, pth);
    if (SF.sens || SF.soil)
      SL("ks_sfc_column", k_sfc_column_split<float>, sgrd(D.ny, D.nx, 1), B, D, G, So, rk == 1 ? So : Sn, T.rt,
         SF.buf, SF.par, SF.tsoil[so], SF.tsoil[rk == 1 ? so : sn], SF.tsoil[sn]);
    const dim3 gc = cgrd(D.ny, D.nx);
    if (s->column_fp64)
      SL("ks_column_ver", ks_column_ver<double>, gc, cblk(), D, G, GF, s->GX, So, Sn, Mo, Mn, T, rk);
    else
      SL("ks_column_ver", ks_column_ver<float>, gc, cblk(), D, G, GF, s->GX, So, Sn, Mo, Mn, T, rk);
    if (tracers) {
      // the two tracer sets fastest (the blocks of a row tile run together), row tiles, columns
      const dim3 gt(2u, (unsigned)((D.ny + 31) / 32), (unsigned)D.nx);
      if (rk == 1) {
        // side (after its tracer tendencies): the first substep's tracer solver and sediment
        // heating, which read w old and new and the gas density (final now) and write the
        // tracer densities and csh, beside the second substep's vorticity and wind update
        SYNC(after(side, stream, EV_C));
        cur = side;
        SLS("ks_column_tracers", ks_column_tracers<true>, gt, dim3(kTrWarps * 32), tracer_smem(D), D, GF, s->GX, So,
            Sn, Mo, Mn, T.rho, C.temperature, s->csh_part);
        if (D.nc > 0) SL("ks_csh_sum", ks_csh_sum, sgrd(D.ny, D.nx, D.nl), B, D, s->csh_part, C.csh);
        if (conc && cudaEventRecord(s->ev[EV_CSH], side) != cudaSuccess) {
          lgame_set_error("split step: event record failed");
          return LGAME_ERR_CUDA;
        }
        cur = stream;
      } else {
        SYNC(after(stream, side, EV_END));
        SLS("ks_column_tracers", ks_column_tracers<false>, gt, dim3(kTrWarps * 32), tracer_smem(D), D, GF, s->GX, So,
            Sn, Mo, Mn, T.rho, C.temperature, s->csh_part);
      }
    }
  }
#undef SL
#undef SLS
#undef SYNC
  *nk = launches;
  return LGAME_OK;
}

}  // namespace lg
