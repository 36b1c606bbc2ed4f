// split.cu -- FP32/FP64 split-precision HEVI step (compiled with -fmad=true, -prec-div=false).
//
// The explicit stencils are the templates of kernels.cuh instantiated for float, reading
// the FP64 state and FP32 copies of the metrics.  This file adds the parts that stay in
// FP64 in this mode -- the pressure gradient and both column solvers -- written for the
// FP64 pipe of this GPU: multiply-adds and reciprocals seeded in FP32 and refined by two
// Newton steps in FP64 instead of FP64 divisions (one division costs ~10 FMA slots), and
// metric reciprocals computed once at set-up.
#include "split.cuh"
#include "common.h"
#include "lgame_gpu.h"

#include <string>
#include <vector>

namespace lg {

namespace {

// 1/x to full FP64 precision: FP32 reciprocal, then two Newton-Raphson steps in FP64
// (relative error 2^-23 -> 2^-46 -> below 2^-52).  |x| must lie in the FP32 normal range.
__device__ __forceinline__ double drcp(double x) {
  double r = (double)__frcp_rn((float)x);
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

constexpr int kMaxL = 128;

struct GridX {  // FP64 reciprocal metrics of the FP64 parts
  const double *inv_dx, *inv_dy, *inv_dz, *inv_volume, *inv_area_z;
};

}  // namespace

struct SplitCtx {
  std::vector<void*> allocs;
  Grid<float> GF{};
  GridX GX{};
  float *gf[40] = {};
  float *ipw[6] = {}, *trsk_u[3] = {}, *trsk_v[2] = {};
  double *inv_dx = nullptr, *inv_dy = nullptr, *inv_dz = nullptr, *inv_volume = nullptr, *inv_area_z = nullptr;
  // FP32 intermediates
  float *th, *gx, *gy, *gz, *divf, *tvu, *tvv, *tpu, *tpv, *ex, *ey, *ez, *uph, *vph, *wph;
  // kinetic energy in FP64: its vertical differences over thin layers cancel most digits
  double* vsq = nullptr;
  SplitCarriedF C{};
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
__global__ void k_to_double(const float* a, double* b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}
__global__ void k_recip(const double* a, double* b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (a[i] != 0.0) ? 1.0 / a[i] : 0.0;
}

// ---- pressure gradient, mo_p_grad.F90:20-120, FP64 products ---------------------------
// gradient of the Exner pressure perturbation in FP64 (the small differences of a small
// field), theta edge values in FP32 (third order) or FP64 (second order), the background
// term theta'*grad(Pi_bg) in FP64, the condensate deceleration factor in FP32.
__global__ void ks_pgrad(Dims D, Grid<double> G, GridX X, State S, const float* tvu, const float* tvv,
                         const float* tpu, const float* tpv, PGrad<double> P, float* pgcw, int lfirst) {
  LG_IDX3;
  const double ubs = D.luse_bg ? 1.0 : 0.0;
  const double* ep = S.ep;
  auto theta = [&](int i, int j, int k) { const long long q = IX(D, i, j, k); return G.theta_v_bg[q] + S.tp[q]; };
  // condensate mass fraction sum(rho_cond)/sum(rho): the reference's rho_g/sum(rho) and
  // rho_g/sum(rho) - 1 (mo_p_grad.F90:86-87, :115-116) rewritten as 1 - f and -f, which
  // is exact for dry air and free of cancellation in FP32
  auto cond_frac = [&](long long q) -> float {
    if (D.nc == 0) return 0.f;
    float c = 0.f;
    for (int jc = 0; jc < D.nc; ++jc) c += float(S.rho[q + (long long)jc * D.fstride]);
    return c / (c + float(S.rho[q + (long long)(D.g - 1) * D.fstride]));
  };
  auto decel = [&](int i, int j, int k) {
    return float(kC_D_P) - float(kC_D_P) * cond_frac(IX(D, i, j, k));
  };
  // vertical gradient of exner_pert at a w point of column (i,j), 0 at the boundary levels
  auto gzp = [&](int i, int j, int k) -> double {
    if (k < 2 || k > D.nl) return 0.0;
    return (ep[IX(D, i, j, k - 1)] - ep[IX(D, i, j, k)]) * X.inv_dz[IX(D, i, j, k)];
  };
  auto remapx = [&](int ji_, int jk_, int jl_) -> double {  // mo_averaging.F90:56-95 on gzp
    const int a = (jk_ == 1 || jk_ == D.nx + 1) ? D.nx : jk_ - 1, b = (jk_ == 1 || jk_ == D.nx + 1) ? 1 : jk_;
    double r = G.ipw[4][IX(D, ji_, a, jl_)] * gzp(ji_, a, jl_) + G.ipw[4][IX(D, ji_, b, jl_)] * gzp(ji_, b, jl_);
    if (jl_ < D.nl || D.freeslip)
      r += G.ipw[5][IX(D, ji_, a, jl_)] * gzp(ji_, a, jl_ + 1) + G.ipw[5][IX(D, ji_, b, jl_)] * gzp(ji_, b, jl_ + 1);
    return 0.5 * r;
  };
  auto remapy = [&](int ji_, int jk_, int jl_) -> double {
    const int a = (ji_ == 1 || ji_ == D.ny + 1) ? D.ny : ji_ - 1, b = (ji_ == 1 || ji_ == D.ny + 1) ? 1 : ji_;
    double r = G.ipw[4][IX(D, a, jk_, jl_)] * gzp(a, jk_, jl_) + G.ipw[4][IX(D, b, jk_, jl_)] * gzp(b, jk_, jl_);
    if (jl_ < D.nl || D.freeslip)
      r += G.ipw[5][IX(D, a, jk_, jl_)] * gzp(a, jk_, jl_ + 1) + G.ipw[5][IX(D, b, jk_, jl_)] * gzp(b, jk_, jl_ + 1);
    return 0.5 * r;
  };
  if (jl <= D.nl && ji <= D.ny && jk <= D.nx + 1) {
    const long long q = IX(D, ji, jk, jl);
    const bool inner = jk >= 2 && jk <= D.nx;
    const double nl_prev = P.nl_u[q], l_prev = P.l_u[q];
    if (!lfirst) P.old_u[q] = -nl_prev - ubs * l_prev;
    if (inner || D.periodic) {
      const int kk = inner ? jk : 1, ka = inner ? jk - 1 : D.nx;
      const long long qr = IX(D, ji, kk, jl);
      double g = (ep[qr] - ep[IX(D, ji, ka, jl)]) * X.inv_dx[qr];
      if (jl > D.nf) g -= G.slope_x[qr] * remapx(ji, kk, jl);
      const double te = (D.theta_order == 2) ? 0.5 * (theta(ji, ka, jl) + theta(ji, kk, jl)) : (double)tvu[qr];
      const double de = 0.5 * ((double)decel(ji, ka, jl) + (double)decel(ji, kk, jl));
      const double nlv = de * (te * g);
      double lv = l_prev;
      if (D.luse_bg) {
        const double tp = (D.theta_order == 2) ? 0.5 * (S.tp[IX(D, ji, ka, jl)] + S.tp[qr]) : (double)tpu[qr];
        lv = de * (tp * G.egu[qr]);
        P.l_u[q] = lv;
      }
      P.nl_u[q] = nlv;
      if (lfirst) P.old_u[q] = -nlv - ubs * lv;
    } else if (lfirst) {
      P.old_u[q] = -nl_prev - ubs * l_prev;
    }
  }
  if (jl <= D.nl && ji <= D.ny + 1 && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    const bool inner = ji >= 2 && ji <= D.ny;
    const double nl_prev = P.nl_v[q], l_prev = P.l_v[q];
    if (!lfirst) P.old_v[q] = -nl_prev - ubs * l_prev;
    if (inner || D.periodic) {
      const int ii = inner ? ji : 1, ia = inner ? ji - 1 : D.ny;
      const long long qr = IX(D, ii, jk, jl);
      double g = (ep[IX(D, ia, jk, jl)] - ep[qr]) * X.inv_dy[qr];
      if (jl > D.nf) g -= G.slope_y[qr] * remapy(ii, jk, jl);
      const double te = (D.theta_order == 2) ? 0.5 * (theta(ia, jk, jl) + theta(ii, jk, jl)) : (double)tvv[qr];
      const double de = 0.5 * ((double)decel(ia, jk, jl) + (double)decel(ii, jk, jl));
      const double nlv = de * (te * g);
      double lv = l_prev;
      if (D.luse_bg) {
        const double tp = (D.theta_order == 2) ? 0.5 * (S.tp[IX(D, ia, jk, jl)] + S.tp[qr]) : (double)tpv[qr];
        lv = de * (tp * G.egv[qr]);
        P.l_v[q] = lv;
      }
      P.nl_v[q] = nlv;
      if (lfirst) P.old_v[q] = -nlv - ubs * lv;
    } else if (lfirst) {
      P.old_v[q] = -nl_prev - ubs * l_prev;
    }
  }
  if (jl >= 2 && jl <= D.nl && ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl), qa = IX(D, ji, jk, jl - 1);
    const double de = 0.5 * ((double)decel(ji, jk, jl - 1) + (double)decel(ji, jk, jl));
    P.nl_w[q] = de * (0.5 * (theta(ji, jk, jl - 1) + theta(ji, jk, jl)) * gzp(ji, jk, jl));
    if (D.luse_bg) P.l_w[q] = de * (0.5 * (S.tp[qa] + S.tp[q]) * G.egw[q]);
    const float da = -cond_frac(qa), db = -cond_frac(q);
    pgcw[q] = 0.5f * (da + db) * float(G.gm[q]);
  }
}

// ---- three_band_solver_ver, mo_column_solvers.F90:21-351, FP64 --------------------------
// Same system as the reference; the explicit predictions take the FP32 tendencies, the
// partial derivatives alpha, beta, gamma are formed unscaled and multiplied by the
// reciprocal volume, divisions are drcp() multiplications.
__global__ void ks_column_ver(Dims D, Grid<double> G, GridX X, State So, State Sn, Tend<float> Tn, int rk_step) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const int nl = D.nl;
  const double dt = D.dtime, idt = 1.0 / D.dtime;
  const long long goff = (long long)(D.g - 1) * D.fstride;
  const State& Su = (rk_step == 1) ? So : Sn;
  const double* rho_o = So.rho + goff;
  const double* rho_u = Su.rho + goff;
  double* rho_n = Sn.rho + goff;
  const float* t_rho = Tn.rho + goff;
  const double rdcv = kR_D / kC_D_V;
  const double ic2 = 1.0 / (kIMPL_THERMO_WEIGHT * (dt * dt) * kC_D_P);
  const double ic1 = 1.0 / (kIMPL_THERMO_WEIGHT * dt * kC_D_P);

  double au[kMaxL + 1], bu[kMaxL + 1], gu[kMaxL + 1];     // unscaled partial derivatives
  double rho_e[kMaxL + 1], rt_e[kMaxL + 1], ep_e[kMaxL + 1], tp_e[kMaxL + 1], thu[kMaxL + 1];
  double irio[kMaxL + 1], rie[kMaxL + 1], ti[kMaxL + 1];
  double cv[kMaxL + 1], dv[kMaxL + 1], ev[kMaxL + 1], rv[kMaxL + 1], epr[kMaxL + 1], rpr[kMaxL + 1];

  for (int jl = 1; jl <= nl; ++jl) {
    const long long i = IX(D, ji, jk, jl);
    const double tr = (double)t_rho[i], trt = (double)Tn.rt[i];
    const double ro = rho_o[i], rto = So.rt[i];
    rho_e[jl] = fma(dt, tr, ro);
    rt_e[jl] = fma(dt, trt, rto);
    const double iro = drcp(ro), irto = drcp(rto);
    double a = -rto * iro * iro, b = iro, g = rdcv * irto * (G.exner_bg[i] + So.ep[i]);
    if (rk_step == 2) {
      const double ru = rho_u[i], rtu = Su.rt[i];
      const double iru = drcp(ru), irtu = drcp(rtu);
      a = 0.5 * (a - rtu * iru * iru);
      b = 0.5 * (b + iru);
      g = 0.5 * (g + rdcv * irtu * (G.exner_bg[i] + Su.ep[i]));
      thu[jl] = rtu * iru;
    } else {
      thu[jl] = rto * iro;
    }
    au[jl] = a; bu[jl] = b; gu[jl] = g;
    tp_e[jl] = So.tp[i] + dt * (a * tr + b * trt);
    ep_e[jl] = So.ep[i] + dt * g * trt;
  }
  for (int jl = 1; jl <= nl - 1; ++jl) {
    const long long a = IX(D, ji, jk, jl), b = IX(D, ji, jk, jl + 1);
    irio[jl] = drcp(0.5 * (rho_o[a] + rho_o[b]));
    rie[jl] = 0.5 * (rho_e[jl] + rho_e[jl + 1]);
    ti[jl] = 0.5 * (thu[jl] + thu[jl + 1]);
  }
  for (int jl = 1; jl <= nl - 1; ++jl) {
    const long long a = IX(D, ji, jk, jl), b = IX(D, ji, jk, jl + 1);
    const double iva = X.inv_volume[a], ivb = X.inv_volume[b];
    const double dz = G.z_scalar[a] - G.z_scalar[b];
    const double deb = G.exner_bg[a] - G.exner_bg[b];
    const double dp = G.damp[b];
    const double wo = So.w[b];
    const double t = ti[jl];
    // scaled derivatives (divided by the volume) as in the reference
    const double al0 = au[jl] * iva, al1 = au[jl + 1] * ivb, be0 = bu[jl] * iva, be1 = bu[jl + 1] * ivb;
    const double ga0 = gu[jl] * iva, ga1 = gu[jl + 1] * ivb;
    dv[jl] = -(t * t) * (ga0 + ga1) + 0.5 * deb * (al1 - al0 + t * (be1 - be0))
             - dz * ic2 * irio[jl] * (2.0 * X.inv_area_z[b] + dt * wo * 0.5 * (ivb - iva)) * dp;
    rv[jl] = -(wo + dt * (double)Tn.w[b]) * dz * ic2 + t * (ep_e[jl] - ep_e[jl + 1]) * idt
             + 0.5 * idt * (tp_e[jl] + tp_e[jl + 1]) * deb - dz * ic2 * wo * rie[jl] * irio[jl];
  }
  for (int jl = 1; jl <= nl - 2; ++jl) {
    const long long a = IX(D, ji, jk, jl), b = IX(D, ji, jk, jl + 1), c = IX(D, ji, jk, jl + 2);
    const double ivb = X.inv_volume[b];
    const double al1 = au[jl + 1] * ivb, be1 = bu[jl + 1] * ivb, ga1 = gu[jl + 1] * ivb;
    cv[jl] = ti[jl + 1] * ga1 * ti[jl] + 0.5 * (G.exner_bg[b] - G.exner_bg[c]) * (al1 + be1 * ti[jl])
             - (G.z_scalar[b] - G.z_scalar[c]) * ic1 * 0.5 * So.w[c] * ivb * irio[jl + 1] * G.damp[c];
    ev[jl] = ti[jl] * ga1 * ti[jl + 1] - 0.5 * (G.exner_bg[a] - G.exner_bg[b]) * (al1 + be1 * ti[jl + 1])
             + (G.z_scalar[a] - G.z_scalar[b]) * ic1 * 0.5 * So.w[b] * ivb * irio[jl] * G.damp[b];
  }
  // Thomas, one reciprocal per row
  const int n = nl - 1;
  {
    const double id = drcp(dv[1]);
    epr[1] = ev[1] * id;
    rpr[1] = rv[1] * id;
    for (int jl = 2; jl <= n; ++jl) {
      const double iden = drcp(dv[jl] - epr[jl - 1] * cv[jl - 1]);
      if (jl <= n - 1) epr[jl] = ev[jl] * iden;
      rpr[jl] = (rv[jl] - rpr[jl - 1] * cv[jl - 1]) * iden;
    }
    double s = rpr[n];
    rv[n] = s;
    for (int jl = n - 1; jl >= 1; --jl) {
      s = rpr[jl] - epr[jl] * s;
      rv[jl] = s;  // solution
    }
  }
  const double* sol = rv;
  for (int jl = 1; jl <= nl; ++jl) {
    const long long i = IX(D, ji, jk, jl);
    const double iv = X.inv_volume[i];
    const double s0 = (jl >= 2) ? sol[jl - 1] : 0.0;
    const double s1 = (jl <= nl - 1) ? sol[jl] : 0.0;
    const double t0 = (jl >= 2) ? ti[jl - 1] : 0.0;
    const double t1 = (jl <= nl - 1) ? ti[jl] : 0.0;
    const double rn = rho_e[jl] + dt * (s1 - s0) * iv;
    const double rtn = rt_e[jl] + dt * (t1 * s1 - t0 * s0) * iv;
    rho_n[i] = rn;
    Sn.rt[i] = rtn;
    Sn.ep[i] = So.ep[i] + gu[jl] * (rtn - So.rt[i]);
    Sn.tp[i] = rtn * drcp(rn) - G.theta_v_bg[i];
  }
  for (int jl = 2; jl <= nl; ++jl) {
    const long long i = IX(D, ji, jk, jl);
    const double rin = 0.5 * (rho_n[IX(D, ji, jk, jl - 1)] + rho_n[i]);
    Sn.w[i] = (2.0 * sol[jl - 1] * X.inv_area_z[i] - rin * So.w[i]) * irio[jl - 1];
  }
  if (D.freeslip) {
    const int m = nl;
    Sn.w[IX(D, ji, jk, m + 1)] =
        G.ipw[0][IX(D, ji, jk, m)] * Sn.u[IX(D, ji, jk + 1, m)] * G.slope_x[IX(D, ji, jk + 1, m)]
      + G.ipw[1][IX(D, ji, jk, m)] * Sn.v[IX(D, ji, jk, m)] * G.slope_y[IX(D, ji, jk, m)]
      + G.ipw[2][IX(D, ji, jk, m)] * Sn.u[IX(D, ji, jk, m)] * G.slope_x[IX(D, ji, jk, m)]
      + G.ipw[3][IX(D, ji, jk, m)] * Sn.v[IX(D, ji + 1, jk, m)] * G.slope_y[IX(D, ji + 1, jk, m)];
  }
}

// v_fall_liquid, mo_derived.F90:218-263, in FP32
__device__ __forceinline__ float vfall_liquid_f(const Dims& D, const Grid<float>& GF, const double* rho_g,
                                                const float* Tm, float radius, int ji, int jk, int jl) {
  float g;
  if (jl == 1) g = GF.gm[IX(D, ji, jk, jl + 1)];
  else if (jl == D.nl) g = GF.gm[IX(D, ji, jk, jl)];
  else g = GF.ipw[4][IX(D, ji, jk, jl)] * GF.gm[IX(D, ji, jk, jl)] + GF.ipw[5][IX(D, ji, jk, jl)] * GF.gm[IX(D, ji, jk, jl + 1)];
  const long long i = IX(D, ji, jk, jl);
  const float rg = float(rho_g[i]);
  const float pm = float(kM_D / kN_A);
  const float tv = sqrtf(8.f * float(kK_B) / (float(kPI) * pm) * Tm[i]);
  const float mfp = 1.f / (1.41421356f * (rg / pm) * (4.f * float(kPI) * (130e-12f * 130e-12f)));
  const float nu = (1.f / 3.f) * tv * mfp;
  float v = 2.f * (radius * radius) * (float(kRHO_H2O) - rg) * g / (9.f * rg * nu);
  if (v * radius / nu > 10.f) v = sqrtf(8.f * radius * float(kRHO_H2O) * g / (3.f * rg * 0.8f));
  return v;
}

// ---- three_band_solver_gen_densities, mo_column_solvers.F90:353-604 ----------------------
// fall speeds, vertical fluxes and matrix coefficients in FP32; the explicit prediction
// rho_old + dt*tendency and the Thomas solve in FP64.
__global__ void ks_column_tracers(Dims D, Grid<double> G, Grid<float> GF, GridX X, State So, State Sn,
                                  const float* t_rho_all, const float* Tm, float* csh, int rk_step) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (ji > D.ny || jk > D.nx) return;
  const int nl = D.nl, NL = D.NL, nc = D.nc;
  const float dt = float(D.dtime);
  const double dtd = D.dtime;
  const float itw = 0.5f, ew = 0.5f;
  const double* rho_g_o = So.rho + (long long)(D.g - 1) * D.fstride;
  float vfi[kMaxL + 1], vfr[kMaxL + 1], vefv[kMaxL + 1], vcl[kMaxL + 1], itv[kMaxL + 1], cpi[kMaxL + 2], cpw[kMaxL + 2];
  double cv[kMaxL + 1], dv[kMaxL + 1], ev[kMaxL + 1], rv[kMaxL + 1], epr[kMaxL + 1], rpr[kMaxL + 1];
  for (int jl = 1; jl <= nl; ++jl) {
    const long long i = IX(D, ji, jk, jl);
    itv[jl] = itw * dt * float(X.inv_volume[i]);
    vcl[jl] = vfall_liquid_f(D, GF, rho_g_o, Tm, 12.e-6f, ji, jk, jl);
    if (jl >= 2) { cpi[jl] = c_p_ice(Tm[i]); cpw[jl] = c_p_water(Tm[i]); }
  }
  for (int jc = 1; jc <= D.ncons; ++jc) {
    if (jc == D.g) continue;
    const double* rho_o = So.rho + (long long)(jc - 1) * D.fstride;
    double* rho_n = Sn.rho + (long long)(jc - 1) * D.fstride;
    const float* t_rho = t_rho_all + (long long)(jc - 1) * D.fstride;
    const bool ice = (jc - 1) % 2 == 0;
    float vsurf = 0.f;
    for (int jl = 1; jl <= nl - 1; ++jl) {
      const long long a = IX(D, ji, jk, jl), b = IX(D, ji, jk, jl + 1);
      if (rk_step == 1 && jc == 1) csh[a] = 0.f;
      float vf = 0.f;
      if (jc == 1) vf = 1.f;               // snow radius 500 um > 250 um
      else if (jc == 3) vf = 0.001f;       // cloud ice
      else if (jc == 4) vf = 0.5f * (vcl[jl] + vcl[jl + 1]);
      const float az = GF.area_z[b];
      vfi[jl] = az * (float(So.w[b]) - vf);
      float fr = az * (float(Sn.w[b]) - vf);
      fr = ((fr >= 0.f) ? float(rho_o[b]) : float(rho_o[a])) * fr;
      vfr[jl] = fr;
      const float toi = Tm[b];
      vefv[jl] = (jc <= nc) ? (ice ? cpi[jl + 1] : cpw[jl + 1]) * toi * fr : 0.f;
    }
    if (rk_step == 1 && jc == 1) csh[IX(D, ji, jk, nl)] = 0.f;
    if (jc == 1) vsurf = 1.f;
    else if (jc == 3) vsurf = 0.001f;
    else if (jc == 4) vsurf = vcl[nl];
    for (int jl = 1; jl <= nl - 1; ++jl) {
      if (vfi[jl] >= 0.f) { cv[jl] = 0.0; ev[jl] = -(double)(itv[jl] * vfi[jl]); }
      else { cv[jl] = (double)(itv[jl + 1] * vfi[jl]); ev[jl] = 0.0; }
    }
    for (int jl = 1; jl <= nl; ++jl) {
      const long long i = IX(D, ji, jk, jl);
      const float iv = float(X.inv_volume[i]);
      float d;
      if (jl == 1) {
        d = (vfi[1] >= 0.f) ? 1.f : 1.f - itv[1] * vfi[1];
      } else if (jl == nl) {
        d = (vfi[jl - 1] >= 0.f) ? 1.f + itv[jl] * vfi[jl - 1] : 1.f;
        if (jc <= nc) d += itw * vsurf * dt * GF.area_z[IX(D, ji, jk, jl + 1)] * iv;
      } else {
        d = 1.f;
        if (vfi[jl - 1] >= 0.f) d += itv[jl] * vfi[jl - 1];
        if (vfi[jl] < 0.f) d -= itv[jl] * vfi[jl];
      }
      dv[jl] = d;
      double r = fma(dtd, (double)t_rho[i], rho_o[i]);
      float fl;
      if (jl == 1) {
        fl = ew * dt * vfr[jl] * iv;
        if (rk_step == 1 && jc <= nc) csh[i] += vefv[jl] * iv;
      } else if (jl == nl) {
        fl = -ew * dt * vfr[jl - 1] * iv;
        if (rk_step == 1 && jc <= nc) csh[i] -= vefv[jl - 1] * iv;
        if (jc <= nc) {
          fl -= ew * vsurf * dt * float(rho_o[i]) * GF.area_z[IX(D, ji, jk, jl + 1)] * iv;
          if (jc > nc / 4 && rk_step == 1) {
            const float Tn = Tm[IX(D, ji, jk, nl)];
            csh[i] -= vsurf * Tn * (ice ? cpi[nl] : cpw[nl]) * float(rho_o[IX(D, ji, jk, nl)]) *
                      GF.area_z[IX(D, ji, jk, NL)] * iv;
          }
        }
      } else {
        fl = ew * dt * (vfr[jl] - vfr[jl - 1]) * iv;
        if (rk_step == 1 && jc <= nc) csh[i] += (vefv[jl] - vefv[jl - 1]) * iv;
      }
      rv[jl] = r + (double)fl;
    }
    // Thomas in FP64, one reciprocal per row
    double id = drcp(dv[1]);
    epr[1] = ev[1] * id;
    rpr[1] = rv[1] * id;
    for (int jl = 2; jl <= nl; ++jl) {
      id = drcp(dv[jl] - epr[jl - 1] * cv[jl - 1]);
      if (jl <= nl - 1) epr[jl] = ev[jl] * id;
      rpr[jl] = (rv[jl] - rpr[jl - 1] * cv[jl - 1]) * id;
    }
    double s = rpr[nl];
    rho_n[IX(D, ji, jk, nl)] = s < 0.0 ? 0.0 : s;
    for (int jl = nl - 1; jl >= 1; --jl) {
      s = rpr[jl] - epr[jl] * s;
      rho_n[IX(D, ji, jk, jl)] = s < 0.0 ? 0.0 : s;
    }
  }
}

dim3 sblk() { return dim3(32, 8, 1); }
dim3 sgrd(int rows, int cols, int levs) {
  return dim3((unsigned)((rows + 31) / 32), (unsigned)((cols + 7) / 8), (unsigned)levs);
}

}  // namespace

int split_create(const Dims& D, SplitCtx** out, long long* bytes) {
  auto* s = new SplitCtx();
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
  float** scratch[] = {&s->th, &s->gx, &s->gy, &s->gz, &s->divf, &s->tvu, &s->tvv, &s->tpu, &s->tpv,
                       &s->ex, &s->ey, &s->ez, &s->uph, &s->vph, &s->wph};
  for (float** p : scratch) if ((rc = salloc(s, p, F, bytes))) return fail(rc);
  if ((rc = salloc(s, &s->vsq, F, bytes))) return fail(rc);
  SplitCarriedF& C = s->C;
  float** car[] = {&C.pgcw, &C.vsg_x, &C.vsg_y, &C.vsg_z, &C.pvt_x, &C.pvt_y, &C.pvt_z, &C.csh, &C.rad, &C.temperature,
                   &C.tend.rt, &C.tend.u, &C.tend.v, &C.tend.w};
  for (float** p : car) if ((rc = salloc(s, p, F, bytes))) return fail(rc);
  if ((rc = salloc(s, &C.tend.rho, F * D.ncons, bytes))) return fail(rc);
  *out = s;
  return LGAME_OK;
}

void split_destroy(SplitCtx* s) {
  if (!s) return;
  for (void* p : s->allocs) cudaFree(p);
  delete s;
}

SplitCarriedF split_carried(SplitCtx* s) { return s->C; }

int split_convert(const double* src, float* dst, long long n, cudaStream_t stream) {
  k_to_float<<<1216, 256, 0, stream>>>(src, dst, n);
  return cudaGetLastError() == cudaSuccess ? LGAME_OK : LGAME_ERR_CUDA;
}
int split_convert_back(const float* src, double* dst, long long n, cudaStream_t stream) {
  k_to_double<<<1216, 256, 0, stream>>>(src, dst, n);
  return cudaGetLastError() == cudaSuccess ? LGAME_OK : LGAME_ERR_CUDA;
}

int split_set_grid(SplitCtx* s, const Dims& D, const Grid<double>& G, cudaStream_t stream) {
  const long long F = D.fstride;
  const double* src[] = {G.z_scalar, G.z_u, G.z_v, G.z_w, G.dx, G.dy, G.dz, G.volume, G.area_x, G.area_y, G.area_z,
                         G.area_dual_x, G.area_dual_y, G.area_dual_z, G.z_area_dual_z, G.slope_x, G.slope_y,
                         G.theta_v_bg, G.exner_bg, G.egu, G.egv, G.egw, G.gm, G.gp, G.fvec_x, G.fvec_y, G.fvec_z,
                         G.damp};
  const int nsrc = sizeof(src) / sizeof(src[0]);
  for (int k = 0; k < nsrc; ++k) {
    const long long n = (src[k] == G.fvec_x || src[k] == G.fvec_y || src[k] == G.fvec_z) ? D.plane : F;
    if (split_convert(src[k], s->gf[k], n, stream)) return LGAME_ERR_CUDA;
  }
  for (int k = 0; k < 6; ++k) if (split_convert(G.ipw[k], s->ipw[k], F, stream)) return LGAME_ERR_CUDA;
  for (int k = 0; k < 3; ++k) if (split_convert(G.trsk_u[k], s->trsk_u[k], D.P, stream)) return LGAME_ERR_CUDA;
  for (int k = 0; k < 2; ++k) if (split_convert(G.trsk_v[k], s->trsk_v[k], D.P, stream)) return LGAME_ERR_CUDA;
  k_recip<<<1216, 256, 0, stream>>>(G.dx, s->inv_dx, F);
  k_recip<<<1216, 256, 0, stream>>>(G.dy, s->inv_dy, F);
  k_recip<<<1216, 256, 0, stream>>>(G.dz, s->inv_dz, F);
  k_recip<<<1216, 256, 0, stream>>>(G.volume, s->inv_volume, F);
  k_recip<<<1216, 256, 0, stream>>>(G.area_z, s->inv_area_z, F);
  if (cudaGetLastError() != cudaSuccess) return LGAME_ERR_CUDA;
  Grid<float>& GF = s->GF;
  float** g = s->gf;
  GF.z_scalar = g[0]; GF.z_u = g[1]; GF.z_v = g[2]; GF.z_w = g[3]; GF.dx = g[4]; GF.dy = g[5]; GF.dz = g[6];
  GF.volume = g[7]; GF.area_x = g[8]; GF.area_y = g[9]; GF.area_z = g[10]; GF.area_dual_x = g[11];
  GF.area_dual_y = g[12]; GF.area_dual_z = g[13]; GF.z_area_dual_z = g[14]; GF.slope_x = g[15]; GF.slope_y = g[16];
  GF.theta_v_bg = g[17]; GF.exner_bg = g[18]; GF.egu = g[19]; GF.egv = g[20]; GF.egw = g[21]; GF.gm = g[22];
  GF.gp = g[23]; GF.fvec_x = g[24]; GF.fvec_y = g[25]; GF.fvec_z = g[26]; GF.damp = g[27];
  for (int k = 0; k < 6; ++k) GF.ipw[k] = s->ipw[k];
  for (int k = 0; k < 3; ++k) GF.trsk_u[k] = s->trsk_u[k];
  for (int k = 0; k < 2; ++k) GF.trsk_v[k] = s->trsk_v[k];
  s->GX = GridX{s->inv_dx, s->inv_dy, s->inv_dz, s->inv_volume, s->inv_area_z};
  return LGAME_OK;
}

int split_step(SplitCtx* s, const Dims& D, const Grid<double>& G, const State& So, const State& Sn,
               const PGrad<double>& pg, int step, cudaStream_t stream, int* nk,
               int (*tb)(void*, const char*), void (*te)(void*, int), void* tracer) {
  const Grid<float>& GF = s->GF;
  const SplitCarriedF& C = s->C;
  const Tend<float> T = C.tend;
  int launches = 0;
#define SL(name, kernel, grid_, ...)                                            \
  do {                                                                          \
    const int tr_ = tb ? tb(tracer, name) : -1;                                 \
    kernel<<<grid_, sblk(), 0, stream>>>(__VA_ARGS__);                          \
    if (tr_ >= 0) te(tracer, tr_);                                              \
    cudaError_t e_ = cudaGetLastError();                                        \
    if (e_ != cudaSuccess) {                                                    \
      lgame_set_error((std::string("launch of ") + name + ": " + cudaGetErrorString(e_)).c_str()); \
      return LGAME_ERR_CUDA;                                                    \
    }                                                                           \
    ++launches;                                                                 \
  } while (0)
  auto theta3f = [&](const double* tp, int mode, const double* u, const double* v, float* ou, float* ov) -> int {
    SL("ks_theta", k_theta<float>, sgrd(D.ny, D.nx, D.nl), D, GF, tp, s->th, mode);
    SL("ks_grad_vert", (k_grad_vert<float, float>), sgrd(D.ny, D.nx, D.nl - 1), D, GF, s->th, s->gz);
    SL("ks_grad_hor", (k_grad_hor<float, float>), sgrd(D.ny + 1, D.nx + 1, D.nl), D, GF, s->th, s->gz, s->gx, s->gy);
    SL("ks_div_h", k_div_h<float>, sgrd(D.ny, D.nx, D.nl), D, GF, s->gx, s->gy, s->divf);
    SL("ks_theta_edges", k_theta_edges<float>, sgrd(D.ny + 1, D.nx + 1, D.nl), D, GF, s->th, s->divf, u, v, ou, ov);
    return LGAME_OK;
  };
  SL("ks_temperature", k_temperature<float>, sgrd(D.ny, D.nx, D.nl), D, GF, So, C.temperature);
  Carried<float> CC{pg.nl_u, pg.nl_v, pg.nl_w, pg.l_u, pg.l_v, pg.l_w, pg.old_u, pg.old_v, C.pgcw,
                    C.vsg_x, C.vsg_y, C.vsg_z, C.pvt_x, C.pvt_y, C.pvt_z};
  for (int rk = 1; rk <= 2; ++rk) {
    const State& Sv = (rk == 1) ? So : Sn;
    if (rk == 1) {
      if (D.theta_order == 3) {
        int rc = theta3f(So.tp, 0, So.u, So.v, s->tvu, s->tvv);
        if (rc) return rc;
        if (D.luse_bg) { rc = theta3f(So.tp, 1, So.u, So.v, s->tpu, s->tpv); if (rc) return rc; }
      }
      SL("ks_pgrad", ks_pgrad, sgrd(D.ny + 1, D.nx + 1, D.nl), D, G, s->GX, So, s->tvu, s->tvv, s->tpu, s->tpv, pg,
         C.pgcw, step == 0 ? 1 : 0);
    }
    if ((rk == 2 || step == 0) && (!D.llinear || D.lcorio)) {
      SL("ks_eta_xy", k_eta_xy<float>, sgrd(D.ny + 1, D.nx + 1, D.NL), D, GF, Sv, s->ex, s->ey);
      SL("ks_eta_z", k_eta_z<float>, sgrd(D.ny + 1, D.nx + 1, D.nl), D, GF, Sv, s->ez);
      SL("ks_mass_flux", k_mass_flux<float>, sgrd(D.ny + 1, D.nx + 1, D.nl), D, GF, Sv, s->uph, s->vph, s->wph);
      SL("ks_vort_flux", k_vort_flux<float>, sgrd(D.ny + 1, D.nx + 1, D.nl), D, GF, Sv, s->ex, s->ey, s->ez, s->uph,
         s->vph, s->wph, C.pvt_x, C.pvt_y, C.pvt_z);
      if (!D.llinear) {
        SL("ks_ke", k_ke<double>, sgrd(D.ny, D.nx, D.nl), D, G, Sv, s->vsq);
        SL("ks_grad_vert", (k_grad_vert<float, double>), sgrd(D.ny, D.nx, D.nl - 1), D, GF, s->vsq, C.vsg_z);
        SL("ks_grad_hor", (k_grad_hor<float, double>), sgrd(D.ny + 1, D.nx + 1, D.nl), D, GF, s->vsq, C.vsg_z,
           C.vsg_x, C.vsg_y);
      }
    }
    SL("ks_tend_wind", k_tend_wind<float>, sgrd(D.ny + 1, D.nx + 1, D.NL), D, So, Sn, T, CC, rk);
    const State& Ss = (rk == 1) ? So : Sn;
    if (D.ncons > 1) SL("ks_tracers", k_tracers<float>, sgrd(D.ny, D.nx, D.nl), D, GF, Ss, Sn.u, Sn.v, T.rho, rk);
    if (D.theta_order == 3) {
      int rc = theta3f(Ss.tp, 0, Ss.u, Ss.v, s->tvu, s->tvv);
      if (rc) return rc;
    }
    SL("ks_gas_theta", k_gas_theta<float>, sgrd(D.ny, D.nx, D.nl), D, GF, Ss, Sn.u, Sn.v, s->tvu, s->tvv,
       C.temperature, C.rad, C.csh, T.rho, T.rt);
    const dim3 g2 = sgrd(D.ny, D.nx, 1);
    SL("ks_column_ver", ks_column_ver, g2, D, G, s->GX, So, Sn, T, rk);
    if (D.ncons > 1)
      SL("ks_column_tracers", ks_column_tracers, g2, D, G, GF, s->GX, So, Sn, T.rho, C.temperature, C.csh, rk);
  }
#undef SL
  *nk = launches;
  return LGAME_OK;
}

}  // namespace lg
