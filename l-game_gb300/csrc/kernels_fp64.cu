// kernels_fp64.cu -- the FP64 pressure-gradient kernel of the HEVI step (compiled with
// -fmad=false).  The other explicit kernels are templates in kernels.cuh, instantiated
// for double by lgame_gpu.cu (same compiler flags).
#include "kernels.cuh"

namespace lg {

// manage_p_grad, mo_p_grad.F90:20-104, after the gradients of exner_pert (gx,gy,gz)
// and, for theta_adv_order 3, the edge values of theta (tvu,tvv) and theta' (tpu,tpv)
// are known; also calc_p_grad_condensates_v, mo_p_grad.F90:106-120 (identical at both
// substeps because it always reads state_old).
__global__ void k_pgrad(Dims D, Grid<double> G, State S, const double* gx, const double* gy, const double* gz,
                        const double* tvu, const double* tvv, const double* tpu, const double* tpv,
                        PGrad<double> P, int lfirst) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.y + 1;
  const double use_bg_switch = D.luse_bg ? 1.0 : 0.0;
  auto theta = [&](int i, int j, int k) { const long long q = IX(D, i, j, k); return G.theta_v_bg[q] + S.tp[q]; };
  auto thetap = [&](int i, int j, int k) { return S.tp[IX(D, i, j, k)]; };
  auto decel = [&](int i, int j, int k) {
    const long long q = IX(D, i, j, k);
    return kC_D_P * S.rho[q + (long long)(D.g - 1) * D.fstride] / rho_sum_cond_gas<double>(D, S.rho, q);
  };
  // u points.  Periodic jk = nx+1 ends as a copy of jk = 1 (scalar_times_vector_h2
  // copies it last), so it is evaluated from column 1.  Non-periodic boundary edges stay
  // at their initial zero in every array of the reference (no operator writes them and
  // whole-array products multiply zeros), so only p_grad_acc_old is refreshed there.
  if (jl <= D.nl && ji <= D.ny && jk <= D.nx + 1) {
    const long long q = IX(D, ji, jk, jl);
    const bool inner = jk >= 2 && jk <= D.nx;
    const double nl_prev = P.nl_u[q], l_prev = P.l_u[q];
    if (!lfirst) P.old_u[q] = -nl_prev - use_bg_switch * l_prev;
    if (inner || D.periodic) {
      const int kk = inner ? jk : 1;
      const int ka = inner ? jk - 1 : D.nx, kb = kk;
      const long long qr = IX(D, ji, kk, jl);
      double nlv = gx[qr];
      if (D.theta_order == 2) nlv = 0.5 * (theta(ji, ka, jl) + theta(ji, kb, jl)) * nlv;
      else nlv = tvu[qr] * nlv;
      double lv = l_prev;
      if (D.luse_bg) {
        if (D.theta_order == 2) lv = 0.5 * (thetap(ji, ka, jl) + thetap(ji, kb, jl)) * G.egu[qr];
        else lv = tpu[qr] * G.egu[qr];
      }
      const double de = 0.5 * (decel(ji, ka, jl) + decel(ji, kb, jl));
      nlv = de * nlv;
      if (D.luse_bg) lv = de * lv;
      P.nl_u[q] = nlv;
      if (D.luse_bg) P.l_u[q] = lv;
      if (lfirst) P.old_u[q] = -nlv - use_bg_switch * lv;
    } else if (lfirst) {
      P.old_u[q] = -nl_prev - use_bg_switch * l_prev;
    }
  }
  // v points (periodic ji = ny+1 from row 1)
  if (jl <= D.nl && ji <= D.ny + 1 && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    const bool inner = ji >= 2 && ji <= D.ny;
    const double nl_prev = P.nl_v[q], l_prev = P.l_v[q];
    if (!lfirst) P.old_v[q] = -nl_prev - use_bg_switch * l_prev;
    if (inner || D.periodic) {
      const int ii = inner ? ji : 1;
      const int ia = inner ? ji - 1 : 1, ib = inner ? ji : D.ny;  // periodic: s(1)+s(ny)
      const long long qr = IX(D, ii, jk, jl);
      double nlv = gy[qr];
      if (D.theta_order == 2) nlv = 0.5 * (theta(ia, jk, jl) + theta(ib, jk, jl)) * nlv;
      else nlv = tvv[qr] * nlv;
      double lv = l_prev;
      if (D.luse_bg) {
        if (D.theta_order == 2) lv = 0.5 * (thetap(ia, jk, jl) + thetap(ib, jk, jl)) * G.egv[qr];
        else lv = tpv[qr] * G.egv[qr];
      }
      const double de = 0.5 * (decel(ia, jk, jl) + decel(ib, jk, jl));
      nlv = de * nlv;
      if (D.luse_bg) lv = de * lv;
      P.nl_v[q] = nlv;
      if (D.luse_bg) P.l_v[q] = lv;
      if (lfirst) P.old_v[q] = -nlv - use_bg_switch * lv;
    } else if (lfirst) {
      P.old_v[q] = -nl_prev - use_bg_switch * l_prev;
    }
  }
  // w points, levels 2..nl
  if (jl >= 2 && jl <= D.nl && ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    double nlv = 0.5 * (theta(ji, jk, jl - 1) + theta(ji, jk, jl)) * gz[q];
    const double de = 0.5 * (decel(ji, jk, jl - 1) + decel(ji, jk, jl));
    nlv = de * nlv;
    P.nl_w[q] = nlv;
    if (D.luse_bg) {
      double lv = 0.5 * (thetap(ji, jk, jl - 1) + thetap(ji, jk, jl)) * G.egw[q];
      P.l_w[q] = de * lv;
    }
    // p_grad_condensates_w
    const long long qa = IX(D, ji, jk, jl - 1);
    const double da = S.rho[qa + (long long)(D.g - 1) * D.fstride] / rho_sum_cond_gas<double>(D, S.rho, qa) - 1.0;
    const double db = S.rho[q + (long long)(D.g - 1) * D.fstride] / rho_sum_cond_gas<double>(D, S.rho, q) - 1.0;
    P.pgcw[q] = 0.5 * (da + db) * G.gm[q];
  }
}

}  // namespace lg
