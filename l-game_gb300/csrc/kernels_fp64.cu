// kernels_fp64.cu -- FP64 kernels of the HEVI step (compiled with -fmad=false).
//
// Each kernel evaluates, for the points it owns, the same expressions as the reference
// loop bodies cited beside it; inputs that the reference reads from a scratch array
// (scalar_placeholder, flux_density_u, ...) are recomputed inline with the identical
// expression, which yields identical bits.  Boundary points that the reference leaves
// untouched in the non-periodic case are not written here either (device buffers start
// at zero like the reference's arrays, src/control.F90:274-444).
#include "kernels.cuh"

namespace lg {

// ---- temperature_diagnostics, mo_derived.F90:18-38 ----------------------------
__global__ void k_temperature(Dims D, Grid<double> G, State S, double* T) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  if (ji > D.ny || jk > D.nx) return;
  const long long i = IX(D, ji, jk, jl);
  double t = (G.theta_v_bg[i] + S.tp[i]) * (G.exner_bg[i] + S.ep[i]);
  if (D.lmoist) {
    const double rg = S.rho[i + (long long)(D.g - 1) * D.fstride];
    const double rv = S.rho[i + (long long)D.g * D.fstride];
    t = t / (1.0 + rv / rg * (kM_D / kM_V - 1.0));
  }
  T[i] = t;
}

// diag%scalar_placeholder = theta_v_bg + theta_v_pert (mode 0) or theta_v_pert (mode 1)
__global__ void k_theta(Dims D, Grid<double> G, const double* tp, double* out, int mode) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  if (ji > D.ny || jk > D.nx) return;
  const long long i = IX(D, ji, jk, jl);
  out[i] = mode == 0 ? G.theta_v_bg[i] + tp[i] : tp[i];
}

// grad_vert, mo_gradient_operators.F90:65-83 (levels 2..nl)
__global__ void k_grad_vert(Dims D, Grid<double> G, const double* s, double* rz) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 2;
  if (ji > D.ny || jk > D.nx || jl > D.nl) return;
  rz[IX(D, ji, jk, jl)] = (s[IX(D, ji, jk, jl - 1)] - s[IX(D, ji, jk, jl)]) / G.dz[IX(D, ji, jk, jl)];
}

// grad_hor, mo_gradient_operators.F90:17-63 + :85-130, u and v points of layer jl
__global__ void k_grad_hor(Dims D, Grid<double> G, const double* s, const double* rz, double* rx, double* ry) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  if (ji <= D.ny && jk <= D.nx + 1) {
    double r;
    if (grad_x_cov(D, G, s, ji, jk, jl, &r)) {
      if (jl > D.nf) r = r - G.slope_x[IX(D, ji, jk, jl)] * remap_x<double, double>(D, G, rz, ji, jk, jl);
      rx[IX(D, ji, jk, jl)] = r;
    }
  }
  if (ji <= D.ny + 1 && jk <= D.nx) {
    double r;
    if (grad_y_cov(D, G, s, ji, jk, jl, &r)) {
      if (jl > D.nf) r = r - G.slope_y[IX(D, ji, jk, jl)] * remap_y<double, double>(D, G, rz, ji, jk, jl);
      ry[IX(D, ji, jk, jl)] = r;
    }
  }
}

// div_h, mo_divergence_operators.F90:16-68
__global__ void k_div_h(Dims D, Grid<double> G, const double* vx, const double* vy, double* out) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  if (ji > D.ny || jk > D.nx) return;
  auto fx = [&](int i, int j, int k) { return vx[IX(D, i, j, k)]; };
  auto fy = [&](int i, int j, int k) { return vy[IX(D, i, j, k)]; };
  out[IX(D, ji, jk, jl)] = div_h_at<double>(D, G, fx, fy, ji, jk, jl);
}

// theta_v_adv_3rd_order edge values, mo_multiplications.F90:134-202
__global__ void k_theta_edges(Dims D, Grid<double> G, const double* th, const double* Dv,
                              const double* u, const double* v, double* tvu, double* tvv) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  const double c = 1.0 / 8.0 * D.dyn * D.dxn;
  if (ji <= D.ny && jk <= D.nx + 1) {
    double t;
    if (theta_edge_u(D, th, Dv, u, c, ji, jk, jl, &t)) tvu[IX(D, ji, jk, jl)] = t;
  }
  if (ji <= D.ny + 1 && jk <= D.nx) {
    double t;
    if (theta_edge_v(D, th, Dv, v, c, ji, jk, jl, &t)) tvv[IX(D, ji, jk, jl)] = t;
  }
}

// manage_p_grad, mo_p_grad.F90:20-104, after the gradients of exner_pert (gx,gy,gz)
// and, for theta_adv_order 3, the edge values of theta (tvu,tvv) and theta' (tpu,tpv)
// are known; also calc_p_grad_condensates_v, mo_p_grad.F90:106-120 (identical at both
// substeps because it always reads state_old).
__global__ void k_pgrad(Dims D, Grid<double> G, State S, const double* gx, const double* gy, const double* gz,
                        const double* tvu, const double* tvv, const double* tpu, const double* tpv,
                        PGrad P, int lfirst) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  const double use_bg_switch = D.luse_bg ? 1.0 : 0.0;
  auto theta = [&](int i, int j, int k) { const long long q = IX(D, i, j, k); return G.theta_v_bg[q] + S.tp[q]; };
  auto thetap = [&](int i, int j, int k) { return S.tp[IX(D, i, j, k)]; };
  auto decel = [&](int i, int j, int k) {
    const long long q = IX(D, i, j, k);
    return kC_D_P * S.rho[q + (long long)(D.g - 1) * D.fstride] / rho_sum_cond_gas(D, S.rho, q);
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
    const double da = S.rho[qa + (long long)(D.g - 1) * D.fstride] / rho_sum_cond_gas(D, S.rho, qa) - 1.0;
    const double db = S.rho[q + (long long)(D.g - 1) * D.fstride] / rho_sum_cond_gas(D, S.rho, q) - 1.0;
    P.pgcw[q] = 0.5 * (da + db) * G.gm[q];
  }
}

// calc_pot_vort, mo_vorticities.F90:189-421 with rel_vort :19-187 inlined:
// eta_x (ny+1,nx,nl+1) and eta_y (ny,nx+1,nl+1)
__global__ void k_eta_xy(Dims D, Grid<double> G, State S, double* ex, double* ey) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  if (jl > D.NL) return;
  if (ji <= D.ny + 1 && jk <= D.nx) ex[IX(D, ji, jk, jl)] = eta_x_at(D, G, S, ji, jk, jl);
  if (ji <= D.ny && jk <= D.nx + 1) ey[IX(D, ji, jk, jl)] = eta_y_at(D, G, S, ji, jk, jl);
}

// eta_z (ny+1,nx+1,nl)
__global__ void k_eta_z(Dims D, Grid<double> G, State S, double* ez) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  if (ji > D.ny + 1 || jk > D.nx + 1) return;
  ez[IX(D, ji, jk, jl)] = eta_z_at(D, G, S, ji, jk, jl);
}

// mass flux densities, mo_vector_tend_expl.F90:64-66 (scalar_times_vector_h/_v)
__global__ void k_mass_flux(Dims D, Grid<double> G, State S, double* uph, double* vph, double* wph) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  const double* rg = S.rho + (long long)(D.g - 1) * D.fstride;
  if (jl <= D.nl && ji <= D.ny && jk <= D.nx + 1) {
    double f;
    if (stv_h_x(D, rg, S.u, ji, jk, jl, &f)) uph[IX(D, ji, jk, jl)] = f;
  }
  if (jl <= D.nl && ji <= D.ny + 1 && jk <= D.nx) {
    double f;
    if (stv_h_y(D, rg, S.v, ji, jk, jl, &f)) vph[IX(D, ji, jk, jl)] = f;
  }
  if (jl >= 2 && jl <= D.nl && ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    wph[q] = 0.5 * (rg[IX(D, ji, jk, jl - 1)] + rg[q]) * S.w[q];
  }
}

// calc_vorticity_flux_term, mo_vorticity_flux.F90:16-171
__global__ void k_vort_flux(Dims D, Grid<double> G, State S, const double* ex, const double* ey, const double* ez,
                            const double* uph, const double* vph, const double* wph,
                            double* px, double* py, double* pz) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  // vertical mass flux with the free-slip surface value, mo_vector_tend_expl.F90:68-80
  auto wp = [&](int i, int j, int k) -> double {
    if (k == D.NL) {
      if (!D.freeslip) return 0.0;
      const double* rg = S.rho + (long long)(D.g - 1) * D.fstride;
      const double dv = rg[IX(D, i, j, D.nl)] + (rg[IX(D, i, j, D.nl - 1)] - rg[IX(D, i, j, D.nl)])
                        / (G.z_scalar[IX(D, i, j, D.nl - 1)] - G.z_scalar[IX(D, i, j, D.nl)])
                        * (G.z_w[IX(D, i, j, D.NL)] - G.z_scalar[IX(D, i, j, D.nl)]);
      return dv * S.w[IX(D, i, j, D.NL)];
    }
    return wph[IX(D, i, j, k)];
  };
  if (jl <= D.nl && ji <= D.ny && jk <= D.nx + 1) {
    const bool inner = jk >= 2 && jk <= D.nx;
    if (inner || D.periodic) {
      const int kk = inner ? jk : 1, km = inner ? jk - 1 : D.nx, kp = kk + 1;
      double r = trsk_u(D, G, vph, uph, ez, ji, km, kk, kp, jl);
      r = r - 0.5 * W_(5, ji, km, jl) * wp(ji, km, jl) * ey[IX(D, ji, kk, jl)]
            - 0.5 * W_(6, ji, km, jl) * wp(ji, km, jl + 1) * ey[IX(D, ji, kk, jl + 1)]
            - 0.5 * W_(5, ji, kk, jl) * wp(ji, kk, jl) * ey[IX(D, ji, kk, jl)]
            - 0.5 * W_(6, ji, kk, jl) * wp(ji, kk, jl + 1) * ey[IX(D, ji, kk, jl + 1)];
      px[IX(D, ji, jk, jl)] = r;
    }
  }
  if (jl <= D.nl && ji <= D.ny + 1 && jk <= D.nx) {
    const bool inner = ji >= 2 && ji <= D.ny;
    if (inner || D.periodic) {
      const int ii = inner ? ji : 1, im = inner ? ji - 1 : D.ny;
      double r = trsk_v(D, G, uph, ez, im, ii, jk, jl);
      r = r + 0.5 * W_(5, im, jk, jl) * wp(im, jk, jl) * ex[IX(D, ii, jk, jl)]
            + 0.5 * W_(6, im, jk, jl) * wp(im, jk, jl + 1) * ex[IX(D, ii, jk, jl + 1)]
            + 0.5 * W_(5, ii, jk, jl) * wp(ii, jk, jl) * ex[IX(D, ii, jk, jl)]
            + 0.5 * W_(6, ii, jk, jl) * wp(ii, jk, jl + 1) * ex[IX(D, ii, jk, jl + 1)];
      py[IX(D, ji, jk, jl)] = r;
    }
  }
  if (jl >= 2 && jl <= D.nl && ji <= D.ny && jk <= D.nx) {
    pz[IX(D, ji, jk, jl)] = 0.5 * (
        W_(1, ji, jk, jl - 1) * uph[IX(D, ji, jk + 1, jl - 1)] * ey[IX(D, ji, jk + 1, jl)]
      - W_(2, ji, jk, jl - 1) * vph[IX(D, ji, jk, jl - 1)] * ex[IX(D, ji, jk, jl)]
      + W_(3, ji, jk, jl - 1) * uph[IX(D, ji, jk, jl - 1)] * ey[IX(D, ji, jk, jl)]
      - W_(4, ji, jk, jl - 1) * vph[IX(D, ji + 1, jk, jl - 1)] * ex[IX(D, ji + 1, jk, jl)]
      + W_(1, ji, jk, jl) * uph[IX(D, ji, jk + 1, jl)] * ey[IX(D, ji, jk + 1, jl)]
      - W_(2, ji, jk, jl) * vph[IX(D, ji, jk, jl)] * ex[IX(D, ji, jk, jl)]
      + W_(3, ji, jk, jl) * uph[IX(D, ji, jk, jl)] * ey[IX(D, ji, jk, jl)]
      - W_(4, ji, jk, jl) * vph[IX(D, ji + 1, jk, jl)] * ex[IX(D, ji + 1, jk, jl)]);
  }
}

// inner_product of the wind with itself, mo_inner_product.F90:16-50
__global__ void k_ke(Dims D, Grid<double> G, State S, double* out) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  if (ji > D.ny || jk > D.nx) return;
  out[IX(D, ji, jk, jl)] = inner_product_at(D, G, S.u, S.v, S.w, ji, jk, jl);
}

// combination of the explicit wind tendencies, mo_vector_tend_expl.F90:258-310, and the
// forward step of the horizontal wind, mo_manage_pchevi.F90:86-89
__global__ void k_tend_wind(Dims D, State So, State Sn, Tend Tn, Carried C, int rk_step) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  const double new_weight = (rk_step == 2) ? 0.5 : 1.0;
  const double old_weight = 1.0 - new_weight;
  const double chw = 0.5 + kIMPL_THERMO_WEIGHT;
  const double ohw = 1.0 - chw;
  const double cvw = 1.0 - kIMPL_THERMO_WEIGHT;
  const double no_bg_switch = D.luse_bg ? 0.0 : 1.0;
  if (jl <= D.nl && ji <= D.ny && jk <= D.nx + 1) {
    const long long q = IX(D, ji, jk, jl);
    const double t = old_weight * Tn.u[q] + new_weight * (ohw * C.old_u[q] - chw * (C.nl_u[q] + C.l_u[q])
                     - 0.5 * C.vsg_x[q] + C.pvt_x[q]);
    Tn.u[q] = t;
    Sn.u[q] = So.u[q] + D.dtime * t;
  }
  if (jl <= D.nl && ji <= D.ny + 1 && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    const double t = old_weight * Tn.v[q] + new_weight * (ohw * C.old_v[q] - chw * (C.nl_v[q] + C.l_v[q])
                     - 0.5 * C.vsg_y[q] + C.pvt_y[q]);
    Tn.v[q] = t;
    Sn.v[q] = So.v[q] + D.dtime * t;
  }
  if (jl <= D.NL && ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    Tn.w[q] = old_weight * Tn.w[q] + new_weight * (-(cvw * (C.nl_w[q] + C.l_w[q]))
              - no_bg_switch * (1.0 - cvw) * C.l_w[q] - 0.5 * C.vsg_z[q] + C.pvt_z[q] + C.pgcw[q]);
  }
}

// scalar_tend_expl for every constituent other than the gas, mo_scalar_tend_expl.F90:102-128
// with scalar_times_vector_h_upstream (mo_multiplications.F90:206-287) and div_h_tracers
// (mo_divergence_operators.F90:70-147) evaluated inline.
__global__ void k_tracers(Dims D, Grid<double> G, State Ss, const double* u_new, const double* v_new,
                          double* t_rho, int rk_step) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl);
  auto wx = [&](int i, int j, int k) { return u_new[IX(D, i, j, k)]; };
  auto wy = [&](int i, int j, int k) { return v_new[IX(D, i, j, k)]; };
  // contravariant vertical velocity corrections do not depend on the constituent
  double cu = 0.0, cl = 0.0;
  if (jl == D.nf) cl = vcc<double>(D, G, wx, wy, ji, jk, jl + 1);
  else if (jl == D.nl) cu = vcc<double>(D, G, wx, wy, ji, jk, jl);
  else if (jl > D.nf) { cu = vcc<double>(D, G, wx, wy, ji, jk, jl); cl = vcc<double>(D, G, wx, wy, ji, jk, jl + 1); }
  const double new_weight = (rk_step == 2) ? 0.5 : 1.0;
  const double old_weight = 1.0 - new_weight;
  for (int jc = 1; jc <= D.ncons; ++jc) {
    if (jc == D.g) continue;
    const double* r = Ss.rho + (long long)(jc - 1) * D.fstride;
    auto fx = [&](int i, int j, int k) { double f; return upstream_x(D, r, u_new, i, j, k, &f) ? f : 0.0; };
    auto fy = [&](int i, int j, int k) { double f; return upstream_y(D, r, v_new, i, j, k, &f) ? f : 0.0; };
    const double comp_h = fx(ji, jk + 1, jl) * G.area_x[IX(D, ji, jk + 1, jl)]
                        + fy(ji, jk, jl) * G.area_y[IX(D, ji, jk, jl)]
                        - fx(ji, jk, jl) * G.area_x[IX(D, ji, jk, jl)]
                        - fy(ji + 1, jk, jl) * G.area_y[IX(D, ji + 1, jk, jl)];
    double comp_v = 0.0;
    if (jl == D.nf) {
      const double dl = (cl <= 0.0) ? r[IX(D, ji, jk, jl)] : r[IX(D, ji, jk, jl + 1)];
      comp_v = -dl * cl * G.area_z[IX(D, ji, jk, jl + 1)];
    } else if (jl == D.nl) {
      const double du = (cu <= 0.0) ? r[IX(D, ji, jk, jl - 1)] : r[IX(D, ji, jk, jl)];
      comp_v = du * cu * G.area_z[IX(D, ji, jk, jl)];
    } else if (jl > D.nf) {
      const double du = (cu <= 0.0) ? r[IX(D, ji, jk, jl - 1)] : r[IX(D, ji, jk, jl)];
      const double dl = (cl <= 0.0) ? r[IX(D, ji, jk, jl)] : r[IX(D, ji, jk, jl + 1)];
      comp_v = du * cu * G.area_z[IX(D, ji, jk, jl)] - dl * cl * G.area_z[IX(D, ji, jk, jl + 1)];
    }
    const double div = (comp_h + comp_v) / G.volume[q];
    double* t = t_rho + (long long)(jc - 1) * D.fstride;
    t[q] = old_weight * t[q] + new_weight * (-div);
  }
}

// scalar_tend_expl for the gas and the rho*theta_v tendency, mo_scalar_tend_expl.F90:106-177
__global__ void k_gas_theta(Dims D, Grid<double> G, State Ss, const double* u_new, const double* v_new,
                            const double* tvu, const double* tvv, const double* T, const double* rad,
                            const double* csh, double* t_rho, double* t_rt) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.z + 1;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl);
  const double* rg = Ss.rho + (long long)(D.g - 1) * D.fstride;
  auto fx = [&](int i, int j, int k) { double f; return stv_h_x(D, rg, u_new, i, j, k, &f) ? f : 0.0; };
  auto fy = [&](int i, int j, int k) { double f; return stv_h_y(D, rg, v_new, i, j, k, &f) ? f : 0.0; };
  const double div_m = div_h_at<double>(D, G, fx, fy, ji, jk, jl);
  t_rho[q + (long long)(D.g - 1) * D.fstride] = -div_m;  // old_weight 0, new_weight 1 for the gas
  double div_t;
  if (D.theta_order == 2) {
    auto th = [&](int i, int j, int k) { const long long p = IX(D, i, j, k); return G.theta_v_bg[p] + Ss.tp[p]; };
    auto gx = [&](int i, int j, int k) { double f; return stv_h_x_fn(D, th, fx, i, j, k, &f) ? f : 0.0; };
    auto gy = [&](int i, int j, int k) { double f; return stv_h_y_fn(D, th, fy, i, j, k, &f) ? f : 0.0; };
    div_t = div_h_at<double>(D, G, gx, gy, ji, jk, jl);
  } else {
    auto gx = [&](int i, int j, int k) { return tvu[IX(D, i, j, k)] * fx(i, j, k); };
    auto gy = [&](int i, int j, int k) { return tvv[IX(D, i, j, k)] * fy(i, j, k); };
    div_t = div_h_at<double>(D, G, gx, gy, ji, jk, jl);
  }
  const double heat = rad[q] + csh[q];
  double x = 0.0;
  if (heat != 0.0) {
    const double cv = c_v_mass_weighted_air(D, Ss.rho, T, q);
    x = kC_D_V * rg[q] / cv * heat / (kC_D_P * (G.exner_bg[q] + Ss.ep[q]));
  }
  t_rt[q] = -div_t + x;
}

}  // namespace lg
