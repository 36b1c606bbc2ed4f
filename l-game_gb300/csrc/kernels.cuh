// kernels.cuh -- pointwise helpers and kernel declarations of the FP64 HEVI step.
#pragma once

#include "dev.cuh"

namespace lg {

struct PGrad {  // pressure-gradient arrays of t_diag (mo_definitions.F90:137-146)
  double *nl_u, *nl_v, *nl_w, *l_u, *l_v, *l_w, *old_u, *old_v, *pgcw;
};

struct Tend {  // t_tend (mo_definitions.F90:108-116)
  double *rho, *rt, *u, *v, *w;
};

struct Carried {  // read-only view of the diagnostics combined into the wind tendency
  const double *nl_u, *nl_v, *nl_w, *l_u, *l_v, *l_w, *old_u, *old_v, *pgcw;
  const double *vsg_x, *vsg_y, *vsg_z, *pvt_x, *pvt_y, *pvt_z;
};

// ---- edge operators with the reference's boundary branches --------------------
// Each returns false where the reference leaves the output point untouched
// (non-periodic boundary edges); periodic jk=nx+1 / ji=ny+1 evaluate the copy source.

// grad_hor_cov x-component at a u point, mo_gradient_operators.F90:33-52
__device__ __forceinline__ bool grad_x_cov(const Dims& D, const Grid<double>& G, const double* s, int ji, int jk, int jl, double* r) {
  if (jk >= 2 && jk <= D.nx) {
    *r = (s[IX(D, ji, jk, jl)] - s[IX(D, ji, jk - 1, jl)]) / G.dx[IX(D, ji, jk, jl)];
    return true;
  }
  if (!D.periodic) return false;
  *r = (s[IX(D, ji, 1, jl)] - s[IX(D, ji, D.nx, jl)]) / G.dx[IX(D, ji, 1, jl)];
  return true;
}

// grad_hor_cov y-component at a v point, mo_gradient_operators.F90:39-60
__device__ __forceinline__ bool grad_y_cov(const Dims& D, const Grid<double>& G, const double* s, int ji, int jk, int jl, double* r) {
  if (ji >= 2 && ji <= D.ny) {
    *r = (s[IX(D, ji - 1, jk, jl)] - s[IX(D, ji, jk, jl)]) / G.dy[IX(D, ji, jk, jl)];
    return true;
  }
  if (!D.periodic) return false;
  *r = (s[IX(D, D.ny, jk, jl)] - s[IX(D, 1, jk, jl)]) / G.dy[IX(D, 1, jk, jl)];
  return true;
}

// theta_v_adv_3rd_order x edge, mo_multiplications.F90:136-183
__device__ __forceinline__ bool theta_edge_u(const Dims& D, const double* th, const double* Dv, const double* u,
                                             double c, int ji, int jk, int jl, double* out) {
  if (jk >= 2 && jk <= D.nx) {
    double t = 0.5 * (th[IX(D, ji, jk - 1, jl)] + th[IX(D, ji, jk, jl)]);
    if (u[IX(D, ji, jk, jl)] >= 0.0) t = t - c * Dv[IX(D, ji, jk - 1, jl)];
    else t = t - c * Dv[IX(D, ji, jk, jl)];
    *out = t;
    return true;
  }
  if (!D.periodic) return false;
  double t = 0.5 * (th[IX(D, ji, D.nx, jl)] + th[IX(D, ji, 1, jl)]);
  if (u[IX(D, ji, 1, jl)] >= 0.0) t = t - c * Dv[IX(D, ji, D.nx, jl)];
  else t = t - c * Dv[IX(D, ji, 1, jl)];
  *out = t;
  return true;
}

// theta_v_adv_3rd_order y edge, mo_multiplications.F90:152-200
__device__ __forceinline__ bool theta_edge_v(const Dims& D, const double* th, const double* Dv, const double* v,
                                             double c, int ji, int jk, int jl, double* out) {
  if (ji >= 2 && ji <= D.ny) {
    double t = 0.5 * (th[IX(D, ji, jk, jl)] + th[IX(D, ji - 1, jk, jl)]);
    if (v[IX(D, ji, jk, jl)] >= 0.0) t = t - c * Dv[IX(D, ji, jk, jl)];
    else t = t - c * Dv[IX(D, ji - 1, jk, jl)];
    *out = t;
    return true;
  }
  if (!D.periodic) return false;
  double t = 0.5 * (th[IX(D, 1, jk, jl)] + th[IX(D, D.ny, jk, jl)]);
  if (v[IX(D, 1, jk, jl)] >= 0.0) t = t - c * Dv[IX(D, 1, jk, jl)];
  else t = t - c * Dv[IX(D, D.ny, jk, jl)];
  *out = t;
  return true;
}

// scalar_times_vector_h x-component, mo_multiplications.F90:34-54
__device__ __forceinline__ bool stv_h_x(const Dims& D, const double* s, const double* vx, int ji, int jk, int jl, double* r) {
  if (jk >= 2 && jk <= D.nx) {
    *r = 0.5 * (s[IX(D, ji, jk - 1, jl)] + s[IX(D, ji, jk, jl)]) * vx[IX(D, ji, jk, jl)];
    return true;
  }
  if (!D.periodic) return false;
  *r = 0.5 * (s[IX(D, ji, 1, jl)] + s[IX(D, ji, D.nx, jl)]) * vx[IX(D, ji, 1, jl)];
  return true;
}
__device__ __forceinline__ bool stv_h_y(const Dims& D, const double* s, const double* vy, int ji, int jk, int jl, double* r) {
  if (ji >= 2 && ji <= D.ny) {
    *r = 0.5 * (s[IX(D, ji - 1, jk, jl)] + s[IX(D, ji, jk, jl)]) * vy[IX(D, ji, jk, jl)];
    return true;
  }
  if (!D.periodic) return false;
  *r = 0.5 * (s[IX(D, 1, jk, jl)] + s[IX(D, D.ny, jk, jl)]) * vy[IX(D, 1, jk, jl)];
  return true;
}
// the same with the scalar and the vector given as functions of the index
template <class FS, class FV>
__device__ __forceinline__ bool stv_h_x_fn(const Dims& D, FS s, FV vx, int ji, int jk, int jl, double* r) {
  if (jk >= 2 && jk <= D.nx) { *r = 0.5 * (s(ji, jk - 1, jl) + s(ji, jk, jl)) * vx(ji, jk, jl); return true; }
  if (!D.periodic) return false;
  *r = 0.5 * (s(ji, 1, jl) + s(ji, D.nx, jl)) * vx(ji, 1, jl);
  return true;
}
template <class FS, class FV>
__device__ __forceinline__ bool stv_h_y_fn(const Dims& D, FS s, FV vy, int ji, int jk, int jl, double* r) {
  if (ji >= 2 && ji <= D.ny) { *r = 0.5 * (s(ji - 1, jk, jl) + s(ji, jk, jl)) * vy(ji, jk, jl); return true; }
  if (!D.periodic) return false;
  *r = 0.5 * (s(1, jk, jl) + s(D.ny, jk, jl)) * vy(1, jk, jl);
  return true;
}

// scalar_times_vector_h_upstream, mo_multiplications.F90:222-285
__device__ __forceinline__ bool upstream_x(const Dims& D, const double* s, const double* vx, int ji, int jk, int jl, double* r) {
  if (jk >= 2 && jk <= D.nx) {
    const double u = vx[IX(D, ji, jk, jl)];
    *r = (u >= 0.0) ? s[IX(D, ji, jk - 1, jl)] * u : s[IX(D, ji, jk, jl)] * u;
    return true;
  }
  if (!D.periodic) return false;
  const double u = vx[IX(D, ji, 1, jl)];
  *r = (u >= 0.0) ? s[IX(D, ji, D.nx, jl)] * u : s[IX(D, ji, 1, jl)] * u;
  return true;
}
__device__ __forceinline__ bool upstream_y(const Dims& D, const double* s, const double* vy, int ji, int jk, int jl, double* r) {
  if (ji >= 2 && ji <= D.ny) {
    const double v = vy[IX(D, ji, jk, jl)];
    *r = (v >= 0.0) ? s[IX(D, ji, jk, jl)] * v : s[IX(D, ji - 1, jk, jl)] * v;
    return true;
  }
  if (!D.periodic) return false;
  const double v = vy[IX(D, 1, jk, jl)];
  *r = (v >= 0.0) ? s[IX(D, 1, jk, jl)] * v : s[IX(D, D.ny, jk, jl)] * v;
  return true;
}

// sum(state%rho(:,:,:,1:nc+1),4) in constituent order
__device__ __forceinline__ double rho_sum_cond_gas(const Dims& D, const double* rho, long long q) {
  double s = 0.0;
  for (int jc = 0; jc <= D.nc; ++jc) s = s + rho[q + (long long)jc * D.fstride];
  return s;
}

// c_v_mass_weighted_air, mo_derived.F90:157-187
__device__ __forceinline__ double c_v_mass_weighted_air(const Dims& D, const double* rho, const double* T, long long q) {
  double c = 0.0;
  for (int jc = 1; jc <= D.nc; ++jc) c = c + rho[q + (long long)(jc - 1) * D.fstride] * c_p_cond(jc, T[q]);
  if (D.lmoist) {
    c = c + (rho[q + (long long)D.nc * D.fstride] - rho[q + (long long)(D.nc + 1) * D.fstride]) * kC_D_V;
    c = c + rho[q + (long long)(D.nc + 1) * D.fstride] * kC_V_V;
  } else {
    c = rho[q + (long long)D.nc * D.fstride] * kC_D_V;
  }
  return c;
}

// inner_product, mo_inner_product.F90:16-50 (both vectors the same)
__device__ __forceinline__ double inner_product_at(const Dims& D, const Grid<double>& G, const double* u, const double* v,
                                                   const double* w, int ji, int jk, int jl) {
  const double a = u[IX(D, ji, jk + 1, jl)], b = v[IX(D, ji, jk, jl)], c = u[IX(D, ji, jk, jl)];
  const double d = v[IX(D, ji + 1, jk, jl)], e = w[IX(D, ji, jk, jl)], f = w[IX(D, ji, jk, jl + 1)];
  return W_(1, ji, jk, jl) * a * a + W_(2, ji, jk, jl) * b * b + W_(3, ji, jk, jl) * c * c
       + W_(4, ji, jk, jl) * d * d + W_(5, ji, jk, jl) * e * e + W_(6, ji, jk, jl) * f * f;
}

// ---- potential vorticity, mo_vorticities.F90 -----------------------------------

// rel_vort x-component before the division by the area, mo_vorticities.F90:33-93
// (ji in 1..ny+1, already mapped to 1 for the periodic copy row when appropriate)
__device__ __forceinline__ double zeta_x_raw(const Dims& D, const Grid<double>& G, const State& S, int ji, int jk, int jl) {
  const double* v = S.v; const double* w = S.w;
  if (jl <= D.nl) {  // levels 2..nl
    const bool inner = ji >= 2 && ji <= D.ny;
    if (!inner && !D.periodic) return 0.0;
    const int ii = inner ? ji : 1, im = inner ? ji - 1 : D.ny;
    return G.dz[IX(D, im, jk, jl)] * w[IX(D, im, jk, jl)]
         - G.dy[IX(D, ii, jk, jl - 1)] * hcov_y<double, double>(D, G, v, w, ii, jk, jl - 1)
         - G.dz[IX(D, ii, jk, jl)] * w[IX(D, ii, jk, jl)]
         + G.dy[IX(D, ii, jk, jl)] * hcov_y<double, double>(D, G, v, w, ii, jk, jl);
  }
  // surface level NL
  const int nl = D.nl, NL = D.NL;
  const bool inner = ji >= 2 && ji <= D.ny;
  int ii = ji;
  if (D.freeslip && D.periodic && ji == D.ny + 1) ii = 1;  // copy made after the free-slip addition
  double r = -G.dy[IX(D, ii, jk, nl)] * hcov_y<double, double>(D, G, v, w, ii, jk, nl);
  if (D.freeslip && (inner || (D.periodic && ii == 1))) {
    const int im = (ii == 1) ? D.ny : ii - 1;
    r = r + 0.5 * G.dz[IX(D, im, jk, NL)] * w[IX(D, im, jk, NL)]
          - 0.5 * G.dz[IX(D, ii, jk, NL)] * w[IX(D, ii, jk, NL)]
          + G.dy[IX(D, ii, jk, nl)] * (v[IX(D, ii, jk, nl)]
          + (v[IX(D, ii, jk, nl - 1)] - v[IX(D, ii, jk, nl)]) / (G.z_v[IX(D, ii, jk, nl - 1)] - G.z_v[IX(D, ii, jk, nl)])
          * (0.5 * (G.z_w[IX(D, im, jk, NL)] + G.z_w[IX(D, ii, jk, NL)]) - G.z_v[IX(D, ii, jk, nl)])
          + 0.5 * (w[IX(D, im, jk, NL)] + w[IX(D, ii, jk, NL)])
          * (G.z_w[IX(D, im, jk, NL)] - G.z_w[IX(D, ii, jk, NL)]) / G.dy[IX(D, ii, jk, nl)]);
  }
  return r;
}

// rel_vort y-component before the division, mo_vorticities.F90:104-165
__device__ __forceinline__ double zeta_y_raw(const Dims& D, const Grid<double>& G, const State& S, int ji, int jk, int jl) {
  const double* u = S.u; const double* w = S.w;
  if (jl <= D.nl) {
    const bool inner = jk >= 2 && jk <= D.nx;
    if (!inner && !D.periodic) return 0.0;
    const int kk = inner ? jk : 1, km = inner ? jk - 1 : D.nx;
    return -G.dz[IX(D, ji, kk, jl)] * w[IX(D, ji, kk, jl)]
         - G.dx[IX(D, ji, kk, jl)] * hcov_x<double, double>(D, G, u, w, ji, kk, jl)
         + G.dz[IX(D, ji, km, jl)] * w[IX(D, ji, km, jl)]
         + G.dx[IX(D, ji, kk, jl - 1)] * hcov_x<double, double>(D, G, u, w, ji, kk, jl - 1);
  }
  const int nl = D.nl, NL = D.NL;
  const bool inner = jk >= 2 && jk <= D.nx;
  int kk = jk;
  if (D.freeslip && D.periodic && jk == D.nx + 1) kk = 1;
  double r = G.dx[IX(D, ji, kk, nl)] * hcov_x<double, double>(D, G, u, w, ji, kk, nl);
  if (D.freeslip && (inner || (D.periodic && kk == 1))) {
    const int km = (kk == 1) ? D.nx : kk - 1;
    r = r + 0.5 * G.dz[IX(D, ji, km, NL)] * w[IX(D, ji, km, NL)]
          - 0.5 * G.dz[IX(D, ji, kk, NL)] * w[IX(D, ji, kk, NL)]
          - G.dx[IX(D, ji, kk, nl)] * (u[IX(D, ji, kk, nl)]
          + (u[IX(D, ji, kk, nl - 1)] - u[IX(D, ji, kk, nl)]) / (G.z_u[IX(D, ji, kk, nl - 1)] - G.z_u[IX(D, ji, kk, nl)])
          * (0.5 * (G.z_w[IX(D, ji, km, NL)] + G.z_w[IX(D, ji, kk, NL)]) - G.z_u[IX(D, ji, kk, nl)])
          + 0.5 * (w[IX(D, ji, km, NL)] + w[IX(D, ji, kk, NL)])
          * (G.z_w[IX(D, ji, kk, NL)] - G.z_w[IX(D, ji, km, NL)]) / G.dx[IX(D, ji, kk, nl)]);
  }
  return r;
}

// density at a horizontal vorticity point (two scalar columns a and b), mo_vorticities.F90:240-266
__device__ __forceinline__ double rho_avg_h(const Dims& D, const Grid<double>& G, const double* rho,
                                            int ia, int ka, int ib, int kb, int jl) {
  const double* zs = G.z_scalar;
  if (jl == 1) {
    return 0.5 * (rho[IX(D, ia, ka, jl)]
      + (D.toa - zs[IX(D, ia, ka, jl)]) * (rho[IX(D, ia, ka, jl)] - rho[IX(D, ia, ka, jl + 1)])
        / (zs[IX(D, ia, ka, jl)] - zs[IX(D, ia, ka, jl + 1)])
      + rho[IX(D, ib, kb, jl)]
      + (D.toa - zs[IX(D, ib, kb, jl)]) * (rho[IX(D, ib, kb, jl)] - rho[IX(D, ib, kb, jl + 1)])
        / (zs[IX(D, ib, kb, jl)] - zs[IX(D, ib, kb, jl + 1)]));
  }
  if (jl == D.NL) {
    const double* zw = G.z_w;
    return 0.5 * (rho[IX(D, ia, ka, jl - 1)]
      + (zw[IX(D, ia, ka, jl)] - zs[IX(D, ia, ka, jl - 1)]) * (rho[IX(D, ia, ka, jl - 2)] - rho[IX(D, ia, ka, jl - 1)])
        / (zs[IX(D, ia, ka, jl - 2)] - zs[IX(D, ia, ka, jl - 1)])
      + rho[IX(D, ib, kb, jl - 1)]
      + (zw[IX(D, ib, kb, jl)] - zs[IX(D, ib, kb, jl - 1)]) * (rho[IX(D, ib, kb, jl - 2)] - rho[IX(D, ib, kb, jl - 1)])
        / (zs[IX(D, ib, kb, jl - 2)] - zs[IX(D, ib, kb, jl - 1)]));
  }
  return 0.25 * (rho[IX(D, ia, ka, jl - 1)] + rho[IX(D, ib, kb, jl - 1)] + rho[IX(D, ia, ka, jl)] + rho[IX(D, ib, kb, jl)]);
}

// eta_x at (ji,jk,jl), jl in 1..nl+1
__device__ __forceinline__ double eta_x_at(const Dims& D, const Grid<double>& G, const State& S, int ji, int jk, int jl) {
  if (D.periodic && ji == D.ny + 1) ji = 1;  // eta_x(ny+1,:,:) = eta_x(1,:,:) after the division
  double z = 0.0;
  if (!D.llinear) {
    const int lev = (jl == 1) ? 2 : jl;  // zeta_x(:,:,1) = zeta_x(:,:,2) after the division
    z = zeta_x_raw(D, G, S, ji, jk, lev) / G.area_dual_x[IX(D, ji, jk, lev)];
  }
  double e = D.lcorio ? z + G.fvec_x[IX(D, ji, jk, 1)] : z;
  const bool inner = ji >= 2 && ji <= D.ny;
  if (inner || D.periodic) {
    const int ia = inner ? ji - 1 : D.ny, ib = inner ? ji : 1;
    e = e / rho_avg_h(D, G, S.rho + (long long)(D.g - 1) * D.fstride, ia, jk, ib, jk, jl);
  }
  return e;
}

// eta_y at (ji,jk,jl)
__device__ __forceinline__ double eta_y_at(const Dims& D, const Grid<double>& G, const State& S, int ji, int jk, int jl) {
  if (D.periodic && jk == D.nx + 1) jk = 1;
  double z = 0.0;
  if (!D.llinear) {
    const int lev = (jl == 1) ? 2 : jl;
    z = zeta_y_raw(D, G, S, ji, jk, lev) / G.area_dual_y[IX(D, ji, jk, lev)];
  }
  double e = D.lcorio ? z + G.fvec_y[IX(D, ji, jk, 1)] : z;
  const bool inner = jk >= 2 && jk <= D.nx;
  if (inner || D.periodic) {
    const int ka = inner ? jk - 1 : D.nx, kb = inner ? jk : 1;
    e = e / rho_avg_h(D, G, S.rho + (long long)(D.g - 1) * D.fstride, ji, ka, ji, kb, jl);
  }
  return e;
}

// eta_z at (ji,jk,jl), mo_vorticities.F90:176-186 and :377-419
__device__ __forceinline__ double eta_z_at(const Dims& D, const Grid<double>& G, const State& S, int ji, int jk, int jl) {
  if (D.periodic) {
    if (ji == D.ny + 1) ji = 1;
    if (jk == D.nx + 1) jk = 1;
  }
  double z = 0.0;
  if (!D.llinear) z = rel_vort_z_local<double, double>(D, G, S.u, S.v, ji, jk, jl) / G.area_dual_z[IX(D, ji, jk, jl)];
  double e = D.lcorio ? z + G.fvec_z[IX(D, ji, jk, 1)] : z;
  const bool inner = ji >= 2 && ji <= D.ny && jk >= 2 && jk <= D.nx;
  if (inner || D.periodic) {
    const double* rg = S.rho + (long long)(D.g - 1) * D.fstride;
    const int km = (jk == 1) ? D.nx : jk - 1, im = (ji == 1) ? D.ny : ji - 1;
    e = e / (0.25 * (rg[IX(D, ji, km, jl)] + rg[IX(D, ji, jk, jl)] + rg[IX(D, im, jk, jl)] + rg[IX(D, im, km, jl)]));
  }
  return e;
}

// TRSK term for u, mo_vorticity_flux.F90:33-45 (km, kk, kp: columns jk-1, jk, jk+1)
__device__ __forceinline__ double trsk_u(const Dims& D, const Grid<double>& G, const double* vp, const double* up,
                                         const double* ez, int ji, int km, int kk, int kp, int jl) {
  const double w1 = G.trsk_u[0][ji - 1], w2 = G.trsk_u[1][ji - 1], w3 = G.trsk_u[2][ji - 1];
#define EZ(i, k) ez[IX(D, i, k, jl)]
  return w1 * vp[IX(D, ji, km, jl)] * 0.25 * (EZ(ji, km) + EZ(ji, kk) + EZ(ji, kk) + EZ(ji + 1, kk))
       + w2 * up[IX(D, ji, km, jl)] * 0.25 * (EZ(ji, km) + EZ(ji + 1, km) + EZ(ji, kk) + EZ(ji + 1, kk))
       + w3 * vp[IX(D, ji + 1, km, jl)] * 0.25 * (EZ(ji + 1, km) + EZ(ji + 1, kk) + EZ(ji, kk) + EZ(ji + 1, kk))
       + w3 * vp[IX(D, ji + 1, kk, jl)] * 0.25 * (EZ(ji + 1, kk) + EZ(ji + 1, kp) + EZ(ji, kk) + EZ(ji + 1, kk))
       + w2 * up[IX(D, ji, kp, jl)] * 0.25 * (EZ(ji + 1, kp) + EZ(ji, kp) + EZ(ji, kk) + EZ(ji + 1, kk))
       + w1 * vp[IX(D, ji, kk, jl)] * 0.25 * (EZ(ji, kk) + EZ(ji, kp) + EZ(ji, kk) + EZ(ji + 1, kk));
}

// TRSK term for v, mo_vorticity_flux.F90:72-80 (im, ii: rows ji-1, ji)
__device__ __forceinline__ double trsk_v(const Dims& D, const Grid<double>& G, const double* up, const double* ez,
                                         int im, int ii, int jk, int jl) {
  const double w1 = G.trsk_v[0][ii - 1], w2 = G.trsk_v[1][ii - 1];
  return w1 * up[IX(D, ii, jk, jl)] * 0.25 * (EZ(ii, jk) + EZ(ii + 1, jk) + EZ(ii, jk) + EZ(ii, jk + 1))
       + w1 * up[IX(D, ii, jk + 1, jl)] * 0.25 * (EZ(ii, jk + 1) + EZ(ii + 1, jk + 1) + EZ(ii, jk) + EZ(ii, jk + 1))
       + w2 * up[IX(D, im, jk + 1, jl)] * 0.25 * (EZ(im, jk + 1) + EZ(ii, jk + 1) + EZ(ii, jk) + EZ(ii, jk + 1))
       + w2 * up[IX(D, im, jk, jl)] * 0.25 * (EZ(im, jk) + EZ(ii, jk) + EZ(ii, jk) + EZ(ii, jk + 1));
#undef EZ
}

// ---- kernels (kernels_fp64.cu, column_fp64.cu) ----------------------------------
__global__ void k_temperature(Dims D, Grid<double> G, State S, double* T);
__global__ void k_theta(Dims D, Grid<double> G, const double* tp, double* out, int mode);
__global__ void k_grad_vert(Dims D, Grid<double> G, const double* s, double* rz);
__global__ void k_grad_hor(Dims D, Grid<double> G, const double* s, const double* rz, double* rx, double* ry);
__global__ void k_div_h(Dims D, Grid<double> G, const double* vx, const double* vy, double* out);
__global__ void k_theta_edges(Dims D, Grid<double> G, const double* th, const double* Dv, const double* u,
                              const double* v, double* tvu, double* tvv);
__global__ void k_pgrad(Dims D, Grid<double> G, State S, const double* gx, const double* gy, const double* gz,
                        const double* tvu, const double* tvv, const double* tpu, const double* tpv, PGrad P, int lfirst);
__global__ void k_eta_xy(Dims D, Grid<double> G, State S, double* ex, double* ey);
__global__ void k_eta_z(Dims D, Grid<double> G, State S, double* ez);
__global__ void k_mass_flux(Dims D, Grid<double> G, State S, double* uph, double* vph, double* wph);
__global__ void k_vort_flux(Dims D, Grid<double> G, State S, const double* ex, const double* ey, const double* ez,
                            const double* uph, const double* vph, const double* wph, double* px, double* py, double* pz);
__global__ void k_ke(Dims D, Grid<double> G, State S, double* out);
__global__ void k_tend_wind(Dims D, State So, State Sn, Tend Tn, Carried C, int rk_step);
__global__ void k_tracers(Dims D, Grid<double> G, State Ss, const double* u_new, const double* v_new,
                          double* t_rho, int rk_step);
__global__ void k_gas_theta(Dims D, Grid<double> G, State Ss, const double* u_new, const double* v_new,
                            const double* tvu, const double* tvv, const double* T, const double* rad,
                            const double* csh, double* t_rho, double* t_rt);
__global__ void k_column_ver(Dims D, Grid<double> G, State So, State Sn, Tend Tn, int rk_step);
__global__ void k_column_tracers(Dims D, Grid<double> G, State So, State Sn, const double* t_rho, const double* T,
                                 double* csh, int rk_step);

}  // namespace lg
