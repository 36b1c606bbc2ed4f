// kernels.cuh -- pointwise helpers and the explicit-tendency kernels of the HEVI step,
// templated on the type T of the grid metrics, the intermediate fields and the
// arithmetic.  The state is always FP64.
//
//   T = double: the FP64 step (kernels_fp64.cu, -fmad=false): every expression keeps the
//               reference's operands and left-to-right order, so the results are the
//               reference's bits.
//   T = float:  the explicit stencils of the split-precision step (split.cu): the same
//               expressions in FP32 on FP32 copies of the metrics.
#pragma once

#include "dev.cuh"

namespace lg {

template <class T>
struct PGrad {  // pressure-gradient arrays of t_diag (mo_definitions.F90:137-146), always FP64
  double *nl_u, *nl_v, *nl_w, *l_u, *l_v, *l_w, *old_u, *old_v;
  T* pgcw;
};

template <class T>
struct Tend {  // t_tend (mo_definitions.F90:108-116)
  T *rho, *rt, *u, *v, *w;
};

template <class T>
struct Carried {  // read-only view of the diagnostics combined into the wind tendency
  const double *nl_u, *nl_v, *nl_w, *l_u, *l_v, *l_w, *old_u, *old_v;
  const T *pgcw, *vsg_x, *vsg_y, *vsg_z, *pvt_x, *pvt_y, *pvt_z;
  const T *mdt_x = nullptr, *mdt_y = nullptr, *mdt_z = nullptr;  // momentum diffusion (null: off)
};

// ---- edge operators with the reference's boundary branches --------------------
// Each returns false where the reference leaves the output point untouched
// (non-periodic boundary edges); periodic jk=nx+1 / ji=ny+1 evaluate the copy source.

// grad_hor_cov x-component at a u point, mo_gradient_operators.F90:33-52.  The difference
// is taken in the source type S and rounded to T afterwards (FP64 field, FP32 result).
template <class T, class S>
__device__ __forceinline__ bool grad_x_cov(const Dims& D, const Grid<T>& G, const S* s, int ji, int jk, int jl, T* r) {
  if (jk >= 2 && jk <= D.nx) {
    *r = cvt<T>(s[IX(D, ji, jk, jl)] - s[IX(D, ji, jk - 1, jl)]) / G.dx[IX(D, ji, jk, jl)];
    return true;
  }
  if (!D.periodic) return false;
  *r = cvt<T>(s[IX(D, ji, 1, jl)] - s[IX(D, ji, D.nx, jl)]) / G.dx[IX(D, ji, 1, jl)];
  return true;
}

// grad_hor_cov y-component at a v point, mo_gradient_operators.F90:39-60
template <class T, class S>
__device__ __forceinline__ bool grad_y_cov(const Dims& D, const Grid<T>& G, const S* s, int ji, int jk, int jl, T* r) {
  if (ji >= 2 && ji <= D.ny) {
    *r = cvt<T>(s[IX(D, ji - 1, jk, jl)] - s[IX(D, ji, jk, jl)]) / G.dy[IX(D, ji, jk, jl)];
    return true;
  }
  if (!D.periodic) return false;
  *r = cvt<T>(s[IX(D, D.ny, jk, jl)] - s[IX(D, 1, jk, jl)]) / G.dy[IX(D, 1, jk, jl)];
  return true;
}

// theta_v_adv_3rd_order x edge, mo_multiplications.F90:136-183
template <class T, class V>
__device__ __forceinline__ bool theta_edge_u(const Dims& D, const T* th, const T* Dv, const V* u,
                                             T c, int ji, int jk, int jl, T* out) {
  if (jk >= 2 && jk <= D.nx) {
    T t = T(0.5) * (th[IX(D, ji, jk - 1, jl)] + th[IX(D, ji, jk, jl)]);
    if (u[IX(D, ji, jk, jl)] >= V(0)) t = t - c * Dv[IX(D, ji, jk - 1, jl)];
    else t = t - c * Dv[IX(D, ji, jk, jl)];
    *out = t;
    return true;
  }
  if (!D.periodic) return false;
  T t = T(0.5) * (th[IX(D, ji, D.nx, jl)] + th[IX(D, ji, 1, jl)]);
  if (u[IX(D, ji, 1, jl)] >= V(0)) t = t - c * Dv[IX(D, ji, D.nx, jl)];
  else t = t - c * Dv[IX(D, ji, 1, jl)];
  *out = t;
  return true;
}

// theta_v_adv_3rd_order y edge, mo_multiplications.F90:152-200
template <class T, class V>
__device__ __forceinline__ bool theta_edge_v(const Dims& D, const T* th, const T* Dv, const V* v,
                                             T c, int ji, int jk, int jl, T* out) {
  if (ji >= 2 && ji <= D.ny) {
    T t = T(0.5) * (th[IX(D, ji, jk, jl)] + th[IX(D, ji - 1, jk, jl)]);
    if (v[IX(D, ji, jk, jl)] >= V(0)) t = t - c * Dv[IX(D, ji, jk, jl)];
    else t = t - c * Dv[IX(D, ji - 1, jk, jl)];
    *out = t;
    return true;
  }
  if (!D.periodic) return false;
  T t = T(0.5) * (th[IX(D, 1, jk, jl)] + th[IX(D, D.ny, jk, jl)]);
  if (v[IX(D, 1, jk, jl)] >= V(0)) t = t - c * Dv[IX(D, 1, jk, jl)];
  else t = t - c * Dv[IX(D, D.ny, jk, jl)];
  *out = t;
  return true;
}

// scalar_times_vector_h, mo_multiplications.F90:34-54 (state scalar and vector)
template <class T, class V>
__device__ __forceinline__ bool stv_h_x(const Dims& D, const V* s, const V* vx, int ji, int jk, int jl, T* r) {
  if (jk >= 2 && jk <= D.nx) {
    *r = T(0.5) * (T(s[IX(D, ji, jk - 1, jl)]) + T(s[IX(D, ji, jk, jl)])) * T(vx[IX(D, ji, jk, jl)]);
    return true;
  }
  if (!D.periodic) return false;
  *r = T(0.5) * (T(s[IX(D, ji, 1, jl)]) + T(s[IX(D, ji, D.nx, jl)])) * T(vx[IX(D, ji, 1, jl)]);
  return true;
}
template <class T, class V>
__device__ __forceinline__ bool stv_h_y(const Dims& D, const V* s, const V* vy, int ji, int jk, int jl, T* r) {
  if (ji >= 2 && ji <= D.ny) {
    *r = T(0.5) * (T(s[IX(D, ji - 1, jk, jl)]) + T(s[IX(D, ji, jk, jl)])) * T(vy[IX(D, ji, jk, jl)]);
    return true;
  }
  if (!D.periodic) return false;
  *r = T(0.5) * (T(s[IX(D, 1, jk, jl)]) + T(s[IX(D, D.ny, jk, jl)])) * T(vy[IX(D, 1, jk, jl)]);
  return true;
}
// the same with the scalar and the vector given as functions of the index
template <class T, class FS, class FV>
__device__ __forceinline__ bool stv_h_x_fn(const Dims& D, FS s, FV vx, int ji, int jk, int jl, T* r) {
  if (jk >= 2 && jk <= D.nx) { *r = T(0.5) * (s(ji, jk - 1, jl) + s(ji, jk, jl)) * vx(ji, jk, jl); return true; }
  if (!D.periodic) return false;
  *r = T(0.5) * (s(ji, 1, jl) + s(ji, D.nx, jl)) * vx(ji, 1, jl);
  return true;
}
template <class T, class FS, class FV>
__device__ __forceinline__ bool stv_h_y_fn(const Dims& D, FS s, FV vy, int ji, int jk, int jl, T* r) {
  if (ji >= 2 && ji <= D.ny) { *r = T(0.5) * (s(ji - 1, jk, jl) + s(ji, jk, jl)) * vy(ji, jk, jl); return true; }
  if (!D.periodic) return false;
  *r = T(0.5) * (s(1, jk, jl) + s(D.ny, jk, jl)) * vy(1, jk, jl);
  return true;
}

// scalar_times_vector_h_upstream, mo_multiplications.F90:222-285
template <class T, class V>
__device__ __forceinline__ bool upstream_x(const Dims& D, const V* s, const V* vx, int ji, int jk, int jl, T* r) {
  if (jk >= 2 && jk <= D.nx) {
    const V u = vx[IX(D, ji, jk, jl)];
    *r = (u >= V(0)) ? T(s[IX(D, ji, jk - 1, jl)]) * T(u) : T(s[IX(D, ji, jk, jl)]) * T(u);
    return true;
  }
  if (!D.periodic) return false;
  const V u = vx[IX(D, ji, 1, jl)];
  *r = (u >= V(0)) ? T(s[IX(D, ji, D.nx, jl)]) * T(u) : T(s[IX(D, ji, 1, jl)]) * T(u);
  return true;
}
template <class T, class V>
__device__ __forceinline__ bool upstream_y(const Dims& D, const V* s, const V* vy, int ji, int jk, int jl, T* r) {
  if (ji >= 2 && ji <= D.ny) {
    const V v = vy[IX(D, ji, jk, jl)];
    *r = (v >= V(0)) ? T(s[IX(D, ji, jk, jl)]) * T(v) : T(s[IX(D, ji - 1, jk, jl)]) * T(v);
    return true;
  }
  if (!D.periodic) return false;
  const V v = vy[IX(D, 1, jk, jl)];
  *r = (v >= V(0)) ? T(s[IX(D, 1, jk, jl)]) * T(v) : T(s[IX(D, D.ny, jk, jl)]) * T(v);
  return true;
}

// sum(state%rho(:,:,:,1:nc+1),4) in constituent order
template <class T, class V>
__device__ __forceinline__ T rho_sum_cond_gas(const Dims& D, const V* rho, long long q) {
  T s = T(0);
  for (int jc = 0; jc <= D.nc; ++jc) s = s + T(rho[q + (long long)jc * D.fstride]);
  return s;
}

// c_p of the condensates, mo_dictionary.F90:112-189 (float: the same formulas in FP32)
__device__ __forceinline__ float c_p_water(float temperature) {
  float tc = temperature - float(kT_0), c;
  if (tc >= 0.f) {
    if (tc > 35.f) tc = 35.f;
    const float a = tc - 35.f, a2 = a * a;
    c = 0.9979f + 3.1e-6f * a2 + 3.8e-9f * (a2 * a2);
  } else {
    if (tc < -37.f) tc = -37.f;
    const float t2 = tc * tc;
    c = 1.000938f - 2.7052e-3f * tc - 2.3235e-5f * t2 + 4.3778e-6f * (t2 * tc) + 2.7136e-7f * (t2 * t2);
  }
  return 4186.8f * c;
}
__device__ __forceinline__ float c_p_ice(float temperature) {
  float tl = temperature;
  if (tl > float(kT_0)) tl = float(kT_0);
  if (tl < 20.f) tl = 20.f;
  const float q = tl * (1.f / 125.1f);
  const float c = -2.0572f + 0.14644f * tl + 0.06163f * tl * __expf(-(q * q));
  return c * float(1.0 / kM_V);
}
__device__ __forceinline__ float c_p_cond(int jc, float temperature) {
  return ((jc - 1) % 2 == 0) ? c_p_ice(temperature) : c_p_water(temperature);
}

// c_v_mass_weighted_air, mo_derived.F90:157-187
template <class T, class V>
__device__ __forceinline__ T c_v_mass_weighted_air(const Dims& D, const V* rho, const T* Tm, long long q) {
  T c = T(0);
  for (int jc = 1; jc <= D.nc; ++jc) c = c + T(rho[q + (long long)(jc - 1) * D.fstride]) * c_p_cond(jc, Tm[q]);
  if (D.lmoist) {
    c = c + (T(rho[q + (long long)D.nc * D.fstride]) - T(rho[q + (long long)(D.nc + 1) * D.fstride])) * T(kC_D_V);
    c = c + T(rho[q + (long long)(D.nc + 1) * D.fstride]) * T(kC_V_V);
  } else {
    c = T(rho[q + (long long)D.nc * D.fstride]) * T(kC_D_V);
  }
  return c;
}

// inner_product, mo_inner_product.F90:16-50 (both vectors the state wind)
template <class T, class V>
__device__ __forceinline__ T inner_product_at(const Dims& D, const Grid<T>& G, const V* u, const V* v,
                                              const V* w, int ji, int jk, int jl) {
  const T a = T(u[IX(D, ji, jk + 1, jl)]), b = T(v[IX(D, ji, jk, jl)]), c = T(u[IX(D, ji, jk, jl)]);
  const T d = T(v[IX(D, ji + 1, jk, jl)]), e = T(w[IX(D, ji, jk, jl)]), f = T(w[IX(D, ji, jk, jl + 1)]);
  return W_(1, ji, jk, jl) * a * a + W_(2, ji, jk, jl) * b * b + W_(3, ji, jk, jl) * c * c
       + W_(4, ji, jk, jl) * d * d + W_(5, ji, jk, jl) * e * e + W_(6, ji, jk, jl) * f * f;
}

// ---- potential vorticity, mo_vorticities.F90 -----------------------------------

// rel_vort x-component before the division by the area, mo_vorticities.F90:33-93
template <class T, class V>
__device__ __forceinline__ T zeta_x_raw(const Dims& D, const Grid<T>& G, const StateT<V>& S, int ji, int jk, int jl) {
  const V* v = S.v; const V* w = S.w;
  if (jl <= D.nl) {  // levels 2..nl
    const bool inner = ji >= 2 && ji <= D.ny;
    if (!inner && !D.periodic) return T(0);
    const int ii = inner ? ji : 1, im = inner ? ji - 1 : D.ny;
    return G.dz[IX(D, im, jk, jl)] * T(w[IX(D, im, jk, jl)])
         - G.dy[IX(D, ii, jk, jl - 1)] * hcov_y<T, V>(D, G, v, w, ii, jk, jl - 1)
         - G.dz[IX(D, ii, jk, jl)] * T(w[IX(D, ii, jk, jl)])
         + G.dy[IX(D, ii, jk, jl)] * hcov_y<T, V>(D, G, v, w, ii, jk, jl);
  }
  // surface level NL
  const int nl = D.nl, NL = D.NL;
  const bool inner = ji >= 2 && ji <= D.ny;
  int ii = ji;
  if (D.freeslip && D.periodic && ji == D.ny + 1) ii = 1;  // copy made after the free-slip addition
  T r = -G.dy[IX(D, ii, jk, nl)] * hcov_y<T, V>(D, G, v, w, ii, jk, nl);
  if (D.freeslip && (inner || (D.periodic && ii == 1))) {
    const int im = (ii == 1) ? D.ny : ii - 1;
    r = r + T(0.5) * G.dz[IX(D, im, jk, NL)] * T(w[IX(D, im, jk, NL)])
          - T(0.5) * G.dz[IX(D, ii, jk, NL)] * T(w[IX(D, ii, jk, NL)])
          + G.dy[IX(D, ii, jk, nl)] * (T(v[IX(D, ii, jk, nl)])
          + (T(v[IX(D, ii, jk, nl - 1)]) - T(v[IX(D, ii, jk, nl)])) / (G.z_v[IX(D, ii, jk, nl - 1)] - G.z_v[IX(D, ii, jk, nl)])
          * (T(0.5) * (G.z_w[IX(D, im, jk, NL)] + G.z_w[IX(D, ii, jk, NL)]) - G.z_v[IX(D, ii, jk, nl)])
          + T(0.5) * (T(w[IX(D, im, jk, NL)]) + T(w[IX(D, ii, jk, NL)]))
          * (G.z_w[IX(D, im, jk, NL)] - G.z_w[IX(D, ii, jk, NL)]) / G.dy[IX(D, ii, jk, nl)]);
  }
  return r;
}

// rel_vort y-component before the division, mo_vorticities.F90:104-165
template <class T, class V>
__device__ __forceinline__ T zeta_y_raw(const Dims& D, const Grid<T>& G, const StateT<V>& S, int ji, int jk, int jl) {
  const V* u = S.u; const V* w = S.w;
  if (jl <= D.nl) {
    const bool inner = jk >= 2 && jk <= D.nx;
    if (!inner && !D.periodic) return T(0);
    const int kk = inner ? jk : 1, km = inner ? jk - 1 : D.nx;
    return -G.dz[IX(D, ji, kk, jl)] * T(w[IX(D, ji, kk, jl)])
         - G.dx[IX(D, ji, kk, jl)] * hcov_x<T, V>(D, G, u, w, ji, kk, jl)
         + G.dz[IX(D, ji, km, jl)] * T(w[IX(D, ji, km, jl)])
         + G.dx[IX(D, ji, kk, jl - 1)] * hcov_x<T, V>(D, G, u, w, ji, kk, jl - 1);
  }
  const int nl = D.nl, NL = D.NL;
  const bool inner = jk >= 2 && jk <= D.nx;
  int kk = jk;
  if (D.freeslip && D.periodic && jk == D.nx + 1) kk = 1;
  T r = G.dx[IX(D, ji, kk, nl)] * hcov_x<T, V>(D, G, u, w, ji, kk, nl);
  if (D.freeslip && (inner || (D.periodic && kk == 1))) {
    const int km = (kk == 1) ? D.nx : kk - 1;
    r = r + T(0.5) * G.dz[IX(D, ji, km, NL)] * T(w[IX(D, ji, km, NL)])
          - T(0.5) * G.dz[IX(D, ji, kk, NL)] * T(w[IX(D, ji, kk, NL)])
          - G.dx[IX(D, ji, kk, nl)] * (T(u[IX(D, ji, kk, nl)])
          + (T(u[IX(D, ji, kk, nl - 1)]) - T(u[IX(D, ji, kk, nl)])) / (G.z_u[IX(D, ji, kk, nl - 1)] - G.z_u[IX(D, ji, kk, nl)])
          * (T(0.5) * (G.z_w[IX(D, ji, km, NL)] + G.z_w[IX(D, ji, kk, NL)]) - G.z_u[IX(D, ji, kk, nl)])
          + T(0.5) * (T(w[IX(D, ji, km, NL)]) + T(w[IX(D, ji, kk, NL)]))
          * (G.z_w[IX(D, ji, kk, NL)] - G.z_w[IX(D, ji, km, NL)]) / G.dx[IX(D, ji, kk, nl)]);
  }
  return r;
}

// density at a horizontal vorticity point (two scalar columns a and b), mo_vorticities.F90:240-266
template <class T, class V>
__device__ __forceinline__ T rho_avg_h(const Dims& D, const Grid<T>& G, const V* rho, int ia, int ka, int ib,
                                       int kb, int jl) {
  const T* zs = G.z_scalar;
  auto R = [&](int i, int k, int l) { return T(rho[IX(D, i, k, l)]); };
  if (jl == 1) {
    return T(0.5) * (R(ia, ka, jl)
      + (cvt<T>(D.toa) - zs[IX(D, ia, ka, jl)]) * (R(ia, ka, jl) - R(ia, ka, jl + 1))
        / (zs[IX(D, ia, ka, jl)] - zs[IX(D, ia, ka, jl + 1)])
      + R(ib, kb, jl)
      + (cvt<T>(D.toa) - zs[IX(D, ib, kb, jl)]) * (R(ib, kb, jl) - R(ib, kb, jl + 1))
        / (zs[IX(D, ib, kb, jl)] - zs[IX(D, ib, kb, jl + 1)]));
  }
  if (jl == D.NL) {
    const T* zw = G.z_w;
    return T(0.5) * (R(ia, ka, jl - 1)
      + (zw[IX(D, ia, ka, jl)] - zs[IX(D, ia, ka, jl - 1)]) * (R(ia, ka, jl - 2) - R(ia, ka, jl - 1))
        / (zs[IX(D, ia, ka, jl - 2)] - zs[IX(D, ia, ka, jl - 1)])
      + R(ib, kb, jl - 1)
      + (zw[IX(D, ib, kb, jl)] - zs[IX(D, ib, kb, jl - 1)]) * (R(ib, kb, jl - 2) - R(ib, kb, jl - 1))
        / (zs[IX(D, ib, kb, jl - 2)] - zs[IX(D, ib, kb, jl - 1)]));
  }
  return T(0.25) * (R(ia, ka, jl - 1) + R(ib, kb, jl - 1) + R(ia, ka, jl) + R(ib, kb, jl));
}

// eta_x at (ji,jk,jl), jl in 1..nl+1
template <class T, class V>
__device__ __forceinline__ T eta_x_at(const Dims& D, const Grid<T>& G, const StateT<V>& S, int ji, int jk, int jl) {
  if (D.periodic && ji == D.ny + 1) ji = 1;  // eta_x(ny+1,:,:) = eta_x(1,:,:) after the division
  T z = T(0);
  if (!D.llinear) {
    const int lev = (jl == 1) ? 2 : jl;  // zeta_x(:,:,1) = zeta_x(:,:,2) after the division
    z = zeta_x_raw<T>(D, G, S, ji, jk, lev) / G.area_dual_x[IX(D, ji, jk, lev)];
  }
  T e = D.lcorio ? z + G.fvec_x[IX(D, ji, jk, 1)] : z;
  const bool inner = ji >= 2 && ji <= D.ny;
  if (inner || D.periodic) {
    const int ia = inner ? ji - 1 : D.ny, ib = inner ? ji : 1;
    e = e / rho_avg_h<T>(D, G, S.rho + (long long)(D.g - 1) * D.fstride, ia, jk, ib, jk, jl);
  }
  return e;
}

// eta_y at (ji,jk,jl)
template <class T, class V>
__device__ __forceinline__ T eta_y_at(const Dims& D, const Grid<T>& G, const StateT<V>& S, int ji, int jk, int jl) {
  if (D.periodic && jk == D.nx + 1) jk = 1;
  T z = T(0);
  if (!D.llinear) {
    const int lev = (jl == 1) ? 2 : jl;
    z = zeta_y_raw<T>(D, G, S, ji, jk, lev) / G.area_dual_y[IX(D, ji, jk, lev)];
  }
  T e = D.lcorio ? z + G.fvec_y[IX(D, ji, jk, 1)] : z;
  const bool inner = jk >= 2 && jk <= D.nx;
  if (inner || D.periodic) {
    const int ka = inner ? jk - 1 : D.nx, kb = inner ? jk : 1;
    e = e / rho_avg_h<T>(D, G, S.rho + (long long)(D.g - 1) * D.fstride, ji, ka, ji, kb, jl);
  }
  return e;
}

// eta_z at (ji,jk,jl), mo_vorticities.F90:176-186 and :377-419
template <class T, class V>
__device__ __forceinline__ T eta_z_at(const Dims& D, const Grid<T>& G, const StateT<V>& S, int ji, int jk, int jl) {
  if (D.periodic) {
    if (ji == D.ny + 1) ji = 1;
    if (jk == D.nx + 1) jk = 1;
  }
  T z = T(0);
  if (!D.llinear) z = rel_vort_z_local<T, V>(D, G, S.u, S.v, ji, jk, jl) / G.area_dual_z[IX(D, ji, jk, jl)];
  T e = D.lcorio ? z + G.fvec_z[IX(D, ji, jk, 1)] : z;
  const bool inner = ji >= 2 && ji <= D.ny && jk >= 2 && jk <= D.nx;
  if (inner || D.periodic) {
    const V* rg = S.rho + (long long)(D.g - 1) * D.fstride;
    const int km = (jk == 1) ? D.nx : jk - 1, im = (ji == 1) ? D.ny : ji - 1;
    e = e / (T(0.25) * (T(rg[IX(D, ji, km, jl)]) + T(rg[IX(D, ji, jk, jl)]) + T(rg[IX(D, im, jk, jl)]) +
                        T(rg[IX(D, im, km, jl)])));
  }
  return e;
}

// TRSK term for u, mo_vorticity_flux.F90:33-45 (km, kk, kp: columns jk-1, jk, jk+1)
template <class T>
__device__ __forceinline__ T trsk_u(const Dims& D, const Grid<T>& G, const T* vp, const T* up, const T* ez,
                                    int ji, int km, int kk, int kp, int jl) {
  const T w1 = G.trsk_u[0][ji - 1], w2 = G.trsk_u[1][ji - 1], w3 = G.trsk_u[2][ji - 1];
#define EZ(i, k) ez[IX(D, i, k, jl)]
  return w1 * vp[IX(D, ji, km, jl)] * T(0.25) * (EZ(ji, km) + EZ(ji, kk) + EZ(ji, kk) + EZ(ji + 1, kk))
       + w2 * up[IX(D, ji, km, jl)] * T(0.25) * (EZ(ji, km) + EZ(ji + 1, km) + EZ(ji, kk) + EZ(ji + 1, kk))
       + w3 * vp[IX(D, ji + 1, km, jl)] * T(0.25) * (EZ(ji + 1, km) + EZ(ji + 1, kk) + EZ(ji, kk) + EZ(ji + 1, kk))
       + w3 * vp[IX(D, ji + 1, kk, jl)] * T(0.25) * (EZ(ji + 1, kk) + EZ(ji + 1, kp) + EZ(ji, kk) + EZ(ji + 1, kk))
       + w2 * up[IX(D, ji, kp, jl)] * T(0.25) * (EZ(ji + 1, kp) + EZ(ji, kp) + EZ(ji, kk) + EZ(ji + 1, kk))
       + w1 * vp[IX(D, ji, kk, jl)] * T(0.25) * (EZ(ji, kk) + EZ(ji, kp) + EZ(ji, kk) + EZ(ji + 1, kk));
}

// TRSK term for v, mo_vorticity_flux.F90:72-80 (im, ii: rows ji-1, ji)
template <class T>
__device__ __forceinline__ T trsk_v(const Dims& D, const Grid<T>& G, const T* up, const T* ez, int im, int ii, int jk,
                                    int jl) {
  const T w1 = G.trsk_v[0][ii - 1], w2 = G.trsk_v[1][ii - 1];
  return w1 * up[IX(D, ii, jk, jl)] * T(0.25) * (EZ(ii, jk) + EZ(ii + 1, jk) + EZ(ii, jk) + EZ(ii, jk + 1))
       + w1 * up[IX(D, ii, jk + 1, jl)] * T(0.25) * (EZ(ii, jk + 1) + EZ(ii + 1, jk + 1) + EZ(ii, jk) + EZ(ii, jk + 1))
       + w2 * up[IX(D, im, jk + 1, jl)] * T(0.25) * (EZ(im, jk + 1) + EZ(ii, jk + 1) + EZ(ii, jk) + EZ(ii, jk + 1))
       + w2 * up[IX(D, im, jk, jl)] * T(0.25) * (EZ(im, jk) + EZ(ii, jk) + EZ(ii, jk) + EZ(ii, jk + 1));
#undef EZ
}

// 3-D launches: blockIdx.x tiles the rows (ji), blockIdx.y is the level and blockIdx.z tiles
// the columns (jk), so blocks launched one after another cover one level's row tiles and then
// the same rows one level down: the vertical neighbours a stencil reads are still in L2
// (with the columns in blockIdx.y they were a whole level plane of blocks apart)
#define LG_IDX3                                              \
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;  \
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;  \
  const int jl = blockIdx.y + 1

// ---- kernels --------------------------------------------------------------------

// temperature_diagnostics, mo_derived.F90:18-38
template <class T, class V = double>
__global__ void k_temperature(Dims D, Grid<T> G, StateT<V> S, T* Tm) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  const long long i = IX(D, ji, jk, jl);
  T t = (G.theta_v_bg[i] + T(S.tp[i])) * (G.exner_bg[i] + T(S.ep[i]));
  if (D.lmoist) {
    const T rg = T(S.rho[i + (long long)(D.g - 1) * D.fstride]);
    const T rv = T(S.rho[i + (long long)D.g * D.fstride]);
    t = t / (T(1) + rv / rg * T(kM_D / kM_V - 1.0));
  }
  Tm[i] = t;
}

// diag%scalar_placeholder = theta_v_bg + theta_v_pert (mode 0) or theta_v_pert (mode 1)
template <class T, class V = double>
__global__ void k_theta(Dims D, Grid<T> G, const V* tp, T* out, int mode) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  const long long i = IX(D, ji, jk, jl);
  out[i] = mode == 0 ? G.theta_v_bg[i] + T(tp[i]) : T(tp[i]);
}

// grad_vert, mo_gradient_operators.F90:65-83 (levels 2..nl); launched with blockIdx.y = jl-2
template <class T, class S>
__global__ void k_grad_vert(Dims D, Grid<T> G, const S* s, T* rz) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.y + 2;
  if (ji > D.ny || jk > D.nx || jl > D.nl) return;
  rz[IX(D, ji, jk, jl)] = cvt<T>(s[IX(D, ji, jk, jl - 1)] - s[IX(D, ji, jk, jl)]) / G.dz[IX(D, ji, jk, jl)];
}

// grad_hor, mo_gradient_operators.F90:17-63 + :85-130, u and v points of layer jl
template <class T, class S>
__global__ void k_grad_hor(Dims D, Grid<T> G, const S* s, const T* rz, T* rx, T* ry) {
  LG_IDX3;
  if (ji <= D.ny && jk <= D.nx + 1) {
    T r;
    if (grad_x_cov<T, S>(D, G, s, ji, jk, jl, &r)) {
      if (jl > D.nf) r = r - G.slope_x[IX(D, ji, jk, jl)] * remap_x<T, T>(D, G, rz, ji, jk, jl);
      rx[IX(D, ji, jk, jl)] = r;
    }
  }
  if (ji <= D.ny + 1 && jk <= D.nx) {
    T r;
    if (grad_y_cov<T, S>(D, G, s, ji, jk, jl, &r)) {
      if (jl > D.nf) r = r - G.slope_y[IX(D, ji, jk, jl)] * remap_y<T, T>(D, G, rz, ji, jk, jl);
      ry[IX(D, ji, jk, jl)] = r;
    }
  }
}

// div_h, mo_divergence_operators.F90:16-68
template <class T>
__global__ void k_div_h(Dims D, Grid<T> G, const T* vx, const T* vy, T* out) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  auto fx = [&](int i, int j, int k) { return vx[IX(D, i, j, k)]; };
  auto fy = [&](int i, int j, int k) { return vy[IX(D, i, j, k)]; };
  out[IX(D, ji, jk, jl)] = div_h_at<T>(D, G, fx, fy, ji, jk, jl);
}

// theta_v_adv_3rd_order edge values, mo_multiplications.F90:134-202
template <class T, class V = double>
__global__ void k_theta_edges(Dims D, Grid<T> G, const T* th, const T* Dv, const V* u, const V* v,
                              T* tvu, T* tvv) {
  LG_IDX3;
  const T c = cvt<T>(D.theta_edge_c);
  if (ji <= D.ny && jk <= D.nx + 1) {
    T t;
    if (theta_edge_u<T>(D, th, Dv, u, c, ji, jk, jl, &t)) tvu[IX(D, ji, jk, jl)] = t;
  }
  if (ji <= D.ny + 1 && jk <= D.nx) {
    T t;
    if (theta_edge_v<T>(D, th, Dv, v, c, ji, jk, jl, &t)) tvv[IX(D, ji, jk, jl)] = t;
  }
}

// calc_pot_vort, mo_vorticities.F90:189-421 with rel_vort :19-187 inlined:
// eta_x (ny+1,nx,nl+1) and eta_y (ny,nx+1,nl+1)
template <class T, class V = double>
__global__ void k_eta_xy(Dims D, Grid<T> G, StateT<V> S, T* ex, T* ey) {
  LG_IDX3;
  if (jl > D.NL) return;
  if (ji <= D.ny + 1 && jk <= D.nx) ex[IX(D, ji, jk, jl)] = eta_x_at<T>(D, G, S, ji, jk, jl);
  if (ji <= D.ny && jk <= D.nx + 1) ey[IX(D, ji, jk, jl)] = eta_y_at<T>(D, G, S, ji, jk, jl);
}

// eta_z (ny+1,nx+1,nl)
template <class T, class V = double>
__global__ void k_eta_z(Dims D, Grid<T> G, StateT<V> S, T* ez) {
  LG_IDX3;
  if (ji > D.ny + 1 || jk > D.nx + 1) return;
  ez[IX(D, ji, jk, jl)] = eta_z_at<T>(D, G, S, ji, jk, jl);
}

// mass flux densities, mo_vector_tend_expl.F90:64-66 (scalar_times_vector_h/_v)
template <class T, class V = double>
__global__ void k_mass_flux(Dims D, Grid<T> G, StateT<V> S, T* uph, T* vph, T* wph) {
  LG_IDX3;
  const V* rg = S.rho + (long long)(D.g - 1) * D.fstride;
  if (jl <= D.nl && ji <= D.ny && jk <= D.nx + 1) {
    T f;
    if (stv_h_x<T>(D, rg, S.u, ji, jk, jl, &f)) uph[IX(D, ji, jk, jl)] = f;
  }
  if (jl <= D.nl && ji <= D.ny + 1 && jk <= D.nx) {
    T f;
    if (stv_h_y<T>(D, rg, S.v, ji, jk, jl, &f)) vph[IX(D, ji, jk, jl)] = f;
  }
  if (jl >= 2 && jl <= D.nl && ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    wph[q] = T(0.5) * (T(rg[IX(D, ji, jk, jl - 1)]) + T(rg[q])) * T(S.w[q]);
  }
}

// calc_vorticity_flux_term, mo_vorticity_flux.F90:16-171
template <class T, class V = double>
__device__ __forceinline__ void vort_flux_body(const Dims& D, const Grid<T>& G, const StateT<V>& S, const T* ex,
                                               const T* ey, const T* ez, const T* uph, const T* vph, const T* wph,
                                               T* px, T* py, T* pz) {
  LG_IDX3;
  // vertical mass flux with the free-slip surface value, mo_vector_tend_expl.F90:68-80
  auto wp = [&](int i, int j, int k) -> T {
    if (k == D.NL) {
      if (!D.freeslip) return T(0);
      const V* rg = S.rho + (long long)(D.g - 1) * D.fstride;
      const T dv = T(rg[IX(D, i, j, D.nl)]) + (T(rg[IX(D, i, j, D.nl - 1)]) - T(rg[IX(D, i, j, D.nl)]))
                   / (G.z_scalar[IX(D, i, j, D.nl - 1)] - G.z_scalar[IX(D, i, j, D.nl)])
                   * (G.z_w[IX(D, i, j, D.NL)] - G.z_scalar[IX(D, i, j, D.nl)]);
      return dv * T(S.w[IX(D, i, j, D.NL)]);
    }
    return wph[IX(D, i, j, k)];
  };
  if (jl <= D.nl && ji <= D.ny && jk <= D.nx + 1) {
    const bool inner = jk >= 2 && jk <= D.nx;
    if (inner || D.periodic) {
      const int kk = inner ? jk : 1, km = inner ? jk - 1 : D.nx, kp = kk + 1;
      T r = trsk_u<T>(D, G, vph, uph, ez, ji, km, kk, kp, jl);
      r = r - T(0.5) * W_(5, ji, km, jl) * wp(ji, km, jl) * ey[IX(D, ji, kk, jl)]
            - T(0.5) * W_(6, ji, km, jl) * wp(ji, km, jl + 1) * ey[IX(D, ji, kk, jl + 1)]
            - T(0.5) * W_(5, ji, kk, jl) * wp(ji, kk, jl) * ey[IX(D, ji, kk, jl)]
            - T(0.5) * W_(6, ji, kk, jl) * wp(ji, kk, jl + 1) * ey[IX(D, ji, kk, jl + 1)];
      px[IX(D, ji, jk, jl)] = r;
    }
  }
  if (jl <= D.nl && ji <= D.ny + 1 && jk <= D.nx) {
    const bool inner = ji >= 2 && ji <= D.ny;
    if (inner || D.periodic) {
      const int ii = inner ? ji : 1, im = inner ? ji - 1 : D.ny;
      T r = trsk_v<T>(D, G, uph, ez, im, ii, jk, jl);
      r = r + T(0.5) * W_(5, im, jk, jl) * wp(im, jk, jl) * ex[IX(D, ii, jk, jl)]
            + T(0.5) * W_(6, im, jk, jl) * wp(im, jk, jl + 1) * ex[IX(D, ii, jk, jl + 1)]
            + T(0.5) * W_(5, ii, jk, jl) * wp(ii, jk, jl) * ex[IX(D, ii, jk, jl)]
            + T(0.5) * W_(6, ii, jk, jl) * wp(ii, jk, jl + 1) * ex[IX(D, ii, jk, jl + 1)];
      py[IX(D, ji, jk, jl)] = r;
    }
  }
  if (jl >= 2 && jl <= D.nl && ji <= D.ny && jk <= D.nx) {
    pz[IX(D, ji, jk, jl)] = T(0.5) * (
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

template <class T, class V = double>
__global__ void k_vort_flux(Dims D, Grid<T> G, StateT<V> S, const T* ex, const T* ey, const T* ez, const T* uph,
                            const T* vph, const T* wph, T* px, T* py, T* pz) {
  vort_flux_body<T, V>(D, G, S, ex, ey, ez, uph, vph, wph, px, py, pz);
}

// inner_product of the wind with itself, mo_inner_product.F90:16-50
template <class T, class V = double>
__global__ void k_ke(Dims D, Grid<T> G, StateT<V> S, T* out) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  out[IX(D, ji, jk, jl)] = inner_product_at<T>(D, G, S.u, S.v, S.w, ji, jk, jl);
}

// combination of the explicit wind tendencies, mo_vector_tend_expl.F90:258-310, and the
// forward step of the horizontal wind, mo_manage_pchevi.F90:86-89 (in FP64)
template <class T>
// mu, mv (may be null): FP32 mirrors of the new u, v, written beside the FP64 values
__global__ void k_tend_wind(Dims D, State So, State Sn, Tend<T> Tn, Carried<T> C, int rk_step, float* mu, float* mv) {
  LG_IDX3;
  const T new_weight = (rk_step == 2) ? T(0.5) : T(1);
  const T old_weight = T(1) - new_weight;
  // the pressure-gradient combinations are formed in FP64 (the products are FP64; without a
  // background state they are O(g) and cancel gravity), in the reference's operation order
  const double chw_d = 0.5 + kIMPL_THERMO_WEIGHT, ohw_d = 1.0 - (0.5 + kIMPL_THERMO_WEIGHT);
  const double cvw_d = 1.0 - kIMPL_THERMO_WEIGHT, no_bg_d = D.luse_bg ? 0.0 : 1.0;
  // FP32 tendencies with a background state: the sum nl + l, where the two products cancel,
  // is the only FP64 operation; the previous substep's value (already a net force) and that
  // sum are rounded to FP32 and combined there, as the FP32 tendency is rounded anyway
  constexpr bool f32 = sizeof(T) == 4;
  const bool pg32 = f32 && D.luse_bg;
  auto pg_h = [&](const double* old, const double* nl, const double* l, long long q) -> T {
    if (pg32) return T(ohw_d) * cvt<T>(old[q]) - T(chw_d) * cvt<T>(nl[q] + l[q]);
    return cvt<T>(ohw_d * old[q] - chw_d * (nl[q] + l[q]));
  };
  if (jl <= D.nl && ji <= D.ny && jk <= D.nx + 1) {
    const long long q = IX(D, ji, jk, jl);
    T f = pg_h(C.old_u, C.nl_u, C.l_u, q) - T(0.5) * C.vsg_x[q] + C.pvt_x[q];
    if (C.mdt_x) f = f + C.mdt_x[q];
    const T t = old_weight * Tn.u[q] + new_weight * f;
    Tn.u[q] = t;
    const double un = So.u[q] + D.dtime * cvt<double>(t);
    Sn.u[q] = un;
    if (mu) mu[q] = narrow(un);
  }
  if (jl <= D.nl && ji <= D.ny + 1 && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    T f = pg_h(C.old_v, C.nl_v, C.l_v, q) - T(0.5) * C.vsg_y[q] + C.pvt_y[q];
    if (C.mdt_y) f = f + C.mdt_y[q];
    const T t = old_weight * Tn.v[q] + new_weight * f;
    Tn.v[q] = t;
    const double vn = So.v[q] + D.dtime * cvt<double>(t);
    Sn.v[q] = vn;
    if (mv) mv[q] = narrow(vn);
  }
  if (jl <= D.NL && ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    T pg;
    if (pg32) pg = -(T(cvw_d) * cvt<T>(C.nl_w[q] + C.l_w[q]));
    else pg = cvt<T>(-(cvw_d * (C.nl_w[q] + C.l_w[q])) - no_bg_d * (1.0 - cvw_d) * C.l_w[q]);
    T f = pg - T(0.5) * C.vsg_z[q] + C.pvt_z[q] + C.pgcw[q];
    if (C.mdt_z) f = f + C.mdt_z[q];
    Tn.w[q] = old_weight * Tn.w[q] + new_weight * f;
  }
}

// scalar_tend_expl for every constituent other than the gas, mo_scalar_tend_expl.F90:102-128
// with scalar_times_vector_h_upstream (mo_multiplications.F90:206-287) and div_h_tracers
// (mo_divergence_operators.F90:70-147) evaluated inline.
template <class T, class V = double>
__device__ __forceinline__ void tracers_body(const Dims& D, const Grid<T>& G, const StateT<V>& Ss, const V* u_new,
                                             const V* v_new, T* t_rho, int rk_step, const T* mdt,
                                             const T* ptr) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl);
  auto wx = [&](int i, int j, int k) { return T(u_new[IX(D, i, j, k)]); };
  auto wy = [&](int i, int j, int k) { return T(v_new[IX(D, i, j, k)]); };
  // contravariant vertical velocity corrections do not depend on the constituent
  T cu = T(0), cl = T(0);
  if (jl == D.nf) cl = vcc<T>(D, G, wx, wy, ji, jk, jl + 1);
  else if (jl == D.nl) cu = vcc<T>(D, G, wx, wy, ji, jk, jl);
  else if (jl > D.nf) { cu = vcc<T>(D, G, wx, wy, ji, jk, jl); cl = vcc<T>(D, G, wx, wy, ji, jk, jl + 1); }
  const T new_weight = (rk_step == 2) ? T(0.5) : T(1);
  const T old_weight = T(1) - new_weight;
  for (int jc = 1; jc <= D.ncons; ++jc) {
    if (jc == D.g) continue;
    const V* r = Ss.rho + (long long)(jc - 1) * D.fstride;
    auto fx = [&](int i, int j, int k) { T f; return upstream_x<T>(D, r, u_new, i, j, k, &f) ? f : T(0); };
    auto fy = [&](int i, int j, int k) { T f; return upstream_y<T>(D, r, v_new, i, j, k, &f) ? f : T(0); };
    const T comp_h = fx(ji, jk + 1, jl) * G.area_x[IX(D, ji, jk + 1, jl)]
                   + fy(ji, jk, jl) * G.area_y[IX(D, ji, jk, jl)]
                   - fx(ji, jk, jl) * G.area_x[IX(D, ji, jk, jl)]
                   - fy(ji + 1, jk, jl) * G.area_y[IX(D, ji + 1, jk, jl)];
    T comp_v = T(0);
    if (jl == D.nf) {
      const T dl = (cl <= T(0)) ? T(r[IX(D, ji, jk, jl)]) : T(r[IX(D, ji, jk, jl + 1)]);
      comp_v = -dl * cl * G.area_z[IX(D, ji, jk, jl + 1)];
    } else if (jl == D.nl) {
      const T du = (cu <= T(0)) ? T(r[IX(D, ji, jk, jl - 1)]) : T(r[IX(D, ji, jk, jl)]);
      comp_v = du * cu * G.area_z[IX(D, ji, jk, jl)];
    } else if (jl > D.nf) {
      const T du = (cu <= T(0)) ? T(r[IX(D, ji, jk, jl - 1)]) : T(r[IX(D, ji, jk, jl)]);
      const T dl = (cl <= T(0)) ? T(r[IX(D, ji, jk, jl)]) : T(r[IX(D, ji, jk, jl + 1)]);
      comp_v = du * cu * G.area_z[IX(D, ji, jk, jl)] - dl * cl * G.area_z[IX(D, ji, jk, jl + 1)];
    }
    const T div = (comp_h + comp_v) / G.volume[q];
    T* t = t_rho + (long long)(jc - 1) * D.fstride;
    T f = -div;
    if (mdt) f = f + mdt[q + (long long)(jc - 1) * D.fstride];  // mass diffusion
    // phase transitions (null: off, the reference's zero); vapour takes rate nc+1
    if (ptr) f = f + ptr[q + (long long)((jc < D.g ? jc : D.g) - 1) * D.fstride];
    t[q] = old_weight * t[q] + new_weight * f;
  }
}

template <class T, class V = double>
__global__ void k_tracers(Dims D, Grid<T> G, StateT<V> Ss, const V* u_new, const V* v_new, T* t_rho, int rk_step,
                          const T* mdt, const T* ptr) {
  tracers_body<T, V>(D, G, Ss, u_new, v_new, t_rho, rk_step, mdt, ptr);
}

// scalar_tend_expl for the gas and the rho*theta_v tendency, mo_scalar_tend_expl.F90:106-177
template <class T, class V = double>
__global__ void k_gas_theta(Dims D, Grid<T> G, StateT<V> Ss, const V* u_new, const V* v_new, const T* tvu,
                            const T* tvv, const T* Tm, const T* hd, const T* rad, const T* csh, T* t_rho,
                            T* t_rt, const T* mdt, const T* tdh, const T* ptr, const T* pth) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl);
  const V* rg = Ss.rho + (long long)(D.g - 1) * D.fstride;
  auto fx = [&](int i, int j, int k) { T f; return stv_h_x<T>(D, rg, u_new, i, j, k, &f) ? f : T(0); };
  auto fy = [&](int i, int j, int k) { T f; return stv_h_y<T>(D, rg, v_new, i, j, k, &f) ? f : T(0); };
  const T div_m = div_h_at<T>(D, G, fx, fy, ji, jk, jl);
  // old_weight 0, new_weight 1 for the gas; mass diffusion and the phase transitions' vapour
  // rate (null: off)
  const T mdg = mdt ? mdt[q + (long long)(D.g - 1) * D.fstride] : T(0);
  const T ptg = ptr ? ptr[q + (long long)(D.g - 1) * D.fstride] : T(0);
  T tg = mdt ? -div_m + mdg : -div_m;
  if (ptr) tg = tg + ptg;
  t_rho[q + (long long)(D.g - 1) * D.fstride] = tg;
  T div_t;
  if (D.theta_order == 2) {
    auto th = [&](int i, int j, int k) { const long long p = IX(D, i, j, k); return G.theta_v_bg[p] + T(Ss.tp[p]); };
    auto gx = [&](int i, int j, int k) { T f; return stv_h_x_fn<T>(D, th, fx, i, j, k, &f) ? f : T(0); };
    auto gy = [&](int i, int j, int k) { T f; return stv_h_y_fn<T>(D, th, fy, i, j, k, &f) ? f : T(0); };
    div_t = div_h_at<T>(D, G, gx, gy, ji, jk, jl);
  } else {
    auto gx = [&](int i, int j, int k) { return tvu[IX(D, i, j, k)] * fx(i, j, k); };
    auto gy = [&](int i, int j, int k) { return tvv[IX(D, i, j, k)] * fy(i, j, k); };
    div_t = div_h_at<T>(D, G, gx, gy, ji, jk, jl);
  }
  // dissipative heating, radiation, phase transitions (null: off), sediment heating and
  // temperature diffusion, in the reference's order
  T heat = hd[q] + rad[q];
  if (pth) heat = heat + pth[q];
  heat = heat + csh[q];
  if (tdh) heat = heat + tdh[q];
  T x = T(0);
  if (heat != T(0)) {
    const T cv = c_v_mass_weighted_air<T>(D, Ss.rho, Tm, q);
    x = T(kC_D_V) * T(rg[q]) / cv * heat / (T(kC_D_P) * (G.exner_bg[q] + T(Ss.ep[q])));
  }
  T r = -div_t + x;
  // (phase transition rate + mass diffusion of the gas) * theta_v
  if (ptr) r = r + (ptg + mdg) * (G.theta_v_bg[q] + T(Ss.tp[q]));
  else if (mdt) r = r + mdg * (G.theta_v_bg[q] + T(Ss.tp[q]));
  t_rt[q] = r;
}

// ---- FP64-only kernels (kernels_fp64.cu, column_fp64.cu) -------------------------------
__global__ void k_pgrad(Dims D, Grid<double> G, State S, const double* gx, const double* gy, const double* gz,
                        const double* tvu, const double* tvv, const double* tpu, const double* tpv, PGrad<double> P,
                        int lfirst);
__global__ void k_column_ver(Dims D, Grid<double> G, State So, State Sn, Tend<double> Tn, int rk_step);
__global__ void k_column_tracers(Dims D, Grid<double> G, State So, State Sn, const double* t_rho, const double* T,
                                 double* csh, int rk_step);

}  // namespace lg
