// diffusion.cuh -- the diffusion closure of the HEVI step (TKE, Smagorinsky/TKE horizontal
// viscosity, momentum diffusion, temperature and mass diffusion), templated like kernels.cuh
// on the type T of the metrics and the arithmetic and the type V of the state read:
//
//   T = double, V = double: the FP64 step (lgame_gpu.cu, -fmad=false), every expression in the
//                           reference's operand order;
//   T = float,  V = float:  the split step (split.cu), the same expressions in FP32 on the FP32
//                           metric copies and the FP32 mirror of the state; its temperature and
//                           mass diffusion is the fused kernel k_diff_scalar_col (FP32 only).
//
// Reference routines: update_n_squared, tke2hor/vert_diff_coeff, hor_viscosity(_smag/_tke),
// hor_diff_coeff_postprocessing, vert_vert_mom_viscosity, scalar_diff_coeffs
// (src/subgrid_scale/mo_eff_diff_coeffs.F90), tke_update (mo_tke.F90:19-66), mom_diff_h and
// mom_diff_v (mo_momentum_diff_diss.F90:25-331), the diffusion part of scalar_tend_expl
// (mo_scalar_tend_expl.F90:60-101) and add_vertical_div (mo_divergence_operators.F90:149-186).
//
// The reference passes these quantities through shared work arrays (scalar_placeholder,
// u/v/w_placeholder, flux_density_*), some of whose points an operator reads without having
// written them.  What such a point holds is fixed by the step's order of operations:
//   - grad_vert writes w levels 2..nl only; w_placeholder's levels 1 and n_levels are written
//     only by whole-array products of zeros (the copy of mom_diff_tend_z, whose top and bottom
//     levels no operator writes, and the free-slip reset), so every vertical gradient below is
//     0 at those levels;
//   - at non-periodic boundary edges grad_hor and scalar_times_vector_h write nothing: the
//     diffusive flux densities stay at their initial zero there, and the gradient read by
//     tke_update's inner product holds the zero that the previous step's whole-array writers
//     left (mom_diff_v's products with vert_hor_viscosity, which the reference never sets, or
//     theta_v_adv_3rd_order's theta_v_u*flux_density_u); lgame_gpu_create accepts
//     non-periodic diffusion only in those configurations;
//   - vert_hor_mom_viscosity is never called, so vert_hor_viscosity_u/v keep their initial
//     zeros: the vertical diffusion of u and v and the horizontal diffusion of w in mom_diff_v
//     add exact zeros and are not evaluated.
#pragma once

#include "kernels.cuh"

namespace lg {

// device buffers of the closure (T: FP64 step double, split step float)
template <class T>
struct DiffBuf {
  T *tke, *tke_new;      // specific TKE (carried) and its update of this step
  T *visc, *vmol;        // viscosity (rho * (molecular + eddy), carried) and viscosity_molecular
  T *nsq;                // n_squared at scalar points
  T *vz;                 // viscosity_dual * zeta_z at dual points (ny+1, nx+1, nl)
  T *mdtx, *mdty, *mdtz; // mom_diff_tend_x/y/z (carried)
  T *mdt, *tdh;          // mass_diff_tendency (ncons fields), temp_diff_heating
  T* hd;                 // heating_diss (carried; formed by the dissipation kernel)
  T *flx, *fly, *flw;    // diffusive flux densities of the scalar diffusion, one field per constituent
                         // (FP64 step only: the split step forms its faces in shared memory)
  T *zz;                 // zeta_z at dual points (rel_vort of the state of the first substep)
  T *vdiv;               // viscosity * div_h(wind) at scalar points (mom_diff_h's scalar_placeholder)
};

// run-time constants of the closure
struct DiffPar {
  double mva;            // mean_velocity_area, mo_grid_generator.F90:1111
  double eff_hor_res;    // sqrt(dx*dy), mo_run_nml.F90:93
  double c_s, bg_shear;  // Smagorinsky parameter, minimum shear
  int tke_h;             // diff_coeff_scheme_h == "tke"
  int mom_v;             // lmom_diff_v
};

template <class T> __device__ __forceinline__ T dsqrt(T x) { return sqrt(x); }
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }

// tke2hor_diff_coeff, mo_eff_diff_coeffs.F90:671-686.  (2*tke)**0.5: the square root, the
// correctly rounded value of the power (the reference's pow differs from it by at most the
// last bit in rare cases)
template <class T>
__device__ __forceinline__ T tke2hor(const DiffPar& P, T tke) {
  const T mean_velocity = dsqrt<T>(T(2) * tke);
  const T mean_free_path = T(P.eff_hor_res) / T(6);
  return T(1.0 / 6.0) * mean_free_path * mean_velocity;
}

// tke2vert_diff_coeff, mo_eff_diff_coeffs.F90:688-713
template <class T>
__device__ __forceinline__ T tke2vert(T tke, T n_squared, T layer_thickness) {
  const T tke_vert = T(3.0 * 1e-3) * tke;
  const T mean_velocity = dsqrt<T>(T(2) * tke_vert);
  const T n_used = dsqrt<T>(n_squared > T(1e-4) ? n_squared : T(1e-4));
  T mean_free_path = dsqrt<T>(T(2) * tke_vert) / n_used;
  mean_free_path = mean_free_path < layer_thickness ? mean_free_path : layer_thickness;
  return T(1.0 / 6.0) * mean_free_path * mean_velocity;
}

// calc_diff_coeff, mo_derived.F90:189-216, in type T
template <class T>
__device__ __forceinline__ T diff_coeff_t(T temperature, T density) {
  if constexpr (sizeof(T) == 8) {
    return calc_diff_coeff(temperature, density);
  } else {
    const float particle_mass = float(kM_D / kN_A);
    const float thermal_velocity = sqrtf(float(8.0 * kK_B) * temperature / float(kPI * (kM_D / kN_A)));
    const float particle_density = density / particle_mass;
    const float cross_section = float(4.0 * kPI * (130e-12 * 130e-12));
    const float mean_free_path = 1.f / (1.4142135f * particle_density * cross_section);
    return (1.f / 3.f) * thermal_velocity * mean_free_path;
  }
}

// relative vorticity at a dual point, rel_vort (mo_vorticities.F90:181)
template <class T, class V>
__device__ __forceinline__ T zeta_z_at(const Dims& D, const Grid<T>& G, const StateT<V>& S, int ji, int jk, int jl) {
  return rel_vort_z_local<T, V>(D, G, S.u, S.v, ji, jk, jl) / G.area_dual_z[IX(D, ji, jk, jl)];
}

// divergence of the horizontal wind at a scalar point, div_h (mo_divergence_operators.F90:16-68)
template <class T, class V>
__device__ __forceinline__ T div_wind_at(const Dims& D, const Grid<T>& G, const StateT<V>& S, int ji, int jk, int jl) {
  auto fx = [&](int i, int j, int k) { return T(S.u[IX(D, i, j, k)]); };
  auto fy = [&](int i, int j, int k) { return T(S.v[IX(D, i, j, k)]); };
  return div_h_at<T>(D, G, fx, fy, ji, jk, jl);
}

// ---- 1. update_n_squared and tke_update (first substep, any horizontal diffusion on) ----------
// One thread per scalar point.  Reads the old TKE, viscosity and heating_diss; writes the
// updated TKE to tke_new (the old one is still read by neighbours) and n_squared.
template <class T, class V>
__global__ void k_diff_tke(Dims D, Grid<T> G, StateT<V> S, DiffBuf<T> B, DiffPar P) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl);
  // update_n_squared, mo_eff_diff_coeffs.F90:620-669: g * 0.5*(1/theta(l-1) + 1/theta(l)) *
  // dtheta/dz at w level l in 2..nl, zero at levels 1 and nl+1
  auto nz = [&](int l) -> T {
    if (l < 2 || l > D.nl) return T(0);
    const long long a = IX(D, ji, jk, l - 1), b = IX(D, ji, jk, l);
    const T th_a = G.theta_v_bg[a] + T(S.tp[a]), th_b = G.theta_v_bg[b] + T(S.tp[b]);
    const T grad = (th_a - th_b) / G.dz[b];
    return G.gm[b] * (T(0.5) * (T(1) / th_a + T(1) / th_b) * grad);
  };
  T nsq;
  if (jl == 1) nsq = nz(1);
  else if (jl == D.nl) nsq = nz(D.nl + 1);
  else nsq = W_(5, ji, jk, jl) * nz(jl) + W_(6, ji, jk, jl) * nz(jl + 1);
  B.nsq[q] = nsq;
  // tke_update, mo_tke.F90:19-66: the inner product of the wind with grad(tke)
  const T* tke = B.tke;
  auto gz = [&](int i, int j, int l) -> T {  // grad_vert(tke), zero at levels 1 and nl+1
    if (l < 2 || l > D.nl) return T(0);
    return (tke[IX(D, i, j, l - 1)] - tke[IX(D, i, j, l)]) / G.dz[IX(D, i, j, l)];
  };
  auto remap_gx = [&](int i, int j, int l) -> T {  // remap_ver2hor_x of gz
    T r = T(0);
    if (j == 1 || j == D.nx + 1) {
      if (!D.periodic) return r;
      r = r + W_(5, i, D.nx, l) * gz(i, D.nx, l);
      r = r + W_(5, i, 1, l) * gz(i, 1, l);
      if (l < D.nl || D.freeslip) { r = r + W_(6, i, D.nx, l) * gz(i, D.nx, l + 1); r = r + W_(6, i, 1, l) * gz(i, 1, l + 1); }
    } else {
      r = r + W_(5, i, j - 1, l) * gz(i, j - 1, l);
      r = r + W_(5, i, j, l) * gz(i, j, l);
      if (l < D.nl || D.freeslip) { r = r + W_(6, i, j - 1, l) * gz(i, j - 1, l + 1); r = r + W_(6, i, j, l) * gz(i, j, l + 1); }
    }
    return T(0.5) * r;
  };
  auto remap_gy = [&](int i, int j, int l) -> T {  // remap_ver2hor_y of gz
    T r = T(0);
    if (i == 1 || i == D.ny + 1) {
      if (!D.periodic) return r;
      r = r + W_(5, D.ny, j, l) * gz(D.ny, j, l);
      r = r + W_(5, 1, j, l) * gz(1, j, l);
      if (l < D.nl || D.freeslip) { r = r + W_(6, D.ny, j, l) * gz(D.ny, j, l + 1); r = r + W_(6, 1, j, l) * gz(1, j, l + 1); }
    } else {
      r = r + W_(5, i - 1, j, l) * gz(i - 1, j, l);
      r = r + W_(5, i, j, l) * gz(i, j, l);
      if (l < D.nl || D.freeslip) { r = r + W_(6, i - 1, j, l) * gz(i - 1, j, l + 1); r = r + W_(6, i, j, l) * gz(i, j, l + 1); }
    }
    return T(0.5) * r;
  };
  auto gx = [&](int i, int j, int l) -> T {  // grad_hor x at a u point; non-periodic boundary: 0
    T r;
    if (!grad_x_cov<T, T>(D, G, tke, i, j, l, &r)) return T(0);
    if (l > D.nf) r = r - G.slope_x[IX(D, i, j, l)] * remap_gx(i, j, l);
    return r;
  };
  auto gy = [&](int i, int j, int l) -> T {
    T r;
    if (!grad_y_cov<T, T>(D, G, tke, i, j, l, &r)) return T(0);
    if (l > D.nf) r = r - G.slope_y[IX(D, i, j, l)] * remap_gy(i, j, l);
    return r;
  };
  const T adv = W_(1, ji, jk, jl) * T(S.u[IX(D, ji, jk + 1, jl)]) * gx(ji, jk + 1, jl)
              + W_(2, ji, jk, jl) * T(S.v[q]) * gy(ji, jk, jl)
              + W_(3, ji, jk, jl) * T(S.u[q]) * gx(ji, jk, jl)
              + W_(4, ji, jk, jl) * T(S.v[IX(D, ji + 1, jk, jl)]) * gy(ji + 1, jk, jl)
              + W_(5, ji, jk, jl) * T(S.w[q]) * gz(ji, jk, jl)
              + W_(6, ji, jk, jl) * T(S.w[q + D.plane]) * gz(ji, jk, jl + 1);
  const T rg = T(S.rho[q + (long long)(D.g - 1) * D.fstride]);
  const T decay_constant = T(8.0 * (kPI * kPI)) / T(P.mva) * B.visc[q] / rg;
  T t = tke[q] + T(D.dtime) * (-adv + B.hd[q] / rg - decay_constant * tke[q]);
  if (t < T(0)) t = T(0);
  B.tke_new[q] = t;
}

// ---- 2. hor_viscosity (mo_eff_diff_coeffs.F90:24-159) -------------------------------------
// One thread per scalar point: viscosity_molecular, the eddy viscosity (Smagorinsky from the
// vorticity averaged to the cell and the divergence of the wind, or from the updated TKE), their
// sum times the gas density.  Also moves the updated TKE into place.
template <class T, class V>
__global__ void k_diff_visc(Dims D, Grid<T> G, StateT<V> S, const T* Tm, DiffBuf<T> B, DiffPar P) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl);
  const T rg = T(S.rho[q + (long long)(D.g - 1) * D.fstride]);
  const T tke = B.tke_new[q];
  const T vmol = diff_coeff_t<T>(Tm[q], rg);
  const T dv = div_wind_at<T, V>(D, G, S, ji, jk, jl);
  T eddy;
  if (P.tke_h) {
    eddy = tke2hor<T>(P, tke);
  } else {
    const T* zz = B.zz;
    const T vac = T(0.25) * (zz[q] + zz[q + D.P] + zz[q + 1] + zz[q + D.P + 1]);
    const T a = vac * vac + dv * dv, b = T(P.bg_shear) * T(P.bg_shear);
    eddy = T(P.c_s) * T(P.mva) * dsqrt<T>(a > b ? a : b);
  }
  const T visc = rg * (vmol + eddy);
  B.vmol[q] = vmol;
  B.visc[q] = visc;
  B.vdiv[q] = visc * dv;
  B.tke[q] = tke;
}

// zeta_z of the wind at the dual points (ny+1, nx+1, nl), rel_vort (mo_vorticities.F90:19-187)
template <class T, class V>
__global__ void k_diff_zeta(Dims D, Grid<T> G, StateT<V> S, DiffBuf<T> B) {
  LG_IDX3;
  if (ji > D.ny + 1 || jk > D.nx + 1) return;
  B.zz[IX(D, ji, jk, jl)] = zeta_z_at<T, V>(D, G, S, ji, jk, jl);
}

// ---- 3. hor_diff_coeff_postprocessing (mo_eff_diff_coeffs.F90:161-310) and rel_vort ----------
// One thread per dual point (ny+1, nx+1, nl): viscosity_dual (the molecular pass the reference
// makes first is overwritten by the turbulent one, which already holds both parts) times
// zeta_z, the product mom_diff_h differentiates.  Non-periodic boundary dual points keep the
// initial zero of viscosity_dual.
template <class T, class V>
__global__ void k_diff_vz(Dims D, Grid<T> G, StateT<V> S, DiffBuf<T> B) {
  LG_IDX3;
  if (ji > D.ny + 1 || jk > D.nx + 1) return;
  const long long q = IX(D, ji, jk, jl);
  const T* v = B.visc;
  const V* rg = S.rho + (long long)(D.g - 1) * D.fstride;
  auto vs = [&](int i, int j) { return v[IX(D, i, j, jl)]; };
  auto rs = [&](int i, int j) { return T(rg[IX(D, i, j, jl)]); };
  const bool in_i = ji >= 2 && ji <= D.ny, in_k = jk >= 2 && jk <= D.nx;
  T vd = T(0);
  if (in_i && in_k) {
    vd = T(0.25) * (vs(ji - 1, jk - 1) + vs(ji - 1, jk) + vs(ji, jk - 1) + vs(ji, jk));
    vd = T(0.25) * (rs(ji - 1, jk - 1) + rs(ji - 1, jk) + rs(ji, jk - 1) + rs(ji, jk)) * vd;
  } else if (D.periodic) {
    if (in_k) {  // ji = 1 or ny+1 (the copy of 1)
      vd = T(0.25) * (vs(1, jk - 1) + vs(D.ny, jk - 1) + vs(1, jk) + vs(D.ny, jk));
      vd = vd * (T(0.25) * (rs(1, jk - 1) + rs(D.ny, jk - 1) + rs(1, jk) + rs(D.ny, jk)));
    } else if (in_i) {  // jk = 1 or nx+1
      vd = T(0.25) * (vs(ji - 1, D.nx) + vs(ji - 1, 1) + vs(ji, D.nx) + vs(ji, 1));
      vd = vd * (T(0.25) * (rs(ji - 1, D.nx) + rs(ji - 1, 1) + rs(ji, D.nx) + rs(ji, 1)));
    } else {  // corners
      vd = T(0.25) * (vs(1, 1) + vs(D.ny, 1) + vs(1, D.nx) + vs(D.ny, D.nx));
      vd = vd * (T(0.25) * (rs(D.ny, D.nx) + rs(D.ny, 1) + rs(1, D.nx) + rs(1, 1)));
    }
  }
  B.vz[q] = vd * B.zz[q];
}

// ---- 4. mom_diff_h (mo_momentum_diff_diss.F90:25-160) ----------------------------------------
// u and v points: the gradient of viscosity*divergence (grad_hor, whose terrain correction
// reads mom_diff_tend_z as the previous step left it: the reference passes that array as
// grad_hor's vertical component without forming it first), plus the curl of viscosity_dual *
// zeta_z with its terrain-following correction, divided by the averaged density.  The thread
// of jk = 1 (ji = 1) also writes the copy at nx+1 (ny+1); at non-periodic boundary edges the
// reference keeps the previous value (less slope times a zero remap).
template <class T, class V>
__global__ void k_mom_diff_h(Dims D, Grid<T> G, StateT<V> S, DiffBuf<T> B) {
  LG_IDX3;
  auto sdiv = [&](int i, int j, int l) { return B.vdiv[IX(D, i, j, l)]; };
  auto rsum = [&](int i, int j, int l) { return rho_sum_cond_gas<T, V>(D, S.rho, IX(D, i, j, l)); };
  const T* vz = B.vz;
  const T* zd = G.z_area_dual_z;
  const int ui = jl - 1 > 1 ? jl - 1 : 1, li = jl + 1 < D.nl ? jl + 1 : D.nl;
  // u points
  if (ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    const bool inner = jk >= 2;
    T r;
    if (inner || D.periodic) {
      const int kk = jk;  // jk = 1 evaluates the periodic formula; nx+1 is its copy
      const int ka = inner ? jk - 1 : D.nx;
      r = (sdiv(ji, kk, jl) - sdiv(ji, ka, jl)) / G.dx[IX(D, ji, kk, jl)];
      if (jl > D.nf) r = r - G.slope_x[q] * remap_x<T, T>(D, G, B.mdtz, ji, kk, jl);
      const T dyd = G.dy_dual[q];
      T up = (vz[IX(D, ji + 1, kk, jl)] - vz[IX(D, ji, kk, jl)]) / dyd;
      const T slope = (zd[IX(D, ji + 1, kk, jl)] - zd[IX(D, ji, kk, jl)]) / dyd;
      const T vg = T(0.5) * (vz[IX(D, ji + 1, kk, ui)] - vz[IX(D, ji + 1, kk, li)])
                     / (zd[IX(D, ji + 1, kk, ui)] - zd[IX(D, ji + 1, kk, li)])
                 + T(0.5) * (vz[IX(D, ji, kk, ui)] - vz[IX(D, ji, kk, li)])
                     / (zd[IX(D, ji, kk, ui)] - zd[IX(D, ji, kk, li)]);
      up = up - slope * vg;
      r = (r + up) / (T(0.5) * (rsum(ji, ka, jl) + rsum(ji, kk, jl)));
    } else {
      r = B.mdtx[q];
      if (jl > D.nf) r = r - G.slope_x[q] * T(0);
    }
    B.mdtx[q] = r;
    if (jk == 1) B.mdtx[IX(D, ji, D.nx + 1, jl)] = r;
  }
  // v points
  if (ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    const bool inner = ji >= 2;
    T r;
    if (inner || D.periodic) {
      const int ia = inner ? ji - 1 : D.ny;
      r = (sdiv(ia, jk, jl) - sdiv(ji, jk, jl)) / G.dy[q];
      if (jl > D.nf) r = r - G.slope_y[q] * remap_y<T, T>(D, G, B.mdtz, ji, jk, jl);
      const T dxd = G.dx_dual[q];
      T vp = (vz[IX(D, ji, jk + 1, jl)] - vz[q]) / dxd;
      const T slope = (zd[IX(D, ji, jk + 1, jl)] - zd[q]) / dxd;
      const T vg = T(0.5) * (vz[IX(D, ji, jk + 1, ui)] - vz[IX(D, ji, jk + 1, li)])
                     / (zd[IX(D, ji, jk + 1, ui)] - zd[IX(D, ji, jk + 1, li)])
                 + T(0.5) * (vz[IX(D, ji, jk, ui)] - vz[IX(D, ji, jk, li)])
                     / (zd[IX(D, ji, jk, ui)] - zd[IX(D, ji, jk, li)]);
      vp = vp - slope * vg;
      r = (r + vp) / (T(0.5) * (rsum(ia, jk, jl) + rsum(ji, jk, jl)));
    } else {
      r = B.mdty[q];
      if (jl > D.nf) r = r - G.slope_y[q] * T(0);
    }
    B.mdty[q] = r;
    if (ji == 1) B.mdty[IX(D, D.ny + 1, jk, jl)] = r;
  }
}

// ---- 5. mom_diff_v, vertical diffusion of w (mo_momentum_diff_diss.F90:277-329) -----------------
// w levels 2..nl: grad_vert of rho_g * (viscosity_molecular + the TKE's vertical coefficient) *
// add_vertical_div(w), divided by the averaged density (the horizontal diffusion of w in
// between adds zeros).  Levels 1 and nl+1 are not written.
template <class T, class V>
__global__ void k_mom_diff_v(Dims D, Grid<T> G, StateT<V> S, DiffBuf<T> B) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int jk = blockIdx.z * blockDim.y + threadIdx.y + 1;
  const int jl = blockIdx.y + 2;
  if (ji > D.ny || jk > D.nx || jl > D.nl) return;
  auto sp = [&](int l) -> T {
    const long long p = IX(D, ji, jk, l);
    const T cu = (l == 1) ? T(0) : T(S.w[p]);
    const T cl = (l == D.nl) ? T(0) : T(S.w[p + D.plane]);
    const T comp_v = cu * G.area_z[p] - cl * G.area_z[p + D.plane];
    const T dwdz = T(0) + comp_v / G.volume[p];
    const T coeff = B.vmol[p] + tke2vert<T>(B.tke[p], B.nsq[p], G.layer_thickness[p]);
    return T(S.rho[p + (long long)(D.g - 1) * D.fstride]) * coeff * dwdz;
  };
  const long long q = IX(D, ji, jk, jl);
  T m = (sp(jl - 1) - sp(jl)) / G.dz[q];
  m = m / (T(0.5) * (rho_sum_cond_gas<T, V>(D, S.rho, q - D.plane) + rho_sum_cond_gas<T, V>(D, S.rho, q)));
  B.mdtz[q] = m;
}

// ---- 6. simple_dissipation_rate (mo_momentum_diff_diss.F90:333-389) ------------------------------
// One thread per scalar point: the inner product of the wind with the momentum diffusion
// acceleration, whose w part carries the Klemp swamp layer's deceleration at w levels
// 2..n_damping_levels (damping_prefactor = damp, the column solver's prefactor), times
// -sum(rho(1:nc+1)).
// kdamp (split step, may be null): (1/damping_prefactor - 1)/dtime formed in FP64 per w point,
// so that the deceleration is w*kdamp without the cancellation of w/p - w in FP32
template <class T, class V>
__global__ void k_diss_rate(Dims D, Grid<T> G, StateT<V> S, DiffBuf<T> B, const T* damp, const T* kdamp) {
  LG_IDX3;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl), b = q + D.plane;
  auto wp = [&](long long p, int lev) -> T {
    T x = B.mdtz[p];
    if (D.lklemp && lev >= 2 && lev <= D.ndamp) {
      const T w = T(S.w[p]);
      x = x + (kdamp ? w * kdamp[p] : (w / damp[p] - w) / T(D.dtime));
    }
    return x;
  };
  const long long qu = IX(D, ji, jk + 1, jl), qv = IX(D, ji + 1, jk, jl);
  const T ip = W_(1, ji, jk, jl) * T(S.u[qu]) * B.mdtx[qu] + W_(2, ji, jk, jl) * T(S.v[q]) * B.mdty[q]
             + W_(3, ji, jk, jl) * T(S.u[q]) * B.mdtx[q] + W_(4, ji, jk, jl) * T(S.v[qv]) * B.mdty[qv]
             + W_(5, ji, jk, jl) * T(S.w[q]) * wp(q, jl) + W_(6, ji, jk, jl) * T(S.w[b]) * wp(b, jl + 1);
  B.hd[q] = -rho_sum_cond_gas<T, V>(D, S.rho, q) * ip;
}

// ---- 7. temperature and mass diffusion (mo_scalar_tend_expl.F90:60-101) ----------------------------
// The effective coefficients of scalar_diff_coeffs (mo_eff_diff_coeffs.F90:526-618) at a scalar
// point: horizontal and vertical, for mass (kind 0) and temperature (kind 1).  The specific
// heat c_g_v of spec_heat_cap_diagnostics_v (mo_derived.F90:40-68) is rho_g/rho_g*c_d_v.
template <class T, class V>
__device__ __forceinline__ T diff_coeff_h(const Dims& D, const StateT<V>& S, const DiffBuf<T>& B, int kind, long long p) {
  const T rg = T(S.rho[p + (long long)(D.g - 1) * D.fstride]);
  if (kind == 0) return B.visc[p] / rg;
  const T c_g_v = T(0) + rg / rg * T(kC_D_V);
  return c_g_v * B.visc[p];
}
template <class T, class V>
__device__ __forceinline__ T diff_coeff_v(const Dims& D, const Grid<T>& G, const StateT<V>& S, const DiffBuf<T>& B,
                                          int kind, long long p) {
  const T t2v = B.vmol[p] + tke2vert<T>(B.tke[p], B.nsq[p], G.layer_thickness[p]);
  if (kind == 0) return t2v;
  const T rg = T(S.rho[p + (long long)(D.g - 1) * D.fstride]);
  const T c_g_v = T(0) + rg / rg * T(kC_D_V);
  return rg * c_g_v * t2v;
}

// (the FP64 step's form of the scalar diffusion; the split step runs k_diff_scalar_col below)
// diffusive flux densities of nf scalar fields s0 + f*fstride (f = 0..nf-1): grad_hor with
// grad_vert of the field as its vertical component (mo_gradient_operators.F90:65-130; the
// vertical gradient formed inline, zero at levels 1 and nl+1), then scalar_times_vector_h/_v
// with the coefficients of `kind`, which are formed once per point for all fields.  fx, fy at
// u and v points (zero at non-periodic boundary edges, which the reference never writes), fw at
// w levels 2..nl (only with the vertical diffusion on); field f at offset f*fstride.  The
// addresses of the two cells of an edge and their metrics are formed once for all fields.
template <class T, class V, class SF, int NF>
__global__ void k_diff_fluxes(Dims D, Grid<T> G, StateT<V> S, DiffBuf<T> B, const SF* __restrict__ s0, int kind,
                              int vertical, T* __restrict__ fx, T* __restrict__ fy, T* __restrict__ fw) {
  LG_IDX3;
  constexpr int nf = NF;
  const long long pl = D.plane;
  const bool terrain = jl > D.nf;
  const bool lower = jl < D.nl || D.freeslip;
  const bool g_up = jl >= 2, g_lo = jl + 1 <= D.nl;  // grad_vert levels jl and jl+1 exist
  // the edge between cells a and b (b - a is the difference grad_hor_cov takes): slope, the
  // remap weights and the dz of the two vertical gradients of each cell
  struct Edge { long long a, b; T h, dxy, slope, w5a, w5b, w6a, w6b, dza, dzb, dza1, dzb1; };
  auto edge = [&](long long a, long long b, T h, T dxy, T slope) {
    Edge e{a, b, h, dxy, slope, T(0), T(0), T(0), T(0), T(1), T(1), T(1), T(1)};
    if (terrain) {
      e.w5a = G.ipw[4][a]; e.w5b = G.ipw[4][b];
      if (g_up) { e.dza = G.dz[a]; e.dzb = G.dz[b]; }
      if (lower) {
        e.w6a = G.ipw[5][a]; e.w6b = G.ipw[5][b];
        if (g_lo) { e.dza1 = G.dz[a + pl]; e.dzb1 = G.dz[b + pl]; }
      }
    }
    return e;
  };
  // grad_hor of one field at the edge: grad_hor_cov, minus slope times remap_ver2hor of the
  // vertical gradient (mo_averaging.F90:56-136, same order)
  auto grad = [&](const SF* s, const Edge& e, bool x) -> T {
    T g = x ? cvt<T>(s[e.b] - s[e.a]) / e.dxy : cvt<T>(s[e.a] - s[e.b]) / e.dxy;
    if (terrain) {
      const T gza = g_up ? cvt<T>(s[e.a - pl] - s[e.a]) / e.dza : T(0);
      const T gzb = g_up ? cvt<T>(s[e.b - pl] - s[e.b]) / e.dzb : T(0);
      T r = T(0);
      r = r + e.w5a * gza;
      r = r + e.w5b * gzb;
      if (lower) {
        const T gza1 = g_lo ? cvt<T>(s[e.a] - s[e.a + pl]) / e.dza1 : T(0);
        const T gzb1 = g_lo ? cvt<T>(s[e.b] - s[e.b + pl]) / e.dzb1 : T(0);
        r = r + e.w6a * gza1;
        r = r + e.w6b * gzb1;
      }
      g = g - e.slope * (T(0.5) * r);
    }
    return g;
  };
  auto ch = [&](long long p) { return diff_coeff_h<T, V>(D, S, B, kind, p); };
  if (ji <= D.ny && jk <= D.nx + 1) {
    const long long q = IX(D, ji, jk, jl);
    const bool inner = jk >= 2 && jk <= D.nx;
    if (!inner && !D.periodic) {
#pragma unroll
      for (int f = 0; f < nf; ++f) fx[q + (long long)f * D.fstride] = T(0);
    } else {
      // cells west (a = jk-1, periodic nx) and east (b = jk, periodic 1) of the u point
      const long long a = inner ? q - D.P : IX(D, ji, D.nx, jl), b = inner ? q : IX(D, ji, 1, jl);
      const T h = inner ? T(0.5) * (ch(a) + ch(b)) : T(0.5) * (ch(b) + ch(a));
      const Edge e = edge(a, b, h, G.dx[b], G.slope_x[q]);
#pragma unroll
      for (int f = 0; f < nf; ++f) fx[q + (long long)f * D.fstride] = e.h * grad(s0 + (long long)f * D.fstride, e, true);
    }
  }
  if (ji <= D.ny + 1 && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    const bool inner = ji >= 2 && ji <= D.ny;
    if (!inner && !D.periodic) {
#pragma unroll
      for (int f = 0; f < nf; ++f) fy[q + (long long)f * D.fstride] = T(0);
    } else {
      // cells north (a = ji-1, periodic ny) and south (b = ji, periodic 1) of the v point
      const long long a = inner ? q - 1 : IX(D, D.ny, jk, jl), b = inner ? q : IX(D, 1, jk, jl);
      const T h = inner ? T(0.5) * (ch(a) + ch(b)) : T(0.5) * (ch(b) + ch(a));
      const Edge e = edge(a, b, h, G.dy[b], G.slope_y[q]);
#pragma unroll
      for (int f = 0; f < nf; ++f) fy[q + (long long)f * D.fstride] = e.h * grad(s0 + (long long)f * D.fstride, e, false);
    }
  }
  if (vertical && jl >= 2 && ji <= D.ny && jk <= D.nx) {
    const long long q = IX(D, ji, jk, jl);
    const T h = T(0.5) * (diff_coeff_v<T, V>(D, G, S, B, kind, q - pl) + diff_coeff_v<T, V>(D, G, S, B, kind, q));
    const T dz = G.dz[q];
#pragma unroll
    for (int f = 0; f < nf; ++f) {
      const SF* s = s0 + (long long)f * D.fstride;
      fw[q + (long long)f * D.fstride] = h * (cvt<T>(s[q - pl] - s[q]) / dz);
    }
  }
}

// div_h of the flux densities of each of nf fields plus, with the vertical diffusion on,
// add_vertical_div of its fw (mo_divergence_operators.F90:16-68, 149-186).  The same expressions
// and order as div_h_at / vertical_contravariant_corr (mo_averaging.F90:16-54), with the
// addresses of the cell's faces and the metrics of the three layers the contravariant
// corrections read formed once per cell for all fields.
template <class T, int NF>
__global__ void k_diff_divs(Dims D, Grid<T> G, const T* __restrict__ fx, const T* __restrict__ fy,
                            const T* __restrict__ fw, int vertical, T* __restrict__ out) {
  LG_IDX3;
  constexpr int nf = NF;
  if (ji > D.ny || jk > D.nx) return;
  const long long q = IX(D, ji, jk, jl);
  const long long qe = q + D.P, qs = q + 1, pl = D.plane;
  // metrics of layer l (dl = -1, 0, +1 relative to jl) for the correction terms
  struct LM { T sxe, sy, sx, sys, w1, w2, w3, w4; };
  auto lm = [&](long long d) {
    LM m;
    m.sxe = G.slope_x[qe + d]; m.sy = G.slope_y[q + d]; m.sx = G.slope_x[q + d]; m.sys = G.slope_y[qs + d];
    m.w1 = G.ipw[0][q + d]; m.w2 = G.ipw[1][q + d]; m.w3 = G.ipw[2][q + d]; m.w4 = G.ipw[3][q + d];
    return m;
  };
  // which interfaces carry a correction: upper (jl) and lower (jl+1)
  const bool up_t = jl >= D.nf + 1, lo_t = jl + 1 >= D.nf + 1 && jl < D.nl;
  LM mu{}, mc{}, md{};
  if (jl >= D.nf + 2) mu = lm(-pl);
  if (jl >= D.nf) mc = lm(0);
  if (jl + 1 >= D.nf + 1 && jl < D.nl) md = lm(pl);
  const T ax_e = G.area_x[qe], ay_n = G.area_y[q], ax_w = G.area_x[q], ay_s = G.area_y[qs];
  const T az_u = G.area_z[q], az_l = G.area_z[q + pl], vol = G.volume[q];
#pragma unroll
  for (int f = 0; f < nf; ++f) {
    const long long o = (long long)f * D.fstride;
    const T* X = fx + o;
    const T* Y = fy + o;
    // r - 0.5*vx(e)*slope_x(e)*W1 - 0.5*vy(n)*slope_y(n)*W2 - 0.5*vx(w)*slope_x(w)*W3 - 0.5*vy(s)*slope_y(s)*W4
    auto terms = [&](T r, const LM& m, long long d) {
      return r - T(0.5) * X[qe + d] * m.sxe * m.w1 - T(0.5) * Y[q + d] * m.sy * m.w2
               - T(0.5) * X[q + d] * m.sx * m.w3 - T(0.5) * Y[qs + d] * m.sys * m.w4;
    };
    // vertical_contravariant_corr at interface jl (cu) and jl+1 (cl)
    T cu = T(0), cl = T(0);
    if (up_t) cu = (jl == D.nf + 1) ? terms(T(0), mc, 0) : terms(terms(T(0), mu, -pl), mc, 0);
    if (lo_t) cl = (jl + 1 == D.nf + 1) ? terms(T(0), md, pl) : terms(terms(T(0), mc, 0), md, pl);
    const T comp_h = X[qe] * ax_e + Y[q] * ay_n - X[q] * ax_w - Y[qs] * ay_s;
    T comp_v = T(0);
    if (jl == D.nf) comp_v = -cl * az_l;
    else if (jl == D.nl) comp_v = cu * az_u;
    else if (jl > D.nf) comp_v = cu * az_u - cl * az_l;
    T r = (comp_h + comp_v) / vol;
    if (vertical) {
      const T wu = (jl == 1) ? T(0) : fw[o + q];
      const T wl = (jl == D.nl) ? T(0) : fw[o + q + pl];
      r = r + (wu * az_u - wl * az_l) / vol;
    }
    out[o + q] = r;
  }
}

// ---- 7b. temperature and mass diffusion of the split step, fluxes and divergence fused ----------
// k_diff_fluxes followed by k_diff_divs, for the NM mass fields and (HT) the temperature
// together, in FP32, in one launch that marches down the levels: the flux densities never reach
// HBM and the metrics and coefficients are read once for all fields.  A block owns a tile of
// DS_X rows (ji, a lane each) by DS_Y columns (jk, a warp each) and walks it from the top layer to
// the bottom; three more warps hold the tile's halo: the columns jk0-1 and jk0+DS_Y, and the rows
// ji0-1 and ji0+DS_X (a lane per column).  Each level takes three phases, separated by barriers:
//   A  every slot (tile or halo cell, the periodic wrap applied) puts into shared memory its half
//      of the terrain remap of each field's vertical gradients, hc = ipw5*gz(l) + ipw6*gz(l+1),
//      and its horizontal coefficients;
//   B  each face is formed once, by the slot east (u point) or south (v point) of it:
//      h*((s_b - s_a)/dx - slope*0.5*(hc_a + hc_b)) with h = 0.5*(coef_a + coef_b);
//   C  each tile cell adds its four faces and the contravariant corrections of its two
//      interfaces.  The correction at an interface is the sum of the slope-weighted face terms of
//      the layers above and below it; a layer's term is formed once and carried to the next
//      level, and so is the divergence itself, which is finished one level later, when its
//      lower interface's correction and vertical flux are known.
// The field values arrive by cp.async into a ring of three levels (issued two levels ahead), so
// they take no registers; the metrics of phases B and C are issued at the top of the level and
// those of phase A a level ahead.  A column's vertical gradients and layer terms stay in shared
// memory.  The reference's sums (grad_hor's remap, vertical_contravariant_corr, div_h plus
// add_vertical_div: mo_averaging.F90:16-136, mo_divergence_operators.F90:16-68, 149-186) are
// regrouped, so the FP32 results differ from the two-kernel form in the last bits; the FP64 step
// keeps the two kernels and the reference's order.  Coefficients (scalar_diff_coeffs): mass
// viscosity/rho_gas and, vertically, the TKE one; temperature c_d_v times both, the vertical one
// also times rho_gas.
constexpr int DS_X = 32, DS_Y = 8, DS_THREADS = 32 * (DS_Y + 3);
constexpr int DS_SLOTS = (DS_X + 2) * (DS_Y + 2), DS_CELLS = DS_X * DS_Y;
// dynamic shared memory of k_diff_scalar_col for nf fields in all: the field values of three
// levels, the remap halves, the two coefficients, the vertical gradients of two levels and the
// carried layer terms of the slots, and the faces of one level
__host__ __device__ constexpr size_t diff_scalar_smem(int nf) {
  return sizeof(float) * ((size_t)3 * nf * DS_SLOTS + (size_t)nf * DS_SLOTS + 2 * DS_SLOTS +
                          (size_t)2 * nf * DS_SLOTS + (size_t)nf * DS_CELLS + (size_t)nf * (DS_Y + 1) * DS_X +
                          (size_t)nf * DS_Y * (DS_X + 1));
}

// all eight fields (seven constituents and the temperature) within the 227 KB a block may opt into
static_assert(diff_scalar_smem(8) <= 227 * 1024, "k_diff_scalar_col: shared memory of 8 fields");

// asynchronous 4-byte copy global -> shared (cp.async, no register staging) and its groups
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// NM mass fields at sm (fstride apart; results into out_m, vertical part with vert_m) and, with
// HT, the temperature at st (into out_t, vertical part with vert_t)
template <int NM, int HT>
__global__ void __launch_bounds__(DS_THREADS, 2)
k_diff_scalar_col(Dims D, Grid<float> G, StateF S, DiffBuf<float> B, const float* __restrict__ sm, int vert_m,
                  float* __restrict__ out_m, const float* __restrict__ st, int vert_t, float* __restrict__ out_t) {
  constexpr int NF = NM + HT, SX = DS_X + 2, NS = DS_SLOTS;
  extern __shared__ float4 ds_smem[];
  float* const ring = reinterpret_cast<float*>(ds_smem);  // [3][NF][NS]: level m at (m-1) % 3
  float* const sh_h = ring + 3 * NF * NS;                 // [NF][NS]
  float* const sh_c = sh_h + NF * NS;                     // [2][NS]: mass, temperature
  float* const sh_g = sh_c + 2 * NS;                      // [2][NF][NS]: gz(m) at m % 2
  float* const sh_t = sh_g + 2 * NF * NS;                 // [NF][DS_CELLS]
  float* const sh_fx = sh_t + NF * DS_CELLS;              // [NF][DS_Y+1][DS_X]
  float* const sh_fy = sh_fx + NF * (DS_Y + 1) * DS_X;    // [NF][DS_Y][DS_X+1]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ji0 = blockIdx.x * DS_X + 1, jk0 = blockIdx.y * DS_Y + 1;
  // the slot: role 0 tile, 1 west halo, 2 east halo, 3 north halo, 4 south halo, -1 none
  int ji = ji0, jk = jk0, role = -1;
  if (warp < DS_Y) { ji = ji0 + lane; jk = jk0 + warp; role = 0; }
  else if (warp == DS_Y) { ji = ji0 + lane; jk = jk0 - 1; role = 1; }
  else if (warp == DS_Y + 1) { ji = ji0 + lane; jk = jk0 + DS_Y; role = 2; }
  else if (lane < DS_Y) { ji = ji0 - 1; jk = jk0 + lane; role = 3; }
  else if (lane < 2 * DS_Y) { ji = ji0 + DS_X; jk = jk0 + lane - DS_Y; role = 4; }
  const int slot = (jk - jk0 + 1) * SX + (ji - ji0 + 1);
  // the cell whose values the slot holds: itself, or its image across a periodic edge
  bool has = role >= 0 && ji >= 0 && ji <= D.ny + 1 && jk >= 0 && jk <= D.nx + 1;
  if (!D.periodic) has = has && ji >= 1 && ji <= D.ny && jk >= 1 && jk <= D.nx;
  const int ci = ji < 1 ? D.ny : (ji > D.ny ? 1 : ji), ck = jk < 1 ? D.nx : (jk > D.nx ? 1 : jk);
  // the faces formed here: the u point (ji, jk) west of the slot and the v point (ji, jk) north of
  // it, zero at non-periodic edges (where the reference writes none)
  const bool fx_own = (role == 0 || role == 2) && ji >= 1 && ji <= D.ny && jk <= D.nx + 1;
  const bool fy_own = (role == 0 || role == 4) && ji <= D.ny + 1 && jk <= D.nx;
  const bool fx_zero = !D.periodic && (jk == 1 || jk == D.nx + 1);
  const bool fy_zero = !D.periodic && (ji == 1 || ji == D.ny + 1);
  const bool cell = role == 0 && ji <= D.ny && jk <= D.nx;
  const bool vm = NM > 0 && vert_m != 0 && cell, vt = HT > 0 && vert_t != 0 && cell;
  const int fr = jk - jk0, fc = ji - ji0;  // the slot's u point in sh_fx, v point in sh_fy
  const int tc = warp * DS_X + lane;       // the tile cell's index in sh_t
  const long long F = D.fstride, pl = D.plane, gF = (long long)(D.g - 1) * D.fstride;
  const int nl = D.nl, nf = D.nf;
  // u and v points of the slot at level 1 (dx, dy at the wrapped cell, slopes at the point itself)
  const long long qu1 = IX(D, ji >= 1 ? ji : 1, jk >= 1 ? jk : 1, 1);
  const long long qdx1 = IX(D, ji >= 1 ? ji : 1, jk == D.nx + 1 ? 1 : (jk >= 1 ? jk : 1), 1);
  const long long qdy1 = IX(D, ji == D.ny + 1 ? 1 : (ji >= 1 ? ji : 1), jk >= 1 ? jk : 1, 1);
  const long long c1 = has ? IX(D, ci, ck, 1) : 0;
  auto field = [&](int f) { return f < NM ? sm + (long long)f * F : st; };
  // the field values of level m into the ring (one commit group per level, empty past the bottom)
  auto fetch = [&](int m) {
    if (has && m <= nl) {
      float* dst = ring + ((m - 1) % 3) * NF * NS + slot;
      const long long o = c1 + (long long)(m - 1) * pl;
#pragma unroll
      for (int f = 0; f < NF; ++f) cp_async4(dst + f * NS, field(f) + o);
    }
    cp_async_commit();
  };
  // the inputs of phase A at one level, loaded a level ahead
  struct AIn { float w5, w6, dz1, vi, rg, vmol, tke, nsq, lt; };
  auto load_a = [&](int l) {
    AIn a{0.f, 0.f, 1.f, 0.f, 1.f, 0.f, 0.f, 0.f, 0.f};
    if (!has || l > nl) return a;
    const long long q = c1 + (long long)(l - 1) * pl;
    if (l > nf) {
      a.w5 = G.ipw[4][q];
      if (l < nl || D.freeslip) a.w6 = G.ipw[5][q];
    }
    if (l < nl) a.dz1 = G.dz[q + pl];
    a.vi = B.visc[q];
    a.rg = S.rho[q + gF];
    if (vm || vt) { a.vmol = B.vmol[q]; a.tke = B.tke[q]; a.nsq = B.nsq[q]; a.lt = G.layer_thickness[q]; }
    return a;
  };
  float P[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    P[f] = 0.f;
    if (has) sh_g[NF * NS + f * NS + slot] = 0.f;  // gz(1) (buffer 1 % 2): no gradient above the top layer
  }
  fetch(1);
  fetch(2);
  AIn ai = load_a(1);
  float cvp0 = 0.f, cvp1 = 0.f, volp = 1.f;
  for (int l = 1; l <= nl; ++l) {
    const long long lo = (long long)(l - 1) * pl, q = c1 + lo;
    const bool terrain = l > nf, g_lo = l < nl;
    // level l+2 into the slot of level l-1 (free since the last level's faces were formed);
    // then levels l and l+1 are complete
    fetch(l + 2);
    cp_async_wait1();
    // the metrics of phases B and C, issued first so that they arrive during phase A
    float bdx = 1.f, bsx = 0.f, bdy = 1.f, bsy = 0.f;
    if (fx_own && !fx_zero) {
      bdx = G.dx[qdx1 + lo];
      if (terrain) bsx = G.slope_x[qu1 + lo];
    }
    if (fy_own && !fy_zero) {
      bdy = G.dy[qdy1 + lo];
      if (terrain) bsy = G.slope_y[qu1 + lo];
    }
    float ax_w = 0.f, ax_e = 0.f, ay_n = 0.f, ay_s = 0.f, az = 0.f, vol = 1.f;
    float sxe = 0.f, sy = 0.f, sx = 0.f, sys = 0.f, i0 = 0.f, i1 = 0.f, i2 = 0.f, i3 = 0.f;
    if (cell) {
      ax_w = G.area_x[q]; ax_e = G.area_x[q + D.P]; ay_n = G.area_y[q]; ay_s = G.area_y[q + 1];
      az = G.area_z[q]; vol = G.volume[q];
      if (terrain) {
        sxe = G.slope_x[q + D.P]; sy = G.slope_y[q]; sx = G.slope_x[q]; sys = G.slope_y[q + 1];
        i0 = G.ipw[0][q]; i1 = G.ipw[1][q]; i2 = G.ipw[2][q]; i3 = G.ipw[3][q];
      }
    }
    const float* sc = ring + ((l - 1) % 3) * NF * NS;  // level l
    const float* sd = ring + (l % 3) * NF * NS;        // level l+1
    float* const gzl = sh_g + (l & 1) * NF * NS;       // gz(l)
    float* const gzn = sh_g + ((l + 1) & 1) * NF * NS;  // gz(l+1)
    // ---- A: the slot's remap halves and coefficients; the cell's vertical coefficients
    float hv0 = 0.f, hv1 = 0.f;
    if (has) {
      const float idz = g_lo ? 1.f / ai.dz1 : 0.f;
      if (NM > 0) sh_c[slot] = ai.vi / ai.rg;
      if (HT > 0) sh_c[NS + slot] = float(kC_D_V) * ai.vi;
      if (vm || vt) {  // diff_coeff_v at the cell; the interface above takes the mean with the layer above
        const float t2v = ai.vmol + tke2vert<float>(ai.tke, ai.nsq, ai.lt);
        const float cv1 = ai.rg * float(kC_D_V) * t2v;
        hv0 = 0.5f * (cvp0 + t2v);
        hv1 = 0.5f * (cvp1 + cv1);
        cvp0 = t2v;
        cvp1 = cv1;
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const float gn = g_lo ? (sc[f * NS + slot] - sd[f * NS + slot]) * idz : 0.f;
        if (terrain) sh_h[f * NS + slot] = ai.w5 * gzl[f * NS + slot] + ai.w6 * gn;
        gzn[f * NS + slot] = gn;
      }
    }
    ai = load_a(l + 1);
    __syncthreads();
    // ---- B: the faces
    if (fx_own) {
      const int a = slot - SX;
      const float h0 = fx_zero ? 0.f : 0.5f * (sh_c[a] + sh_c[slot]);
      const float h1 = fx_zero ? 0.f : 0.5f * (sh_c[NS + a] + sh_c[NS + slot]);
      const float idx = 1.f / bdx, sl = 0.5f * bsx;
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        float g = 0.f;
        if (!fx_zero) {
          g = (sc[f * NS + slot] - sc[f * NS + a]) * idx;
          if (terrain) g = g - sl * (sh_h[f * NS + a] + sh_h[f * NS + slot]);
        }
        sh_fx[(f * (DS_Y + 1) + fr) * DS_X + fc] = (f < NM ? h0 : h1) * g;
      }
    }
    if (fy_own) {
      const int a = slot - 1;
      const float h0 = fy_zero ? 0.f : 0.5f * (sh_c[a] + sh_c[slot]);
      const float h1 = fy_zero ? 0.f : 0.5f * (sh_c[NS + a] + sh_c[NS + slot]);
      const float idy = 1.f / bdy, sl = 0.5f * bsy;
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        float g = 0.f;
        if (!fy_zero) {
          g = (sc[f * NS + a] - sc[f * NS + slot]) * idy;
          if (terrain) g = g - sl * (sh_h[f * NS + a] + sh_h[f * NS + slot]);
        }
        sh_fy[(f * DS_Y + fr) * (DS_X + 1) + fc] = (f < NM ? h0 : h1) * g;
      }
    }
    __syncthreads();
    // ---- C: the divergence of the tile's cells
    if (cell) {
      // a layer's slope-weighted face terms (vertical_contravariant_corr)
      const float k1 = 0.5f * sxe * i0, k2 = 0.5f * sy * i1, k3 = 0.5f * sx * i2, k4 = 0.5f * sys * i3;
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const float* X = sh_fx + f * (DS_Y + 1) * DS_X;
        const float* Y = sh_fy + f * DS_Y * (DS_X + 1);
        const float xw = X[fr * DS_X + fc], xe = X[(fr + 1) * DS_X + fc];
        const float yn = Y[fr * (DS_X + 1) + fc], ys = Y[fr * (DS_X + 1) + fc + 1];
        const float comp_h = xe * ax_e + yn * ay_n - xw * ax_w - ys * ay_s;
        const float t = terrain ? -(xe * k1 + yn * k2 + xw * k3 + ys * k4) : 0.f;
        // the interface above the layer: correction (none above the terrain-following layers)
        // and vertical flux density (none at the top)
        float* const tpf = sh_t + f * DS_CELLS + tc;
        const float corr = !terrain ? 0.f : (l == nf + 1 ? t : *tpf + t);
        const bool vk = f < NM ? vm : vt;
        const float fw = (vk && l >= 2) ? (f < NM ? hv0 : hv1) * gzl[f * NS + slot] : 0.f;
        const float U = (corr + fw) * az;
        float* const o = f < NM ? out_m + (long long)f * F : out_t;
        if (l >= 2) o[q - pl] = (P[f] - U) / volp;
        P[f] = comp_h + U;
        *tpf = t;
      }
      volp = vol;
    }
  }
  if (cell) {
    const long long q = c1 + (long long)(nl - 1) * pl;
#pragma unroll
    for (int f = 0; f < NF; ++f) (f < NM ? out_m + (long long)f * F : out_t)[q] = P[f] / volp;
  }
}

}  // namespace lg
