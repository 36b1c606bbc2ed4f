// dev.cuh -- device data layout and the pointwise C-grid operators of the HEVI step.
//
// Layout in HBM: every 3-D field, whatever its staggering, is stored with the same
// padded shape [nl+1 planes][nx+1 columns][P rows], P = ny+1 rounded up to 32, with
// ji (y) fastest.  One index function serves scalar, u, v, w and dual points, so a
// thread that handles (ji,jk,jl) reads all staggered neighbours with fixed offsets:
// +-1 in ji is +-8 bytes, +-1 in jk is +-8*P bytes, +-1 in jl is +-8*P*(nx+1) bytes.
// Rows start on 256-byte boundaries, so a warp reading 32 consecutive ji of one row
// issues two fully used 128-byte transactions.  The extra row (ny+1), column (nx+1)
// and level (nl+1) hold the staggered points; padding is never read as data.
//
// Every operator below evaluates one output point exactly as the reference's loop
// body does (same operands, same left-to-right order, same boundary branches), so a
// fused kernel that recomputes an input inline produces the bits the reference would
// produce from the stored array.  The kernels are compiled with -fmad=false for the
// FP64 path so that no multiply-add is contracted.
#pragma once

#include <cstdint>

namespace lg {

struct Dims {
  int ny, nx, nl, NL, nf;   // NL = nl+1 levels, nf = n_flat_layers
  int P, NX1;               // padded row pitch (>= ny+1, multiple of 32), nx+1
  long long plane;          // P*NX1
  long long fstride;        // elements per field = plane*(nl+1)
  int nc, ncons, g;         // condensates, constituents, gas index (1-based) = nc+1
  int periodic, freeslip, lcorio, llinear, luse_bg, lmoist, theta_order, lklemp;
  double dtime, toa, dxn, dyn;  // namelist dx, dy
  double theta_edge_c;          // 1/8*dy*dx of the third-order theta edges, formed once on the host
  int ndamp;                    // n_damping_levels: levels whose highest z_w lies above klemp_begin_rel*toa
};

// ---- FP32 <-> FP64 conversions in integer operations ------------------------------
// On this GPU a hardware conversion between FP32 and FP64 issues on the FP64 pipe (about
// two per clock per SM, against 128 FP32 operations), so the split-precision kernels,
// which convert every value they move between the two precisions, do it with integer
// operations.  Both give the hardware's results bit for bit.

// FP32 -> FP64, exact: the exponent is rebiased (127 -> 1023) and the 23 mantissa bits
// shifted into place.  Zero keeps its sign; subnormals, infinities and NaN take the
// hardware conversion.
__device__ __forceinline__ double wide(float f) {
  const unsigned u = __float_as_uint(f), a = u & 0x7FFFFFFFu;
  if (a - 0x00800000u < 0x7F000000u)  // normal numbers
    return __hiloint2double((int)((u & 0x80000000u) | ((a >> 3) + (896u << 20))), (int)(a << 29));
  if (a == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
  return (double)f;
}

// FP64 -> FP32, rounded to nearest (ties to even), for results in the normal FP32 range
// (2^-126 <= |x| < 2^128): the top 23 of the 52 mantissa bits are kept and the 29 dropped
// bits decide the rounding; a carry out of the mantissa moves into the exponent (up to
// infinity, as the rounding requires).  Zero, FP32-subnormal results, overflow and NaN take
// the hardware conversion.
__device__ __forceinline__ float narrow(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned e = (hi >> 20) & 0x7FFu;
  if (e - 897u < 254u) {
    const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const unsigned f = (hi & 0x80000000u) | ((e - 896u) << 23) | m;
    const unsigned rest = lo & 0x1FFFFFFFu;
    return __uint_as_float(f + ((rest + (m & 1u) + 0x0FFFFFFFu) >> 29));
  }
  return (float)x;
}

// conversion of a value of type S to type T (identity when the types agree)
template <class T, class S>
__device__ __forceinline__ T cvt(S x) {
  if constexpr (sizeof(T) == 4 && sizeof(S) == 8) return narrow(x);
  else if constexpr (sizeof(T) == 8 && sizeof(S) == 4) return wide(x);
  else return T(x);
}

// Offset of point (i, j, k) in a field.  A field's padded extent (fstride) is below 2^31
// (lgame_gpu_create checks it), so the offset is formed in 32-bit signed arithmetic: two
// integer multiply-adds, and the compiler folds the offsets of neighbouring points (+-1, +-P,
// +-plane) into one base; offsets of further fields (constituents) are added in 64 bits.
__host__ __device__ __forceinline__ long long IX(const Dims& d, int i, int j, int k) {
  return (long long)((i - 1) + d.P * ((j - 1) + d.NX1 * (k - 1)));
}

// grid metrics (read-only), one pointer per reference array; ipw = inner_product_weights
template <class T>
struct Grid {
  const T *z_scalar, *z_u, *z_v, *z_w, *dx, *dy, *dz, *volume, *area_x, *area_y, *area_z;
  const T *area_dual_x, *area_dual_y, *area_dual_z, *z_area_dual_z, *slope_x, *slope_y;
  const T* ipw[6];
  const T *theta_v_bg, *exner_bg, *egu, *egv, *egw, *gm, *gp;
  const T *fvec_x, *fvec_y, *fvec_z;        // one plane each
  const T *trsk_u[3], *trsk_v[2];           // length P each
  const T* damp;                            // Klemp prefactor 1+damping_coeff*dtime at w points
  const T *dx_dual, *dy_dual, *layer_thickness;  // diffusion closure: dual distances (v, u points), layers
};

// prognostic state on the device; V = double: the state proper, V = float: the FP32 mirror
// of the split-precision step (rounded copies written by the kernels that update the state)
template <class V>
struct StateT {
  V *rho, *rt, *tp, *ep, *u, *v, *w;  // rho: ncons fields of fstride each
};
using State = StateT<double>;
using StateF = StateT<float>;

// physical constants, src/mo_constants.F90:12-37
constexpr double kR_E = 6371000.789927;
constexpr double kK_B = 1.380649e-23;
constexpr double kN_A = 6.02214076e23;
constexpr double kT_0 = 273.15;
constexpr double kRHO_H2O = 1024.0;
constexpr double kR_D = 287.057811;
constexpr double kC_D_V = 717.942189;
constexpr double kC_V_V = 1396.475121;
constexpr double kC_D_P = 1005.0;
constexpr double kP_0 = 100000.0;
constexpr double kR_V = 461.524879;
constexpr double kM_D = 6.02214076e23 * 0.004810e-23;
constexpr double kM_V = 6.02214076e23 * 0.002991e-23;
constexpr double kIMPL_THERMO_WEIGHT = 717.942189 / 1005.0;
constexpr double kPI = 3.14159265358979323846;

#define W_(n, i, j, k) (G.ipw[(n) - 1][IX(D, i, j, k)])

// ---- mo_averaging.F90 --------------------------------------------------------

// vertical_contravariant_corr, mo_averaging.F90:16-54; FX/FY return the horizontal
// vector components at u/v points (stored arrays or fluxes computed on the fly).
template <class T, class FX, class FY>
__device__ __forceinline__ T vcc(const Dims& D, const Grid<T>& G, FX vx, FY vy, int ji, int jk, int jl) {
  T r = T(0);
  if (jl >= D.nf + 1) {
    if (jl == D.nf + 1) {
      r = r - T(0.5) * vx(ji, jk + 1, jl) * G.slope_x[IX(D, ji, jk + 1, jl)] * W_(1, ji, jk, jl)
            - T(0.5) * vy(ji, jk, jl) * G.slope_y[IX(D, ji, jk, jl)] * W_(2, ji, jk, jl)
            - T(0.5) * vx(ji, jk, jl) * G.slope_x[IX(D, ji, jk, jl)] * W_(3, ji, jk, jl)
            - T(0.5) * vy(ji + 1, jk, jl) * G.slope_y[IX(D, ji + 1, jk, jl)] * W_(4, ji, jk, jl);
    } else {
      r = r - T(0.5) * vx(ji, jk + 1, jl - 1) * G.slope_x[IX(D, ji, jk + 1, jl - 1)] * W_(1, ji, jk, jl - 1)
            - T(0.5) * vy(ji, jk, jl - 1) * G.slope_y[IX(D, ji, jk, jl - 1)] * W_(2, ji, jk, jl - 1)
            - T(0.5) * vx(ji, jk, jl - 1) * G.slope_x[IX(D, ji, jk, jl - 1)] * W_(3, ji, jk, jl - 1)
            - T(0.5) * vy(ji + 1, jk, jl - 1) * G.slope_y[IX(D, ji + 1, jk, jl - 1)] * W_(4, ji, jk, jl - 1);
      r = r - T(0.5) * vx(ji, jk + 1, jl) * G.slope_x[IX(D, ji, jk + 1, jl)] * W_(1, ji, jk, jl)
            - T(0.5) * vy(ji, jk, jl) * G.slope_y[IX(D, ji, jk, jl)] * W_(2, ji, jk, jl)
            - T(0.5) * vx(ji, jk, jl) * G.slope_x[IX(D, ji, jk, jl)] * W_(3, ji, jk, jl)
            - T(0.5) * vy(ji + 1, jk, jl) * G.slope_y[IX(D, ji + 1, jk, jl)] * W_(4, ji, jk, jl);
    }
  }
  return r;
}

// remap_ver2hor_x, mo_averaging.F90:56-95 (vc: w-point field, read as type V)
template <class T, class V>
__device__ __forceinline__ T remap_x(const Dims& D, const Grid<T>& G, const V* vc, int ji, int jk, int jl) {
  T r = T(0);
  if (jk == 1 || jk == D.nx + 1) {
    if (!D.periodic) return r;
    r = r + W_(5, ji, D.nx, jl) * T(vc[IX(D, ji, D.nx, jl)]);
    r = r + W_(5, ji, 1, jl) * T(vc[IX(D, ji, 1, jl)]);
    if (jl < D.nl || D.freeslip) {
      r = r + W_(6, ji, D.nx, jl) * T(vc[IX(D, ji, D.nx, jl + 1)]);
      r = r + W_(6, ji, 1, jl) * T(vc[IX(D, ji, 1, jl + 1)]);
    }
  } else {
    r = r + W_(5, ji, jk - 1, jl) * T(vc[IX(D, ji, jk - 1, jl)]);
    r = r + W_(5, ji, jk, jl) * T(vc[IX(D, ji, jk, jl)]);
    if (jl < D.nl || D.freeslip) {
      r = r + W_(6, ji, jk - 1, jl) * T(vc[IX(D, ji, jk - 1, jl + 1)]);
      r = r + W_(6, ji, jk, jl) * T(vc[IX(D, ji, jk, jl + 1)]);
    }
  }
  return T(0.5) * r;
}

// remap_ver2hor_y, mo_averaging.F90:97-136
template <class T, class V>
__device__ __forceinline__ T remap_y(const Dims& D, const Grid<T>& G, const V* vc, int ji, int jk, int jl) {
  T r = T(0);
  if (ji == 1 || ji == D.ny + 1) {
    if (!D.periodic) return r;
    r = r + W_(5, D.ny, jk, jl) * T(vc[IX(D, D.ny, jk, jl)]);
    r = r + W_(5, 1, jk, jl) * T(vc[IX(D, 1, jk, jl)]);
    if (jl < D.nl || D.freeslip) {
      r = r + W_(6, D.ny, jk, jl) * T(vc[IX(D, D.ny, jk, jl + 1)]);
      r = r + W_(6, 1, jk, jl) * T(vc[IX(D, 1, jk, jl + 1)]);
    }
  } else {
    r = r + W_(5, ji - 1, jk, jl) * T(vc[IX(D, ji - 1, jk, jl)]);
    r = r + W_(5, ji, jk, jl) * T(vc[IX(D, ji, jk, jl)]);
    if (jl < D.nl || D.freeslip) {
      r = r + W_(6, ji - 1, jk, jl) * T(vc[IX(D, ji - 1, jk, jl + 1)]);
      r = r + W_(6, ji, jk, jl) * T(vc[IX(D, ji, jk, jl + 1)]);
    }
  }
  return T(0.5) * r;
}

// horizontal_covariant_x/y, mo_averaging.F90:138-176
template <class T, class V>
__device__ __forceinline__ T hcov_x(const Dims& D, const Grid<T>& G, const V* hx, const V* vc, int ji, int jk, int jl) {
  T r = T(hx[IX(D, ji, jk, jl)]);
  if (jl > D.nf) r = r + G.slope_x[IX(D, ji, jk, jl)] * remap_x<T, V>(D, G, vc, ji, jk, jl);
  return r;
}
template <class T, class V>
__device__ __forceinline__ T hcov_y(const Dims& D, const Grid<T>& G, const V* hy, const V* vc, int ji, int jk, int jl) {
  T r = T(hy[IX(D, ji, jk, jl)]);
  if (jl > D.nf) r = r + G.slope_y[IX(D, ji, jk, jl)] * remap_y<T, V>(D, G, vc, ji, jk, jl);
  return r;
}

// ---- mo_divergence_operators.F90 -------------------------------------------

// div_h, mo_divergence_operators.F90:16-68, one scalar point
template <class T, class FX, class FY>
__device__ __forceinline__ T div_h_at(const Dims& D, const Grid<T>& G, FX vx, FY vy, int ji, int jk, int jl) {
  const T comp_h = vx(ji, jk + 1, jl) * G.area_x[IX(D, ji, jk + 1, jl)]
                 + vy(ji, jk, jl) * G.area_y[IX(D, ji, jk, jl)]
                 - vx(ji, jk, jl) * G.area_x[IX(D, ji, jk, jl)]
                 - vy(ji + 1, jk, jl) * G.area_y[IX(D, ji + 1, jk, jl)];
  T comp_v = T(0);
  if (jl == D.nf) {
    const T cl = vcc<T>(D, G, vx, vy, ji, jk, jl + 1);
    comp_v = -cl * G.area_z[IX(D, ji, jk, jl + 1)];
  } else if (jl == D.nl) {
    const T cu = vcc<T>(D, G, vx, vy, ji, jk, jl);
    comp_v = cu * G.area_z[IX(D, ji, jk, jl)];
  } else if (jl > D.nf) {
    const T cu = vcc<T>(D, G, vx, vy, ji, jk, jl);
    const T cl = vcc<T>(D, G, vx, vy, ji, jk, jl + 1);
    comp_v = cu * G.area_z[IX(D, ji, jk, jl)] - cl * G.area_z[IX(D, ji, jk, jl + 1)];
  }
  return (comp_h + comp_v) / G.volume[IX(D, ji, jk, jl)];
}

// ---- mo_vorticities.F90 ------------------------------------------------------

// rel_vort_z_local, mo_vorticities.F90:423-538
template <class T, class V>
__device__ __forceinline__ T rel_vort_z_local(const Dims& D, const Grid<T>& G, const V* u, const V* v, int ji, int jk, int jl) {
  int j_i[4] = {ji, ji - 1, ji, ji};
  int j_k[4] = {jk, jk, jk - 1, jk};
  T r = T(0);
  if (ji == 1 || jk == 1 || ji == D.ny + 1 || jk == D.nx + 1) {
    if (!D.periodic) return r;
    j_i[0] = ji; j_k[0] = (jk == D.nx + 1) ? 1 : jk;
    j_i[1] = (ji == 1) ? D.ny : ji - 1; j_k[1] = jk;
    j_i[2] = ji; j_k[2] = (jk == 1) ? D.nx : jk - 1;
    j_i[3] = (ji == D.ny + 1) ? 1 : ji; j_k[3] = jk;
  }
  if (jl <= D.nf) {
    r = r + G.dy[IX(D, j_i[0], j_k[0], jl)] * T(v[IX(D, j_i[0], j_k[0], jl)])
          + T(-1) * G.dx[IX(D, j_i[1], j_k[1], jl)] * T(u[IX(D, j_i[1], j_k[1], jl)])
          + T(-1) * G.dy[IX(D, j_i[2], j_k[2], jl)] * T(v[IX(D, j_i[2], j_k[2], jl)])
          + G.dx[IX(D, j_i[3], j_k[3], jl)] * T(u[IX(D, j_i[3], j_k[3], jl)]);
  } else {
    const T zd = G.z_area_dual_z[IX(D, ji, jk, jl)];
#pragma unroll
    for (int jm = 0; jm < 4; ++jm) {
      const int ii = j_i[jm], kk = j_k[jm];
      const T sgn = (jm == 0 || jm == 3) ? T(1) : T(-1);
      if (jm == 0 || jm == 2) {
        const T zv = G.z_v[IX(D, ii, kk, jl)];
        const T l_rescale = (T(kR_E) + zd) / (T(kR_E) + zv);
        const T delta_z = zd - zv;
        int sh = 1;
        if (delta_z > T(0) || jl == D.nl) sh = -1;
        if (jl == 1) sh = 1;
        const T vv = T(v[IX(D, ii, kk, jl)]);
        const T vg = (vv - T(v[IX(D, ii, kk, jl + sh)])) / (zv - G.z_v[IX(D, ii, kk, jl + sh)]);
        r = r + sgn * l_rescale * G.dy[IX(D, ii, kk, jl)] * (vv + delta_z * vg);
      } else {
        const T zu = G.z_u[IX(D, ii, kk, jl)];
        const T l_rescale = (T(kR_E) + zd) / (T(kR_E) + zu);
        const T delta_z = zd - zu;
        int sh = 1;
        if (delta_z > T(0) || jl == D.nl) sh = -1;
        if (jl == 1) sh = 1;
        const T uu = T(u[IX(D, ii, kk, jl)]);
        const T vg = (uu - T(u[IX(D, ii, kk, jl + sh)])) / (zu - G.z_u[IX(D, ii, kk, jl + sh)]);
        r = r + sgn * l_rescale * G.dx[IX(D, ii, kk, jl)] * (uu + delta_z * vg);
      }
    }
  }
  return r;
}

// ---- mo_dictionary.F90 / mo_derived.F90 ---------------------------------------

// c_p_water, mo_dictionary.F90:112-145
__device__ __forceinline__ double c_p_water(double temperature) {
  double tc = temperature - kT_0, c;
  if (tc >= 0.0) {
    if (tc > 35.0) tc = 35.0;
    const double a = tc - 35.0;
    const double a2 = a * a;
    c = 0.9979 + 3.1e-6 * a2 + 3.8e-9 * (a2 * a2);
  } else {
    if (tc < -37.0) tc = -37.0;
    const double t2 = tc * tc;
    c = 1.000938 - 2.7052e-3 * tc - 2.3235e-5 * t2 + 4.3778e-6 * (t2 * tc) + 2.7136e-7 * (t2 * t2);
  }
  return 4186.8 * c;
}

// c_p_ice, mo_dictionary.F90:147-173
__device__ __forceinline__ double c_p_ice(double temperature) {
  double tl = temperature;
  if (tl > kT_0) tl = kT_0;
  if (tl < 20.0) tl = 20.0;
  const double q = tl / 125.1;
  const double c = -2.0572 + 0.14644 * tl + 0.06163 * tl * exp(-(q * q));
  return c / kM_V;
}

// saturation_pressure_ice_huang and _murphy, mo_dictionary.F90:416-442
__device__ __forceinline__ double sat_ice_huang(double temperature) {
  const double temp_c = temperature - kT_0;
  const double d = temp_c + 868.0;
  return exp(43.494 - 6545.8 / (temp_c + 278.0)) / (d * d);
}
__device__ __forceinline__ double sat_ice_murphy(double temperature) {
  return exp(9.550426 - 5723.265 / temperature + 3.53068 * log(temperature) - 0.00728332 * temperature);
}
// saturation_pressure_over_ice, mo_dictionary.F90:318-353 (its blend is written "+ (1-w) +")
__device__ __forceinline__ double sat_ice(double temperature) {
  double t_local = temperature;
  const double temp_c = t_local - kT_0;
  if (temp_c >= -80.0) {
    if (t_local > kT_0) t_local = kT_0;
    return sat_ice_huang(t_local);
  } else if (temp_c >= -100.0) {
    const double huang_weight = (temp_c + 100.0) / 20.0;
    return huang_weight * sat_ice_huang(t_local) + (1.0 - huang_weight) + sat_ice_murphy(t_local);
  }
  if (t_local < 110.0) t_local = 110.0;
  return sat_ice_murphy(t_local);
}
// c_p_cond, mo_dictionary.F90:175-189 (odd constituents are ice, even are water)
__device__ __forceinline__ double c_p_cond(int jc, double temperature) {
  return ((jc - 1) % 2 == 0) ? c_p_ice(temperature) : c_p_water(temperature);
}

// calc_diff_coeff, mo_derived.F90:189-216
__device__ __forceinline__ double calc_diff_coeff(double temperature, double density) {
  const double particle_radius = 130e-12;
  const double particle_mass = kM_D / kN_A;
  const double thermal_velocity = sqrt(8.0 * kK_B * temperature / (kPI * particle_mass));
  const double particle_density = density / particle_mass;
  const double cross_section = 4.0 * kPI * (particle_radius * particle_radius);
  const double mean_free_path = 1.0 / (1.4142135623730951 * particle_density * cross_section);
  return 1.0 / 3.0 * thermal_velocity * mean_free_path;
}

}  // namespace lg
