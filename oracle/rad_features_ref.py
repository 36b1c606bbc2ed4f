"""Oracle of the radiation emulator's column features -- TEST INFRASTRUCTURE ONLY.

A numpy FP64 restatement of the inputs the reference hands to its radiation scheme for one
column, in the feature layout of include/lgame_emulator.h (4*nlev+2 floats per column,
column index ji + ny*(jk-1)), used by tests/ to check lgame_gpu_rad_features:

- temperature: temperature_diagnostics, src/constituents/mo_derived.F90:26-36,
  (theta_v_bg + theta_v_pert)*(exner_bg + exner_pert), divided in moist runs by
  1 + rho(nc+2)/rho(nc+1)*(m_d/m_v - 1);
- pressure: r_d*rho(nc+1)*T, src/radiation/mo_rterrtmgp_coupler.F90:161-167;
- water vapour density: rho(nc+2) (0 in dry runs);
- ozone density: calc_o3_vmr(z_scalar), src/constituents/mo_dictionary.F90:66-86 (a Gaussian
  of FWHM 20 km around 34 km with maximum 8.5e-6), times rho(nc+1)*M_O3/M_dry;
- surface albedo;
- cosine of the zenith angle: coszenith, src/radiation/mo_rterrtmgp_coupler.F90:550-629
  (the Earth's rotation and revolution relative to the winter solstice 2019-12-20 12:00 UTC,
  0 at night).

Every expression keeps the reference's operands and order; the GPU kernel computes in FP64
and rounds each feature to float once, so the two agree to a unit in the last place of the
float (the transcendental functions of the two libraries may differ in their last FP64 bit).
"""
from __future__ import annotations

import numpy as np

R_D = 287.057811
N_A = 6.02214076e23
M_D = N_A * 0.004810e-23
M_V = N_A * 0.002991e-23
M_O3 = 0.0479982  # kg/mol


def coszenith(lat, lon, t):
    """mo_rterrtmgp_coupler.F90:550-629, elementwise over lat/lon arrays (radians)."""
    omega, omega_rev, obliquity = 7.292115e-5, 1.99099e-7, 0.409092592843564
    t_transformed = t - 1576843200.0
    rot = omega * t_transformed - 0.0
    n = np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)])
    trans = np.array([[-np.cos(rot) * np.cos(obliquity), np.sin(rot) * np.cos(obliquity), np.sin(obliquity)],
                      [-np.sin(rot), -np.cos(rot), 0.0],
                      [np.cos(rot) * np.sin(obliquity), -np.sin(rot) * np.sin(obliquity), np.cos(obliquity)]])
    rel_sun = [trans[r, 0] * n[0] + trans[r, 1] * n[1] + trans[r, 2] * n[2] for r in range(3)]
    s2e = [np.cos(omega_rev * t_transformed + 0.0), np.sin(omega_rev * t_transformed + 0.0), 0.0]
    c = rel_sun[0] * -s2e[0] + rel_sun[1] * -s2e[1] + rel_sun[2] * -s2e[2]
    return np.where(c < 0.0, 0.0, c)


def calc_o3_vmr(height):
    """mo_dictionary.F90:66-86."""
    fwhm, max_height, max_vmr = 20e3, 34e3, 8.5e-6
    sigma = fwhm / (8.0 * np.log(2.0)) ** 0.5
    distance = height - max_height
    return max_vmr * np.exp(-distance ** 2 / (2.0 * sigma ** 2))


def features(state: dict, grid: dict, albedo, lat, lon, t: float, lmoist: bool) -> np.ndarray:
    """Feature rows (ny*nx, 4*nl+2) in float64 before the final rounding to float."""
    rho = state["rho"]
    ny, nx, nl = rho.shape[:3]
    nc = 5 if lmoist else 0
    rd = rho[..., nc]
    rv = rho[..., nc + 1] if lmoist else np.zeros_like(rd)
    T = (grid["theta_v_bg"] + state["theta_v_pert"]) * (grid["exner_bg"] + state["exner_pert"])
    if lmoist:
        T = T / (1.0 + rv / rd * (M_D / M_V - 1.0))
    p = R_D * rd * T
    o3 = calc_o3_vmr(grid["z_scalar"]) * rd * M_O3 / M_D

    def col(a):  # (ny, nx, nl) -> (ny*nx, nl), column ji + ny*(jk-1)
        return np.asarray(a).reshape(ny * nx, nl, order="F")

    x = np.empty((ny * nx, 4 * nl + 2))
    x[:, :nl] = col(T)
    x[:, nl:2 * nl] = col(p)
    x[:, 2 * nl:3 * nl] = col(rv)
    x[:, 3 * nl:4 * nl] = col(o3)
    x[:, 4 * nl] = np.asarray(albedo).reshape(-1, order="F")
    x[:, 4 * nl + 1] = coszenith(np.asarray(lat).reshape(-1, order="F"), np.asarray(lon).reshape(-1, order="F"), t)
    return x
