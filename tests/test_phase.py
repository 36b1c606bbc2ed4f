"""Phase transitions of the water constituents (calc_h2otracers_source_rates,
src/constituents/mo_phase_trans.F90:22-330) behind the lphase_trans extension switch: the
reference compiles the routine but never calls it, so its step keeps the rates at zero (which the
other tests check by running with the switch off).

CPU: the oracle's rates, heating rate and surface latent heat fluxes against a second, vectorised
numpy restatement (mo_dictionary.F90's saturation pressures, their derivatives, enhancement
factors and enthalpies); the rates conserve water in every cell away from the surface; the
switch changes the step; the library rejects it without moisture.  GPU: the FP64 step against the
oracle (state, rates, heating, latent fluxes) with and without the surface layer, and the split
step against the FP64 step.
"""
import numpy as np
import pytest

import cases
import lgame_gpu as L
import oracle as O
from test_surface import DIFF_ON, SFC_ON, with_land

T0, R_V, R_D, C_D_V, C_V_V = 273.15, 461.524879, 287.057811, 717.942189, 1396.475121
M_V = 6.02214076e23 * 0.002991e-23


def phase_case(key="jet", surface=True, **kw):
    cfg_name, ov = cases.SMALL[key]
    extra = {**DIFF_ON, **SFC_ON} if surface else {}
    return cases.namelist(cfg_name, **{**ov, **extra, "lphase_trans": True, **kw})


# ---- numpy restatement of mo_dictionary.F90 and mo_phase_trans.F90 ------------------------------------

def sat_water(t):
    tc = np.minimum(t - T0, 100.0)
    warm = np.exp(34.494 - 4924.99 / (tc + 237.1)) / (tc + 105.0) ** 1.57
    c = np.maximum(tc, -50.0)
    cold = (6.107799961 + 4.436518521e-1 * c + 1.428945805e-2 * c ** 2 + 2.650648471e-4 * c ** 3
            + 3.031240396e-6 * c ** 4 + 2.034080948e-8 * c ** 5 + 6.136820929e-11 * c ** 6)
    return np.where(tc > 0.0, warm, cold)


def sat_ice_huang(t):
    tc = t - T0
    return np.exp(43.494 - 6545.8 / (tc + 278.0)) / (tc + 868.0) ** 2


def sat_ice_murphy(t):
    return np.exp(9.550426 - 5723.265 / t + 3.53068 * np.log(t) - 0.00728332 * t)


def sat_ice(t):
    tc = t - T0
    w = (tc + 100.0) / 20.0
    return np.where(tc >= -80.0, sat_ice_huang(np.minimum(t, T0)),
                    np.where(tc >= -100.0, w * sat_ice_huang(t) + (1.0 - w) + sat_ice_murphy(t),
                             sat_ice_murphy(np.maximum(t, 110.0))))


def dsat_water(t):
    tc = t - T0
    d = sat_water(t) * (4924.99 / (tc + 237.1) ** 2 - 1.57 / (tc + 105.0))
    return np.where((tc > 100.0) | (tc < 0.0), 0.0, d)


def dsat_ice(t):
    tc = t - T0
    dh = sat_ice_huang(t) * (6545.8 / (tc + 278.0) ** 2 - 2.0 / (tc + 868.0))
    dm = sat_ice_murphy(t) * (5723.265 / t ** 2 + 3.53068 / t - 0.00728332)
    w = (tc + 100.0) / 20.0
    return np.where(tc > 0.0, 0.0, np.where(tc >= -80.0, dh, np.where(
        tc >= -100.0, w * dh + (1.0 - w) + dm, np.where(t >= 110.0, dm, 0.0))))


def h_evap(t):
    cold = (56579.0 - 42.212 * np.maximum(t, 30.0) + np.exp(0.1149 * (281.6 - np.maximum(t, 30.0)))) / M_V
    warm = 3151378.0 - 2386.0 * np.minimum(t, T0 + 100.0)
    return np.where(t < T0, cold, warm)


def h_subl(t):
    tl = np.minimum(np.maximum(t, 30.0), T0)
    return (46782.5 + 35.8925 * tl - 0.07414 * tl ** 2 + 541.5 * np.exp(-(tl / 123.75) ** 2)) / M_V


def c_p_water(t):
    tc = t - T0
    a = np.minimum(tc, 35.0) - 35.0
    c2 = np.maximum(tc, -37.0)
    return 4186.8 * np.where(tc >= 0.0, 0.9979 + 3.1e-6 * a ** 2 + 3.8e-9 * a ** 4,
                             1.000938 - 2.7052e-3 * c2 - 2.3235e-5 * c2 ** 2 + 4.3778e-6 * c2 ** 3
                             + 2.7136e-7 * c2 ** 4)


def c_p_ice(t):
    tl = np.maximum(np.minimum(t, T0), 20.0)
    return (-2.0572 + 0.14644 * tl + 0.06163 * tl * np.exp(-(tl / 125.1) ** 2)) / M_V


def np_rates(rho, t, dtime, sfc=None):
    """calc_h2otracers_source_rates over all cells: (rates (…, 6), heating, lat_lake, lat_sea)."""
    rv, rg = rho[..., 6], rho[..., 5]
    warm = t >= T0
    wvp = rv * R_V * t
    air = (rg - rv) * R_D * t + wvp
    ef = np.where(warm, 1.00071 * np.exp(0.000000045 * air), 0.99882 * np.exp(0.00000008 * air))
    sp = ef * np.where(warm, sat_water(t), sat_ice(t))
    cv = sum(rho[..., jc - 1] * (c_p_ice(t) if (jc - 1) % 2 == 0 else c_p_water(t)) for jc in range(1, 6))
    cv = cv + (rg - rv) * C_D_V + rv * C_V_V
    h = np.where(warm, h_evap(t), h_subl(t))
    h3 = h_subl(t) - h_evap(t)
    a = -R_V * h / cv
    b = R_V * t - R_V * rv * h / cv + ef * np.where(warm, dsat_water(t), dsat_ice(t)) * h / cv
    p, q = b / a, (wvp - sp) / a
    dd = -0.5 * p - np.sqrt(0.25 * p ** 2 - q)
    unsat = sp >= wvp
    ptd = np.where(unsat, np.minimum(np.where(warm, rho[..., 3], rho[..., 2]), dd), dd)
    r = np.zeros(rho.shape[:-1] + (6,))
    r[..., 2] = np.where(warm, -rho[..., 2] / dtime, rho[..., 3] / dtime - ptd / dtime)
    r[..., 3] = np.where(warm, rho[..., 2] / dtime - ptd / dtime, -rho[..., 3] / dtime)
    r[..., 5] = ptd / dtime
    heat = np.where(warm, r[..., 2] * h3, -r[..., 3] * h3) - ptd * h / dtime
    r[..., 0] = np.where(~warm, np.maximum(rho[..., 2] - 0.2e-3 * rg, 0.0) / 1000.0, 0.0)
    r[..., 1] = np.where(warm, np.maximum(rho[..., 3] - 0.2e-3 * rg, 0.0) / 1000.0, 0.0)
    r[..., 2] -= r[..., 0]
    r[..., 3] -= r[..., 1]
    melt = warm & (rho[..., 0] > 0.0)
    r[..., 0] = np.where(melt, -rho[..., 0] / dtime, r[..., 0])
    r[..., 1] = np.where(melt, r[..., 1] - r[..., 0], r[..., 1])
    heat = np.where(melt, heat + r[..., 0] * h3, heat)
    frz = ~warm & (rho[..., 1] > 0.0)
    r[..., 1] = np.where(frz, -rho[..., 1] / dtime, r[..., 1])
    r[..., 0] = np.where(frz, r[..., 0] - r[..., 1], r[..., 0])
    heat = np.where(frz, heat - r[..., 1] * h3, heat)
    lat_lake = lat_sea = None
    if sfc is not None:
        land, lake, ts, sst, sfr, lt = sfc
        airN, rvN = air[:, :, -1], rv[:, :, -1]

        def sat_sfc(x):
            return np.where(x >= T0, 1.00071 * np.exp(0.000000045 * airN) * sat_water(x),
                            0.99882 * np.exp(0.00000008 * airN) * sat_ice(x))
        dd_sea = (1.0 - land - lake) * (sat_sfc(sst) / (R_V * sst) - rvN)
        dd_lake = lake * (sat_sfc(ts) / (R_V * ts) - rvN)
        e_sea, e_lake = np.maximum(0.0, dd_sea / sfr), np.maximum(0.0, dd_lake / sfr)
        on = land < 1.0
        r[:, :, -1, 5] = np.where(on, r[:, :, -1, 5] + e_sea / lt + e_lake / lt, r[:, :, -1, 5])
        lat_lake = np.where(on, -np.where(ts >= T0, h_evap(ts), h_subl(ts)) * e_lake, 0.0)
        lat_sea = np.where(on, -np.where(sst >= T0, h_evap(sst), h_subl(sst)) * e_sea, 0.0)
    return r, heat, lat_lake, lat_sea


def _setup(surface):
    """The moist jet; with the surface layer, land and lake columns (test_surface.with_land) and
    sea and soil warmer than the air above them, so that water evaporates from both."""
    n = phase_case(surface=surface)
    hm = L.HostModel(n)
    if not surface:
        return n, hm, hm.grid, hm.diag, hm.copy_state()
    grid, diag = with_land(hm)
    state = hm.copy_state()
    state["temperature_soil"][...] = 300.0
    diag["sst"] = np.asfortranarray(np.full((hm.ny, hm.nx), 302.0))
    return n, hm, grid, diag, state


def _oracle_step(n, grid, diag, state=None):
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    o = O.Oracle(cfg, grid)
    st = state if state is not None else hm.state
    o.set_state(0, st)
    o.set_state(1, st)
    o.set_diag(diag)
    o.pchevi(0, 1, 0)
    d = o.get_diag()
    o.close()
    return hm, cfg, d


@pytest.mark.parametrize("surface", [False, True])
def test_oracle_rates_numpy(surface):
    """The rates and the heating rate formed at the first substep from the initial state and its
    temperature; with the surface layer, the evaporation from sea and lakes into the lowest layer
    and the latent heat flux densities (land and lake columns, sea elsewhere)."""
    n, hm0, grid, diag, state = _setup(surface)
    hm, cfg, d = _oracle_step(n, grid, diag, state)
    rho, t = state["rho"], d["temperature"]
    sfc = None
    if surface:
        sfc = (grid["land_fraction"], grid["lake_fraction"], state["temperature_soil"][:, :, 0], diag["sst"],
               d["scalar_flux_resistance"], grid["layer_thickness"][:, :, -1])
    r, heat, lat_lake, lat_sea = np_rates(rho, t, cfg.dtime, sfc)
    got = d["phase_trans_rates"]
    for k in (0, 1, 2, 3, 5):
        assert np.abs(r[..., k]).max() > 0.0, k
        err = np.abs(got[..., k] - r[..., k]).max() / np.abs(r[..., k]).max()
        assert err <= 1e-10, (k, err)
    assert np.all(got[..., 4] == 0.0)  # graupel's rate is never written
    assert cases.rel_err(d["phase_trans_heating_rate"], heat) <= 1e-10
    if surface:
        assert np.abs(lat_lake).max() > 0.0 and np.abs(lat_sea).max() > 0.0
        assert cases.rel_err(d["power_flux_density_lat_lake"], lat_lake) <= 1e-12
        assert cases.rel_err(d["power_flux_density_lat_sea"], lat_sea) <= 1e-12


def test_oracle_rates_conserve_water():
    """Away from the surface every cell's rates add up to zero: what one water constituent loses
    another gains (the surface evaporation is the only source)."""
    n = phase_case(surface=False)
    hm = L.HostModel(n)
    _, _, d = _oracle_step(n, hm.grid, hm.diag)
    r = d["phase_trans_rates"]
    total = r[..., :5].sum(axis=-1) + r[..., 5]
    scale = np.abs(r).max()
    assert np.abs(total).max() <= 1e-12 * scale


def test_oracle_phase_transitions_change_the_step():
    """With the switch the water constituents and rhotheta_v of the step differ from the run
    without (whose rates stay zero, as in the reference's step)."""
    outs = []
    for on in (True, False):
        n = phase_case(surface=False, lphase_trans=on)
        hm = L.HostModel(n)
        _, cfg, d = _oracle_step(n, hm.grid, hm.diag)
        outs.append(d)
    assert np.all(outs[1]["phase_trans_rates"] == 0.0) and np.all(outs[1]["phase_trans_heating_rate"] == 0.0)
    assert np.abs(outs[0]["tend_rho"] - outs[1]["tend_rho"]).max() > 0.0
    assert np.abs(outs[0]["tend_rhotheta_v"] - outs[1]["tend_rhotheta_v"]).max() > 0.0


def test_create_rejects_phase_transitions_without_moisture():
    import ctypes as C
    n = cases.small_case("schaer")
    cfg = L.config_from_namelist(n)
    cfg.lphase_trans = 1
    h = C.c_void_p()
    rc = L.load_library().lgame_gpu_create(C.byref(cfg), C.byref(h))
    assert rc == L.ERR_BAD_CONFIG and not h.value


# ---- GPU --------------------------------------------------------------------------------------------

PHASE_DIAG = ["phase_trans_rates", "phase_trans_heating_rate", "power_flux_density_lat_lake",
              "power_flux_density_lat_sea", "tend_rho", "tend_rhotheta_v"]


@pytest.mark.gpu
@pytest.mark.parametrize("surface", [False, True])
def test_fp64_phase_transitions_match_oracle(surface):
    n, hm, grid, diag, state = _setup(surface)
    cfg = L.config_from_namelist(n)
    o = O.Oracle(cfg, grid)
    cfg.precision = L.PRECISION_FP64
    g = L.GpuModel(cfg, grid)
    for m in (o, g):
        m.set_state(0, state)
        m.set_state(1, state)
        m.set_diag(diag)
    nsteps = 4
    for k in range(nsteps):
        o.pchevi(k % 2, (k + 1) % 2, k)
        g.pchevi(k % 2, (k + 1) % 2, k)
    so, sg = o.get_state(nsteps % 2), g.get_state(nsteps % 2)
    do, dgpu = o.get_diag(), g.get_diag()
    g.close()
    o.close()
    for f in so:
        assert cases.rel_err(sg[f], so[f]) <= 1e-12, (f, cases.rel_err(sg[f], so[f]))
    for f in PHASE_DIAG:
        assert cases.rel_err(dgpu[f], do[f]) <= 1e-10, (f, cases.rel_err(dgpu[f], do[f]))
    assert np.abs(do["phase_trans_rates"]).max() > 0.0


@pytest.mark.gpu
def test_split_phase_transitions_close_to_fp64():
    """The split step with the phase transitions against the FP64 step: the state after ten steps
    within the split step's bar (3e-5 of each field's maximum)."""
    from test_split import field_errors
    n, hm, grid, diag, state = _setup(True)
    gs = []
    for prec in (L.PRECISION_FP64, L.PRECISION_SPLIT):
        cfg = L.config_from_namelist(n)
        cfg.precision = prec
        g = L.GpuModel(cfg, grid)
        g.set_state(0, state)
        g.set_state(1, state)
        g.set_diag(diag)
        gs.append(g)
    for step in range(10):
        for g in gs:
            g.pchevi(step % 2, (step + 1) % 2, step)
    a, b = gs[1].get_state(0), gs[0].get_state(0)
    da, db = gs[1].get_diag(), gs[0].get_diag()
    for g in gs:
        g.close()
    errs = field_errors(a, b)
    assert max(errs.values()) <= 3e-5, errs
    assert np.all(np.isfinite(da["phase_trans_rates"]))
    assert cases.rel_err(da["phase_trans_heating_rate"], db["phase_trans_heating_rate"]) <= 1e-2
