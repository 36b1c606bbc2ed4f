"""Lateral boundary relaxation of non-periodic runs (src/io/mo_boundaries.F90).

CPU: the oracle's rescale factors (setup_bc_factor, :125-170) and its update
(update_boundaries, :19-97) against a numpy restatement of the Fortran, including the
level swap when the old weight turns negative (the loader is asked for t_latest_bc +
dtime_bc into the old index, the indices swap, t_latest_bc advances, the weights are not
recomputed) and the step hook (mo_manage_pchevi.F90:114-116).

GPU: the FP64 step with the relaxation against the oracle, <= 1e-12 per field (the blend
is evaluated in the oracle's order without fused multiply-adds; exner_pert goes through
pow(), which need not round as the C library's does), over steps that cross two level
swaps, dry and moist; the split step against the FP64 step with the FP32/FP64 split's bar.
"""
import math

import numpy as np
import pytest

import cases
import lgame_gpu as L
import oracle as O

R_D, C_D_V, P_0 = 287.057811, 717.942189, 100000.0


def _namelist(key):
    if key == "jet_nonperiodic":
        return cases.namelist("jet_1024x1024x80", **{**cases.SMALL["jet"][1], "lperiodic": False, "lfreeslip": False})
    return cases.small_case(key)


def _level(hm, t):
    """A boundary level for valid time t: the initial state with seeded perturbations."""
    rng = np.random.default_rng(int(round(t)) + 1)
    st = hm.copy_state()
    return {"rho": st["rho"] * (1.0 + 1e-3 * rng.standard_normal(st["rho"].shape)),
            "rhotheta_v": st["rhotheta_v"] * (1.0 + 1e-3 * rng.standard_normal(st["rhotheta_v"].shape)),
            "wind_u": st["wind_u"] + rng.standard_normal(st["wind_u"].shape),
            "wind_v": st["wind_v"] + rng.standard_normal(st["wind_v"].shape),
            "wind_w": st["wind_w"] + 0.01 * rng.standard_normal(st["wind_w"].shape)}


def _factors_ref(n_swamp, n1, n2):
    f = np.zeros((n1, n2))
    for ji in range(1, n1 + 1):
        for jk in range(1, n2 + 1):
            d = float(min(ji - 1, jk - 1, n1 - ji, n2 - jk))
            f[ji - 1, jk - 1] = math.sin(0.5 * math.pi * max(1.0 - d / n_swamp, 0.0)) ** 2
    return f


def _oracle(key, loader_log=None, n_swamp=3, dtime_bc=15):
    n = _namelist(key)
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    o = O.Oracle(cfg, hm.grid)
    o.set_state(0, hm.state)
    o.set_state(1, hm.state)
    o.set_diag(hm.diag)

    def loader(t, idx):
        if loader_log is not None:
            loader_log.append((t, idx))
        return _level(hm, t)
    o.bc_setup(n_swamp, dtime_bc, 0.0, loader)
    o.set_bc(1, _level(hm, 0.0))
    o.set_bc(2, _level(hm, float(dtime_bc)))
    return hm, cfg, o


@pytest.mark.parametrize("n_swamp", [1, 3, 40])
def test_bc_factors(n_swamp):
    hm, cfg, o = _oracle("hills_nonperiodic", n_swamp=n_swamp)
    fs, fu, fv = o.bc_factors()
    ny, nx = cfg.ny, cfg.nx
    np.testing.assert_array_equal(fs, _factors_ref(n_swamp, ny, nx))
    np.testing.assert_array_equal(fu, _factors_ref(n_swamp, ny, nx + 1))
    np.testing.assert_array_equal(fv, _factors_ref(n_swamp, ny + 1, nx))
    assert np.all(fs[0, :] == 1.0) and np.all(fs[:, -1] == 1.0)
    if n_swamp < min(ny, nx) // 2:
        assert fs[ny // 2, nx // 2] == 0.0
    o.close()


def test_update_boundaries_formula_and_swap():
    log = []
    hm, cfg, o = _oracle("hills_nonperiodic", loader_log=log)
    fs, fu, fv = o.bc_factors()
    lev = {1: _level(hm, 0.0), 2: _level(hm, 15.0)}
    grid = hm.grid
    slot = 1
    t_latest, io, inew = 0.0, 1, 2
    for t_now in (6.0, 14.0, 21.0, 29.0, 52.0):
        s = o.get_state(slot)
        ow = 1.0 - (t_now - t_latest) / 15
        if ow < 0.0:
            lev[io] = _level(hm, t_latest + 15)
            io, inew = inew, (2 if inew == 1 else 1)
            t_latest += 15
        nw = 1.0 - ow
        o.update_boundaries(slot, t_now)
        r = o.get_state(slot)
        exp = {}
        for f, fac in (("rho", fs), ("rhotheta_v", fs), ("wind_w", fs), ("wind_u", fu), ("wind_v", fv)):
            b = fac[:, :, None, None] if f == "rho" else fac[:, :, None]
            exp[f] = b * (ow * lev[io][f] + nw * lev[inew][f]) + (1.0 - b) * s[f]
            np.testing.assert_allclose(r[f], exp[f], rtol=1e-15, atol=0, err_msg=f"t={t_now} {f}")
        g = hm.ncons - 2 if hm.ncons > 1 else 0
        tp = exp["rhotheta_v"] / exp["rho"][..., g] - grid["theta_v_bg"]
        ep = (R_D * exp["rhotheta_v"] / P_0) ** (R_D / C_D_V) - grid["exner_bg"]
        np.testing.assert_allclose(r["theta_v_pert"], tp, rtol=0, atol=1e-12 * np.abs(tp).max())
        np.testing.assert_allclose(r["exner_pert"], ep, rtol=0, atol=1e-13)
        assert o.bc_state() == (io, inew, t_latest)
    # loads at t = 21 (old weight -0.4) and t = 52 (-1.47, one load only)
    assert log == [(15.0, 1), (30.0, 2)]
    o.close()


def test_update_boundaries_without_loader_fails():
    n = cases.small_case("hills_nonperiodic")
    hm = L.HostModel(n)
    o = O.Oracle(L.config_from_namelist(n), hm.grid)
    o.set_state(0, hm.state)
    o.bc_setup(3, 15, 0.0, None)
    o.update_boundaries(0, 10.0)  # old weight 1/3: no new level needed
    with pytest.raises(RuntimeError):
        o.update_boundaries(0, 16.0)
    o.close()


def test_bc_setup_rejected_when_periodic():
    n = cases.small_case("hills")
    hm = L.HostModel(n)
    o = O.Oracle(L.config_from_namelist(n), hm.grid)
    with pytest.raises(RuntimeError):
        o.bc_setup(3, 15, 0.0, None)
    o.close()


def test_oracle_step_relaxes_the_rim():
    """With both levels equal to the initial state, the outer ring keeps the initial
    values to the blend's round-off, and the step hook is active (without boundary data
    the ring evolves freely)."""
    n = _namelist("jet_nonperiodic")
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    runs = []
    for with_bc in (True, False):
        o = O.Oracle(cfg, hm.grid)
        o.set_state(0, hm.state)
        o.set_state(1, hm.state)
        o.set_diag(hm.diag)
        if with_bc:
            o.bc_setup(3, 10800, 0.0, None)
            st = hm.copy_state()
            lev = {f: st[f] for f in L.BC_FIELDS}
            o.set_bc(1, lev)
            o.set_bc(2, lev)
        for k in range(3):
            o.pchevi(k % 2, (k + 1) % 2, k)
        runs.append(o.get_state(1))
        o.close()
    ring = np.zeros(runs[0]["rhotheta_v"].shape[:2], bool)
    ring[0, :] = ring[-1, :] = ring[:, 0] = ring[:, -1] = True
    for f in ("rho", "rhotheta_v", "wind_w"):
        a, b = runs[0][f][ring], hm.state[f][ring]
        np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-14 * np.abs(b).max(), err_msg=f)
    assert all(np.isfinite(v).all() for v in runs[0].values())
    assert not np.array_equal(runs[0]["rhotheta_v"][ring], runs[1]["rhotheta_v"][ring])


def test_golden_boundaries_and_output():
    """The oracle reproduces the committed vectors of tests/golden/hills_nonperiodic_bc.npz
    (five relaxed steps and the output fields, from tests/golden/make_golden.py)."""
    import importlib.util
    from pathlib import Path
    here = Path(__file__).resolve().parent / "golden"
    spec = importlib.util.spec_from_file_location("make_golden", here / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g = np.load(here / "hills_nonperiodic_bc.npz")
    st, out, bc = mg.boundary_output_case()
    np.testing.assert_array_equal(bc, g["bc_state"])
    for f in L.ATMOS_FIELDS:
        assert cases.rel_err(st[f], g[f]) <= 1e-12, f
    for f, v in out.items():
        np.testing.assert_allclose(v, g["out_" + f], rtol=1e-6, atol=0, err_msg=f)


# ---- GPU ------------------------------------------------------------------------------
def _gpu_pair(key, precision=L.PRECISION_FP64, with_oracle=True):
    n = _namelist(key)
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    cfg.precision = precision
    g = L.GpuModel(cfg, hm.grid)
    models = [g]
    if with_oracle:
        models.append(O.Oracle(L.config_from_namelist(n), hm.grid))
    for m in models:
        m.set_state(0, hm.state)
        m.set_state(1, hm.state)
        m.set_diag(hm.diag)
        m.bc_setup(3, 15, 0.0, lambda t, idx: _level(hm, t))
        m.set_bc(1, _level(hm, 0.0))
        m.set_bc(2, _level(hm, 15.0))
    return hm, models


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["hills_nonperiodic", "jet_nonperiodic"])
def test_bc_step_parity_fp64(key):
    hm, (g, o) = _gpu_pair(key)
    for step in range(5):  # dtime ~ 8-10 s: level swaps inside the run
        so, sn = step % 2, (step + 1) % 2
        g.pchevi(so, sn, step)
        o.pchevi(so, sn, step)
        sg, sr = g.get_state(sn), o.get_state(sn)
        bad = [(f, cases.rel_err(sg[f], sr[f])) for f in L.STATE_FIELDS
               if not np.isfinite(sg[f]).all() or cases.rel_err(sg[f], sr[f]) > 1e-12]
        assert not bad, f"{key} step {step}: {bad}"
        assert g.bc_state() == o.bc_state(), step
    assert g.bc_state()[2] > 0.0  # at least one swap happened
    g.close()
    o.close()


@pytest.mark.gpu
def test_bc_split_close_to_fp64():
    from test_split import field_errors
    hm, (g64,) = _gpu_pair("jet_nonperiodic", L.PRECISION_FP64, with_oracle=False)
    _, (gsp,) = _gpu_pair("jet_nonperiodic", L.PRECISION_SPLIT, with_oracle=False)
    for step in range(6):
        for g in (g64, gsp):
            g.pchevi(step % 2, (step + 1) % 2, step)
    a, b = gsp.get_state(0), g64.get_state(0)
    for f in L.STATE_FIELDS:
        assert np.isfinite(a[f]).all(), f
    errs = field_errors(a, b)
    assert max(errs.values()) <= 3e-5, errs
    assert gsp.bc_state() == g64.bc_state()
    g64.close()
    gsp.close()


@pytest.mark.gpu
def test_bc_setup_rejected_when_periodic_gpu():
    n = cases.small_case("hills")
    hm = L.HostModel(n)
    g = L.GpuModel(L.config_from_namelist(n), hm.grid)
    with pytest.raises(L.LgameError):
        g.bc_setup(3, 15, 0.0, None)
    g.close()
