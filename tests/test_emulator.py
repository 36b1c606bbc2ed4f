"""Radiation emulator: the stand-in teacher and the MLP oracle on the CPU; the tensor-core
GEMM, the gradients (against the oracle), training and the coupling on the GPU."""
import sys
from pathlib import Path

import numpy as np
import pytest

import cases
import lgame_gpu as L
from lgame_gpu import emulator as E

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
import emulator_ref as R  # noqa: E402


def synthetic_columns(n: int, nlev: int, seed: int) -> np.ndarray:
    """Feature rows of plausible columns: a standard-atmosphere-like profile with random
    surface temperature, lapse rate, humidity, albedo and zenith angle (CPU tests)."""
    rng = np.random.default_rng(seed)
    z = np.linspace(20000.0, 50.0, nlev)  # layer 1 = top
    t_sfc = rng.uniform(270.0, 305.0, (n, 1))
    lapse = rng.uniform(0.005, 0.0075, (n, 1))
    T = np.maximum(t_sfc - lapse * z, 210.0)
    p = 101325.0 * np.exp(-z / 8000.0) * np.ones((n, 1))
    rho_d = p / (287.057811 * T)
    rh = rng.uniform(0.2, 0.95, (n, 1))
    es = 611.2 * np.exp(17.67 * (T - 273.15) / (T - 29.65))
    rv = rh * es / (461.5 * T) * np.exp(-z / 12000.0)
    o3 = 8.5e-6 * np.exp(-(z - 34e3) ** 2 / (2 * (20e3 / np.sqrt(8 * np.log(2))) ** 2)) * rho_d * 1.657
    alb = rng.uniform(0.05, 0.8, (n, 1))
    mu = rng.uniform(0.0, 1.0, (n, 1))
    mu[rng.uniform(size=(n, 1)) < 0.2] = 0.0
    return np.hstack([T, p, rv, o3, alb, mu]).astype(np.float32)


# ---- CPU ---------------------------------------------------------------------------------
def test_teacher_physics():
    nlev = 40
    x = synthetic_columns(64, nlev, 1)
    h = E.teacher(x, nlev)
    assert h.shape == (64, 2 * nlev) and np.isfinite(h).all()
    sw, lw = h[:, :nlev], h[:, nlev:]
    night = x[:, -1] == 0.0
    assert np.all(sw[night] == 0.0)
    assert np.all(sw[~night] >= -1e-6) and sw[~night].max() > 0.1
    # longwave: net cooling of the column as a whole
    assert np.all(lw.mean(1) < 0.0)
    assert np.abs(h).max() < 200.0
    np.testing.assert_array_equal(h, E.teacher(x, nlev))  # deterministic


def test_teacher_rejects_bad_column():
    x = synthetic_columns(2, 10, 2)
    x[1, 0] = -1.0
    with pytest.raises(L.LgameError):
        E.teacher(x, 10)


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(3)
    nin, hidden, nout, B = 6, 5, 4, 7
    n = hidden * nin + hidden + 2 * (hidden * hidden + hidden) + nout * hidden + nout
    p = rng.normal(0, 0.4, n)
    x = rng.normal(size=(B, nin))
    y = rng.normal(size=(B, nout))
    _, g = R.loss_grad(p, x, y, nin, hidden, nout, bf16=False)
    eps = 1e-6
    for k in rng.choice(n, 25, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (R.loss_grad(pp, x, y, nin, hidden, nout, bf16=False)[0] -
              R.loss_grad(pm, x, y, nin, hidden, nout, bf16=False)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


# ---- GPU ---------------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("m,n,k", [(128, 64, 64), (128, 128, 128), (256, 192, 192), (128, 256, 512), (384, 512, 256)])
def test_tensor_core_gemm(m, n, k):
    rng = np.random.default_rng(m + n + k)
    a = E.bf16_bits(rng.normal(size=(m, k)))
    b = E.bf16_bits(rng.normal(size=(n, k)))
    emu = E.Emulator(nlev=8, hidden=256, batch_max=128)
    c = emu.gemm_bf16(a, b)
    af = (a.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    bf = (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    ref = af @ bf.T
    scale = np.abs(af) @ np.abs(bf).T
    assert np.all(np.abs(c - ref) <= 1e-5 * scale + 1e-6), np.max(np.abs(c - ref) / (scale + 1e-30))
    emu.close()


def _emu_and_data(nlev=20, hidden=256, batch=256, seed=5):
    x = synthetic_columns(batch, nlev, seed)
    y = E.teacher(x, nlev)
    emu = E.Emulator(nlev=nlev, hidden=hidden, batch_max=batch, seed=seed)
    norm = E.normalization_from(x, y)
    emu.set_normalization(*norm)
    return emu, x, y, norm


@pytest.mark.gpu
def test_gradients_match_oracle():
    emu, x, y, norm = _emu_and_data()
    p = emu.get_params()
    loss, g = emu.loss_grad(x, y)
    lo, go = R.loss_grad(p, x, y, emu.nin, emu.hidden, emu.nout, norm=norm, bf16=True)
    assert abs(loss - lo) <= 1e-4 * lo
    for name, a, b in zip(["W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"], emu.split_params(g), emu.split_params(go)):
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert rel < 1e-2, (name, rel)
    emu.close()


@pytest.mark.gpu
def test_inference_matches_oracle_and_pinned_equals_pageable():
    """Inference over a ragged number of columns (several batches, the last one padded)
    against the oracle's forward pass, and the direct path for page-locked host arrays
    against the copy path for ordinary ones, bit for bit."""
    torch = pytest.importorskip("torch")
    emu, _, _, norm = _emu_and_data()
    n = 700
    x = synthetic_columns(n, 20, 11)
    y = emu.infer(x)
    yo = R.predict(emu.get_params(), x, emu.nin, emu.hidden, emu.nout, norm)
    ys = norm[3].astype(np.float64)
    assert np.linalg.norm((y - yo) / ys) / np.linalg.norm((yo - norm[2]) / ys) < 1e-3
    assert np.max(np.abs(y - yo) / ys) < 2e-2
    xp = torch.empty((n, emu.nin), dtype=torch.float32, pin_memory=True).numpy()
    yp = torch.zeros((n, emu.nout), dtype=torch.float32, pin_memory=True).numpy()
    xp[...] = x
    emu.infer(xp, out=yp)
    np.testing.assert_array_equal(yp, y)
    emu.close()


@pytest.mark.gpu
def test_params_roundtrip_and_determinism():
    emu, x, y, _ = _emu_and_data()
    p = emu.get_params()
    emu.set_params(p)
    np.testing.assert_array_equal(emu.get_params(), p)
    l1, g1 = emu.loss_grad(x, y)
    l2, g2 = emu.loss_grad(x, y)
    assert l1 == l2
    np.testing.assert_array_equal(g1, g2)
    emu.close()


@pytest.mark.gpu
def test_training_beats_the_method_without_network():
    """Trained on teacher targets, the network's error on held-out columns is far below the
    error of the best profile that ignores the state (the training-set mean heating)."""
    nlev, hidden = 20, 256
    xtr = synthetic_columns(4096, nlev, 11)
    ytr = E.teacher(xtr, nlev)
    xva = synthetic_columns(1024, nlev, 12)
    yva = E.teacher(xva, nlev)
    emu = E.Emulator(nlev=nlev, hidden=hidden, batch_max=512, seed=7)
    emu.set_normalization(*E.normalization_from(xtr, ytr))
    emu.set_dataset(xtr, ytr)
    first = emu.train_epoch(512, 2e-3, 1)
    for ep in range(40):
        last = emu.train_epoch(512, 2e-3 if ep < 30 else 5e-4, ep + 2)
    assert last < 0.2 * first
    rmse_net = float(np.sqrt(np.mean((emu.infer(xva) - yva) ** 2)))
    rmse_mean = float(np.sqrt(np.mean((ytr.mean(0) - yva) ** 2)))
    assert rmse_net < 0.3 * rmse_mean, (rmse_net, rmse_mean)
    emu.close()


@pytest.mark.gpu
def test_coupling_features_and_update():
    n = cases.small_case("jet")
    hm = L.HostModel(n)
    g = L.GpuModel(L.config_from_namelist(n), hm.grid)
    g.set_state(0, hm.state)
    g.set_state(1, hm.state)
    g.set_diag(hm.diag)
    ny, nx, nl = n.ny, n.nx, n.n_layers
    E.rad_set_surface(g, hm.surface["sfc_albedo"], hm.surface["lat_geo_scalar"], hm.surface["lon_geo_scalar"])
    t = 1576843200.0 + 6 * 3600.0
    x = E.rad_features(g, 0, t)
    assert x.shape == (ny * nx, 4 * nl + 2) and np.isfinite(x).all()
    T = x[:, :nl]
    assert 150.0 < T.min() and T.max() < 340.0
    assert np.all(x[:, nl:2 * nl] > 0.0) and np.all(x[:, 2 * nl:3 * nl] >= 0.0)
    assert np.all((x[:, -1] >= 0.0) & (x[:, -1] <= 1.0))
    # teacher heating -> radiation tendency (W m^-3) = rate/86400 * rho_gas * c_p
    h = E.teacher(x, nl)
    E.rad_apply_heating(g, 0, h)
    rad = g.get_diag()["radiation_tendency"]
    rho = hm.state["rho"][..., -2] + hm.state["rho"][..., -1]
    def col(a):  # (ny, nx, nl) Fortran array -> (column ji + ny*(jk-1), layer)
        return np.asarray(a).reshape(ny * nx, nl, order="F")

    expect = (h[:, :nl] + h[:, nl:]) / 86400.0 * col(rho) * 1005.0
    np.testing.assert_allclose(col(rad), expect, rtol=1e-5, atol=1e-12)
    # emulator update with every column sampled and a bound it cannot meet untrained: fallback
    emu = E.Emulator(nlev=nl, hidden=256, batch_max=256, seed=3)
    rep = E.rad_update(g, emu, 0, t, 1, 1e-6)
    assert rep["fallback"] and rep["sampled"] == ny * nx
    np.testing.assert_allclose(col(g.get_diag()["radiation_tendency"]), expect, rtol=1e-5, atol=1e-12)
    # and the step runs with the radiation tendency
    g.pchevi(0, 1, 0)
    assert all(np.isfinite(v).all() for v in g.get_state(1).values())
    emu.close()


@pytest.mark.gpu
def test_lrad_update_drives_attached_emulator():
    """pchevi(..., lrad_update=1, t_0) with an attached emulator equals the host calling
    lgame_gpu_rad_update(old slot, t_0 + dtime_rad/2) itself before the step
    (mo_manage_pchevi.F90:56-58, mo_manage_radiation_calls.F90:46-51), bit for bit; with
    lrad_update=0, or with no emulator attached, the radiation tendency is left alone."""
    n = cases.small_case("jet")
    hm = L.HostModel(n)
    nl = n.n_layers
    emu = E.Emulator(nlev=nl, hidden=256, batch_max=256, seed=3)
    t0, dtime_rad = 1576843200.0 + 5 * 3600.0, 900.0
    models = []
    for _ in range(2):
        g = L.GpuModel(L.config_from_namelist(n), hm.grid)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(hm.diag)
        E.rad_set_surface(g, hm.surface["sfc_albedo"], hm.surface["lat_geo_scalar"], hm.surface["lon_geo_scalar"])
        models.append(g)
    a, b = models
    E.rad_attach(a, emu, dtime_rad, 4, 1e9)
    a.pchevi(0, 1, 0, 1, t0)
    rep = E.rad_last_report(a)
    assert rep["updates"] == 1 and rep["sampled"] > 0 and not rep["fallback"]
    E.rad_update(b, emu, 0, t0 + 0.5 * dtime_rad, 4, 1e9)
    b.pchevi(0, 1, 0, 0, t0)
    for f, v in a.get_state(1).items():
        np.testing.assert_array_equal(v, b.get_state(1)[f], err_msg=f)
    rad = a.get_diag()["radiation_tendency"]
    assert np.abs(rad).max() > 0.0
    np.testing.assert_array_equal(rad, b.get_diag()["radiation_tendency"])
    # lrad_update = 0 runs no update; detached, lrad_update = 1 is ignored
    a.pchevi(1, 0, 1, 0, t0 + 4.0)
    assert E.rad_last_report(a)["updates"] == 1
    E.rad_attach(a, None, 0.0, 0, 0.0)
    a.pchevi(0, 1, 2, 1, t0 + 8.0)
    np.testing.assert_array_equal(a.get_diag()["radiation_tendency"], rad)
    a.close()
    b.close()
    emu.close()
