"""Output fields of the time loop (control.F90:535-537): linear_combine_two_states
(mo_linear_combination.F90:15-37) and the variables write_output stores
(mo_write_out.F90:167-217) as floats, with the crash check (:60-67).

CPU: the oracle against a numpy restatement of the Fortran; density, temperature and the
centred winds bit for bit (same operations, same order, then rounded to float), relative
humidity within two float ulps (exp, log and pow of two libraries), over every branch of
its saturation pressures.  GPU: lgame_gpu_output
against the oracle on the same two states, with the same bars, in both precision modes (the
output reads the FP64 state either way).
"""
import numpy as np
import pytest

import cases
import lgame_gpu as L
import oracle as O

T_0, R_V = 273.15, 461.524879
ULP = 2.4e-7  # two float32 ulps, relative


def _sat_ice_huang(t):
    tc = t - T_0
    d = tc + 868.0
    return np.exp(43.494 - 6545.8 / (tc + 278.0)) / (d * d)


def _sat_ice_murphy(t):
    return np.exp(9.550426 - 5723.265 / t + 3.53068 * np.log(t) - 0.00728332 * t)


def _rel_humidity(rho_v, t):
    vp = rho_v * R_V * t
    tcw = np.minimum(t - T_0, 100.0)
    with np.errstate(invalid="ignore"):  # the warm formula at cold points, discarded below
        warm = np.exp(34.494 - 4924.99 / (tcw + 237.1)) / np.power(tcw + 105.0, 1.57)
    tc = t - T_0
    ice = np.where(tc >= -80.0, _sat_ice_huang(np.minimum(t, T_0)),
                   np.where(tc >= -100.0,
                            (tc + 100.0) / 20.0 * _sat_ice_huang(t) + (1.0 - (tc + 100.0) / 20.0) + _sat_ice_murphy(t),
                            _sat_ice_murphy(np.maximum(t, 110.0))))
    return vp / np.where(t > T_0, warm, ice)


def _expected(a, b, grid, c1, c2, ncons):
    comb = {f: c1 * a[f] + c2 * b[f] for f in ("rho", "rhotheta_v", "exner_pert", "wind_u", "wind_v", "wind_w")}
    g = ncons - 2 if ncons > 1 else 0
    tp = comb["rhotheta_v"] / comb["rho"][..., g] - grid["theta_v_bg"]
    t = (grid["theta_v_bg"] + tp) * (grid["exner_bg"] + comb["exner_pert"])
    u, v, w = comb["wind_u"], comb["wind_v"], comb["wind_w"]
    zs, zw = grid["z_scalar"], grid["z_w"]
    uw = (zs - zw[..., 1:]) / (zw[..., :-1] - zw[..., 1:])
    out = {"rho": comb["rho"].astype(np.float32), "temperature": t.astype(np.float32),
           "wind_u": (0.5 * (u[:, :-1] + u[:, 1:])).astype(np.float32),
           "wind_v": (0.5 * (v[:-1] + v[1:])).astype(np.float32),
           "wind_w": (uw * w[..., :-1] + (1.0 - uw) * w[..., 1:]).astype(np.float32)}
    if ncons > 1:
        out["rel_humidity"] = _rel_humidity(comb["rho"][..., g + 1], t).astype(np.float32)
    return out, bool(np.isnan(comb["exner_pert"]).any())


def _compare(got, exp):
    assert set(got) == set(exp)
    for f in exp:
        if f == "rel_humidity":
            rel = np.abs(got[f].astype(np.float64) - exp[f]) / np.maximum(np.abs(exp[f]), 1e-30)
            assert rel.max() <= ULP, (f, rel.max())
        else:
            np.testing.assert_array_equal(got[f], exp[f], err_msg=f)


def _two_states(key, nsteps=2):
    n = cases.small_case(key)
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    o = O.Oracle(cfg, hm.grid)
    o.set_state(0, hm.state)
    o.set_state(1, hm.state)
    o.set_diag(hm.diag)
    for k in range(nsteps):
        o.pchevi(k % 2, (k + 1) % 2, k)
    return hm, cfg, o


@pytest.mark.parametrize("key", ["hills", "jet"])
def test_output_oracle_against_numpy(key):
    hm, cfg, o = _two_states(key)
    a, b = o.get_state(0), o.get_state(1)
    got, crashed = o.output(0, 1, 0.3, 0.7)
    exp, nan = _expected(a, b, hm.grid, 0.3, 0.7, hm.ncons)
    _compare(got, exp)
    assert crashed is False and nan is False
    o.close()


def test_output_crash_flag_oracle():
    hm, cfg, o = _two_states("hills", 1)
    st = o.get_state(0)
    st["exner_pert"][3, 4, 5] = np.nan
    o.set_state(0, st)
    _, crashed = o.output(0, 1, 0.0, 1.0)  # 0*NaN is NaN: flagged, as in the reference
    assert crashed is True
    _, crashed = o.output(1, 1, 0.5, 0.5)
    assert crashed is False
    o.close()


def _all_branch_states():
    """The small jet's state with rhotheta_v rewritten so that the output temperature spans
    100-400 K: every branch of rel_humidity (Huang over water with the 100 C clip, Huang over
    ice, the blend between -100 C and -80 C, Murphy with the 110 K clip)."""
    hm, cfg, o = _two_states("jet", 1)
    g = hm.ncons - 2
    out = []
    for slot in (0, 1):
        st = o.get_state(slot)
        exner = hm.grid["exner_bg"] + st["exner_pert"]
        t_target = np.linspace(100.0, 400.0, exner.size).reshape(exner.shape, order="F")
        st["rhotheta_v"] = st["rho"][..., g] * t_target / exner
        o.set_state(slot, st)
        out.append(st)
    return hm, cfg, o, out


def test_output_humidity_all_branches_oracle():
    hm, cfg, o, (a, b) = _all_branch_states()
    got, _ = o.output(0, 1, 0.5, 0.5)
    exp, _ = _expected(a, b, hm.grid, 0.5, 0.5, hm.ncons)
    t = exp["temperature"]
    assert t.min() < 150.0 and t.max() > 380.0
    _compare(got, exp)
    o.close()


@pytest.mark.gpu
def test_output_humidity_all_branches_gpu():
    hm, cfg, o, _ = _all_branch_states()
    g = L.GpuModel(cfg, hm.grid)
    for s in (0, 1):
        g.set_state(s, o.get_state(s))
    got, _ = g.output(0, 1, 0.5, 0.5)
    ref, _ = o.output(0, 1, 0.5, 0.5)
    _compare(got, {f: v.astype(np.float64) if f == "rel_humidity" else v for f, v in ref.items()})
    g.close()
    o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["hills", "jet"])
@pytest.mark.parametrize("precision", [L.PRECISION_FP64, L.PRECISION_SPLIT])
def test_output_parity(key, precision):
    hm, cfg, o = _two_states(key)
    cfg.precision = precision
    g = L.GpuModel(cfg, hm.grid)
    for s in (0, 1):
        g.set_state(s, o.get_state(s))
    for c1, c2 in ((0.3, 0.7), (1.0, 0.0), (-0.25, 1.25)):
        got, crashed = g.output(0, 1, c1, c2)
        ref, rcrash = o.output(0, 1, c1, c2)
        _compare(got, {f: v.astype(np.float64) if f == "rel_humidity" else v for f, v in ref.items()})
        assert crashed == rcrash is False
    g.close()
    o.close()


@pytest.mark.gpu
def test_output_crash_flag_gpu():
    hm, cfg, o = _two_states("hills", 1)
    g = L.GpuModel(cfg, hm.grid)
    st = o.get_state(0)
    st["exner_pert"][3, 4, 5] = np.nan
    g.set_state(0, st)
    g.set_state(1, o.get_state(1))
    assert g.output(0, 1, 0.0, 1.0)[1] is True
    assert g.output(1, 1, 0.5, 0.5)[1] is False
    g.close()
    o.close()
