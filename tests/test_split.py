"""The FP32/FP64 split-precision step against the FP64 step on identical inputs.

The FP64 GPU step equals the oracle to <= 1e-12 per field and step (test_gpu_parity.py),
so it is the reference here.  Error of a field f:

    max|f_split - f_fp64| / max(max|f_fp64|, floor_f)

with a floor at the field's physical scale (1 m/s for the winds, 1 K for theta_v',
1e-3 for exner'), so that fields which stay at round-off level (a fluid at rest over
hills, where the FP64 winds are ~1e-14 m/s) are measured on an absolute scale rather
than relative to their own noise.  Bar: every field finite, error <= 1e-5 after one
step and <= 3e-5 after ten.  The hour-scale error study is l-game_gb300/error_study.py.
"""
import numpy as np
import pytest

import cases
import lgame_gpu as L

KEYS = ["schaer_odd", "mountain_rest", "hills", "jet", "jet_plane", "jet_order2_nobg", "hills_nonperiodic"]


def _models(key):
    n = cases.small_case(key)
    hm = L.HostModel(n)
    out = []
    for prec in (L.PRECISION_FP64, L.PRECISION_SPLIT):
        cfg = L.config_from_namelist(n)
        cfg.precision = prec
        g = L.GpuModel(cfg, hm.grid)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(hm.diag)
        out.append(g)
    return hm, out


FLOOR = {"wind_u": 1.0, "wind_v": 1.0, "wind_w": 1.0, "theta_v_pert": 1.0, "exner_pert": 1e-3}


def field_errors(a, b):
    """max|a-b| over max|b| (or the field's floor) of each atmospheric state field."""
    out = {}
    for f in L.ATMOS_FIELDS:
        d = float(np.abs(a[f] - b[f]).max())
        out[f] = d / max(float(np.abs(b[f]).max()), FLOOR.get(f, 0.0))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("key", KEYS)
def test_split_close_to_fp64(key):
    hm, (g64, gsp) = _models(key)
    for step in range(10):
        for g in (g64, gsp):
            g.pchevi(step % 2, (step + 1) % 2, step)
        if step not in (0, 9):
            continue
        a, b = gsp.get_state((step + 1) % 2), g64.get_state((step + 1) % 2)
        for f in L.STATE_FIELDS:
            assert np.isfinite(a[f]).all(), (key, step, f)
        errs = field_errors(a, b)
        bar = 1e-5 if step == 0 else 3e-5
        assert max(errs.values()) <= bar, (key, step + 1, errs)


@pytest.mark.gpu
def test_split_diag_roundtrip_and_budgets():
    hm, (g64, gsp) = _models("jet")
    for step in range(2):
        gsp.pchevi(step % 2, (step + 1) % 2, step)
        g64.pchevi(step % 2, (step + 1) % 2, step)
    d = gsp.get_diag()
    assert np.isfinite(d["pot_vort_tend_x"]).all() and np.abs(d["pot_vort_tend_x"]).max() > 0
    gsp.set_diag(d)
    d2 = gsp.get_diag()
    for f in L.DIAG_FIELDS:
        np.testing.assert_array_equal(d[f], d2[f])
    b64, bsp = g64.budgets(0), gsp.budgets(0)
    np.testing.assert_allclose(bsp[:-1], b64[:-1], rtol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["schaer_odd", "mountain_rest", "jet", "hills_nonperiodic"])
def test_split_fp64_column_close_to_fp64(key):
    """LGAME_PRECISION_SPLIT_FP64_COLUMN (the vertical acoustic solve wholly in FP64) against
    the FP64 step, with the bars of the split mode; it must not be farther from FP64 than
    the split mode with FP32 coefficients after ten steps."""
    n = cases.small_case(key)
    hm = L.HostModel(n)
    models = []
    for prec in (L.PRECISION_FP64, L.PRECISION_SPLIT, L.PRECISION_SPLIT_FP64_COLUMN):
        cfg = L.config_from_namelist(n)
        cfg.precision = prec
        g = L.GpuModel(cfg, hm.grid)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(hm.diag)
        models.append(g)
    for step in range(10):
        for g in models:
            g.pchevi(step % 2, (step + 1) % 2, step)
        if step not in (0, 9):
            continue
        b = models[0].get_state((step + 1) % 2)
        e32 = field_errors(models[1].get_state((step + 1) % 2), b)
        a = models[2].get_state((step + 1) % 2)
        for f in L.STATE_FIELDS:
            assert np.isfinite(a[f]).all(), (key, step, f)
        e64 = field_errors(a, b)
        bar = 1e-5 if step == 0 else 3e-5
        assert max(e64.values()) <= bar, (key, step + 1, e64)
        if step == 9:
            assert max(e64.values()) <= 2.0 * max(e32.values()), (key, e64, e32)
    for g in models:
        g.close()
