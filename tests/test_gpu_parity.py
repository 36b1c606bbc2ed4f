"""FP64 GPU step vs the CPU oracle on identical inputs, through the C ABI.

Bar: for every prognostic field and every carried diagnostic,
max|gpu - oracle| / max|oracle| <= 1e-12 after each of the first steps (the FP64 path
keeps the reference's operation order, so most fields agree bit for bit; the only
non-correctly-rounded function in the step is exp() in c_p_ice, moist runs only).
"""
import numpy as np
import pytest

import cases
import lgame_gpu as L
import oracle as O

TOL = 1e-12
NSTEPS = 3


def _pair(key):
    n = cases.small_case(key)
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    g = L.GpuModel(cfg, hm.grid)
    o = O.Oracle(cfg, hm.grid)
    st, dg = hm.copy_state(), hm.copy_diag()
    for m in (g, o):
        m.set_state(0, st)
        m.set_state(1, st)
        m.set_diag(dg)
    return hm, g, o


@pytest.mark.gpu
@pytest.mark.parametrize("key", list(cases.SMALL))
def test_step_parity_fp64(key):
    hm, g, o = _pair(key)
    for step in range(NSTEPS):
        so, sn = step % 2, (step + 1) % 2
        g.pchevi(so, sn, step)
        o.pchevi(so, sn, step)
        sg, sr = g.get_state(sn), o.get_state(sn)
        bad = []
        for f in L.STATE_FIELDS:
            e = cases.rel_err(sg[f], sr[f])
            if not np.isfinite(sg[f]).all() or e > TOL:
                bad.append((f, e))
        dgd, drd = g.get_diag(), o.get_diag()
        for f in L.DIAG_FIELDS:
            e = cases.rel_err(dgd[f], drd[f])
            if e > TOL:
                bad.append((f, e))
        assert not bad, f"{key} step {step}: {bad}"


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["schaer", "jet"])
def test_budgets_fp64(key):
    hm, g, o = _pair(key)
    for step in range(2):
        g.pchevi(step % 2, (step + 1) % 2, step)
        o.pchevi(step % 2, (step + 1) % 2, step)
    bg, br = g.budgets(0), o.budgets(0)
    np.testing.assert_allclose(bg, br, rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_host_buffer_step_matches_device_step():
    """lgame_gpu_pchevi_host (host buffers in and out) gives the device-resident result."""
    hm, g, o = _pair("jet")
    st = hm.copy_state()
    out = {f: np.zeros_like(v, order="F") for f, v in st.items()}
    g.pchevi_host(st, out, 0)
    o.pchevi(0, 1, 0)
    ref = o.get_state(1)
    for f in L.STATE_FIELDS:
        assert cases.rel_err(out[f], ref[f]) <= TOL, f
