"""lgame_gpu_budgets_static (budget sums with a fixed scratch array, no allocation)
against lgame_gpu_budgets, both called through the C ABI with ctypes.

The two entry points run the same reduction kernels in the same order, so the sums must
agree to the last bit; the tolerance below (rtol 1e-15) only allows for that.  Two calls in
a row on each state slot check that nothing left in the static scratch by one call changes
the next.  This file is collected last, so that it also runs after every other test in
the same process.
"""
import ctypes as C

import numpy as np
import pytest

import cases
import lgame_gpu as L


def _budgets_static(lib, g, slot, nout=11):
    out = np.full(nout, np.nan)
    rc = lib.lgame_gpu_budgets_static(g.h, slot, out.ctypes.data_as(C.POINTER(C.c_double)), nout)
    return rc, out


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [L.PRECISION_FP64, L.PRECISION_SPLIT])
def test_budgets_static_equals_budgets(precision):
    lib = L.load_library()
    lib.lgame_gpu_budgets_static.restype = C.c_int
    lib.lgame_gpu_budgets_static.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_int]
    n = cases.small_case("jet")
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    cfg.precision = precision
    g = L.GpuModel(cfg, hm.grid)
    g.set_state(0, hm.state)
    g.set_state(1, hm.state)
    g.set_diag(hm.diag)
    for step in range(3):
        g.pchevi(step % 2, (step + 1) % 2, step)
    nq = n.n_constituents + 4
    for slot in (0, 1):
        for _ in range(2):
            ref = g.budgets(slot)
            rc, out = _budgets_static(lib, g, slot)
            assert rc == L.OK, L.last_error()
            assert np.isfinite(out[:nq]).all()
            np.testing.assert_allclose(out[:nq], ref, rtol=1e-15, atol=0.0)
    # an output array shorter than n_constituents + 4 is rejected before any GPU work
    rc, _ = _budgets_static(lib, g, 0, nout=nq - 1)
    assert rc == L.ERR_INVALID_ARG
    assert "output" in L.last_error()
    g.close()
