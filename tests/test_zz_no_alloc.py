"""lgame_gpu_budgets_static (budget sums with a fixed scratch array, no allocation)
against lgame_gpu_budgets, both called through the C ABI with ctypes.

Hosts that run their time loop under an allocation guard, or whose GPU memory is fully
committed to model state, call lgame_gpu_budgets_static instead of lgame_gpu_budgets.
The two entry points run the same reduction kernels in the same order, so the sums must
agree to the last bit: the comparison is of the bit patterns.  Two calls in a row on each
state slot check that nothing left in the shared static scratch by one call changes the
next; two contexts on one device, used one after the other, check that each still gets its
own sums from the one scratch array.  Around a warm call, neither the context's device
bytes nor the device's free memory (cudaMemGetInfo) may change.  This file is collected
last, so that it also runs after every other test in the same process.
"""
import ctypes as C

import numpy as np
import pytest

import cases
import lgame_gpu as L


def _lib():
    lib = L.load_library()
    lib.lgame_gpu_budgets_static.restype = C.c_int
    lib.lgame_gpu_budgets_static.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_int]
    return lib


def _budgets_static(lib, g, slot, nout=11):
    out = np.full(nout, np.nan)
    rc = lib.lgame_gpu_budgets_static(g.h, slot, out.ctypes.data_as(C.POINTER(C.c_double)), nout)
    return rc, out


def _model(key, precision, nsteps=3):
    n = cases.small_case(key)
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    cfg.precision = precision
    g = L.GpuModel(cfg, hm.grid)
    g.set_state(0, hm.state)
    g.set_state(1, hm.state)
    g.set_diag(hm.diag)
    for step in range(nsteps):
        g.pchevi(step % 2, (step + 1) % 2, step)
    return n, g


def _same_bits(out, ref):
    np.testing.assert_array_equal(np.ascontiguousarray(out).view(np.uint64), np.ascontiguousarray(ref).view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [L.PRECISION_FP64, L.PRECISION_SPLIT])
def test_budgets_static_equals_budgets(precision):
    lib = _lib()
    n, g = _model("jet", precision)
    nq = n.n_constituents + 4
    for slot in (0, 1):
        for _ in range(2):
            ref = g.budgets(slot)
            rc, out = _budgets_static(lib, g, slot)
            assert rc == L.OK, L.last_error()
            assert np.isfinite(out[:nq]).all()
            _same_bits(out[:nq], ref)
    # an output array shorter than n_constituents + 4 is rejected before any GPU work
    rc, _ = _budgets_static(lib, g, 0, nout=nq - 1)
    assert rc == L.ERR_INVALID_ARG
    assert "output" in L.last_error()
    g.close()


@pytest.mark.gpu
def test_budgets_static_allocates_nothing():
    torch = pytest.importorskip("torch")
    lib = _lib()
    n, g = _model("jet", L.PRECISION_SPLIT)
    nq = n.n_constituents + 4
    rc, _ = _budgets_static(lib, g, 1)  # warm: every kernel of the call has run once
    assert rc == L.OK, L.last_error()
    torch.cuda.mem_get_info(0)
    lgame_bytes = g.device_bytes()
    free_before, _ = torch.cuda.mem_get_info(0)
    rc, out = _budgets_static(lib, g, 1)
    free_after, _ = torch.cuda.mem_get_info(0)
    assert rc == L.OK, L.last_error()
    assert g.device_bytes() == lgame_bytes
    assert free_after == free_before, (free_before, free_after)
    _same_bits(out[:nq], g.budgets(1))
    g.close()


@pytest.mark.gpu
def test_budgets_static_two_contexts_one_device():
    lib = _lib()
    n1, a = _model("jet", L.PRECISION_FP64, nsteps=2)
    n2, b = _model("hills", L.PRECISION_SPLIT, nsteps=3)
    for _ in range(2):
        for n, g in ((n1, a), (n2, b)):
            nq = n.n_constituents + 4
            ref = g.budgets(0)
            rc, out = _budgets_static(lib, g, 0)
            assert rc == L.OK, L.last_error()
            _same_bits(out[:nq], ref)
    a.close()
    b.close()
