"""lgame_gpu_pchevi_host with page-locked host arrays, which the GPU reads and writes itself
over the CPU-GPU link, against the same call with ordinary (pageable) arrays, which the copy
engines move: the new states must agree bit for bit, in both precisions and over two steps
in a row (the second starting from the first's output)."""
import numpy as np
import pytest

import cases
import lgame_gpu as L


def _pinned_like(a: np.ndarray, keep: list) -> np.ndarray:
    torch = pytest.importorskip("torch")
    t = torch.empty(a.shape[::-1], dtype=torch.float64, pin_memory=True)
    keep.append(t)
    v = t.numpy().T  # Fortran-ordered view of the page-locked buffer
    v[...] = a
    return v


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [L.PRECISION_FP64, L.PRECISION_SPLIT])
def test_pinned_host_step_equals_pageable_host_step(precision):
    n = cases.small_case("jet")
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    cfg.precision = precision
    models = []
    for _ in range(2):
        g = L.GpuModel(cfg, hm.grid)
        g.set_diag(hm.diag)
        models.append(g)
    keep = []
    st = hm.copy_state()
    pin_old = {f: _pinned_like(v, keep) for f, v in st.items()}
    pin_new = {f: _pinned_like(np.zeros_like(v, order="F"), keep) for f, v in st.items()}
    pag_old = {f: np.asfortranarray(v).copy(order="F") for f, v in st.items()}
    pag_new = {f: np.zeros_like(v, order="F") for f, v in st.items()}
    for step in range(2):
        models[0].pchevi_host(pin_old, pin_new, step)
        models[1].pchevi_host(pag_old, pag_new, step)
        for f in L.STATE_FIELDS:
            assert np.isfinite(pag_new[f]).all(), (step, f)
            np.testing.assert_array_equal(pin_new[f], pag_new[f], err_msg=f"step {step} field {f}")
        for f in L.STATE_FIELDS:
            pin_old[f][...] = pin_new[f]
            pag_old[f][...] = pag_new[f]
    for g in models:
        g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [L.PRECISION_FP64, L.PRECISION_SPLIT])
def test_nonfinite_state_is_reported(precision):
    """Failure detection without a fault: a NaN planted in the host state before upload makes
    the step of a context with check_finite return LGAME_ERR_NONFINITE, and the context keeps
    answering (the NaN reaches the carried diagnostics too, so a host that goes on restores
    the state and the diagnostics, as from a restart snapshot)."""
    n = cases.small_case("hills")
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    cfg.precision = precision
    cfg.check_finite = 1
    g = L.GpuModel(cfg, hm.grid)
    g.set_diag(hm.diag)
    bad = hm.copy_state()
    bad["rhotheta_v"][2, 3, 4] = np.nan
    g.set_state(0, bad)
    g.set_state(1, bad)
    with pytest.raises(L.LgameError) as e:
        g.pchevi(0, 1, 0)
    assert e.value.code == L.ERR_NONFINITE
    assert not np.isfinite(g.get_state(1)["rhotheta_v"]).all()
    g.set_state(0, hm.state)
    back = g.get_state(0)
    for f in L.STATE_FIELDS:
        np.testing.assert_array_equal(back[f], hm.state[f], err_msg=f)
    g.close()
