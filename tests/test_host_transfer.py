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
