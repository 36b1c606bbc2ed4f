"""The step launched as a captured CUDA graph (lgame_gpu_set_graphs, the default after step 0)
against the same steps launched kernel by kernel: identical states after five steps, which
cover both slot pairs (0 -> 1, 1 -> 0) and the graphs' replay, in both precisions."""
import numpy as np
import pytest

import cases
import lgame_gpu as L


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [L.PRECISION_FP64, L.PRECISION_SPLIT])
def test_graph_steps_equal_direct_steps(precision):
    n = cases.small_case("jet")
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    cfg.precision = precision
    models = []
    for graphs in (True, False):
        g = L.GpuModel(cfg, hm.grid)
        g.set_graphs(graphs)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(hm.diag)
        models.append(g)
    for step in range(5):
        for g in models:
            g.pchevi(step % 2, (step + 1) % 2, step)
    a, b = models[0].get_state(1), models[1].get_state(1)
    for f in L.STATE_FIELDS:
        assert np.isfinite(a[f]).all(), f
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    assert models[0].kernels_per_step() == models[1].kernels_per_step()
    for g in models:
        g.close()
