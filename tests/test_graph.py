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


# physics switches whose kernels run on the split step's side streams: the closure, the PBL, the
# soil and the phase transitions
BRANCH_PHYSICS = dict(lmom_diff_h=True, lmom_diff_v=True, ltemp_diff_h=True, ltemp_diff_v=True, lmass_diff_h=True,
                      lmass_diff_v=True, lprog_soil_temp=True, lsfc_sensible_heat_flux=True, lsfc_phase_trans=True,
                      lpbl=True, lphase_trans=True)


@pytest.mark.gpu
@pytest.mark.parametrize("physics", [False, True])
def test_split_branches_equal_serial_order(physics):
    """The split step's concurrent branches (side streams joined by events, as the step runs when
    launched kernel by kernel) against the same kernels one after another on one stream (as
    per-kernel tracing and the captured graph run them): the same bits after five steps, with the
    plain step and with every physics switch on (the branches that run the closure, the PBL and
    the phase transitions)."""
    key, ov = cases.SMALL["jet"]
    n = cases.namelist(key, **{**ov, **(BRANCH_PHYSICS if physics else {})})
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    cfg.precision = L.PRECISION_SPLIT
    models = []
    for serial in (False, True):
        g = L.GpuModel(cfg, hm.grid)
        g.set_graphs(False)
        g.set_profiling(serial)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(hm.diag)
        models.append(g)
    for step in range(5):
        for g in models:
            g.pchevi(step % 2, (step + 1) % 2, step)
    a, b = models[0].get_state(1), models[1].get_state(1)
    da, db = models[0].get_diag(), models[1].get_diag()
    for f in L.STATE_FIELDS:
        assert np.isfinite(a[f]).all(), f
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    for f in L.DIAG_FIELDS:
        np.testing.assert_array_equal(da[f], db[f], err_msg=f)
    for g in models:
        g.close()
