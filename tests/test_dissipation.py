"""Dissipative heating of the Klemp swamp layer (simple_dissipation_rate,
src/spatial_operators/mo_momentum_diff_diss.F90:333-389), which the reference's step forms at
its first substep whenever the layer is on (mo_vector_tend_expl.F90:122-125) and adds to the
rho*theta_v tendency of both substeps (mo_scalar_tend_expl.F90:155-160).

CPU: the oracle's heating_diss after one step against a numpy restatement of the Fortran:
n_damping_levels from the highest z_w of each level (mo_grid_generator.F90:1049-1058), the
swamp layer's deceleration (w/(1 + dtime*coeff) - w)/dtime at w levels 2..n_damping_levels,
its inner product with w (the horizontal diffusion accelerations are zero) and the factor
-sum(rho(1:nc+1)).  Zero everywhere with the layer off.
GPU: the FP64 step's heating enters the rho*theta_v tendency as the oracle's does (the
state parity tests cover it); here the split step's FP32 heating against the FP64 step's
state after one step, on the damping layers.
"""
import numpy as np
import pytest

import cases
import lgame_gpu as L
import oracle as O


def _heating_ref(n, cfg, hm, st):
    g = hm.grid
    z_w, w = g["z_w"], st["wind_w"]
    start = n.klemp_begin_rel * n.toa
    ndamp = sum(1 for jl in range(n.n_layers + 1) if z_w[:, :, jl].max() > start)
    wp = np.zeros_like(w)
    for jl in range(2, ndamp + 1):
        za = z_w[:, :, jl - 1] - start
        sv = np.sin(0.5 * np.pi * np.maximum(za, 0.0) / (n.toa - start))
        coeff = np.where(za < 0.0, 0.0, n.klemp_damp_max * (sv * sv))
        pref = 1.0 + cfg.dtime * coeff
        wl = w[:, :, jl - 1]
        wp[:, :, jl - 1] = 0.0 + (wl / pref - wl) / cfg.dtime
    ipw = g["inner_product_weights"]
    ip = ipw[4] * w[:, :, :-1] * wp[:, :, :-1] + ipw[5] * w[:, :, 1:] * wp[:, :, 1:]
    rho = st["rho"]
    nc = 5 if n.lmoist else 0
    rs = np.zeros_like(ip)
    for jc in range(nc + 1):
        rs = rs + rho[..., jc]
    return -rs * ip, ndamp


@pytest.mark.parametrize("key", ["jet", "hills", "schaer", "jet_order2_nobg"])
def test_oracle_heating_diss(key):
    n = cases.small_case(key)
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    o = O.Oracle(cfg, hm.grid)
    o.set_state(0, hm.state)
    o.set_state(1, hm.state)
    o.set_diag(hm.diag)
    # the initial states are at rest vertically (w = 0): two steps first, then the heating the
    # third step forms from its old state
    for step in range(2):
        o.pchevi(step % 2, (step + 1) % 2, step)
    old = o.get_state(0)
    o.pchevi(0, 1, 2)
    hd = o.heating_diss()
    o.close()
    if not n.lklemp:
        assert not np.any(hd), "no swamp layer, no dissipative heating"
        return
    ref, ndamp = _heating_ref(n, cfg, hm, old)
    assert 2 <= ndamp <= n.n_layers
    np.testing.assert_allclose(hd, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
    assert np.abs(hd[:, :, :ndamp]).max() > 0.0
    assert not np.any(hd[:, :, ndamp:])  # below the damping levels nothing


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["jet", "hills"])
def test_split_heating_close_to_fp64(key):
    """The split path's swamp-layer heating: one step of the split and the FP64 path from the
    same state with the radiation tendency zero, so that the diabatic part of the rho*theta_v
    tendency is the dissipative heating (and the sediment heating, moist); theta_v' of the two
    paths in the damping layers then agrees to the split path's bar."""
    from test_split import field_errors
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
        g.pchevi(0, 1, 0)
        out.append(g.get_state(1))
        g.close()
    errs = field_errors(out[1], out[0])
    assert max(errs.values()) <= 1e-5, errs
