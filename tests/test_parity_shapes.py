"""GPU parity on the benchmark shapes themselves, not only on the toy grids of cases.SMALL.

The toy grids have ny <= 20, so the padded row pitch P = round_up(ny+1, 32) is 32 and
every launch has a single row tile.  The shapes here reach what those do not:

- schaer_256x4x60: the Schaer mountain wave exactly as its namelist states it (nl = 60);
- jet_128x128x80: the moist benchmark workload on the 128x128x80 sub-domain that the CPU
  baseline runs (P = 160, five row tiles, nl = 80 in the column solvers);
- hills_512x512x50: the rest-over-hills workload at its full size (13.1 M cells);
- jet_97x65x33 (periodic and non-periodic with the lateral relaxation): sizes that are
  multiples of neither 32 nor 8, so the periodic row ny+1 = 66 lies in the third row tile
  and the column tiles end part-way; and the same two with every physics switch on (the
  reference's default diffusion closure and surface layer, PBL and soil, and the phase
  transitions), whose two-dimensional surface kernels and periodic wrap points then also
  span several row tiles.

Each case runs the FP64 GPU step against the oracle (<= 1e-12 relative per state field and
carried diagnostic, as tests/test_gpu_parity.py) and the split step against the FP64 step
for ten steps (tests/test_split.py's bar: 1e-5 after one step, 3e-5 after ten).
Reference: pchevi, src/time_stepping/mo_manage_pchevi.F90:27-118.
"""
import numpy as np
import pytest

import cases
import lgame_gpu as L
import oracle as O
from test_boundaries import _level
from test_split import field_errors

TOL = 1e-12
# the surface layer's and the phase transitions' diagnostics come out of logarithms, powers and a
# quadratic's root (CUDA's and glibc's functions): their bar is that of tests/test_surface.py and
# tests/test_phase.py
DIAG_TOL = {f: 1e-11 for f in ("roughness_length_diag", "roughness_velocity", "monin_obukhov_length",
                              "scalar_flux_resistance", "power_flux_density_sens_soil",
                              "power_flux_density_sens_sea")}
DIAG_TOL.update({f: 1e-10 for f in ("phase_trans_rates", "phase_trans_heating_rate", "power_flux_density_lat_lake",
                                    "power_flux_density_lat_sea")})
# every physics switch: the reference's default &diff and &surface, and the phase transitions
PHYSICS = dict(lmom_diff_h=True, lmom_diff_v=True, ltemp_diff_h=True, ltemp_diff_v=True, lmass_diff_h=True,
               lmass_diff_v=True, lprog_soil_temp=True, lsfc_sensible_heat_flux=True, lsfc_phase_trans=True,
               lpbl=True, lphase_trans=True)

# key: (namelist, overrides, FP64-vs-oracle steps, lateral relaxation)
SHAPES = {
    "schaer_256x4x60": ("schaer_256x4x60", {}, 3, False),
    "jet_128x128x80": ("jet_1024x1024x80", dict(nx=128, ny=128), 3, False),
    "hills_512x512x50": ("rest_hills_512x512x50", {}, 2, False),
    "jet_97x65x33": ("jet_1024x1024x80", dict(nx=97, ny=65, n_layers=33, n_oro_layers=25), 3, False),
    "jet_97x65x33_nonperiodic": ("jet_1024x1024x80", dict(nx=97, ny=65, n_layers=33, n_oro_layers=25,
                                                          lperiodic=False, lfreeslip=False), 3, True),
    "jet_97x65x33_physics": ("jet_1024x1024x80", dict(nx=97, ny=65, n_layers=33, n_oro_layers=25, **PHYSICS), 3,
                             False),
    "jet_97x65x33_nonperiodic_physics": ("jet_1024x1024x80", dict(nx=97, ny=65, n_layers=33, n_oro_layers=25,
                                                                  lperiodic=False, lfreeslip=False, **PHYSICS), 3,
                                         True),
}


def _start(m, hm, relax):
    m.set_state(0, hm.state)
    m.set_state(1, hm.state)
    m.set_diag(hm.diag)
    if relax:
        m.bc_setup(5, 15, 0.0, lambda t, idx: _level(hm, t))
        m.set_bc(1, _level(hm, 0.0))
        m.set_bc(2, _level(hm, 15.0))


def _setup(key):
    name, ov, nsteps, relax = SHAPES[key]
    n = cases.namelist(name, **ov)
    return n, L.HostModel(n), nsteps, relax


def test_shapes_cover_several_row_tiles():
    """Host-side check of what the shapes exercise: P > 32 and an odd, unaligned grid."""
    pitch = {k: ((SHAPES[k][1].get("ny", 0) + 1 + 31) // 32) * 32 for k in SHAPES if "ny" in SHAPES[k][1]}
    assert pitch["jet_128x128x80"] == 160 and pitch["jet_97x65x33"] == 96
    assert 65 % 32 and 97 % 8 and 33 % 8


@pytest.mark.gpu
@pytest.mark.parametrize("key", list(SHAPES))
def test_fp64_parity_full_shape(key):
    n, hm, nsteps, relax = _setup(key)
    cfg = L.config_from_namelist(n)
    g = L.GpuModel(cfg, hm.grid)
    o = O.Oracle(L.config_from_namelist(n), hm.grid)
    for m in (g, o):
        _start(m, hm, relax)
    try:
        for step in range(nsteps):
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
                if e > DIAG_TOL.get(f, TOL):
                    bad.append((f, e))
            assert not bad, f"{key} step {step}: {bad}"
            if relax:
                assert g.bc_state() == o.bc_state(), step
        # The budget terms are sums of n non-negative cell values, and the GPU's reduction
        # tree adds them in another order than the oracle's threads: any two orders agree to
        # 2(n-1)u relative (u = 2^-53), which at 13 M cells is above 1e-12.  A resting
        # atmosphere's kinetic energy (round-off winds) shows it.
        ncell = n.nx * n.ny * n.n_layers
        bg, br = g.budgets(nsteps % 2), o.budgets(nsteps % 2)
        np.testing.assert_allclose(bg, br, rtol=max(TOL, 2.0 * ncell * 2.0 ** -53), atol=0)
    finally:
        g.close()
        o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("key", list(SHAPES))
def test_split_close_to_fp64_full_shape(key):
    n, hm, _, relax = _setup(key)
    models = []
    for prec in (L.PRECISION_FP64, L.PRECISION_SPLIT):
        cfg = L.config_from_namelist(n)
        cfg.precision = prec
        g = L.GpuModel(cfg, hm.grid)
        _start(g, hm, relax)
        models.append(g)
    g64, gsp = models
    try:
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
    finally:
        g64.close()
        gsp.close()
