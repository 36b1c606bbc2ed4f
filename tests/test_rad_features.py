"""The radiation emulator's column features (k_rad_features, lgame_gpu_rad_features) against
the numpy restatement in oracle/rad_features_ref.py of the reference's definitions:
temperature_diagnostics (mo_derived.F90:18-38), p = r_d*rho_dry*T
(mo_rterrtmgp_coupler.F90:161-167), calc_o3_vmr (mo_dictionary.F90:66-86) and coszenith
(mo_rterrtmgp_coupler.F90:550-629).

CPU: known answers of coszenith (the sun overhead at 23.44 S over Greenwich at the December
solstice 2019-12-20 12:00 UTC, the reference's t_0; night on the far side) and of the ozone
profile (8.5e-6 at 34 km, half of it 10 km away).
GPU: every feature of every column at two times, with latitudes and longitudes spread over
the globe so that each call has day and night columns; the features are FP64 values rounded
once to float, so the bar is two units in the last place of a float (relative 2.4e-7; one
subnormal unit, 1.4e-45, where the ozone density underflows) and 1e-7 absolute for the zenith
cosine near the terminator.
"""
import numpy as np
import pytest

import cases
import lgame_gpu as L
import rad_features_ref as R

T_SOLSTICE = 1576843200.0
OBLIQUITY = 0.409092592843564


def test_coszenith_known_answers():
    c = R.coszenith(np.array([-OBLIQUITY, -OBLIQUITY, OBLIQUITY, 0.0]), np.array([0.0, np.pi, 0.0, 0.0]), T_SOLSTICE)
    assert abs(c[0] - 1.0) < 1e-15  # overhead
    assert c[1] == 0.0  # night
    np.testing.assert_allclose(c[2], np.cos(2 * OBLIQUITY), rtol=1e-14)
    np.testing.assert_allclose(c[3], np.cos(OBLIQUITY), rtol=1e-14)
    # six hours later the sub-solar point has moved to 90 W (the Earth turns by omega*t)
    lon = -7.292115e-5 * 6 * 3600.0
    c6 = R.coszenith(np.array([-OBLIQUITY]), np.array([lon]), T_SOLSTICE + 6 * 3600.0)
    assert c6[0] > 0.9999


def test_ozone_profile():
    v = R.calc_o3_vmr(np.array([34e3, 24e3, 44e3, 0.0]))
    np.testing.assert_allclose(v[0], 8.5e-6, rtol=1e-15)
    np.testing.assert_allclose(v[1:3], 0.5 * 8.5e-6, rtol=1e-14)
    assert 0.0 < v[3] < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["jet", "hills"])
def test_features_match_oracle(key):
    from lgame_gpu import emulator as E
    n = cases.small_case(key)
    hm = L.HostModel(n)
    g = L.GpuModel(L.config_from_namelist(n), hm.grid)
    g.set_state(0, hm.state)
    g.set_state(1, hm.state)
    g.set_diag(hm.diag)
    for step in range(2):  # a state that is not the initial one
        g.pchevi(step % 2, (step + 1) % 2, step)
    st = g.get_state(0)
    rng = np.random.default_rng(5)
    ny, nx, nl = n.ny, n.nx, n.n_layers
    lat = rng.uniform(-0.5 * np.pi, 0.5 * np.pi, (ny, nx))
    lon = rng.uniform(-np.pi, np.pi, (ny, nx))
    alb = rng.uniform(0.05, 0.9, (ny, nx))
    E.rad_set_surface(g, alb, lat, lon)
    for t in (T_SOLSTICE + 3 * 3600.0, T_SOLSTICE + 200 * 86400.0 + 17 * 3600.0):
        x = E.rad_features(g, 0, t)
        ref = R.features(st, hm.grid, alb, lat, lon, t, bool(n.lmoist))
        cz, cz_ref = x[:, -1], ref[:, -1]
        assert (cz_ref == 0.0).any() and (cz_ref > 0.2).any(), "want day and night columns"
        np.testing.assert_allclose(cz, cz_ref, rtol=0, atol=1e-7)
        np.testing.assert_array_equal(cz == 0.0, cz_ref == 0.0)
        # the oracle rounded to float as the kernel rounds its FP64 values; ozone densities
        # far from 34 km underflow into float subnormals, where one unit is 1.4e-45
        np.testing.assert_allclose(x[:, :-1], ref[:, :-1].astype(np.float32), rtol=2.4e-7, atol=1.5e-45)
    g.close()
