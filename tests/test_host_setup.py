"""Host set-up (grid_setup, bg_setup, ideal_init restated in the library's C++ host code):
geometric and hydrostatic invariants of the generated inputs."""
import numpy as np
import pytest

import cases
import lgame_gpu as L


@pytest.fixture(scope="module")
def schaer():
    return L.HostModel(cases.small_case("schaer"))


@pytest.fixture(scope="module")
def hills():
    return L.HostModel(cases.small_case("hills"))


def test_plane_geometry(schaer):
    g, n = schaer.grid, schaer.nml
    np.testing.assert_allclose(g["area_z"], n.dx * n.dy, rtol=1e-15)
    np.testing.assert_allclose(g["dx"], n.dx, rtol=0)
    dzl = g["z_w"][:, :, :-1] - g["z_w"][:, :, 1:]
    np.testing.assert_allclose(g["volume"], n.dx * n.dy * dzl, rtol=1e-14)


def test_levels_are_ordered_and_terrain_following(schaer, hills):
    for m in (schaer, hills):
        zw = m.grid["z_w"]
        assert np.all(zw[:, :, :-1] > zw[:, :, 1:])
        np.testing.assert_array_equal(zw[:, :, -1], m.surface["oro"])
        zs = m.grid["z_scalar"]
        # inner levels sit half-way between the layers (mo_grid_generator.F90:1039-1047)
        np.testing.assert_allclose(zw[:, :, 1:-1], 0.5 * (zs[:, :, :-1] + zs[:, :, 1:]), rtol=1e-15)
        assert np.all(zs < zw[:, :, :-1]) and np.all(zs > zw[:, :, 1:])
        assert np.all(m.grid["z_w"][:, :, 0] == m.nml.toa)


def test_inner_product_weights_reproduce_kinetic_energy_of_uniform_wind(schaer):
    """inner_product of a uniform wind (u0, 0, 0) gives u0^2/2 on a plane grid up to the
    terrain-following face tilt (mo_inner_product.F90:16-50)."""
    w = schaer.grid["inner_product_weights"]
    s = w[0] + w[2]  # weights of the two u faces
    assert np.all(s > 0.9) and np.all(s < 1.1)


def test_background_is_hydrostatic_and_periodic(hills):
    g = hills.grid
    eb, tb = g["exner_bg"], g["theta_v_bg"]
    assert np.all(eb > 0) and np.all(tb > 150)
    # hydrostatic balance c_p*theta*dPi = -dPhi between adjacent layers (the background
    # integration of mo_grid_generator.F90:1405-1429), within the discretisation error
    dpi = eb[:, :, :-1] - eb[:, :, 1:]
    dphi = g["gravity_potential"][:, :, :-1] - g["gravity_potential"][:, :, 1:]
    th = 0.5 * (tb[:, :, :-1] + tb[:, :, 1:])
    np.testing.assert_allclose(1005.0 * th * dpi, -dphi, rtol=1e-3)
    # periodic duplicates (mo_gradient_operators.F90:46-61)
    np.testing.assert_array_equal(g["slope_x"][:, 0, :], g["slope_x"][:, -1, :])
    np.testing.assert_array_equal(g["slope_y"][0, :, :], g["slope_y"][-1, :, :])


def test_random_hills_are_seeded_and_bounded():
    # the arrays are views into each model's memory: keep the models alive while reading them
    ma, mb = L.HostModel(cases.small_case("hills")), L.HostModel(cases.small_case("hills"))
    a, b = ma.surface["oro"], mb.surface["oro"]
    np.testing.assert_array_equal(a, b)
    mc = L.HostModel(cases.namelist(cases.SMALL["hills"][0], **{**cases.SMALL["hills"][1], "seed": 99}))
    assert not np.array_equal(a, mc.surface["oro"])
    assert a.min() >= 0 and a.max() > 100


def test_moist_jet_state(hills):
    m = L.HostModel(cases.small_case("jet"))
    rho = m.state["rho"]
    assert rho.shape[3] == 7
    assert np.all(rho >= 0)
    q = rho[..., 6] / rho[..., 5]
    assert 1e-4 < q.max() < 0.05                # specific humidity below 5 %
    assert np.all(rho[..., 4] == 0)             # graupel zero
    assert np.abs(m.state["wind_u"]).max() == pytest.approx(30.0, abs=0.5)


def test_unknown_orography_reports_error():
    with pytest.raises(L.LgameError) as e:
        L.HostModel(cases.namelist(cases.SMALL["hills"][0], **{**cases.SMALL["hills"][1], "orography_id": 1}))
    assert e.value.code == L.ERR_UNSUPPORTED
