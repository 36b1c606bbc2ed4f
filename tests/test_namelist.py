"""The namelist reader keeps the reference's defaults, derived quantities and sanity
checks (src/namelists/*.F90, src/control.F90:94-97), and never exits the process."""
import math

import pytest

import lgame_gpu as L


def parse(text):
    return L.namelist_from_text(text)


def test_defaults_are_the_reference_defaults():
    n = parse("")
    # mo_run_nml.F90:55-80
    assert (n.ny, n.nx, n.n_layers, n.n_oro_layers) == (35, 37, 50, 40)
    assert n.dx == 25e3 and n.dy == 25e3 and n.toa == 40000.0 and n.stretching_parameter == 1.3
    assert n.scenario == b"standard" and n.lcorio == 1 and n.lplane == 0 and n.theta_adv_order == 2
    assert n.luse_bg_state == 1 and n.llinear == 0 and n.run_span_min == 1440
    # mo_diff_nml.F90:39-53
    assert n.lmom_diff_h == 1 and n.lklemp == 1 and n.klemp_damp_max == 0.25 and n.klemp_begin_rel == 0.53
    assert n.diff_coeff_scheme_h == b"smag" and n.diff_coeff_scheme_v == b"tke"
    # mo_surface_nml.F90:148-154, mo_bc_nml.F90:293-297, mo_constituents_nml.F90:236
    assert n.orography_id == 1 and n.nsoillays == 5 and n.lpbl == 1 and n.lsleve == 0
    assert n.lperiodic == 0 and n.lfreeslip == 0 and n.n_swamp == 5 and n.dtime_bc == 10800
    assert n.lmoist == 1 and n.n_condensed_constituents == 5 and n.n_constituents == 7
    # derived, mo_run_nml.F90:89-94, mo_rad_nml.F90:207, mo_io_nml.F90:266
    assert n.n_levels == 51 and n.n_flat_layers == 10
    assert n.dtime == 1.61 * math.sqrt(25e3 * 25e3) / 1000.0
    assert n.dtime_rad == 60.0 * 25e3 / 1000.0 and n.dt_write == 3600.0


def test_reads_groups_types_and_comments():
    n = parse("""
    ! a comment line
    &run
    ny=3, nx=401   ! two items on a line
    n_layers = 70
    n_oro_layers=69
    toa=21000.0
    dy=500
    dx=5d2
    scenario='schaer'
    run_id="a ""quoted"" id"
    lcorio=.false.
    lplane=T
    theta_adv_order=3
    /
    &constituents lmoist=.false. /
    &unknown_group foo=1 /
    """)
    assert (n.ny, n.nx, n.n_layers, n.n_oro_layers) == (3, 401, 70, 69)
    assert n.dx == 500.0 and n.dy == 500.0 and n.toa == 21000.0
    assert n.scenario == b"schaer" and n.run_id == b'a "quoted" id'
    assert n.lcorio == 0 and n.lplane == 1 and n.theta_adv_order == 3
    assert n.lmoist == 0 and n.n_constituents == 1 and n.n_condensed_constituents == 0
    assert n.dtime == pytest.approx(0.805)


@pytest.mark.parametrize("text,code", [
    ("&run ny=4 /", L.ERR_BAD_DIMS),               # ny must be odd (mo_run_nml.F90:112-115)
    ("&run nx=2 /", L.ERR_BAD_DIMS),               # nx >= 3
    ("&run n_oro_layers=50 /", L.ERR_BAD_DIMS),    # n_oro_layers < n_layers
    ("&run theta_adv_order=4 /", L.ERR_BAD_CONFIG),
    ("&run toa=-1.0 /", L.ERR_BAD_CONFIG),
    ("&run lat_center=2.0 /", L.ERR_BAD_CONFIG),
    ("&diff diff_coeff_scheme_v='smag' /", L.ERR_BAD_CONFIG),
    ("&diff lmom_diff_h=.false. /", L.ERR_BAD_CONFIG),  # lpbl needs lmom_diff_h
    ("&io dt_write_min=0 /", L.ERR_BAD_CONFIG),     # dtime <= dt_write
    ("&run foo=1 /", L.ERR_BAD_CONFIG),             # unknown variable
    ("&run ny=abc /", L.ERR_BAD_CONFIG),
    ("&run ny=3", L.ERR_BAD_CONFIG),                # unterminated group
    ("&gpu precision=7 /", L.ERR_BAD_CONFIG),
])
def test_sanity_checks_return_errors(text, code):
    with pytest.raises(L.LgameError) as e:
        parse(text)
    assert e.value.code == code
    assert L.last_error()


def test_even_sizes_need_the_extension_switch():
    n = parse("&run ny=4 nx=256 / &gpu strict_reference=.false. /")
    assert n.ny == 4 and n.nx == 256


def test_dtime_override_and_config_translation():
    n = parse("&run dx=2500 dy=2500 / &gpu dtime_override=10.0 precision=1 / &bc lperiodic=.true. /")
    assert n.dtime == 10.0
    c = L.config_from_namelist(n)
    assert c.dtime == 10.0 and c.precision == 1 and c.lperiodic == 1 and c.ny == n.ny
    assert c.lmom_diff_h == 1 and c.lpbl == 1   # the reference defaults; the GPU rejects them at create
