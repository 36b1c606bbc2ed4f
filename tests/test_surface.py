"""Surface layer, planetary boundary layer and soil of the HEVI step (src/subgrid_scale/mo_pbl.F90,
the sensible heat flux and soil rows of three_band_solver_ver, mo_column_solvers.F90:80-133,
228-300, 335-340, and their call sites mo_manage_pchevi.F90:51-53, mo_vector_tend_expl.F90:
119-125).

CPU: the namelist defaults of &surface; the host's soil grid, soil and sea temperatures and
surface properties (mo_grid_generator.F90:746-813, 1360-1378, mo_set_initial_state.F90:237-247);
the oracle against a second, vectorised numpy restatement: the surface turbulence quantities
(roughness length over the sea, roughness velocity, Monin-Obukhov length, scalar flux
resistance), the PBL friction of the lowest layer's u and v (as the difference of a step with and
without the PBL from the same state), and the soil temperature (a dense solve of the soil rows
against the oracle's Thomas sweep over the combined atmosphere + soil system); the surface
physics changes the step.  GPU: the FP64 step against the oracle (state with soil temperature and
the surface diagnostics) on moving, resting, non-periodic and land-covered cases, the split step
against the FP64 step, and the host-buffer entry point carrying the soil temperature.
"""
import numpy as np
import pytest

import cases
import lgame_gpu as L
import oracle as O

SFC_ON = dict(lprog_soil_temp=True, lsfc_sensible_heat_flux=True, lsfc_phase_trans=True, lpbl=True)
DIFF_ON = dict(lmom_diff_h=True, lmom_diff_v=True, ltemp_diff_h=True, ltemp_diff_v=True, lmass_diff_h=True,
               lmass_diff_v=True)
SFC_DIAG = ["roughness_length_diag", "roughness_velocity", "monin_obukhov_length", "scalar_flux_resistance",
            "power_flux_density_sens_soil", "power_flux_density_sens_sea", "v_squared", "mom_diff_tend_x",
            "mom_diff_tend_y", "heating_diss", "tend_rhotheta_v"]
GRAVITY, EPS = 9.80616, 1e-10


def sfc_case(key: str, **kw):
    cfg_name, ov = cases.SMALL[key]
    return cases.namelist(cfg_name, **{**ov, **DIFF_ON, **SFC_ON, **kw})


def with_land(hm):
    """The grid with land (and some lake) on a band of columns, soil properties to match
    (mo_grid_generator.F90:782-793), and the host's surface radiation fluxes: exercises the
    soil branch of the sensible heat flux and the radiative terms of the soil rows."""
    grid = dict(hm.grid)
    ny, nx = hm.ny, hm.nx
    land = np.zeros((ny, nx), order="F")
    lake = np.zeros((ny, nx), order="F")
    land[:, nx // 3: 2 * nx // 3] = 1.0
    land[: ny // 2, 2 * nx // 3:] = 0.6
    lake[: ny // 2, 2 * nx // 3:] = 0.3
    on = land > 1e-10
    rhoc = np.full((ny, nx), 1024.0 * 4184.0, order="F")
    tc = np.full((ny, nx), 1.4e-7, order="F")
    rhoc[on] = (land[on] * 1442.0 * 830.0 + lake[on] * 1024.0 * 4184.0) / (land[on] + lake[on])
    tc[on] = (land[on] * 7.5e-7 + lake[on] * 1.4e-7) / (land[on] + lake[on])
    rl = np.asfortranarray(grid["roughness_length"].copy())
    rl[on] = 0.5
    grid.update(land_fraction=land, lake_fraction=lake, sfc_rho_c=rhoc, t_conduc_soil=tc, roughness_length=rl)
    diag = hm.copy_diag()
    diag["roughness_length_diag"] = rl.copy(order="F")
    diag["sfc_sw_in"] = np.asfortranarray(np.full((ny, nx), 300.0))
    diag["sfc_lw_out"] = np.asfortranarray(np.full((ny, nx), 380.0))
    return grid, diag


def _oracle(n, grid=None, diag=None, state=None):
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    o = O.Oracle(cfg, grid if grid is not None else hm.grid)
    st = state if state is not None else hm.state
    o.set_state(0, st)
    o.set_state(1, st)
    o.set_diag(diag if diag is not None else hm.diag)
    return hm, cfg, o


# ---- namelist and host set-up ---------------------------------------------------------------------

def test_namelist_defaults_of_surface():
    """&surface left out: the reference's defaults (mo_surface_nml.F90:30-37), and the surface-layer
    constants of &diff (mo_diff_nml.F90:39, 46) in the step's configuration."""
    text = (cases.CONFIGS / "jet_1024x1024x80.nml").read_text()
    for group in ("&surface", "&diff"):  # the PBL's default needs &diff's default lmom_diff_h
        start = text.index(group)
        end = text.index("/", start)
        text = text[:start] + text[end + 1:]
    n = L.namelist_from_text(text)
    assert (n.lprog_soil_temp, n.nsoillays, n.lsfc_sensible_heat_flux, n.lsfc_phase_trans, n.lpbl) == (1, 5, 1, 1, 1)
    cfg = L.config_from_namelist(n)
    assert (cfg.lprog_soil_temp, cfg.lsfc_sensible_heat_flux, cfg.lsfc_phase_trans, cfg.lpbl) == (1, 1, 1, 1)
    assert (cfg.nsoillays, cfg.h_prandtl, cfg.karman) == (5, 100.0, 0.4)


def test_host_soil_grid_and_initial_soil():
    """Soil interfaces spaced by powers of 0.352 and rescaled to end at z_t_const = -10 m, centres
    halfway; soil and sea at 280 K; the carried roughness length starts at the grid's; water
    everywhere but the seabreeze land band (rho*c_p and conductivity of soil there)."""
    n = sfc_case("jet", nsoillays=5)
    hm = L.HostModel(n)
    zi, zc = hm.grid["z_soil_interface"], hm.grid["z_soil_center"]
    steps = np.array([0.352 ** (5 - jl) for jl in range(2, 7)])
    raw = np.concatenate([[0.0], np.cumsum(steps)])
    np.testing.assert_allclose(zi, -10.0 / raw[-1] * raw, rtol=1e-15, atol=0)
    np.testing.assert_allclose(zc, 0.5 * (zi[:-1] + zi[1:]), rtol=1e-15)
    assert hm.grid["z_t_const"][0] == -10.0 and abs(zi[-1] + 10.0) < 1e-14
    assert np.all(hm.state["temperature_soil"] == 280.0) and np.all(hm.diag["sst"] == 280.0)
    np.testing.assert_array_equal(hm.diag["roughness_length_diag"], hm.grid["roughness_length"])
    assert np.all(hm.grid["land_fraction"] == 0.0) and np.all(hm.grid["roughness_length"] == 0.08)
    sb = L.HostModel(cases.namelist("jet_1024x1024x80", nx=16, ny=8, n_layers=20, n_oro_layers=14,
                                    dx=5000.0, dy=5000.0, scenario="seabreeze", orography_id=0, lmoist=False))
    land = sb.grid["land_fraction"]
    cols = [jk for jk in range(1, 17) if 16 // 4 <= jk <= 3 * 16 // 4]
    assert np.all(land[:, [c - 1 for c in cols]] == 1.0) and land.sum() == 8 * len(cols)
    on = land > 0
    assert np.all(sb.grid["sfc_rho_c"][on] == 1442.0 * 830.0) and np.all(sb.grid["t_conduc_soil"][on] == 7.5e-7)
    lat = sb.surface["lat_geo_scalar"]
    np.testing.assert_allclose(sb.grid["roughness_length"][on], np.maximum(
        1e-4, 20.0 * np.cos(lat[on]) * np.exp(-sb.grid["z_w"][:, :, -1][on] / 1500.0) / 8.0), rtol=1e-15)
    np.testing.assert_allclose(sb.grid["t_const_soil"], 273.15 + 25.0 * np.cos(2.0 * lat), rtol=1e-15)


# ---- numpy restatement of the surface layer -----------------------------------------------------------

def np_turb(grid, st, vsq, rl_prev, dtime, karman=0.4, h_prandtl=100.0):
    """update_sfc_turb_quantities (mo_pbl.F90:19-108) over all columns: (rl, rv, mol, sfr)."""
    zs, zw = grid["z_scalar"], grid["z_w"]
    agl = zs[:, :, -1] - zw[:, :, -1]
    u_low = np.sqrt(vsq[:, :, -1])
    u10 = u_low * np.log(10.0 / rl_prev) / np.log(agl / rl_prev)
    land = grid["land_fraction"]
    swh = 0.0248 * u10 ** 2
    wl = GRAVITY * (0.729 * u10) ** 2 / (2.0 * np.pi)
    rl_sea = np.maximum(1e-4, 1200.0 * swh * (swh / np.maximum(wl, EPS)) ** 4.5)
    rl = np.where(land < 1.0, land * grid["roughness_length"] + (1.0 - land) * rl_sea, rl_prev)
    rv = rough_vel(u_low, agl, rl, karman)
    tv = grid["theta_v_bg"] + st["theta_v_pert"]
    dtv = (tv[:, :, -2] - tv[:, :, -1]) / (zs[:, :, -2] - zs[:, :, -1])
    w_pert = u10 * np.maximum(0.001, 0.02 * (1.0 - dtv / 0.01))
    wt = 0.2 * w_pert * (-0.2 * dtime * w_pert * dtv)
    wt = np.where(np.abs(wt) < EPS, EPS, wt)
    mol = -tv[:, :, -1] * rv ** 3 / (karman * GRAVITY * wt)
    h = np.minimum(agl, h_prandtl)
    sfr = 1.0 / (karman * rv) * (np.log(h / rl) - psi(h, mol, "h") + np.log(7.0))
    sfr = np.maximum(sfr, dtime / agl)
    return rl, rv, mol, sfr


def rough_vel(w, z, rl, karman):
    den = np.log(z / rl)
    den = np.where(np.abs(den) < EPS, EPS, den)
    return np.maximum(EPS, w * karman / den)


def psi(eff, l, kind):
    """psi_h / psi_m, mo_pbl.F90:382-433."""
    ll = np.where(np.abs(l) < EPS, EPS, l)
    with np.errstate(invalid="ignore"):
        x = np.where(ll < 0.0, (1.0 - 15.0 * eff / np.where(ll < 0.0, ll, -1.0)) ** 0.25, 0.0)
    if kind == "h":
        return np.where(ll < 0.0, 2.0 * np.log((1.0 + x ** 2) / 2.0), -4.0 * eff / ll)
    unstable = 2.0 * np.log((1.0 + x) / 2.0) + np.log((1.0 + x ** 2) / 2.0) - 2.0 * np.arctan(x) + np.pi / 2.0
    return np.where(ll < 0.0, unstable, -4.7 * eff / ll)


def np_friction(grid, vsq, rl, mol, wind, z_vec, a, b, dtime, karman=0.4, h_prandtl=100.0):
    """The PBL friction (mo_pbl.F90:133-156) of vector points between the column arrays a and b
    (index tuples into the (ny, nx) planes): the acceleration that is subtracted."""
    zw = grid["z_w"]
    ws = 0.5 * (np.sqrt(vsq[:, :, -1][a]) + np.sqrt(vsq[:, :, -1][b]))
    zs = 0.5 * (zw[:, :, -1][a] + zw[:, :, -1][b])
    z_agl = z_vec - zs
    lt = 0.5 * (zw[:, :, -2][a] + zw[:, :, -2][b]) - zs
    r = 0.5 * (rl[a] + rl[b])
    m = 0.5 * (mol[a] + mol[b])
    h = np.minimum(z_agl, h_prandtl)
    fr = 1.0 / (karman * rough_vel(ws, z_agl, r, karman)) * (np.log(h / r) - psi(h, m, "m"))
    fr = np.maximum(fr, dtime / z_agl)
    wrf = np.where(z_agl > h_prandtl, np.log(h_prandtl / r) / np.log(z_agl / r), 1.0)
    return wrf * wind / fr / lt


def _one_step(n, grid, diag, state, k):
    hm, cfg, o = _oracle(n, grid, diag, state)
    o.pchevi(0, 1, k)
    out = o.get_state(1), o.get_diag()
    o.close()
    return out


def test_oracle_turbulence_quantities_numpy():
    """The surface turbulence quantities of step 1 from state and v_squared after step 0."""
    n = sfc_case("jet")
    hm, cfg, o = _oracle(n)
    o.pchevi(0, 1, 0)
    st0, d0 = o.get_state(1), o.get_diag()
    o.pchevi(1, 0, 1)
    d1 = o.get_diag()
    o.close()
    rl, rv, mol, sfr = np_turb(hm.grid, st0, d0["v_squared"], d0["roughness_length_diag"], cfg.dtime)
    assert np.abs(rv).max() > 1e-3 and np.all(np.isfinite(mol))
    for name, ref in [("roughness_length_diag", rl), ("roughness_velocity", rv), ("monin_obukhov_length", mol),
                      ("scalar_flux_resistance", sfr)]:
        assert cases.rel_err(d1[name], ref) <= 1e-12, (name, cases.rel_err(d1[name], ref))


def test_oracle_pbl_friction_numpy():
    """A step from the same state with and without the PBL: the lowest layer's momentum diffusion
    acceleration differs by the numpy friction at every u and v point, periodic wrap included."""
    n_on = sfc_case("jet")
    hm, cfg, o = _oracle(n_on)
    o.pchevi(0, 1, 0)
    st, dg = o.get_state(1), o.get_diag()
    o.close()
    s_on, d_on = _one_step(n_on, hm.grid, dg, st, 1)
    s_off, d_off = _one_step(sfc_case("jet", lpbl=False), hm.grid, dg, st, 1)
    ny, nx = hm.ny, hm.nx
    g, vsq, rl, mol = hm.grid, dg["v_squared"], d_on["roughness_length_diag"], d_on["monin_obukhov_length"]
    jj, kk = np.meshgrid(np.arange(ny), np.arange(nx + 1), indexing="ij")
    fu = np_friction(g, vsq, rl, mol, st["wind_u"][:, :, -1], g["z_u"][:, :, -1],
                     (jj, (kk - 1) % nx), (jj, kk % nx), cfg.dtime)
    jj, kk = np.meshgrid(np.arange(ny + 1), np.arange(nx), indexing="ij")
    fv = np_friction(g, vsq, rl, mol, st["wind_v"][:, :, -1], g["z_v"][:, :, -1],
                     ((jj - 1) % ny, kk), (jj % ny, kk), cfg.dtime)
    du = d_off["mom_diff_tend_x"][:, :, -1] - d_on["mom_diff_tend_x"][:, :, -1]
    dv = d_off["mom_diff_tend_y"][:, :, -1] - d_on["mom_diff_tend_y"][:, :, -1]
    scale_u = np.abs(d_on["mom_diff_tend_x"]).max() + np.abs(fu).max()
    scale_v = np.abs(d_on["mom_diff_tend_y"]).max() + np.abs(fv).max()
    assert np.abs(fu).max() > 0.0 and np.abs(fv).max() > 0.0
    assert np.abs(du - fu).max() <= 1e-12 * scale_u
    assert np.abs(dv - fv).max() <= 1e-12 * scale_v
    # the layers above are untouched
    np.testing.assert_array_equal(d_off["mom_diff_tend_x"][:, :, :-1], d_on["mom_diff_tend_x"][:, :, :-1])


def test_oracle_soil_rows_numpy():
    """Prognostic soil without the sensible heat flux: the soil temperature after one step is the
    solution of the soil rows (mo_column_solvers.F90:228-300) with the carried sensible flux and
    the radiation fluxes; numpy's dense solve against the oracle's sweep over the combined
    system, whose coupling entries are zero."""
    n = sfc_case("jet", lsfc_sensible_heat_flux=False, lsfc_phase_trans=False, lpbl=False)
    hm = L.HostModel(n)
    grid, diag = with_land(hm)
    rng = np.random.default_rng(7)
    ny, nx, ns = hm.ny, hm.nx, hm.ns
    diag["power_flux_density_sens_soil"] = np.asfortranarray(rng.uniform(-50.0, 50.0, (ny, nx)))
    state = hm.copy_state()
    state["temperature_soil"] = np.asfortranarray(280.0 + rng.uniform(-3.0, 3.0, (ny, nx, ns)))
    hm2, cfg, o = _oracle(n, grid, diag, state)
    o.pchevi(0, 1, 0)
    new = o.get_state(1)["temperature_soil"]
    o.close()
    dt, zi, zc, zt = cfg.dtime, grid["z_soil_interface"], grid["z_soil_center"], grid["z_t_const"][0]
    worst = 0.0
    for ji in range(ny):
        for jk in range(nx):
            rc, tc, ts = grid["sfc_rho_c"][ji, jk], grid["t_conduc_soil"][ji, jk], state["temperature_soil"][ji, jk]
            h = np.empty(ns)
            h[:-1] = -rc * tc * (ts[:-1] - ts[1:]) / (zc[:-1] - zc[1:])
            h[-1] = -rc * tc * (ts[-1] - grid["t_const_soil"][ji, jk]) / (2.0 * (zc[-1] - zt))
            dzi = zi[:-1] - zi[1:]
            r = np.empty(ns)
            r[0] = ts[0] + (diag["power_flux_density_sens_soil"][ji, jk] + diag["sfc_sw_in"][ji, jk]
                            - diag["sfc_lw_out"][ji, jk] + 0.5 * h[0]) / (dzi[0] * rc) * dt
            r[1:] = ts[1:] + 0.5 * (-h[:-1] + h[1:]) / (dzi[1:] * rc) * dt
            q = 0.5 * dt * rc * tc / (dzi * rc)
            inv = 1.0 / (zc[:-1] - zc[1:])
            A = np.zeros((ns, ns))
            for jl in range(ns):
                A[jl, jl] = 1.0 + q[jl] * ((inv[jl - 1] if jl > 0 else 0.0) + (inv[jl] if jl < ns - 1 else 0.0))
            for jl in range(ns - 1):
                A[jl + 1, jl] = -0.5 * dt * rc * tc / (dzi[jl + 1] * rc) * inv[jl]
                A[jl, jl + 1] = -0.5 * dt * rc * tc / (dzi[jl] * rc) * inv[jl]
            x = np.linalg.solve(A, r)
            worst = max(worst, np.abs(x - new[ji, jk]).max() / np.abs(x).max())
    assert worst <= 1e-13, worst
    assert np.abs(new - state["temperature_soil"]).max() > 1e-6


def test_oracle_surface_changes_the_step():
    """The surface physics is live: the lowest layer's wind and rhotheta_v after three steps
    differ from the run without it, everything stays finite, and over land the sensible flux
    into the soil is formed while over the sea the flux into the sea is (and not the other)."""
    outs = []
    for on in (True, False):
        n = sfc_case("jet") if on else sfc_case("jet", lprog_soil_temp=False, lsfc_sensible_heat_flux=False,
                                                 lsfc_phase_trans=False, lpbl=False)
        hm = L.HostModel(n)
        grid, diag = with_land(hm)
        _, cfg, o = _oracle(n, grid, diag)
        for k in range(3):
            o.pchevi(k % 2, (k + 1) % 2, k)
        outs.append((o.get_state(1), o.get_diag(), grid))
        o.close()
    (s_on, d_on, grid), (s_off, _, _) = outs
    for f in ("wind_u", "wind_v", "rhotheta_v"):
        assert np.abs(s_on[f][:, :, -1] - s_off[f][:, :, -1]).max() > 0.0, f
    assert all(np.all(np.isfinite(v)) for v in s_on.values())
    land = grid["land_fraction"] + grid["lake_fraction"]
    ss, se = d_on["power_flux_density_sens_soil"], d_on["power_flux_density_sens_sea"]
    assert np.all(ss[land == 0.0] == 0.0) and np.abs(ss[land > 0.0]).min() > 0.0
    assert np.all(se[land == 1.0] == 0.0) and np.abs(se[land < 1.0]).min() > 0.0
    assert np.abs(s_on["temperature_soil"] - 280.0).max() > 1e-6


# ---- GPU: the FP64 step against the oracle ------------------------------------------------------------

GPU_CASES = {
    "jet": ("jet", {}, False),                         # moving atmosphere, all switches on
    "jet_land": ("jet", {}, True),                     # land and lake columns, radiation fluxes
    "schaer_odd": ("schaer_odd", {}, False),           # uniform flow over a ridge, dry
    "hills": ("hills", {}, False),                     # atmosphere at rest: the resistances' limits
    "hills_nonperiodic": ("hills_nonperiodic", {}, True),  # PBL and fluxes at non-periodic edges
    "jet_soil_only": ("jet", dict(lsfc_sensible_heat_flux=False, lsfc_phase_trans=False, lpbl=False,
                                  lmom_diff_h=False, lmom_diff_v=False, ltemp_diff_h=False, ltemp_diff_v=False,
                                  lmass_diff_h=False, lmass_diff_v=False), True),
    # the PBL alone: the turbulence update without the scalar flux resistance (no soil)
    "jet_pbl_only": ("jet", dict(lprog_soil_temp=False, lsfc_sensible_heat_flux=False, lsfc_phase_trans=False), False),
    # the surface phase-transition switch alone: only the turbulence update runs (the reference's
    # step forms no phase transitions), and its roughness length is carried
    "jet_sfc_phase_switch_only": ("jet", dict(lsfc_sensible_heat_flux=False, lpbl=False, lprog_soil_temp=False),
                                  False),
}


def _gpu_setup(name):
    key, kw, land = GPU_CASES[name]
    n = sfc_case(key, **kw)
    hm = L.HostModel(n)
    grid, diag = with_land(hm) if land else (hm.grid, hm.diag)
    return n, hm, grid, diag


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GPU_CASES))
def test_fp64_surface_matches_oracle(name):
    n, hm, grid, diag = _gpu_setup(name)
    _, cfg, o = _oracle(n, grid, diag)
    cfg.precision = L.PRECISION_FP64
    g = L.GpuModel(cfg, grid)
    for slot in (0, 1):
        g.set_state(slot, hm.state)
    g.set_diag(diag)
    nsteps = 4
    for k in range(nsteps):
        o.pchevi(k % 2, (k + 1) % 2, k)
        g.pchevi(k % 2, (k + 1) % 2, k)
    so, sg = o.get_state(nsteps % 2), g.get_state(nsteps % 2)
    do, dgpu = o.get_diag(), g.get_diag()
    g.close()
    o.close()
    for f in so:
        assert cases.rel_err(sg[f], so[f]) <= 1e-12, (f, cases.rel_err(sg[f], so[f]))
    for f in SFC_DIAG:
        assert cases.rel_err(dgpu[f], do[f]) <= 1e-11, (f, cases.rel_err(dgpu[f], do[f]))
    if n.lprog_soil_temp:  # the soil moved; without prognostic soil it stays as set
        assert np.abs(so["temperature_soil"] - 280.0).max() > 0.0
    else:
        assert np.all(sg["temperature_soil"] == hm.state["temperature_soil"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["jet", "jet_land"])
def test_split_surface_close_to_fp64(name):
    """The split step with the surface physics against the FP64 step: the state after ten steps
    within the split step's bar (3e-5 of each field's maximum), the soil temperature and the
    surface diagnostics close (the surface kernels run in FP64 in both)."""
    from test_split import field_errors
    n, hm, grid, diag = _gpu_setup(name)
    gs = []
    for prec in (L.PRECISION_FP64, L.PRECISION_SPLIT):
        cfg = L.config_from_namelist(n)
        cfg.precision = prec
        g = L.GpuModel(cfg, grid)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(diag)
        gs.append(g)
    for step in range(10):
        for g in gs:
            g.pchevi(step % 2, (step + 1) % 2, step)
    a, b = gs[1].get_state(0), gs[0].get_state(0)
    da, db = gs[1].get_diag(), gs[0].get_diag()
    for g in gs:
        g.close()
    errs = field_errors(a, b)
    assert max(errs.values()) <= 3e-5, errs
    assert cases.rel_err(a["temperature_soil"] - 280.0, b["temperature_soil"] - 280.0) <= 1e-3
    for f in ("roughness_velocity", "monin_obukhov_length", "scalar_flux_resistance", "power_flux_density_sens_sea"):
        assert np.all(np.isfinite(da[f])), f
        assert cases.rel_err(da[f], db[f]) <= 1e-3, (f, cases.rel_err(da[f], db[f]))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [L.PRECISION_FP64, L.PRECISION_SPLIT])
def test_pchevi_host_carries_the_soil(precision):
    """lgame_gpu_pchevi_host with all eight state arrays equals lgame_gpu_pchevi bit for bit, soil
    temperature included, and refuses the atmosphere's seven alone when the soil is prognostic."""
    n, hm, grid, diag = _gpu_setup("jet_land")
    cfg = L.config_from_namelist(n)
    cfg.precision = precision
    out = []
    for host in (False, True):
        g = L.GpuModel(cfg, grid)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(diag)
        if host:
            s = hm.copy_state()
            for k in range(2):
                new = {f: np.zeros_like(v, order="F") for f, v in s.items()}
                g.pchevi_host(s, new, k)
                s = new
            with pytest.raises(L.LgameError):
                g.pchevi_host({f: s[f] for f in L.ATMOS_FIELDS}, {f: new[f] for f in L.ATMOS_FIELDS}, 2)
            out.append(s)
        else:
            for k in range(2):
                g.pchevi(k % 2, (k + 1) % 2, k)
            out.append(g.get_state(0))
        g.close()
    for f in L.STATE_FIELDS:
        np.testing.assert_array_equal(out[0][f], out[1][f], err_msg=f)
