"""Diffusion closure of the HEVI step: TKE, horizontal viscosity (Smagorinsky or TKE),
momentum diffusion, temperature and mass diffusion (src/subgrid_scale/mo_eff_diff_coeffs.F90,
mo_tke.F90, src/spatial_operators/mo_momentum_diff_diss.F90, mo_vector_tend_expl.F90:100-126,
mo_scalar_tend_expl.F90:60-101).

CPU: the oracle's restatement against a second, vectorised numpy restatement on a flat plane
(no terrain terms): the viscosity and the vertical diffusion of w after the first step (the
TKE is still zero then); the gas mass is conserved with mass diffusion on in a periodic
domain; the namelist defaults of &diff are the reference's (all diffusion on, smag, tke); the
split step's fused scalar diffusion, its regrouped sums restated in FP64 numpy, against the
oracle's two-pass form, and its tile, halo and face logic restated for its launch grid (every
cell owned once, every face formed once from the right cells, every index in bounds).
GPU: the FP64 step against the oracle, state and the carried diffusion diagnostics, on
periodic and non-periodic cases with orography, Smagorinsky and TKE horizontal schemes, with
horizontal momentum diffusion alone, and on a grid whose sizes are multiples of the fused
kernel's tile; the split step against the FP64 step, after ten steps and, for the temperature
and mass diffusion, after one.
"""
import numpy as np
import pytest

import cases
import lgame_gpu as L
import oracle as O

DIFF_ON = dict(lmom_diff_h=True, lmom_diff_v=True, ltemp_diff_h=True, ltemp_diff_v=True, lmass_diff_h=True,
               lmass_diff_v=True)
DIFF_FIELDS = ["tke", "viscosity", "heating_diss", "mom_diff_tend_x", "mom_diff_tend_y", "mom_diff_tend_z"]


def diff_case(key: str, **kw):
    cfg_name, ov = cases.SMALL[key]
    return cases.namelist(cfg_name, **{**ov, **DIFF_ON, **kw})


def _oracle(n):
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    o = O.Oracle(cfg, hm.grid)
    o.set_state(0, hm.state)
    o.set_state(1, hm.state)
    o.set_diag(hm.diag)
    return hm, cfg, o


def test_namelist_defaults_of_diff():
    """&diff left out: the reference's defaults (mo_diff_nml.F90:38-53)."""
    text = (cases.CONFIGS / "jet_1024x1024x80.nml").read_text()
    start = text.index("&diff")
    end = text.index("/", start)
    n = L.namelist_from_text(text[:start] + text[end + 1:])
    cfg = L.config_from_namelist(n)
    assert (cfg.lmom_diff_h, cfg.lmom_diff_v, cfg.ltemp_diff_h, cfg.ltemp_diff_v, cfg.lmass_diff_h,
            cfg.lmass_diff_v) == (1, 1, 1, 1, 1, 1)
    assert cfg.diff_coeff_scheme_h == L.DIFF_COEFF_SMAG
    assert (cfg.bg_shear, cfg.c_s) == (1.5e-5, 0.2)
    n2 = cases.namelist("jet_1024x1024x80", diff_coeff_scheme_h="tke", c_s=0.25, bg_shear=2e-5)
    cfg2 = L.config_from_namelist(n2)
    assert (cfg2.diff_coeff_scheme_h, cfg2.c_s, cfg2.bg_shear) == (L.DIFF_COEFF_TKE, 0.25, 2e-5)


# ---- numpy restatement on a flat plane (periodic, no terrain) ---------------------------------

K_B, N_A, M_D = 1.380649e-23, 6.02214076e23, 6.02214076e23 * 0.004810e-23


def _calc_diff_coeff(t, rho):
    """calc_diff_coeff, mo_derived.F90:189-216."""
    m = M_D / N_A
    thermal_velocity = np.sqrt(8.0 * K_B * t / (np.pi * m))
    particle_density = rho / m
    cross_section = 4.0 * np.pi * (130e-12 * 130e-12)
    mean_free_path = 1.0 / (np.sqrt(2.0) * particle_density * cross_section)
    return 1.0 / 3.0 * thermal_velocity * mean_free_path


def _plane_fields(hm, st, nc):
    g = hm.grid
    u, v = st["wind_u"], st["wind_v"]
    rg = st["rho"][..., nc]
    # relative vorticity at the dual points (rel_vort_z_local's flat formula with the periodic
    # wrap, mo_vorticities.F90:423-538): +dy v(i,k) - dx u(i-1,k) - dy v(i,k-1) + dx u(i,k)
    ny, nx = rg.shape[:2]
    dy, dx = g["dy"], g["dx"]
    ii = np.arange(ny + 1)
    kk = np.arange(nx + 1)
    i0 = np.where(ii == ny, 0, ii)            # v row ji (ny+1 -> 1)
    im = np.where(ii == 0, ny - 1, ii - 1)    # u row ji-1 (1 -> ny)
    k0 = np.where(kk == nx, 0, kk)            # u column jk (nx+1 -> 1)
    km = np.where(kk == 0, nx - 1, kk - 1)    # v column jk-1 (1 -> nx)
    A = dy[ii][:, k0] * v[ii][:, k0]
    B = dx[im][:, kk] * u[im][:, kk]
    Cc = dy[ii][:, km] * v[ii][:, km]
    Dd = dx[i0][:, kk] * u[i0][:, kk]
    zeta = (((A + (-1.0) * B) + (-1.0) * Cc) + Dd) / g["area_dual_z"]
    div = (u[:, 1:] * g["area_x"][:, 1:] + v[:-1] * g["area_y"][:-1] - u[:, :-1] * g["area_x"][:, :-1]
           - v[1:] * g["area_y"][1:]) / g["volume"]
    return zeta, div, rg


def test_oracle_viscosity_and_vertical_w_diffusion_plane():
    """After the first step of the flat plane case (TKE zero, so the vertical coefficient is the
    molecular one alone): viscosity = rho_g*(molecular + c_s*mean_velocity_area*max(|(zeta,
    div)|, bg_shear)) and mom_diff_tend_z = grad_vert(rho_g*nu_mol*dw/dz)/rho averaged."""
    n = diff_case("jet_plane")
    hm, cfg, o = _oracle(n)
    nc = 5 if n.lmoist else 0
    st0 = o.get_state(0)
    o.pchevi(0, 1, 0)
    dg = o.get_diag()
    T0 = dg["temperature"]
    o.close()
    g = hm.grid
    zeta, div, rg = _plane_fields(hm, st0, nc)
    vac = 0.25 * (zeta[:-1, :-1] + zeta[:-1, 1:] + zeta[1:, :-1] + zeta[1:, 1:])
    mva = 2.0 * g["area_z"][:, :, -1].sum() / g["area_z"][:, :, -1].size
    eddy = cfg.c_s * mva * np.sqrt(np.maximum(vac * vac + div * div, cfg.bg_shear ** 2))
    vmol = _calc_diff_coeff(T0, rg)
    visc = rg * (vmol + eddy)
    np.testing.assert_allclose(dg["viscosity"], visc, rtol=1e-12)
    assert not np.any(dg["tke"]), "the TKE stays zero in the first step (no gradient, no heating yet)"
    # vertical diffusion of w
    w = st0["wind_w"]
    cu = w[:, :, :-1].copy()
    cu[:, :, 0] = 0.0
    cl = w[:, :, 1:].copy()
    cl[:, :, -1] = 0.0
    az = g["area_z"]
    dwdz = (cu * az[:, :, :-1] - cl * az[:, :, 1:]) / g["volume"]
    sp = rg * vmol * dwdz
    mz = (sp[:, :, :-1] - sp[:, :, 1:]) / g["dz"][:, :, 1:-1]
    rsum = st0["rho"][..., 0].copy()
    for jc in range(1, nc + 1):
        rsum = rsum + st0["rho"][..., jc]
    mz = mz / (0.5 * (rsum[:, :, :-1] + rsum[:, :, 1:]))
    np.testing.assert_allclose(dg["mom_diff_tend_z"][:, :, 1:-1], mz, rtol=1e-10,
                               atol=1e-12 * np.abs(mz).max())
    assert not np.any(dg["mom_diff_tend_z"][:, :, [0, -1]])


@pytest.mark.parametrize("key", ["jet_plane", "hills_nonperiodic"])
def test_oracle_scalar_diffusion_is_conservative(key):
    """The mass and temperature diffusion are flux divergences whose boundary fluxes vanish
    (periodic wrap, or never-written boundary edges): sum(tendency * volume) is zero to
    rounding for every constituent and for the heating, after three steps.  A flat periodic
    plane and a non-periodic domain: where the periodic wrap joins faces of different areas
    (area_y of rows 1 and ny+1 on the rotated sphere; area_x of columns 1 and nx+1 over
    periodic terrain, whose boundary faces the grid generator extrapolates one-sidedly,
    mo_grid_generator.F90:1113-1123), the reference's sums are not zero."""
    n = diff_case(key)
    hm, cfg, o = _oracle(n)
    for k in range(3):
        o.pchevi(k % 2, (k + 1) % 2, k)
    mdt, tdh = o.scalar_diffusion()
    dg = o.get_diag()  # the same arrays as the C ABI's diagnostics
    o.close()
    assert np.array_equal(dg["temp_diff_heating"], tdh) and np.array_equal(dg["mass_diff_tendency"], mdt)
    vol = hm.grid["volume"]
    fields = [tdh] + [mdt[..., jc] for jc in range(mdt.shape[3])]
    nc = 5 if n.lmoist else 0
    assert np.abs(tdh).max() > 0.0 and np.abs(mdt[..., nc]).max() > 0.0
    for jc, x in enumerate(fields):  # constituents absent from the case diffuse nothing
        xv = x * vol
        scale = np.abs(xv).sum()
        assert abs(xv.sum()) <= 1e-12 * scale, (jc, xv.sum(), scale)


def test_oracle_diffusion_changes_the_step():
    """The closure is live: with diffusion on the state after two steps differs from the run
    without, the TKE has grown where the dissipation heats, and the heating is finite."""
    outs = []
    for on in (True, False):
        n = diff_case("jet") if on else cases.small_case("jet")
        hm, cfg, o = _oracle(n)
        for k in range(3):
            o.pchevi(k % 2, (k + 1) % 2, k)
        outs.append((o.get_state(1), o.get_diag()))
        o.close()
    (s_on, d_on), (s_off, _) = outs
    assert np.abs(s_on["wind_u"] - s_off["wind_u"]).max() > 0.0
    assert np.all(np.isfinite(d_on["heating_diss"])) and np.all(d_on["tke"] >= 0.0)
    assert d_on["tke"].max() > 0.0
    assert np.abs(d_on["mom_diff_tend_x"]).max() > 0.0


def fused_scalar_diffusion(grid, s, coef, nf, periodic, freeslip):
    """The split step's column-marching form of the horizontal scalar diffusion
    (k_diff_scalar_col in csrc/diffusion.cuh), restated in FP64 numpy as the kernel regroups it:
    per level each cell's half of the terrain remap, hc = ipw5*gz(l) + ipw6*gz(l+1); each face
    once, h*((s_b - s_a)/dx - slope*0.5*(hc_a + hc_b)); each cell's divergence finished a level
    later, the interface correction being the sum of the layer terms above and below it.
    s, coef: (ny, nx, nl) at scalar points; returns the divergence (ny, nx, nl)."""
    ny, nx, nl = s.shape
    ipw = grid["inner_product_weights"]
    sx, sy, dx, dy = grid["slope_x"], grid["slope_y"], grid["dx"], grid["dy"]
    ax, ay, az, vol, dz = grid["area_x"], grid["area_y"], grid["area_z"], grid["volume"], grid["dz"]
    gz = np.zeros((ny, nx, nl + 1))  # vertical gradients at w levels, zero at the top and bottom
    gz[:, :, 1:nl] = (s[:, :, :-1] - s[:, :, 1:]) / dz[:, :, 1:nl]
    # cells either side of the u points 1..nx+1 (x) and v points 1..ny+1 (y), periodic wrap
    ax_w, ax_e = np.r_[nx - 1, np.arange(nx)], np.r_[np.arange(nx), 0]
    ay_n, ay_s = np.r_[ny - 1, np.arange(ny)], np.r_[np.arange(ny), 0]
    out = np.zeros_like(s)
    P = tp = volp = None
    for l in range(nl):
        terrain = l + 1 > nf
        hc = np.zeros((ny, nx))
        if terrain:
            w6 = ipw[5][:, :, l] if (l + 1 < nl or freeslip) else 0.0
            hc = ipw[4][:, :, l] * gz[:, :, l] + w6 * gz[:, :, l + 1]
        sl, c = s[:, :, l], coef[:, :, l]
        g = (sl[:, ax_e] - sl[:, ax_w]) / dx[:, ax_e, l]
        if terrain:
            g = g - 0.5 * sx[:, :, l] * (hc[:, ax_w] + hc[:, ax_e])
        fx = 0.5 * (c[:, ax_w] + c[:, ax_e]) * g
        g = (sl[ay_n, :] - sl[ay_s, :]) / dy[ay_s, :, l]
        if terrain:
            g = g - 0.5 * sy[:, :, l] * (hc[ay_n, :] + hc[ay_s, :])
        fy = 0.5 * (c[ay_n, :] + c[ay_s, :]) * g
        if not periodic:
            fx[:, [0, nx]] = 0.0
            fy[[0, ny], :] = 0.0
        xw, xe, yn, ys = fx[:, :-1], fx[:, 1:], fy[:-1, :], fy[1:, :]
        comp_h = xe * ax[:, 1:, l] + yn * ay[:-1, :, l] - xw * ax[:, :-1, l] - ys * ay[1:, :, l]
        t = np.zeros((ny, nx))
        if terrain:
            t = -(xe * 0.5 * sx[:, 1:, l] * ipw[0][:, :, l] + yn * 0.5 * sy[:-1, :, l] * ipw[1][:, :, l]
                  + xw * 0.5 * sx[:, :-1, l] * ipw[2][:, :, l] + ys * 0.5 * sy[1:, :, l] * ipw[3][:, :, l])
        corr = 0.0 if not terrain else (t if l + 1 == nf + 1 else tp + t)
        U = corr * az[:, :, l]
        if l >= 1:
            out[:, :, l - 1] = (P - U) / volp
        P, tp, volp = comp_h + U, t, vol[:, :, l]
    out[:, :, nl - 1] = P / volp
    return out


@pytest.mark.parametrize("key", ["jet", "hills_nonperiodic"])
def test_fused_scalar_diffusion_algorithm_matches_oracle(key):
    """The regrouped sums of the split step's fused scalar diffusion kernel, restated in FP64
    (fused_scalar_diffusion), against the oracle's two-pass restatement of the reference
    (fluxes, then div_h with vertical_contravariant_corr): temp_diff_heating and every
    constituent's mass_diff_tendency after one step, horizontal diffusion only, within 1e-11 of
    the field's largest value: the regrouping pinned at FP64 precision, far below the bar of the
    GPU kernel's FP32 comparison (leaving out the contravariant correction moves the result by
    0.1-0.2 of its largest value here)."""
    n = diff_case(key, ltemp_diff_v=False, lmass_diff_v=False)
    hm, cfg, o = _oracle(n)
    state = hm.copy_state()
    o.pchevi(0, 1, 0)
    mdt, tdh = o.scalar_diffusion()
    dg = o.get_diag()
    o.close()
    g = hm.grid
    nf = n.n_layers - n.n_oro_layers
    rho = state["rho"]
    rho_g = rho[..., 5] if rho.shape[3] == 7 else rho[..., 0]
    visc = dg["viscosity"]
    args = (nf, bool(n.lperiodic), bool(n.lfreeslip))
    t_ref = fused_scalar_diffusion(g, dg["temperature"], 717.942189 * visc, *args)
    assert np.abs(tdh).max() > 0.0
    assert cases.rel_err(t_ref, tdh) <= 1e-11, cases.rel_err(t_ref, tdh)
    for jc in range(rho.shape[3]):
        if np.abs(mdt[..., jc]).max() == 0.0:
            continue
        m_ref = fused_scalar_diffusion(g, rho[..., jc], visc / rho_g, *args)
        assert cases.rel_err(m_ref, mdt[..., jc]) <= 1e-11, (jc, cases.rel_err(m_ref, mdt[..., jc]))


def _tile_constants():
    """DS_X, DS_Y of k_diff_scalar_col, read from its source so the check below follows it."""
    import re
    from pathlib import Path
    src = (Path(__file__).resolve().parents[1] / "l-game_gb300" / "csrc" / "diffusion.cuh").read_text()
    m = re.search(r"constexpr int DS_X = (\d+), DS_Y = (\d+), DS_THREADS = 32 \* \(DS_Y \+ 3\);", src)
    assert m, "tile constants of k_diff_scalar_col not found"
    return int(m.group(1)), int(m.group(2))


@pytest.mark.parametrize("ny,nx,periodic", [(4, 40, True), (17, 21, False), (18, 20, True), (32, 24, True),
                                            (65, 97, True), (65, 97, False), (64, 16, False), (3, 3, True)])
def test_fused_scalar_diffusion_tiles_cover_the_grid(ny, nx, periodic):
    """The slot, face and halo logic of k_diff_scalar_col (csrc/diffusion.cuh), restated on the
    CPU for its launch grid: every cell belongs to one tile thread; each face a cell reads is
    formed by exactly one thread of its block from two slots that hold data, the cells either
    side of the face across the periodic edges as the reference's grad_hor takes them; every
    shared-memory index lies in its array and every global point in its field's extent."""
    DX, DY = _tile_constants()
    SX, NS = DX + 2, (DX + 2) * (DY + 2)
    wrap_y = lambda i: ny if i < 1 else (1 if i > ny else i)
    wrap_x = lambda k: nx if k < 1 else (1 if k > nx else k)
    owner = np.zeros((ny + 1, nx + 1), dtype=int)
    for by in range((nx + DY - 1) // DY):
        for bx in range((ny + DX - 1) // DX):
            ji0, jk0 = bx * DX + 1, by * DY + 1
            slots, fxw, fyw, cells = {}, {}, {}, []
            for t in range(32 * (DY + 3)):
                lane, warp = t % 32, t // 32
                if warp < DY:
                    ji, jk, role = ji0 + lane, jk0 + warp, 0
                elif warp == DY:
                    ji, jk, role = ji0 + lane, jk0 - 1, 1
                elif warp == DY + 1:
                    ji, jk, role = ji0 + lane, jk0 + DY, 2
                elif lane < DY:
                    ji, jk, role = ji0 - 1, jk0 + lane, 3
                elif lane < 2 * DY:
                    ji, jk, role = ji0 + DX, jk0 + lane - DY, 4
                else:
                    continue
                slot = (jk - jk0 + 1) * SX + (ji - ji0 + 1)
                assert 0 <= slot < NS and slot not in slots
                has = 0 <= ji <= ny + 1 and 0 <= jk <= nx + 1
                if not periodic:
                    has = has and 1 <= ji <= ny and 1 <= jk <= nx
                slots[slot] = (wrap_y(ji), wrap_x(jk)) if has else None
                if has:
                    assert 1 <= wrap_y(ji) <= ny and 1 <= wrap_x(jk) <= nx
                fr, fc = jk - jk0, ji - ji0
                if role in (0, 2) and 1 <= ji <= ny and jk <= nx + 1:  # u point (ji, jk)
                    assert 0 <= fr <= DY and 0 <= fc < DX and (fr, fc) not in fxw
                    zero = not periodic and jk in (1, nx + 1)
                    fxw[(fr, fc)] = (slot - SX, slot, zero, (ji, jk))
                if role in (0, 4) and ji <= ny + 1 and jk <= nx:  # v point (ji, jk)
                    assert 0 <= fr < DY and 0 <= fc <= DX and (fr, fc) not in fyw
                    zero = not periodic and ji in (1, ny + 1)
                    fyw[(fr, fc)] = (slot - 1, slot, zero, (ji, jk))
                if role == 0 and ji <= ny and jk <= nx:
                    cells.append((ji, jk, fr, fc))
            for (a, b, zero, (ji, jk)) in fxw.values():  # west cell jk-1, east cell jk
                assert 0 <= a < NS
                if not zero:
                    assert slots.get(a) == (wrap_y(ji), wrap_x(jk - 1)) and slots.get(b) == (ji, wrap_x(jk))
            for (a, b, zero, (ji, jk)) in fyw.values():  # north cell ji-1, south cell ji
                assert 0 <= a < NS
                if not zero:
                    assert slots.get(a) == (wrap_y(ji - 1), jk) and slots.get(b) == (wrap_y(ji), jk)
            for ji, jk, fr, fc in cells:
                owner[ji, jk] += 1
                assert fxw[(fr, fc)][3] == (ji, jk) and fxw[(fr + 1, fc)][3] == (ji, jk + 1)
                assert fyw[(fr, fc)][3] == (ji, jk) and fyw[(fr, fc + 1)][3] == (ji + 1, jk)
    assert np.all(owner[1:, 1:] == 1) and not owner[0].any() and not owner[:, 0].any()


# ---- GPU: the FP64 step against the oracle ------------------------------------------------------

GPU_CASES = {
    "jet": {},
    "jet_tke": dict(diff_coeff_scheme_h="tke"),
    "jet_mom_h_only": dict(lmom_diff_v=False, ltemp_diff_h=False, lmass_diff_h=False),
    "hills_nonperiodic": {},
    "schaer": {},
    # ny a multiple of 32 and nx of 8: the split step's fused scalar diffusion forms the periodic
    # wrap faces ny+1 and nx+1 in its halo lanes and warps rather than inside its tiles
    "jet_tiles": dict(ny=32, nx=24),
}


def _gpu_case(name):
    kw = dict(GPU_CASES[name])
    key = name.split("_tke")[0].split("_mom_h_only")[0].split("_tiles")[0]
    return diff_case(key, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GPU_CASES))
def test_fp64_diffusion_matches_oracle(name):
    n = _gpu_case(name)
    hm, cfg, o = _oracle(n)
    cfg.precision = L.PRECISION_FP64
    g = L.GpuModel(cfg, hm.grid)
    g.set_state(0, hm.state)
    g.set_state(1, hm.state)
    g.set_diag(hm.diag)
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
    for f in DIFF_FIELDS + ["temp_diff_heating", "mass_diff_tendency"]:
        assert cases.rel_err(dgpu[f], do[f]) <= 1e-11, (f, cases.rel_err(dgpu[f], do[f]))
    assert do["viscosity"].max() > 0.0 and np.abs(do["mom_diff_tend_x"]).max() > 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["jet", "hills_nonperiodic"])
def test_split_diffusion_close_to_fp64(name):
    """The split step's FP32 closure against the FP64 step: the state after ten steps within
    the split step's bar (3e-5 of each field's maximum), the carried diffusion diagnostics
    within FP32 accuracy of theirs."""
    from test_split import field_errors
    n = _gpu_case(name)
    hm = L.HostModel(n)
    gs = []
    for prec in (L.PRECISION_FP64, L.PRECISION_SPLIT):
        cfg = L.config_from_namelist(n)
        cfg.precision = prec
        g = L.GpuModel(cfg, hm.grid)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(hm.diag)
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
    for f in DIFF_FIELDS:
        assert np.all(np.isfinite(da[f])), f
        assert cases.rel_err(da[f], db[f]) <= 2e-3, (f, cases.rel_err(da[f], db[f]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["jet", "hills_nonperiodic", "schaer", "jet_tiles"])
def test_split_scalar_diffusion_close_to_fp64(name):
    """The split step's temperature and mass diffusion (fluxes and divergence formed in one
    column-marching launch, in FP32) against the FP64 step's two-kernel form, after one step
    from the same state: temp_diff_heating and each constituent's mass_diff_tendency within
    SCALAR_DIFF_TOL of the field's largest value."""
    n = _gpu_case(name)
    hm = L.HostModel(n)
    out = {}
    for prec in (L.PRECISION_FP64, L.PRECISION_SPLIT):
        cfg = L.config_from_namelist(n)
        cfg.precision = prec
        g = L.GpuModel(cfg, hm.grid)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(hm.diag)
        g.pchevi(0, 1, 0)
        out[prec] = g.get_diag()
        g.close()
    a, b = out[L.PRECISION_SPLIT], out[L.PRECISION_FP64]
    errs = {"temp_diff_heating": cases.rel_err(a["temp_diff_heating"], b["temp_diff_heating"])}
    for jc in range(b["mass_diff_tendency"].shape[-1]):
        ref = b["mass_diff_tendency"][..., jc]
        if np.abs(ref).max() > 0.0:
            errs[f"mass_diff_tendency[{jc}]"] = cases.rel_err(a["mass_diff_tendency"][..., jc], ref)
    assert np.abs(b["temp_diff_heating"]).max() > 0.0 and np.abs(b["mass_diff_tendency"]).max() > 0.0
    print(name, errs)
    assert max(errs.values()) <= SCALAR_DIFF_TOL, errs


SCALAR_DIFF_TOL = 1e-3
