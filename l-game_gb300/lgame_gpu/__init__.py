"""Python bindings of liblgame_gpu.so (ctypes over the C ABI of include/lgame_gpu.h and
include/lgame_host.h).

The library is the product: CUDA kernels for sm_103a behind a C ABI.  This module only
marshals numpy arrays (Fortran order, the reference's extents) into it.  There is no
fallback: if the shared library or a CUDA device is missing, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_PKG = _HERE.parent
LIB_PATH = _PKG / "_build" / "liblgame_gpu.so"

# ---- status codes and enums (include/lgame_gpu.h) ------------------------------
OK, ERR_INVALID_ARG, ERR_BAD_DIMS, ERR_BAD_CONFIG, ERR_UNSUPPORTED = 0, -1, -2, -3, -4
ERR_ALLOC, ERR_CUDA, ERR_NONFINITE, ERR_NO_DEVICE, ERR_STATE = -5, -6, -7, -8, -9
PRECISION_FP64, PRECISION_SPLIT, PRECISION_SPLIT_FP64_COLUMN = 0, 1, 2
# diff_coeff_scheme_h (lgame_config)
DIFF_COEFF_SMAG = 0
DIFF_COEFF_TKE = 1

GRID_FIELDS = ["z_scalar", "z_u", "z_v", "z_w", "dx", "dy", "dz", "volume", "area_x", "area_y", "area_z",
               "area_dual_x", "area_dual_y", "area_dual_z", "z_area_dual_z", "slope_x", "slope_y",
               "inner_product_weights", "theta_v_bg", "exner_bg", "exner_bg_grad_u", "exner_bg_grad_v",
               "exner_bg_grad_w", "gravity_m_v", "gravity_potential", "fvec_x", "fvec_y", "fvec_z",
               "trsk_weights_u", "trsk_weights_v", "dx_dual", "dy_dual", "layer_thickness",
               "land_fraction", "lake_fraction", "roughness_length", "sfc_rho_c", "t_conduc_soil", "t_const_soil",
               "z_soil_interface", "z_soil_center", "z_t_const"]
STATE_FIELDS = ["rho", "rhotheta_v", "theta_v_pert", "exner_pert", "wind_u", "wind_v", "wind_w", "temperature_soil"]
# the atmosphere's fields (LGAME_STATE_NFIELDS_ATMOS): a state dict without the soil temperature
ATMOS_FIELDS = STATE_FIELDS[:7]
# fields of an output file (enum lgame_output_field), float32, scalar points
OUTPUT_FIELDS = ["rho", "temperature", "rel_humidity", "wind_u", "wind_v", "wind_w"]
# one level of lateral boundary data (t_bc, mo_definitions.F90:117-131), state-field shapes
BC_FIELDS = ["rho", "rhotheta_v", "wind_u", "wind_v", "wind_w"]
# lgame_bc_loader: (user, t_update, time_index) -> 0 on success
BC_LOADER = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_double, C.c_int)


def output_arrays(ny, nx, nl, ncons, fields=OUTPUT_FIELDS):
    """Fortran-ordered float32 arrays for the selected output fields (no relative humidity in
    dry runs) and the pointer array of lgame_gpu_output / oracle_output."""
    out = {}
    for f in fields:
        if f == "rel_humidity" and ncons == 1:
            continue
        shape = (ny, nx, nl, ncons) if f == "rho" else (ny, nx, nl)
        out[f] = np.zeros(shape, np.float32, order="F")
    fp = C.POINTER(C.c_float)
    ptrs = (fp * len(OUTPUT_FIELDS))(*[out[f].ctypes.data_as(fp) if f in out else fp() for f in OUTPUT_FIELDS])
    return out, ptrs


# ---- raw binary files (include/lgame_host.h) -------------------------------------------------
class BcFiles(C.Structure):
    """lgame_bc_files (include/lgame_host.h)."""
    _fields_ = [("ctx", C.c_void_p), ("root", C.c_char_p), ("t_init", C.c_double), ("ny", C.c_int),
                ("nx", C.c_int), ("n_layers", C.c_int), ("n_constituents", C.c_int)]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def write_snapshot(path, ny, nx, nl, ncons, step, slot0: dict, slot1: dict, diag: dict, ns: int = 0):
    """Restart snapshot of both state slots (ns soil layers), the carried diagnostics and the
    step counter."""
    lib = load_library()
    sh = field_shapes(ny, nx, nl, ncons, ns)
    arr = lambda d, names: [np.asfortranarray(d[f] if f in d else np.zeros(sh[f]), dtype=np.float64) for f in names]
    a0, a1, ad = arr(slot0, STATE_FIELDS), arr(slot1, STATE_FIELDS), arr(diag, DIAG_FIELDS)
    check(lib.lgame_host_write_snapshot(str(path).encode(), ny, nx, nl, ncons, ns, step, ptr_array(a0),
                                        ptr_array(a1), ptr_array(ad)), "lgame_host_write_snapshot")


def read_snapshot(path, ny, nx, nl, ncons, ns: int = 0):
    """(step, slot 0 state, slot 1 state, diagnostics) of a snapshot written for these dimensions."""
    lib = load_library()
    sh = field_shapes(ny, nx, nl, ncons, ns)
    s0 = {f: np.zeros(sh[f], order="F") for f in STATE_FIELDS}
    s1 = {f: np.zeros(sh[f], order="F") for f in STATE_FIELDS}
    dg = {f: np.zeros(sh[f], order="F") for f in DIAG_FIELDS}
    step = C.c_longlong()
    check(lib.lgame_host_read_snapshot(str(path).encode(), ny, nx, nl, ncons, ns, C.byref(step),
                                       ptr_array([s0[f] for f in STATE_FIELDS]), ptr_array([s1[f] for f in STATE_FIELDS]),
                                       ptr_array([dg[f] for f in DIAG_FIELDS])), "lgame_host_read_snapshot")
    return step.value, s0, s1, dg


def write_bc_level(path, ny, nx, nl, ncons, t_valid, level: dict):
    lib = load_library()
    a = [np.asfortranarray(level[f], dtype=np.float64) for f in BC_FIELDS]
    check(lib.lgame_host_write_bc_level(str(path).encode(), ny, nx, nl, ncons, t_valid, *[_dp(x) for x in a]),
          "lgame_host_write_bc_level")


def read_bc_level(path, ny, nx, nl, ncons):
    """(valid time, level) of a boundary level file."""
    lib = load_library()
    sh = field_shapes(ny, nx, nl, ncons)
    lev = {f: np.zeros(sh[f], order="F") for f in BC_FIELDS}
    t = C.c_double()
    check(lib.lgame_host_read_bc_level(str(path).encode(), ny, nx, nl, ncons, C.byref(t),
                                       *[_dp(lev[f]) for f in BC_FIELDS]), "lgame_host_read_bc_level")
    return t.value, lev


def bc_filename(root, t_update, t_init) -> str:
    lib = load_library()
    buf = C.create_string_buffer(4096)
    check(lib.lgame_host_bc_filename(str(root).encode(), t_update, t_init, buf, len(buf)), "lgame_host_bc_filename")
    return buf.value.decode()


def bc_callback(model, loader):
    """A C loader for model.bc_setup: loader(t_update, time_index) returns the level (a dict
    of BC_FIELDS arrays), which goes to model.set_bc(time_index, ...); None gives a null loader."""
    if loader is None:
        return BC_LOADER()

    def cb(user, t_update, time_index):
        try:
            model.set_bc(time_index, loader(t_update, time_index))
            return 0
        except Exception:  # reported to the library as a failed load
            import traceback
            traceback.print_exc()
            return 1
    return BC_LOADER(cb)
DIAG_FIELDS = ["p_grad_acc_neg_nl_u", "p_grad_acc_neg_nl_v", "p_grad_acc_neg_nl_w", "p_grad_acc_neg_l_u",
               "p_grad_acc_neg_l_v", "p_grad_acc_neg_l_w", "p_grad_acc_old_u", "p_grad_acc_old_v",
               "pot_vort_tend_x", "pot_vort_tend_y", "pot_vort_tend_z", "v_squared_grad_x", "v_squared_grad_y",
               "v_squared_grad_z", "condensates_sediment_heat", "radiation_tendency", "temperature",
               "tend_rho", "tend_rhotheta_v", "tend_wind_u", "tend_wind_v", "tend_wind_w",
               "tke", "viscosity", "heating_diss", "mom_diff_tend_x", "mom_diff_tend_y", "mom_diff_tend_z",
               "v_squared", "roughness_length_diag", "roughness_velocity", "monin_obukhov_length",
               "scalar_flux_resistance", "power_flux_density_sens_soil", "power_flux_density_sens_sea", "sst",
               "sfc_sw_in", "sfc_lw_out", "phase_trans_rates", "phase_trans_heating_rate",
               "power_flux_density_lat_lake", "power_flux_density_lat_sea", "temp_diff_heating",
               "mass_diff_tendency"]


class Config(C.Structure):
    """lgame_config (include/lgame_gpu.h)."""
    _fields_ = [("ny", C.c_int), ("nx", C.c_int), ("n_layers", C.c_int), ("n_oro_layers", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("toa", C.c_double), ("dtime", C.c_double),
                ("theta_adv_order", C.c_int), ("llinear", C.c_int), ("lcorio", C.c_int),
                ("luse_bg_state", C.c_int), ("lplane", C.c_int), ("lmoist", C.c_int), ("lklemp", C.c_int),
                ("klemp_damp_max", C.c_double), ("klemp_begin_rel", C.c_double),
                ("lmom_diff_h", C.c_int), ("lmom_diff_v", C.c_int), ("ltemp_diff_h", C.c_int),
                ("ltemp_diff_v", C.c_int), ("lmass_diff_h", C.c_int), ("lmass_diff_v", C.c_int),
                ("lprog_soil_temp", C.c_int), ("lsfc_sensible_heat_flux", C.c_int),
                ("lsfc_phase_trans", C.c_int), ("lpbl", C.c_int), ("lperiodic", C.c_int),
                ("lfreeslip", C.c_int), ("precision", C.c_int), ("check_finite", C.c_int),
                ("device", C.c_int), ("diff_coeff_scheme_h", C.c_int), ("bg_shear", C.c_double),
                ("c_s", C.c_double), ("nsoillays", C.c_int), ("h_prandtl", C.c_double), ("karman", C.c_double),
                ("lphase_trans", C.c_int)]


def _s(n):
    return C.c_char * n


class Namelist(C.Structure):
    """lgame_namelist (include/lgame_host.h)."""
    _fields_ = [
        ("ny", C.c_int), ("nx", C.c_int), ("n_layers", C.c_int), ("n_oro_layers", C.c_int),
        ("dy", C.c_double), ("dx", C.c_double), ("run_span_min", C.c_int), ("stretching_parameter", C.c_double),
        ("theta_adv_order", C.c_int), ("toa", C.c_double), ("scenario", _s(64)), ("llinear", C.c_int),
        ("run_id", _s(64)), ("lcorio", C.c_int), ("lat_center", C.c_double), ("lon_center", C.c_double),
        ("start_year", C.c_int), ("start_month", C.c_int), ("start_day", C.c_int), ("start_hour", C.c_int),
        ("start_minute", C.c_int), ("lplane", C.c_int), ("luse_bg_state", C.c_int),
        ("dt_write_min", C.c_int), ("lread_geo", C.c_int), ("lwrite_grid", C.c_int),
        ("grid_filename", _s(64)), ("restart_filename", _s(64)), ("lwrite_integrals", C.c_int),
        ("lmoist", C.c_int),
        ("lmom_diff_h", C.c_int), ("lmom_diff_v", C.c_int), ("ltemp_diff_h", C.c_int), ("ltemp_diff_v", C.c_int),
        ("lmass_diff_h", C.c_int), ("lmass_diff_v", C.c_int), ("h_prandtl", C.c_double), ("karman", C.c_double),
        ("lklemp", C.c_int), ("klemp_damp_max", C.c_double), ("klemp_begin_rel", C.c_double),
        ("diff_coeff_scheme_h", _s(16)), ("diff_coeff_scheme_v", _s(16)), ("bg_shear", C.c_double),
        ("c_s", C.c_double),
        ("orography_id", C.c_int), ("lprog_soil_temp", C.c_int), ("nsoillays", C.c_int),
        ("lsfc_sensible_heat_flux", C.c_int), ("lsfc_phase_trans", C.c_int), ("lpbl", C.c_int), ("lsleve", C.c_int),
        ("n_swamp", C.c_int), ("lperiodic", C.c_int), ("lfreeslip", C.c_int), ("dtime_bc", C.c_int),
        ("bc_root_filename", _s(64)),
        ("lrad", C.c_int), ("dtime_rad", C.c_double), ("rrtmgp_coefficients_file_sw", _s(128)),
        ("rrtmgp_coefficients_file_lw", _s(128)), ("cloud_coefficients_file_sw", _s(128)),
        ("cloud_coefficients_file_lw", _s(128)),
        ("precision", C.c_int), ("dtime_override", C.c_double), ("strict_reference", C.c_int),
        ("seed", C.c_longlong), ("n_hills", C.c_int), ("hill_height_min", C.c_double),
        ("hill_height_max", C.c_double), ("hill_width_min", C.c_double), ("hill_width_max", C.c_double),
        ("jet_speed", C.c_double), ("jet_pressure", C.c_double), ("t_pert_sigma", C.c_double),
        ("rh_mean", C.c_double), ("check_finite", C.c_int), ("lphase_trans", C.c_int),
        ("n_levels", C.c_int), ("n_flat_layers", C.c_int), ("n_condensed_constituents", C.c_int),
        ("n_constituents", C.c_int), ("eff_hor_res", C.c_double), ("dtime", C.c_double), ("dt_write", C.c_double),
        ("t_init", C.c_double)]


class LgameError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def load_library(path: str | os.PathLike | None = None):
    """Loads liblgame_gpu.so (built by l-game_gb300/build.py); raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: run `python l-game_gb300/build.py` (or __graft_entry__.build())")
    lib = C.CDLL(str(p))
    vp, i, d, ll = C.c_void_p, C.c_int, C.c_double, C.c_longlong
    fp = C.POINTER(C.c_float)
    pp = C.POINTER(C.POINTER(C.c_double))
    sig = {
        "lgame_gpu_create": (i, [C.POINTER(Config), C.POINTER(vp)]),
        "lgame_gpu_set_grid": (i, [vp, pp, i]),
        "lgame_gpu_set_state": (i, [vp, i, pp, i]),
        "lgame_gpu_get_state": (i, [vp, i, pp, i]),
        "lgame_gpu_set_diag": (i, [vp, pp, i]),
        "lgame_gpu_get_diag": (i, [vp, pp, i]),
        "lgame_gpu_pchevi": (i, [vp, i, i, i, i, d]),
        "lgame_gpu_pchevi_host": (i, [vp, pp, pp, i, i, i, d]),
        "lgame_gpu_budgets": (i, [vp, i, C.POINTER(C.c_double), i]),
        "lgame_gpu_synchronize": (i, [vp]),
        "lgame_gpu_kernels_per_step": (i, [vp]),
        "lgame_gpu_device_bytes": (ll, [vp]),
        "lgame_gpu_stream": (vp, [vp]),
        "lgame_gpu_set_profiling": (i, [vp, i]),
        "lgame_gpu_set_graphs": (i, [vp, i]),
        "lgame_gpu_output": (i, [vp, i, i, d, d, C.POINTER(C.POINTER(C.c_float)), i, C.POINTER(i)]),
        "lgame_gpu_bc_setup": (i, [vp, i, i, d, BC_LOADER, vp]),
        "lgame_host_write_snapshot": (i, [C.c_char_p, i, i, i, i, i, ll, pp, pp, pp]),
        "lgame_host_read_snapshot": (i, [C.c_char_p, i, i, i, i, i, C.POINTER(ll), pp, pp, pp]),
        "lgame_host_write_bc_level": (i, [C.c_char_p, i, i, i, i, d] + [C.POINTER(C.c_double)] * 5),
        "lgame_host_read_bc_level": (i, [C.c_char_p, i, i, i, i, C.POINTER(d)] + [C.POINTER(C.c_double)] * 5),
        "lgame_host_bc_filename": (i, [C.c_char_p, d, d, C.c_char_p, i]),
        "lgame_bc_file_loader": (i, [vp, d, i]),
        "lgame_gpu_set_bc": (i, [vp, i] + [C.POINTER(C.c_double)] * 5),
        "lgame_gpu_update_boundaries": (i, [vp, i, d]),
        "lgame_gpu_bc_state": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(d)]),
        "lgame_gpu_profile_report": (i, [vp, C.c_char_p, i]),
        "lgame_gpu_destroy": (None, [vp]),
        "lgame_gpu_last_error": (C.c_char_p, []),
        "lgame_gpu_version": (C.c_char_p, []),
        "lgame_namelist_defaults": (None, [C.POINTER(Namelist)]),
        "lgame_namelist_parse": (i, [C.c_char_p, C.POINTER(Namelist)]),
        "lgame_namelist_read_file": (i, [C.c_char_p, C.POINTER(Namelist)]),
        "lgame_config_from_namelist": (i, [C.POINTER(Namelist), C.POINTER(Config)]),
        "lgame_host_setup": (i, [C.POINTER(Namelist), C.POINTER(vp)]),
        "lgame_host_destroy": (None, [vp]),
        "lgame_host_grid_field": (C.POINTER(C.c_double), [vp, i, C.POINTER(C.c_size_t)]),
        "lgame_host_state_field": (C.POINTER(C.c_double), [vp, i, C.POINTER(C.c_size_t)]),
        "lgame_host_diag_field": (C.POINTER(C.c_double), [vp, i, C.POINTER(C.c_size_t)]),
        "lgame_host_surface_field": (C.POINTER(C.c_double), [vp, i, C.POINTER(C.c_size_t)]),
        "lgame_gpu_budgets_static": (i, [vp, i, C.POINTER(C.c_double), i]),
        # radiation emulator (include/lgame_emulator.h)
        "lgame_rad_teacher": (i, [fp, ll, i, fp]),
        "lgame_emu_create": (i, [i, i, i, C.c_ulonglong, i, C.POINTER(vp)]),
        "lgame_emu_destroy": (None, [vp]),
        "lgame_emu_num_params": (ll, [vp]),
        "lgame_emu_get_params": (i, [vp, fp]),
        "lgame_emu_set_params": (i, [vp, fp]),
        "lgame_emu_set_normalization": (i, [vp, fp, fp, fp, fp]),
        "lgame_emu_loss_grad": (i, [vp, fp, fp, i, fp, fp]),
        "lgame_emu_train_step": (i, [vp, fp, fp, i, C.c_float, fp]),
        "lgame_emu_set_dataset": (i, [vp, fp, fp, ll]),
        "lgame_emu_train_epoch": (i, [vp, i, C.c_float, C.c_ulonglong, fp]),
        "lgame_emu_infer": (i, [vp, fp, ll, fp]),
        "lgame_emu_gemm_bf16": (i, [vp, C.POINTER(C.c_ushort), C.POINTER(C.c_ushort), fp, i, i, i]),
        "lgame_emu_stats": (i, [vp, C.POINTER(ll), C.POINTER(d)]),
        "lgame_emu_time_gemm": (i, [vp, i, i, i, i, C.POINTER(d)]),
        "lgame_gpu_rad_set_surface": (i, [vp, C.POINTER(d), C.POINTER(d), C.POINTER(d)]),
        "lgame_gpu_rad_features": (i, [vp, i, d, fp]),
        "lgame_gpu_rad_apply_heating": (i, [vp, i, fp]),
        "lgame_gpu_rad_update": (i, [vp, vp, i, d, i, d, C.POINTER(d)]),
        "lgame_gpu_rad_attach": (i, [vp, vp, d, i, d]),
        "lgame_gpu_rad_last_report": (i, [vp, C.POINTER(d), C.POINTER(i)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


def last_error() -> str:
    return load_library().lgame_gpu_last_error().decode()


def check(rc: int, what: str = ""):
    if rc != OK:
        raise LgameError(rc, f"{what}: {last_error()}")


# ---- shapes (Fortran order, the reference's extents) ----------------------------
def field_shapes(ny: int, nx: int, nl: int, ncons: int, ns: int = 0) -> dict[str, tuple]:
    """Shapes of every grid, state and diagnostic field; ns = nsoillays."""
    s, u, v, w = (ny, nx, nl), (ny, nx + 1, nl), (ny + 1, nx, nl), (ny, nx, nl + 1)
    p = (ny, nx)
    z, ex, ey = (ny + 1, nx + 1, nl), (ny + 1, nx, nl + 1), (ny, nx + 1, nl + 1)
    return {
        "z_scalar": s, "z_u": u, "z_v": v, "z_w": w, "dx": u, "dy": v, "dz": w, "volume": s,
        "area_x": u, "area_y": v, "area_z": w, "area_dual_x": ex, "area_dual_y": ey, "area_dual_z": z,
        "z_area_dual_z": z, "slope_x": u, "slope_y": v, "inner_product_weights": (6, ny, nx, nl),
        "theta_v_bg": s, "exner_bg": s, "exner_bg_grad_u": u, "exner_bg_grad_v": v, "exner_bg_grad_w": w,
        "gravity_m_v": w, "gravity_potential": s, "fvec_x": (ny + 1, nx), "fvec_y": (ny, nx + 1),
        "fvec_z": (ny + 1, nx + 1), "trsk_weights_u": (3, ny), "trsk_weights_v": (2, ny + 1),
        "rho": (ny, nx, nl, ncons), "rhotheta_v": s, "theta_v_pert": s, "exner_pert": s,
        "wind_u": u, "wind_v": v, "wind_w": w,
        "p_grad_acc_neg_nl_u": u, "p_grad_acc_neg_nl_v": v, "p_grad_acc_neg_nl_w": w,
        "p_grad_acc_neg_l_u": u, "p_grad_acc_neg_l_v": v, "p_grad_acc_neg_l_w": w,
        "p_grad_acc_old_u": u, "p_grad_acc_old_v": v, "pot_vort_tend_x": u, "pot_vort_tend_y": v,
        "pot_vort_tend_z": w, "v_squared_grad_x": u, "v_squared_grad_y": v, "v_squared_grad_z": w,
        "condensates_sediment_heat": s, "radiation_tendency": s, "temperature": s,
        "tend_rho": (ny, nx, nl, ncons), "tend_rhotheta_v": s, "tend_wind_u": u, "tend_wind_v": v, "tend_wind_w": w,
        "dx_dual": v, "dy_dual": u, "layer_thickness": s,
        "tke": s, "viscosity": s, "heating_diss": s, "mom_diff_tend_x": u, "mom_diff_tend_y": v,
        "mom_diff_tend_z": w,
        "land_fraction": p, "lake_fraction": p, "roughness_length": p, "sfc_rho_c": p, "t_conduc_soil": p,
        "t_const_soil": p, "z_soil_interface": (ns + 1,), "z_soil_center": (ns,), "z_t_const": (1,),
        "temperature_soil": (ny, nx, ns),
        "v_squared": s, "roughness_length_diag": p, "roughness_velocity": p, "monin_obukhov_length": p,
        "scalar_flux_resistance": p, "power_flux_density_sens_soil": p, "power_flux_density_sens_sea": p,
        "sst": p, "sfc_sw_in": p, "sfc_lw_out": p,
        "phase_trans_rates": (ny, nx, nl, 6 if ncons == 7 else 1), "phase_trans_heating_rate": s,
        "power_flux_density_lat_lake": p, "power_flux_density_lat_sea": p,
        "temp_diff_heating": s, "mass_diff_tendency": (ny, nx, nl, ncons),
    }


def state_fields(state: dict) -> list:
    """The state fields a dict carries: all of STATE_FIELDS, or the atmosphere's alone."""
    return STATE_FIELDS if "temperature_soil" in state else ATMOS_FIELDS


def ptr_array(arrays: list) -> C.Array:
    """double** for a list of Fortran-ordered float64 arrays (None -> NULL)."""
    arr = (C.POINTER(C.c_double) * len(arrays))()
    for k, a in enumerate(arrays):
        if a is None:
            arr[k] = C.POINTER(C.c_double)()
        else:
            assert a.dtype == np.float64 and a.flags.f_contiguous, "arrays must be float64, Fortran-contiguous"
            arr[k] = a.ctypes.data_as(C.POINTER(C.c_double))
    return arr


# ---- namelist -------------------------------------------------------------------
def namelist_from_text(text: str, defaults: bool = True) -> Namelist:
    lib = load_library()
    n = Namelist()
    if defaults:
        lib.lgame_namelist_defaults(C.byref(n))
    check(lib.lgame_namelist_parse(text.encode(), C.byref(n)), "lgame_namelist_parse")
    return n


def config_from_namelist(n: Namelist) -> Config:
    c = Config()
    check(load_library().lgame_config_from_namelist(C.byref(n), C.byref(c)), "lgame_config_from_namelist")
    return c


class HostModel:
    """Grid, background state and idealised initial state built by the library's host code
    (lgame_host_setup): the inputs a Fortran host would pass to the GPU step.  grid, state,
    diag and surface are numpy views of the library's arrays, valid while this object lives."""

    def __init__(self, nml: Namelist):
        self.lib = load_library()
        self.nml = nml
        self.h = C.c_void_p()
        check(self.lib.lgame_host_setup(C.byref(nml), C.byref(self.h)), "lgame_host_setup")
        self.ny, self.nx, self.nl = nml.ny, nml.nx, nml.n_layers
        self.ncons = nml.n_constituents
        self.ns = nml.nsoillays
        self.shapes = field_shapes(self.ny, self.nx, self.nl, self.ncons, self.ns)
        self.grid = {f: self._view(self.lib.lgame_host_grid_field, k, f) for k, f in enumerate(GRID_FIELDS)}
        self.state = {f: self._view(self.lib.lgame_host_state_field, k, f) for k, f in enumerate(STATE_FIELDS)}
        self.diag = {f: self._view(self.lib.lgame_host_diag_field, k, f) for k, f in enumerate(DIAG_FIELDS)}
        self.surface = {}
        for k, name in enumerate(["oro", "sfc_albedo", "lat_geo_scalar", "lon_geo_scalar"]):
            n = C.c_size_t()
            p = self.lib.lgame_host_surface_field(self.h, k, C.byref(n))
            self.surface[name] = np.ctypeslib.as_array(p, shape=(n.value,)).reshape((self.ny, self.nx), order="F")

    def _view(self, fn, k, name):
        n = C.c_size_t()
        p = fn(self.h, k, C.byref(n))
        shape = self.shapes[name]
        assert int(np.prod(shape)) == n.value, (name, shape, n.value)
        return np.ctypeslib.as_array(p, shape=(n.value,)).reshape(shape, order="F")

    def copy_state(self) -> dict:
        return {k: np.asfortranarray(v.copy(order="F")) for k, v in self.state.items()}

    def copy_diag(self) -> dict:
        return {k: np.asfortranarray(v.copy(order="F")) for k, v in self.diag.items()}

    def close(self):
        if self.h:
            self.lib.lgame_host_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuModel:
    """One GPU context (lgame_gpu_create) with the grid uploaded."""

    def __init__(self, cfg: Config, grid: dict):
        self.lib = load_library()
        self.cfg = cfg
        self.h = C.c_void_p()
        check(self.lib.lgame_gpu_create(C.byref(cfg), C.byref(self.h)), "lgame_gpu_create")
        self.ny, self.nx, self.nl = cfg.ny, cfg.nx, cfg.n_layers
        self.ncons = 7 if cfg.lmoist else 1
        self.ns = cfg.nsoillays
        self.shapes = field_shapes(self.ny, self.nx, self.nl, self.ncons, self.ns)
        arrs = [None if grid.get(f) is None else np.asfortranarray(grid[f], dtype=np.float64) for f in GRID_FIELDS]
        check(self.lib.lgame_gpu_set_grid(self.h, ptr_array(arrs), len(arrs)), "lgame_gpu_set_grid")

    def set_state(self, slot: int, state: dict):
        arrs = [np.asfortranarray(state[f], dtype=np.float64) for f in state_fields(state)]
        check(self.lib.lgame_gpu_set_state(self.h, slot, ptr_array(arrs), len(arrs)), "lgame_gpu_set_state")

    def get_state(self, slot: int) -> dict:
        out = {f: np.zeros(self.shapes[f], order="F") for f in STATE_FIELDS}
        check(self.lib.lgame_gpu_get_state(self.h, slot, ptr_array([out[f] for f in STATE_FIELDS]),
                                           len(STATE_FIELDS)), "lgame_gpu_get_state")
        return out

    def set_diag(self, diag: dict):
        arrs = [None if diag.get(f) is None else np.asfortranarray(diag[f], dtype=np.float64) for f in DIAG_FIELDS]
        check(self.lib.lgame_gpu_set_diag(self.h, ptr_array(arrs), len(arrs)), "lgame_gpu_set_diag")

    def get_diag(self) -> dict:
        out = {f: np.zeros(self.shapes[f], order="F") for f in DIAG_FIELDS}
        check(self.lib.lgame_gpu_get_diag(self.h, ptr_array([out[f] for f in DIAG_FIELDS]), len(DIAG_FIELDS)),
              "lgame_gpu_get_diag")
        return out

    def pchevi(self, old_slot: int, new_slot: int, step: int, lrad_update: int = 0, t0: float = 0.0):
        check(self.lib.lgame_gpu_pchevi(self.h, old_slot, new_slot, step, lrad_update, t0), "lgame_gpu_pchevi")

    def pchevi_host(self, state_old: dict, state_new: dict, step: int):
        names = state_fields(state_old)
        a = [state_old[f] for f in names]
        b = [state_new[f] for f in names]
        check(self.lib.lgame_gpu_pchevi_host(self.h, ptr_array(a), ptr_array(b), len(names), step, 0, 0.0),
              "lgame_gpu_pchevi_host")

    def budgets(self, slot: int) -> np.ndarray:
        out = np.zeros(11)
        check(self.lib.lgame_gpu_budgets(self.h, slot, out.ctypes.data_as(C.POINTER(C.c_double)), 11),
              "lgame_gpu_budgets")
        return out[: self.ncons + 4]

    def synchronize(self):
        check(self.lib.lgame_gpu_synchronize(self.h), "lgame_gpu_synchronize")

    def kernels_per_step(self) -> int:
        return self.lib.lgame_gpu_kernels_per_step(self.h)

    def device_bytes(self) -> int:
        return self.lib.lgame_gpu_device_bytes(self.h)

    def stream_handle(self) -> int:
        """cudaStream_t of the context (for CUDA events recorded by the caller)."""
        return int(self.lib.lgame_gpu_stream(self.h) or 0)

    def set_profiling(self, enable: bool):
        check(self.lib.lgame_gpu_set_profiling(self.h, 1 if enable else 0), "lgame_gpu_set_profiling")

    def set_graphs(self, enable: bool):
        """Launch each step after step 0 as a captured CUDA graph (the default) or kernel by kernel."""
        check(self.lib.lgame_gpu_set_graphs(self.h, 1 if enable else 0), "lgame_gpu_set_graphs")

    def output(self, slot_1: int, slot_2: int, coeff_1: float, coeff_2: float, fields=OUTPUT_FIELDS):
        """The fields of an output file for coeff_1*state[slot_1] + coeff_2*state[slot_2]
        (float32 arrays, scalar points) and the crash flag; `fields` selects which to fetch."""
        out, ptrs = output_arrays(self.ny, self.nx, self.nl, self.ncons, fields)
        crashed = C.c_int()
        check(self.lib.lgame_gpu_output(self.h, slot_1, slot_2, coeff_1, coeff_2, ptrs, len(OUTPUT_FIELDS),
                                        C.byref(crashed)), "lgame_gpu_output")
        return out, bool(crashed.value)

    # lateral boundary relaxation (mo_boundaries.F90)
    def bc_setup(self, n_swamp: int, dtime_bc: int, t_latest_bc: float = 0.0, loader=None):
        """Relaxation toward boundary data at the end of every step of this non-periodic run;
        loader(t_update, time_index) -> dict of BC_FIELDS supplies later levels."""
        self._bc_cb = bc_callback(self, loader)
        check(self.lib.lgame_gpu_bc_setup(self.h, n_swamp, dtime_bc, t_latest_bc, self._bc_cb, None),
              "lgame_gpu_bc_setup")

    def bc_setup_files(self, n_swamp: int, dtime_bc: int, root, t_init: float = 0.0, t_latest_bc: float = 0.0):
        """Relaxation with later levels read by the library's own loader (lgame_bc_file_loader)
        from the files bc_filename(root, t_update, t_init)."""
        self._bc_root = str(root).encode()
        self._bc_files = BcFiles(self.h, self._bc_root, t_init, self.ny, self.nx, self.nl, self.ncons)
        self._bc_cb = C.cast(self.lib.lgame_bc_file_loader, BC_LOADER)
        check(self.lib.lgame_gpu_bc_setup(self.h, n_swamp, dtime_bc, t_latest_bc, self._bc_cb,
                                          C.cast(C.pointer(self._bc_files), C.c_void_p)), "lgame_gpu_bc_setup")

    def set_bc(self, time_index: int, bc: dict):
        arrs = [np.asfortranarray(bc[f], dtype=np.float64) for f in BC_FIELDS]
        dp = C.POINTER(C.c_double)
        check(self.lib.lgame_gpu_set_bc(self.h, time_index, *[a.ctypes.data_as(dp) for a in arrs]), "lgame_gpu_set_bc")

    def update_boundaries(self, slot: int, t_now: float):
        check(self.lib.lgame_gpu_update_boundaries(self.h, slot, t_now), "lgame_gpu_update_boundaries")

    def bc_state(self) -> tuple[int, int, float]:
        io, inew, t = C.c_int(), C.c_int(), C.c_double()
        check(self.lib.lgame_gpu_bc_state(self.h, C.byref(io), C.byref(inew), C.byref(t)), "lgame_gpu_bc_state")
        return io.value, inew.value, t.value

    def profile_report(self) -> dict:
        import json
        n = self.lib.lgame_gpu_profile_report(self.h, None, 0)
        if n < 0:
            check(n, "lgame_gpu_profile_report")
        buf = C.create_string_buffer(n + 1)
        self.lib.lgame_gpu_profile_report(self.h, buf, n + 1)
        return json.loads(buf.value.decode())

    def close(self):
        if self.h:
            self.lib.lgame_gpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
