"""Test cases: the benchmark namelists of l-game_gb300/configs at reduced sizes."""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np

import lgame_gpu as L

CONFIGS = Path(__file__).resolve().parent.parent / "l-game_gb300" / "configs"


def namelist_text(name: str, **overrides) -> str:
    """Text of configs/<name>.nml with `key=value` items replaced (any group) or, for
    keys not present, appended to the &gpu group."""
    text = (CONFIGS / f"{name}.nml").read_text()
    extra = {}
    for k, v in overrides.items():
        if isinstance(v, bool):
            v = ".true." if v else ".false."
        elif isinstance(v, str):
            v = f'"{v}"'
        pat = re.compile(rf"^(\s*){k}\s*=.*$", re.MULTILINE)
        if pat.search(text):
            text = pat.sub(rf"\g<1>{k}={v}", text)
        else:
            extra.setdefault(GROUP_OF.get(k, "gpu"), []).append(f"{k}={v}")
    for group, items in extra.items():
        text += f"\n&{group}\n" + "\n".join(items) + "\n/\n"
    return text


# namelist group of the keys that the overrides may add (defaults to the &gpu extension)
GROUP_OF = {
    "luse_bg_state": "run", "llinear": "run", "lcorio": "run", "lplane": "run", "theta_adv_order": "run",
    "stretching_parameter": "run", "lat_center": "run", "lon_center": "run", "scenario": "run",
    "lklemp": "diff", "klemp_damp_max": "diff", "klemp_begin_rel": "diff", "lmom_diff_h": "diff",
    "lmom_diff_v": "diff", "ltemp_diff_h": "diff", "ltemp_diff_v": "diff", "lmass_diff_h": "diff",
    "lmass_diff_v": "diff", "diff_coeff_scheme_h": "diff", "bg_shear": "diff", "c_s": "diff",
    "lperiodic": "bc", "lfreeslip": "bc", "lmoist": "constituents", "orography_id": "surface", "lsleve": "surface",
    "lprog_soil_temp": "surface", "nsoillays": "surface", "lsfc_sensible_heat_flux": "surface",
    "lsfc_phase_trans": "surface", "lpbl": "surface", "h_prandtl": "diff", "karman": "diff",
}


def namelist(name: str, **overrides) -> L.Namelist:
    return L.namelist_from_text(namelist_text(name, **overrides))


# small variants used by the parity tests: (config, overrides)
SMALL = {
    "schaer": ("schaer_256x4x60", dict(nx=40, ny=4, n_layers=24, n_oro_layers=23)),
    "schaer_odd": ("schaer_256x4x60", dict(nx=41, ny=3, n_layers=20, n_oro_layers=19, strict_reference=True)),
    "mountain_rest": ("schaer_256x4x60", dict(nx=33, ny=5, n_layers=20, n_oro_layers=19, scenario="mountain_rest",
                                              theta_adv_order=2, orography_id=4)),
    "hills": ("rest_hills_512x512x50", dict(nx=24, ny=20, n_layers=16, n_oro_layers=12, dx=6000.0, dy=6000.0,
                                            n_hills=6, hill_width_min=6000.0, hill_width_max=15000.0)),
    "hills_nonperiodic": ("rest_hills_512x512x50", dict(nx=21, ny=17, n_layers=16, n_oro_layers=12, dx=6000.0,
                                                        dy=6000.0, n_hills=6, hill_width_min=6000.0,
                                                        hill_width_max=15000.0, lperiodic=False, lfreeslip=False)),
    "jet": ("jet_1024x1024x80", dict(nx=20, ny=18, n_layers=24, n_oro_layers=18, dx=5000.0, dy=5000.0, n_hills=5,
                                     hill_height_min=200.0, hill_height_max=1500.0,
                                     hill_width_min=8000.0, hill_width_max=20000.0)),
    "jet_plane": ("jet_1024x1024x80", dict(nx=15, ny=13, n_layers=20, n_oro_layers=14, dx=5000.0, dy=5000.0,
                                           lplane=True, orography_id=0, lcorio=False)),
    "jet_order2_nobg": ("jet_1024x1024x80", dict(nx=16, ny=15, n_layers=20, n_oro_layers=14, dx=5000.0, dy=5000.0,
                                                 n_hills=4, hill_height_min=200.0, hill_height_max=1500.0,
                                                 hill_width_min=8000.0, hill_width_max=20000.0,
                                                 theta_adv_order=2, luse_bg_state=False, lklemp=False)),
}


def small_case(key: str):
    cfg_name, ov = SMALL[key]
    return namelist(cfg_name, **ov)


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max|a-b| / max|b| (0 if both are zero)."""
    d = float(np.max(np.abs(a - b))) if a.size else 0.0
    m = float(np.max(np.abs(b))) if b.size else 0.0
    if m == 0.0:
        return d
    return d / m
