"""Python binding of the CPU oracle (TEST INFRASTRUCTURE).

Loads oracle/_build/liblgame_oracle.so (built from oracle/ by `make -C oracle`).  Only the
tests, the smoke check and the CPU-baseline leg of bench.py use this module; the GPU
library never does.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liblgame_oracle.so"

_lib = None


def build(force: bool = False) -> Path:
    srcs = [HERE / "lgame_oracle.c", HERE / "lgame_oracle_ops.inc", HERE / "lgame_oracle_step.inc",
            HERE / "lgame_oracle_diff.inc", HERE / "lgame_oracle_sfc.inc", HERE / "lgame_oracle_phase.inc", HERE / "lgame_oracle.h",
            HERE.parent / "include" / "lgame_gpu.h", HERE / "Makefile"]
    if force or not LIB_PATH.exists() or any(s.stat().st_mtime > LIB_PATH.stat().st_mtime for s in srcs):
        subprocess.run(["make", "-s", "-C", str(HERE), "-B" if force else "all"], check=True)
    return LIB_PATH


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB_PATH))
        vp, i = C.c_void_p, C.c_int
        pp = C.POINTER(C.POINTER(C.c_double))
        from lgame_gpu import BC_LOADER, Config  # same struct layout (include/lgame_gpu.h)
        dp = C.POINTER(C.c_double)
        for name, res, args in [
            ("oracle_create", i, [C.POINTER(Config), C.POINTER(vp)]),
            ("oracle_destroy", None, [vp]),
            ("oracle_set_grid", i, [vp, pp, i]),
            ("oracle_set_state", i, [vp, i, pp, i]),
            ("oracle_get_state", i, [vp, i, pp, i]),
            ("oracle_set_diag", i, [vp, pp, i]),
            ("oracle_get_diag", i, [vp, pp, i]),
            ("oracle_pchevi", i, [vp, i, i, i]),
            ("oracle_budgets", i, [vp, i, C.POINTER(C.c_double), i]),
            ("oracle_num_threads", i, []),
            ("oracle_thomas", None, [C.POINTER(C.c_double)] * 5 + [i]),
            ("oracle_bc_setup", i, [vp, i, i, C.c_double, BC_LOADER, vp]),
            ("oracle_set_bc", i, [vp, i] + [dp] * 5),
            ("oracle_update_boundaries", i, [vp, i, C.c_double]),
            ("oracle_bc_state", i, [vp, C.POINTER(i), C.POINTER(i), dp]),
            ("oracle_bc_factors", i, [vp, dp, dp, dp]),
            ("oracle_heating_diss", i, [vp, C.POINTER(C.c_double)]),
            ("oracle_scalar_diffusion", i, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
            ("oracle_output", i, [vp, i, i, C.c_double, C.c_double, C.POINTER(C.POINTER(C.c_float)), i,
                                  C.POINTER(i)]),
        ]:
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


class Oracle:
    """The oracle's context, with the same calls as lgame_gpu.GpuModel."""

    def __init__(self, cfg, grid: dict):
        from lgame_gpu import GRID_FIELDS, field_shapes, ptr_array
        self.lib = load()
        self.h = C.c_void_p()
        rc = self.lib.oracle_create(C.byref(cfg), C.byref(self.h))
        if rc != 0:
            raise RuntimeError(f"oracle_create failed: {rc}")
        self.ncons = 7 if cfg.lmoist else 1
        self.shapes = field_shapes(cfg.ny, cfg.nx, cfg.n_layers, self.ncons, cfg.nsoillays)
        arrs = [None if grid.get(f) is None else np.asfortranarray(grid[f], dtype=np.float64) for f in GRID_FIELDS]
        rc = self.lib.oracle_set_grid(self.h, ptr_array(arrs), len(arrs))
        if rc != 0:
            raise RuntimeError(f"oracle_set_grid failed: {rc}")

    def set_state(self, slot, state):
        from lgame_gpu import ptr_array, state_fields
        arrs = [np.asfortranarray(state[f], dtype=np.float64) for f in state_fields(state)]
        assert self.lib.oracle_set_state(self.h, slot, ptr_array(arrs), len(arrs)) == 0

    def get_state(self, slot):
        from lgame_gpu import STATE_FIELDS, ptr_array
        out = {f: np.zeros(self.shapes[f], order="F") for f in STATE_FIELDS}
        assert self.lib.oracle_get_state(self.h, slot, ptr_array([out[f] for f in STATE_FIELDS]), len(STATE_FIELDS)) == 0
        return out

    def set_diag(self, diag):
        from lgame_gpu import DIAG_FIELDS, ptr_array
        arrs = [None if diag.get(f) is None else np.asfortranarray(diag[f], dtype=np.float64) for f in DIAG_FIELDS]
        assert self.lib.oracle_set_diag(self.h, ptr_array(arrs), len(arrs)) == 0

    def get_diag(self):
        from lgame_gpu import DIAG_FIELDS, ptr_array
        out = {f: np.zeros(self.shapes[f], order="F") for f in DIAG_FIELDS}
        assert self.lib.oracle_get_diag(self.h, ptr_array([out[f] for f in DIAG_FIELDS]), len(DIAG_FIELDS)) == 0
        return out

    def pchevi(self, old_slot, new_slot, step):
        rc = self.lib.oracle_pchevi(self.h, old_slot, new_slot, step)
        if rc != 0:
            raise RuntimeError(f"oracle_pchevi failed: {rc}")

    def output(self, slot_1, slot_2, coeff_1, coeff_2):
        from lgame_gpu import OUTPUT_FIELDS, output_arrays
        ny, nx, nl = self.shapes["rhotheta_v"]
        out, ptrs = output_arrays(ny, nx, nl, self.ncons)
        crashed = C.c_int()
        rc = self.lib.oracle_output(self.h, slot_1, slot_2, coeff_1, coeff_2, ptrs, len(OUTPUT_FIELDS), C.byref(crashed))
        if rc != 0:
            raise RuntimeError(f"oracle_output failed: {rc}")
        return out, bool(crashed.value)

    # lateral boundary relaxation (mo_boundaries.F90), as lgame_gpu.GpuModel
    def bc_setup(self, n_swamp, dtime_bc, t_latest_bc=0.0, loader=None):
        from lgame_gpu import bc_callback
        self._bc_cb = bc_callback(self, loader)
        rc = self.lib.oracle_bc_setup(self.h, n_swamp, dtime_bc, t_latest_bc, self._bc_cb, None)
        if rc != 0:
            raise RuntimeError(f"oracle_bc_setup failed: {rc}")

    def set_bc(self, time_index, bc):
        from lgame_gpu import BC_FIELDS
        arrs = [np.asfortranarray(bc[f], dtype=np.float64) for f in BC_FIELDS]
        dp = C.POINTER(C.c_double)
        assert self.lib.oracle_set_bc(self.h, time_index, *[a.ctypes.data_as(dp) for a in arrs]) == 0

    def update_boundaries(self, slot, t_now):
        rc = self.lib.oracle_update_boundaries(self.h, slot, t_now)
        if rc != 0:
            raise RuntimeError(f"oracle_update_boundaries failed: {rc}")

    def bc_state(self):
        io, inew, t = C.c_int(), C.c_int(), C.c_double()
        assert self.lib.oracle_bc_state(self.h, C.byref(io), C.byref(inew), C.byref(t)) == 0
        return io.value, inew.value, t.value

    def bc_factors(self):
        ny, nx = self.shapes["rhotheta_v"][:2]
        fs, fu, fv = (np.zeros(sh, order="F") for sh in [(ny, nx), (ny, nx + 1), (ny + 1, nx)])
        dp = C.POINTER(C.c_double)
        assert self.lib.oracle_bc_factors(self.h, *[a.ctypes.data_as(dp) for a in (fs, fu, fv)]) == 0
        return fs, fu, fv

    def scalar_diffusion(self):
        """(mass_diff_tendency (ny, nx, n_layers, ncons), temp_diff_heating (ny, nx, n_layers))
        of the last step."""
        ny, nx, nl = self.shapes["theta_v_pert"]
        mdt = np.zeros((ny, nx, nl, self.shapes["rho"][3]), order="F")
        tdh = np.zeros((ny, nx, nl), order="F")
        rc = self.lib.oracle_scalar_diffusion(self.h, mdt.ctypes.data_as(C.POINTER(C.c_double)),
                                              tdh.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != 0:
            raise RuntimeError(f"oracle_scalar_diffusion failed: {rc}")
        return mdt, tdh

    def heating_diss(self):
        """diag%heating_diss of the last step, (ny, nx, n_layers)."""
        ny, nx, nl = self.shapes["theta_v_pert"]
        out = np.zeros((ny, nx, nl), order="F")
        rc = self.lib.oracle_heating_diss(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != 0:
            raise RuntimeError(f"oracle_heating_diss failed: {rc}")
        return out

    def budgets(self, slot):
        out = np.zeros(11)
        assert self.lib.oracle_budgets(self.h, slot, out.ctypes.data_as(C.POINTER(C.c_double)), 11) == 0
        return out[: self.ncons + 4]

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def thomas(c, d, e, r):
    """mo_column_solvers.F90:606-640 on numpy vectors (len(d) == n, len(c) == len(e) == n-1)."""
    lib = load()
    n = len(d)
    c = np.ascontiguousarray(np.concatenate([c, [0.0]]), dtype=np.float64)
    e = np.ascontiguousarray(np.concatenate([e, [0.0]]), dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    r = np.ascontiguousarray(r, dtype=np.float64)
    x = np.zeros(n)
    P = C.POINTER(C.c_double)
    lib.oracle_thomas(c.ctypes.data_as(P), d.ctypes.data_as(P), e.ctypes.data_as(P), r.ctypes.data_as(P),
                      x.ctypes.data_as(P), n)
    return x
