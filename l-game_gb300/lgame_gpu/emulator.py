"""Radiation emulator (include/lgame_emulator.h) through ctypes: the tensor-core MLP, the
stand-in radiation scheme that provides its targets, and the coupling to a GpuModel.

Feature rows: 4*nlev+2 floats per column (temperature, dry-air pressure, water vapour and
ozone densities per layer, surface albedo, cos(zenith)); heating rows: 2*nlev floats
(shortwave, longwave; K/day)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import LgameError, check, load_library

_F = C.POINTER(C.c_float)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_F)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def bf16_bits(x) -> np.ndarray:
    """float32 -> BF16 bit patterns, round to nearest even."""
    u = _f32(x).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def bf16_round(x) -> np.ndarray:
    return (bf16_bits(x).astype(np.uint32) << 16).view(np.float32)


def teacher(features: np.ndarray, nlev: int) -> np.ndarray:
    """Heating rates (ncol x 2*nlev, K/day) of the stand-in scheme (lgame_rad_teacher)."""
    lib = load_library()
    x = _f32(features)
    n = x.shape[0]
    y = np.zeros((n, 2 * nlev), np.float32)
    check(lib.lgame_rad_teacher(_fp(x), n, nlev, _fp(y)), "lgame_rad_teacher")
    return y


class Emulator:
    """The MLP (4*nlev+2) -> hidden x3 (GELU) -> 2*nlev on one GPU."""

    def __init__(self, nlev: int = 80, hidden: int = 512, batch_max: int = 8192, seed: int = 1, device: int = 0):
        self.lib = load_library()
        self.h = C.c_void_p()
        check(self.lib.lgame_emu_create(nlev, hidden, batch_max, C.c_ulonglong(seed), device, C.byref(self.h)),
              "lgame_emu_create")
        self.nlev, self.hidden, self.batch_max = nlev, hidden, batch_max
        self.nin, self.nout = 4 * nlev + 2, 2 * nlev

    def close(self):
        if self.h:
            self.lib.lgame_emu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        return int(self.lib.lgame_emu_num_params(self.h))

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.num_params, np.float32)
        check(self.lib.lgame_emu_get_params(self.h, _fp(p)), "lgame_emu_get_params")
        return p

    def set_params(self, p: np.ndarray):
        p = _f32(p)
        if p.size != self.num_params:
            raise ValueError("wrong number of parameters")
        check(self.lib.lgame_emu_set_params(self.h, _fp(p)), "lgame_emu_set_params")

    def split_params(self, p: np.ndarray) -> list[np.ndarray]:
        """[W1, b1, W2, b2, W3, b3, W4, b4] views of a flat parameter vector."""
        shapes = [(self.hidden, self.nin), (self.hidden,), (self.hidden, self.hidden), (self.hidden,),
                  (self.hidden, self.hidden), (self.hidden,), (self.nout, self.hidden), (self.nout,)]
        out, off = [], 0
        for s in shapes:
            n = int(np.prod(s))
            out.append(p[off:off + n].reshape(s))
            off += n
        return out

    def set_normalization(self, x_mean, x_std, y_mean, y_std):
        a = [_f32(v) for v in (x_mean, x_std, y_mean, y_std)]
        check(self.lib.lgame_emu_set_normalization(self.h, *[_fp(v) for v in a]), "lgame_emu_set_normalization")
        self.norm = a

    def loss_grad(self, x, y) -> tuple[float, np.ndarray]:
        x, y = _f32(x), _f32(y)
        loss = np.zeros(1, np.float32)
        g = np.zeros(self.num_params, np.float32)
        check(self.lib.lgame_emu_loss_grad(self.h, _fp(x), _fp(y), x.shape[0], _fp(loss), _fp(g)),
              "lgame_emu_loss_grad")
        return float(loss[0]), g

    def train_step(self, x, y, lr: float) -> float:
        x, y = _f32(x), _f32(y)
        loss = np.zeros(1, np.float32)
        check(self.lib.lgame_emu_train_step(self.h, _fp(x), _fp(y), x.shape[0], C.c_float(lr), _fp(loss)),
              "lgame_emu_train_step")
        return float(loss[0])

    def set_dataset(self, x, y):
        x, y = _f32(x), _f32(y)
        check(self.lib.lgame_emu_set_dataset(self.h, _fp(x), _fp(y), x.shape[0]), "lgame_emu_set_dataset")

    def train_epoch(self, batch: int, lr: float, seed: int) -> float:
        loss = np.zeros(1, np.float32)
        check(self.lib.lgame_emu_train_epoch(self.h, batch, C.c_float(lr), C.c_ulonglong(seed), _fp(loss)),
              "lgame_emu_train_epoch")
        return float(loss[0])

    def infer(self, x, out: np.ndarray | None = None) -> np.ndarray:
        """Heating rates of the rows of x (n x nin); `out` (n x nout, C-contiguous float32)
        receives them when given.  Page-locked x and out are read and written by the GPU
        directly."""
        x = _f32(x)
        if out is None:
            out = np.zeros((x.shape[0], self.nout), np.float32)
        if out.dtype != np.float32 or out.shape != (x.shape[0], self.nout) or not out.flags.c_contiguous:
            raise ValueError("infer: out must be a C-contiguous float32 array of shape (n, nout)")
        check(self.lib.lgame_emu_infer(self.h, _fp(x), x.shape[0], _fp(out)), "lgame_emu_infer")
        return out

    def gemm_bf16(self, a_bits: np.ndarray, b_bits: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(a_bits, np.uint16)
        b = np.ascontiguousarray(b_bits, np.uint16)
        m, k = a.shape
        n = b.shape[0]
        c = np.zeros((m, n), np.float32)
        us = C.POINTER(C.c_ushort)
        check(self.lib.lgame_emu_gemm_bf16(self.h, a.ctypes.data_as(us), b.ctypes.data_as(us), _fp(c), m, n, k),
              "lgame_emu_gemm_bf16")
        return c

    def time_gemm(self, m: int, n: int, k: int, reps: int = 20) -> float:
        """Milliseconds per launch of the tensor-core GEMM (M x K by N x K, device data)."""
        ms = C.c_double()
        check(self.lib.lgame_emu_time_gemm(self.h, m, n, k, reps, C.byref(ms)), "lgame_emu_time_gemm")
        return float(ms.value)

    def stats(self) -> tuple[int, float]:
        n, f = C.c_longlong(), C.c_double()
        check(self.lib.lgame_emu_stats(self.h, C.byref(n), C.byref(f)), "lgame_emu_stats")
        return int(n.value), float(f.value)


def normalization_from(x: np.ndarray, y: np.ndarray):
    """Per-feature and per-output mean/std (std floored) of a training set."""
    xm, xs = x.mean(0), x.std(0)
    ym, ys = y.mean(0), y.std(0)
    xs = np.where(xs > 1e-6 * (np.abs(xm) + 1e-30), xs, 1.0)
    ys = np.where(ys > 1e-6, ys, 1.0)
    return xm.astype(np.float32), xs.astype(np.float32), ym.astype(np.float32), ys.astype(np.float32)


def rad_set_surface(model, albedo: np.ndarray, lat: np.ndarray, lon: np.ndarray):
    lib = load_library()
    dp = C.POINTER(C.c_double)
    a = [np.asfortranarray(v, dtype=np.float64) for v in (albedo, lat, lon)]
    check(lib.lgame_gpu_rad_set_surface(model.h, *[v.ctypes.data_as(dp) for v in a]), "lgame_gpu_rad_set_surface")


def rad_features(model, slot: int, t: float) -> np.ndarray:
    lib = load_library()
    nf = 4 * model.nl + 2
    x = np.zeros((model.ny * model.nx, nf), np.float32)
    check(lib.lgame_gpu_rad_features(model.h, slot, C.c_double(t), _fp(x)), "lgame_gpu_rad_features")
    return x


def rad_apply_heating(model, slot: int, heating: np.ndarray):
    lib = load_library()
    h = _f32(heating)
    check(lib.lgame_gpu_rad_apply_heating(model.h, slot, _fp(h)), "lgame_gpu_rad_apply_heating")


def rad_update(model, emu: Emulator, slot: int, t: float, sample_stride: int, bound: float) -> dict:
    lib = load_library()
    rep = np.zeros(4)
    check(lib.lgame_gpu_rad_update(model.h, emu.h, slot, C.c_double(t), sample_stride, C.c_double(bound),
                                   rep.ctypes.data_as(C.POINTER(C.c_double))), "lgame_gpu_rad_update")
    return {"rms_k_per_day": rep[0], "fallback": bool(rep[1]), "sampled": int(rep[2]), "wall_s": rep[3]}


def rad_attach(model, emu, dtime_rad: float, sample_stride: int, bound: float):
    """Lets lgame_gpu_pchevi(..., lrad_update=1, t_0) run the emulator's radiation update
    (emu None: detach)."""
    lib = load_library()
    check(lib.lgame_gpu_rad_attach(model.h, emu.h if emu is not None else None, C.c_double(dtime_rad), sample_stride,
                                   C.c_double(bound)), "lgame_gpu_rad_attach")


def rad_last_report(model) -> dict:
    lib = load_library()
    rep = np.zeros(4)
    n = C.c_int(0)
    check(lib.lgame_gpu_rad_last_report(model.h, rep.ctypes.data_as(C.POINTER(C.c_double)), C.byref(n)),
          "lgame_gpu_rad_last_report")
    return {"rms_k_per_day": rep[0], "fallback": bool(rep[1]), "sampled": int(rep[2]), "wall_s": rep[3],
            "updates": n.value}


__all__ = ["Emulator", "teacher", "bf16_bits", "bf16_round", "normalization_from", "rad_set_surface",
           "rad_features", "rad_apply_heating", "rad_update", "rad_attach", "rad_last_report", "LgameError"]
