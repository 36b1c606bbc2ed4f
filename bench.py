"""Benchmark of the GB300 HEVI step: HEVI steps/s at 1024x1024x80 (moist, rotated lat-lon).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one pchevi call (two predictor-corrector substeps) over the whole domain.
`value` is the device-resident step rate of the headline precision path (FP32/FP64 split
when built, else FP64); the FP64 step is measured beside it.  `e2e` is the same step
through the C ABI with host buffers (lgame_gpu_pchevi_host: state in from pinned host
memory, new state back).  The per-kernel roofline comes from CUDA events the library
records around every launch on its own stream.  The CPU baseline is the oracle (the
FP64 restatement of the reference, the reference itself cannot be built here) on a
bounded sub-domain of the same workload, scaled to the full domain by cell count.

N > 1: the path is run as independent replicas, one per GPU (no collective exists in
the reference's step); value = all replicas' steps / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for p in (ROOT / "l-game_gb300", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

WORKLOAD = "jet_1024x1024x80"
METRIC = "HEVI steps/s at 1024x1024x80, FP32/FP64 split vs FP64 at stated error; HBM GB/s"
# cells of the CPU-baseline sample (same namelist, smaller horizontal extent)
CPU_SAMPLE = dict(nx=128, ny=128)


def read_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "bf16_tflops": d.get("bf16_tflops", 1900.0), "src": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "src": "fallback"}


def emulator_bench(peaks: dict, nlev: int = 80, hidden: int = 512, batch: int = 8192) -> dict:
    """Radiation-emulator MLP (4*nlev+2 -> 3 x hidden GELU -> 2*nlev) on the tensor cores:
    the GEMM of one hidden layer (batch x hidden x hidden) timed with CUDA events against the
    measured BF16 peak and against the time bound of its HBM traffic (A, B and the FP32 C,
    once each), training throughput (whole Adam steps on a device-resident set of 8 batches)
    and inference throughput through the host API (1024*1024 columns; page-locked host
    features in and heating rates out, which the GPU reads and writes itself).  Random
    inputs; the rates do not depend on the values."""
    import torch
    from lgame_gpu import emulator as E
    emu = E.Emulator(nlev=nlev, hidden=hidden, batch_max=batch, seed=1)
    ms = emu.time_gemm(batch, hidden, hidden, reps=50)
    tflops = 2.0 * batch * hidden * hidden / (ms * 1e-3) / 1e12
    gemm_bytes = 2.0 * (batch * hidden + hidden * hidden) + 4.0 * batch * hidden
    t_tensor = 2.0 * batch * hidden * hidden / (peaks["bf16_tflops"] * 1e12)
    t_hbm = gemm_bytes / (peaks["hbm_gbs"] * 1e9)
    # the same layer over the 65,536-row chunks inference streams (several tiles per SM)
    ml = 65536
    ms_l = emu.time_gemm(ml, hidden, hidden, reps=20)
    bytes_l = 2.0 * (ml * hidden + hidden * hidden) + 4.0 * ml * hidden
    roof_l = max(2.0 * ml * hidden * hidden / (peaks["bf16_tflops"] * 1e12), bytes_l / (peaks["hbm_gbs"] * 1e9))
    rng = np.random.default_rng(0)
    nin, nout = 4 * nlev + 2, 2 * nlev
    x = rng.normal(size=(8 * batch, nin)).astype(np.float32)
    y = rng.normal(size=(8 * batch, nout)).astype(np.float32)
    emu.set_dataset(x, y)
    emu.train_epoch(batch, 1e-4, 1)
    emu.stats()
    t = time.perf_counter()
    for ep in range(3):
        emu.train_epoch(batch, 1e-4, ep + 2)
    dt = time.perf_counter() - t
    _, flop = emu.stats()
    ni = 1024 * 1024
    xi = torch.empty((ni, nin), dtype=torch.float32, pin_memory=True).numpy()
    yi = torch.empty((ni, nout), dtype=torch.float32, pin_memory=True).numpy()
    xi[...] = rng.normal(size=(ni, nin)).astype(np.float32)
    emu.infer(xi[:batch], out=yi[:batch])
    t = time.perf_counter()
    emu.infer(xi, out=yi)
    di = time.perf_counter() - t
    emu.close()
    return {"net": f"{nin}->{hidden}x3->{nout} GELU, BF16 operands, FP32 accumulation (tcgen05)",
            "gemm": {"bound": "hbm" if t_hbm > t_tensor else "tensor", "m": batch, "n": hidden, "k": hidden,
                     "avg_launch_ms": ms, "achieved": tflops, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                     "frac": tflops / peaks["bf16_tflops"], "peak_src": peaks["src"] + " (burst)",
                     "hbm_bytes": gemm_bytes, "roofline_ms": max(t_tensor, t_hbm) * 1e3,
                     "frac_of_roofline": max(t_tensor, t_hbm) * 1e3 / ms},
            "gemm_large": {"m": ml, "n": hidden, "k": hidden, "avg_launch_ms": ms_l,
                           "achieved_tflops": 2.0 * ml * hidden * hidden / (ms_l * 1e-3) / 1e12,
                           "hbm_bytes": bytes_l, "roofline_ms": roof_l * 1e3, "frac_of_roofline": roof_l * 1e3 / ms_l},
            "training_columns_per_s": 3 * 8 * batch / dt, "training_tflops_whole_step": flop / dt / 1e12,
            "inference_columns_per_s": ni / di,
            "inference_note": "page-locked host features in, heating rates out, accessed by the GPU directly"}


# Algorithmic (compulsory) bytes per cell of one launch: every distinct array a kernel
# touches, read or written once per cell.  Entries are (n8, nT, n8_oro, nT_oro):
#   n8  arrays stored in FP64 (the state, the pressure-gradient products, the FP64 metrics
#       and reciprocals of the column solvers); the split stencils read the FP32 mirror of
#       the state instead, so there they count 4 B (except the kinetic energy and the wind
#       update, which keep FP64 state arrays),
#   nT  arrays of the kernel's working type (8 B on the FP64 path, 4 B on the split path:
#       FP32 metric copies, intermediates, tendencies, carried stencil diagnostics),
#   *_oro  arrays read only in the terrain-following layers jl >= n_flat_layers (slopes,
#       inner-product weights, area_z), weighted by the fraction of those layers.
# ntr = number of constituents other than the gas.  Data-dependent reads (the diabatic
# branch of k_gas_theta) and 1-D/2-D arrays are left out, so these are lower bounds.
def _kernel_fields(ncons: int) -> dict:
    ntr = ncons - 1
    moist = 2 if ncons > 1 else 0
    return {
        "temperature": (2 + moist, 3, 0, 0),          # theta', exner' (+rho_g, rho_v); bg x2, T out
        "theta": (1, 2, 0, 0),                         # theta'; theta_bg, out
        "grad_vert": (0, 3, 0, 0),                     # field, dz, out
        "grad_hor": (0, 5, 0, 5),                      # field, dx, dy, 2 out; slopes, dz-gradient, 2 weights
        "div_h": (0, 6, 0, 7),                         # 2 in, area_x/y, volume, out; area_z, slopes, 4 weights
        "theta_edges": (2, 4, 0, 0),                   # u, v; theta, div, 2 out
        "eta_xy": (4, 11, 0, 0),                       # u, v, w, rho_g; dx,dy,dz,z_u,z_v,z_w,z_scalar,2 dual areas, 2 out
        "eta_z": (3, 6, 0, 3),                         # u, v, rho_g; dx, dy, area_dual_z, z_area_dual_z, z_scalar, out
        "mass_flux": (4, 3, 0, 0),                     # rho_g, u, v, w; 3 out
        "vort_flux": (0, 15, 0, 0),                    # 3 eta, 3 mass fluxes, 6 weights, 3 out
        "ke": (3, 7, 0, 0),                            # u, v, w; 6 weights, out
        "tend_wind": (12, 13, 0, 0),                   # u, v old/new, 8 pressure-gradient arrays; 3 tendencies r/w, 7 carried
        "tracers": (ntr + 2, 2 * ntr + 3, 0, 7),       # rho_jc, u, v; tend r/w per tracer, area_x/y, volume
        "gas_theta": (3, 9, 0, 7),                     # rho_g, u, v; 2 theta edges, area_x/y, volume, rad, csh, 2 out
        "gas_flux": (0, 9, 0, 0),                      # rho_g, u, v, 2 theta edges; 4 fluxes out
        "gas_div": (0, 11, 0, 7),                      # 4 fluxes, area_x/y, volume, rad, csh; 2 tendencies out
    }


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per cell of one launch of each
# split-step kernel, averaged over its launches, from a one-pass ncu capture of the moist jet
# at 256x256x80 (5.2 M cells, inputs about 5 GB, larger than L2, so the per-cell figures carry
# over to 1024x1024x80).  `roofline.traffic` is this figure times the cells of the run (bytes
# moved per launch of the dominant kernel); traffic above the algorithmic bytes is re-reads and
# per-thread stacks.
MEASURED_DRAM_BYTES_PER_CELL = {
    "ks_column_tracers": 206.0, "ks_column_ver": 228.4, "ks_tracers": 98.5, "ks_pgrad": 213.6,
    "ks_tend_wind": 109.8, "ks_gas_div": 98.7, "ks_eta": 82.9, "ks_vort_flux": 59.6, "ks_div_h": 45.0,
    "ks_ke": 78.6, "ks_theta_edges": 44.7, "ks_gas_flux": 29.4, "ks_gzp": 36.4,
    "ks_temperature": 25.4, "ks_csh_sum": 21.0, "ks_heating_diss": 16.1,
}


def step_bytes_per_cell(ncons: int, split: bool) -> float:
    """Compulsory bytes per cell of one step: reads 2P + P + 2G + T + C, writes 2P + T + C
    with P = ncons + 6 prognostic, T = ncons + 4 tendency, C = 8 carried (+1 sediment
    heating when moist) and G = 29 grid arrays.  FP64 path: all 8 B (952 B dry, 1304 B
    moist).  Split path: state 8 B; grid copies, tendencies and the carried stencil
    diagnostics 4 B; p_grad_acc_old (2 arrays) 8 B."""
    P, T, C, G = ncons + 6, ncons + 4, 8 + (1 if ncons > 1 else 0), 29
    if not split:
        return 8.0 * (3 * P + 2 * G + T + C + 2 * P + T + C)
    c8, c4 = 2, C - 2
    return 8.0 * 5 * P + 4.0 * 2 * G + 4.0 * 2 * T + 2 * (8.0 * c8 + 4.0 * c4)


def kernel_bytes_per_cell(name: str, ncons: int, split: bool, f_oro: float) -> float:
    """Algorithmic bytes per cell (ny*nx*n_layers) of one launch of kernel `name`."""
    ntr = ncons - 1
    fp64_only = {
        # state old (rho_g, rho*theta, exner', theta', w), new at rk2 (half the launches),
        # tendencies, metrics (volume, exner_bg, theta_bg, z_scalar, area_z, damping), 5 writes
        "k_column_ver": 5 + 3 + 2 + 6 + 5,
        # per tracer rho old/tend/new; w old/new, T, volume, area_z, rho_g, csh
        "k_column_tracers": 3 * ntr + 7,
        # grad exner' (3), theta edges (2 + 2 perturbation), all rho, 3 background gradients,
        # gravity, 8 products written, 4 previous products read
        "k_pgrad": 3 + 4 + ncons + 3 + 1 + 8 + 4,
    }
    if not split:
        if name in fp64_only:
            return fp64_only[name] * 8.0
        f = _kernel_fields(ncons).get(name[2:])
        return 0.0 if f is None else 8.0 * (f[0] + f[1] + f_oro * (f[2] + f[3]))
    split_own = {
        # FP64: state old (rho_g, rho*theta, exner', theta', w), theta_bg, 5 new values written;
        # FP32: mirror old (rho_g, rho*theta, exner', w), mirror new at rk2 (3, half the launches),
        # exner_bg, damping, dz, d(exner_bg), 1/volume, 1/area_z, 3 tendencies, 5 mirror values written
        "ks_column_ver": 11 * 8.0 + 19.5 * 4.0,
        # FP64: rho old and new per tracer; FP32: mirror old, tendency and mirror new per tracer,
        # w old/new, rho_g, T, area_z, 1/volume, and one sediment-heating plane per condensate
        # written in the first of the two launches of a step
        "ks_column_tracers": 2 * ntr * 8.0 + (3 * ntr + 6 + 0.5 * max(ncons - 2, 0)) * 4.0,
        # the condensate planes read, their sum written
        "ks_csh_sum": (max(ncons - 2, 0) + 1) * 4.0,
        # FP64: exner', its vertical gradient, 1/dx, 1/dy, slopes, 2 weights, 3 background
        # gradients, gravity, 8 products written, 4 previous read; FP32: all rho (mirror),
        # 4 theta edges, pgcw
        "ks_pgrad": 24 * 8.0 + (ncons + 5) * 4.0,
        # FP64: exner' read, 1/dz read, gradient written
        "ks_gzp": 3 * 8.0,
    }
    if name in split_own:
        return split_own[name]
    base = name[3:]
    f = _kernel_fields(ncons).get(base)
    if f is None:
        return 0.0
    # the split stencils read the FP32 mirror of the state; the kinetic energy and the wind
    # update keep FP64 state arrays (the latter also writes the two mirror winds)
    if base in ("ke", "tend_wind"):
        extra = 2 if base == "tend_wind" else 0
        return 8.0 * (f[0] + f_oro * f[2]) + 4.0 * (f[1] + extra + f_oro * f[3])
    return 4.0 * (f[0] + f[1] + f_oro * (f[2] + f[3]))


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.lines: list[str] = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[3 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    lrank = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, lrank


def dist_init(ws):
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        return dist
    return None


def reduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def time_steps(L, g, steps: int, first_step: int):
    """Device time of `steps` consecutive pchevi calls, CUDA events on the library's stream."""
    import torch
    s = torch.cuda.ExternalStream(g.stream_handle())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g.synchronize()
    e0.record(s)
    for k in range(first_step, first_step + steps):
        g.pchevi(k % 2, (k + 1) % 2, k)
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3


def cpu_baseline(nml_overrides: dict, seconds: float = 12.0, max_steps: int = 8) -> dict:
    """The oracle (CPU FP64 restatement) on a sub-domain of the workload; steps/s scaled
    to the full domain by the ratio of cells."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import cases
    import lgame_gpu as L
    import oracle as O
    full = cases.namelist(WORKLOAD)
    n = cases.namelist(WORKLOAD, **nml_overrides)
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    o = O.Oracle(cfg, hm.grid)
    o.set_state(0, hm.state)
    o.set_state(1, hm.state)
    o.set_diag(hm.diag)
    o.pchevi(0, 1, 0)  # warm-up (first step includes the step-0 advection)
    t0 = time.perf_counter()
    k = 1
    while True:
        o.pchevi(k % 2, (k + 1) % 2, k)
        k += 1
        el = time.perf_counter() - t0
        if el > seconds or k > max_steps:
            break
    per_step = el / (k - 1)
    cells_s = n.nx * n.ny * n.n_layers
    cells_f = full.nx * full.ny * full.n_layers
    return {"value": 1.0 / (per_step * cells_f / cells_s), "unit": "steps/s", "cores": O.load().oracle_num_threads(),
            "kind": "port", "sample": f"{k - 1} oracle steps of the {n.nx}x{n.ny}x{n.n_layers} sub-domain of the same "
                                      f"workload ({per_step:.3f} s/step), scaled by cells x{cells_f / cells_s:.0f}",
            "sample_s_per_step": per_step}


def run_reference(args):
    ws, rank, _ = dist_info()
    dist = dist_init(ws)
    if rank != 0:
        barrier(dist)
        return 0
    sys.path.insert(0, str(ROOT / "oracle"))
    import cases
    import lgame_gpu as L
    import oracle as O
    full = cases.namelist(WORKLOAD)
    n = cases.namelist(WORKLOAD, **CPU_SAMPLE)
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    o = O.Oracle(cfg, hm.grid)
    o.set_state(0, hm.state)
    o.set_state(1, hm.state)
    o.set_diag(hm.diag)
    for k in range(args.warmup):
        o.pchevi(k % 2, (k + 1) % 2, k)
    t0 = time.perf_counter()
    for k in range(args.warmup, args.warmup + args.steps):
        o.pchevi(k % 2, (k + 1) % 2, k)
    el = time.perf_counter() - t0
    scale = (full.nx * full.ny * full.n_layers) / (n.nx * n.ny * n.n_layers)
    value = args.steps / (el * scale)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{WORKLOAD} moist baroclinic jet, rotated lat-lon, dx=2.5 km",
                       "sample": f"{n.nx}x{n.ny}x{n.n_layers} sub-domain per step, scaled by cells x{scale:.0f}",
                       "input_vs_l2": "inputs larger than L2 (CPU run)"},
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": O.load().oracle_num_threads(),
                             "kind": "port",
                             "sample": f"oracle pchevi on {n.nx}x{n.ny}x{n.n_layers}, {args.steps} steps"},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)
    barrier(dist)
    return 0


def profile_kernels(g, steps: int, first_step: int, ncons: int, cells: int, peak_gbs: float, split: bool,
                    f_oro: float):
    g.set_profiling(True)
    for k in range(first_step, first_step + steps):
        g.pchevi(k % 2, (k + 1) % 2, k)
    rep = g.profile_report()
    g.set_profiling(False)
    total = sum(v["ms"] for v in rep.values())
    rows = sorted(rep.items(), key=lambda kv: -kv[1]["ms"])
    top = rows[0]
    name, st = top[0], top[1]
    avg_ms = st["ms"] / st["launches"]
    bpc = kernel_bytes_per_cell(name, ncons, split, f_oro)
    alg = bpc * cells
    achieved = alg / (avg_ms / 1e3) / 1e9 if avg_ms > 0 else 0.0
    shares = {k: round(v["ms"] / total, 4) for k, v in rows}
    dram = MEASURED_DRAM_BYTES_PER_CELL.get(name) if split else None
    return {"kernel": name, "avg_launch_ms": avg_ms, "alg_bytes_per_launch": alg, "achieved_gbs": achieved,
            "frac": achieved / peak_gbs, "shares": shares, "rows": rows,
            "traffic": None if dram is None else dram * cells}


# FP64 thread instructions per cell of one launch of the split step's FP64-heavy kernels:
# sm__inst_executed_pipe_fp64.sum x 32 / cells from an ncu capture of the moist jet at
# 192x192x80 (ks_column_ver: 2,597,768 warp instructions, 2,949,120 cells).  The FP64 pipe
# issues 1.68 operations per clock per SM on this GPU (register-only probe; FMA and add alike).
FP64_INST_PER_CELL = {"ks_column_ver": 28.2}
FP64_OPS_PER_CLK_SM = 1.68


def fp64_pipe_roofline(kernel: str, avg_ms: float, cells: int, clocks) -> dict | None:
    """The FP64-pipe bound of an FP64-heavy split kernel: its FP64 instructions per launch over
    the pipe's rate at the SM clock measured during the run (152 SMs)."""
    per = FP64_INST_PER_CELL.get(kernel)
    mhz = (clocks or {}).get("sm_mhz")
    if per is None or not mhz or avg_ms <= 0:
        return None
    peak = FP64_OPS_PER_CLK_SM * 152 * mhz * 1e6
    achieved = per * cells / (avg_ms * 1e-3)
    return {"achieved_ops_per_s": achieved, "peak_ops_per_s": peak, "frac": achieved / peak,
            "fp64_inst_per_cell": per, "src": "ncu sm__inst_executed_pipe_fp64 at 192x192x80; 1.68 FP64 ops/clk/SM "
                                              "(probe) at the sampled SM clock"}


def size_overrides(args) -> dict:
    """Namelist overrides of a reduced-size run (profiling captures): nx = ny, and n_layers with
    the orography-following layers kept at the workload's fraction."""
    ov = {"nx": args.nx, "ny": args.ny} if args.nx else {}
    if args.nl:
        ov["n_layers"] = args.nl
        ov["n_oro_layers"] = max(1, min(args.nl - 1, round(args.nl * 60 / 80)))
    return ov


def run_ours(args):
    import torch
    import cases
    import lgame_gpu as L
    ws, rank, lrank = dist_info()
    dist = dist_init(ws)
    peaks = read_peaks()
    t_setup = time.perf_counter()
    n = cases.namelist(WORKLOAD, **size_overrides(args))
    hm = L.HostModel(n)
    t_setup = time.perf_counter() - t_setup
    cells = n.nx * n.ny * n.n_layers
    ncons = n.n_constituents
    f_oro = (n.n_oro_layers + 1) / n.n_layers
    results = {}
    precisions = [L.PRECISION_SPLIT, L.PRECISION_FP64, L.PRECISION_SPLIT_FP64_COLUMN]
    if args.fp64_only:
        precisions = [L.PRECISION_FP64]
    elif args.split_only:
        precisions = [L.PRECISION_SPLIT]
    clocks = None
    for prec in precisions:
        cfg = L.config_from_namelist(n)
        cfg.precision = prec
        cfg.device = lrank
        try:
            g = L.GpuModel(cfg, hm.grid)
        except L.LgameError as e:
            if e.code == L.ERR_UNSUPPORTED:
                continue
            raise
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(hm.diag)
        for k in range(args.warmup):
            g.pchevi(k % 2, (k + 1) % 2, k)
        g.synchronize()
        barrier(dist)
        sampler = ClockSampler(lrank) if clocks is None else None
        if sampler:
            sampler.__enter__()
        el = time_steps(L, g, args.steps, args.warmup)
        if sampler:
            sampler.__exit__()
            clocks = sampler.summary()
        barrier(dist)
        el = reduce_max(dist, el)
        nk = g.kernels_per_step()
        prof = profile_kernels(g, 2, args.warmup + args.steps, ncons, cells, peaks["hbm_gbs"],
                               prec != L.PRECISION_FP64, f_oro)
        st = g.get_state((args.warmup + args.steps + 2) % 2)
        finite = all(bool(np.isfinite(v).all()) for v in st.values())
        results[prec] = {"s_per_step": el / args.steps, "kernels_per_step": nk, "profile": prof, "finite": finite,
                         "device_gb": g.device_bytes() / 1e9, "model": g}
        if prec == precisions[0] or len(results) == 1:
            # end to end through the C ABI with pinned host buffers
            e2e = measure_e2e(L, g, hm, args)
            results[prec]["e2e"] = e2e
            if rank == 0 and ws == 1:
                results[prec]["output"] = measure_output(L, g, n, peaks)
        g.close()
        results[prec].pop("model")
        torch.cuda.synchronize()
    if not results:
        raise RuntimeError("no precision path available")
    head_prec = L.PRECISION_SPLIT if L.PRECISION_SPLIT in results else L.PRECISION_FP64
    head = results[head_prec]
    value = ws * 1.0 / head["s_per_step"]
    prof = head["profile"]
    step_b = step_bytes_per_cell(ncons, head_prec == L.PRECISION_SPLIT)
    fp64 = results.get(L.PRECISION_FP64)
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["s_per_step"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32/f64 split" if head_prec == L.PRECISION_SPLIT else "f64",
        "data": "synthetic (seeded moist baroclinic jet over seeded hills; no dataset)",
        "config": {"workload": f"{WORKLOAD}: moist, 7 constituents, rotated lat-lon, dx=2.5 km, theta_adv_order 3, "
                               f"dtime {n.dtime:.3f} s", "nx": n.nx, "ny": n.ny, "n_layers": n.n_layers,
                   "cells": cells, "input_vs_l2": "inputs larger than L2 (device working set "
                                                  f"{head['device_gb']:.1f} GB)",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU", "setup_s": round(t_setup, 1)},
        "column_updates_per_s": value * n.nx * n.ny,
        "roofline": {"bound": "hbm", "kernel": prof["kernel"], "achieved": prof["achieved_gbs"],
                     "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": prof["frac"], "traffic": prof["traffic"],
                     "traffic_src": "ncu dram__bytes_read.sum + dram__bytes_write.sum per cell (one-pass capture "
                                    "of the 256x256x80 jet), times the cells of this run",
                     "peak_src": peaks["src"], "avg_launch_ms": prof["avg_launch_ms"],
                     "alg_bytes_per_launch": prof["alg_bytes_per_launch"], "kernel_shares": prof["shares"],
                     "fp64_pipe": fp64_pipe_roofline(prof["kernel"], prof["avg_launch_ms"], cells, clocks)},
        "step_roofline": {"alg_bytes_per_cell": step_b, "alg_bytes_per_step": step_b * cells,
                          "achieved_gbs": step_b * cells / head["s_per_step"] / 1e9,
                          "peak_gbs": peaks["hbm_gbs"], "frac": step_b * cells / head["s_per_step"] / 1e9 / peaks["hbm_gbs"]},
        "gpu_launches": head["kernels_per_step"] * args.steps,
        "clocks": clocks,
        "finite": head["finite"],
    }
    if fp64 is not None:
        line["fp64"] = {"value": ws / fp64["s_per_step"], "ms_per_step": fp64["s_per_step"] * 1e3,
                        "kernels_per_step": fp64["kernels_per_step"], "top_kernel": fp64["profile"]["kernel"],
                        "kernel_shares": fp64["profile"]["shares"]}
        if head_prec != L.PRECISION_FP64:
            line["split_speedup_vs_fp64"] = fp64["s_per_step"] / head["s_per_step"]
    col64 = results.get(L.PRECISION_SPLIT_FP64_COLUMN)
    if col64 is not None:
        # the split step with the vertical acoustic solve wholly in FP64 (precision mode 2)
        line["split_fp64_column"] = {"value": ws / col64["s_per_step"], "ms_per_step": col64["s_per_step"] * 1e3,
                                     "column_ver_ms_per_launch": {k: v["ms"] / v["launches"]
                                                                  for k, v in col64["profile"]["rows"]}.get("ks_column_ver"),
                                     "speedup_vs_fp64": (fp64["s_per_step"] / col64["s_per_step"]) if fp64 else None}
    if "output" in head:
        line["output"] = head["output"]
    if "e2e" in head:
        line["e2e"] = head["e2e"]
    else:
        for r in results.values():
            if "e2e" in r:
                line["e2e"] = r["e2e"]
    hm = None  # the sub-benchmarks below set up their own host models
    if rank == 0 and ws == 1 and not args.no_boundaries:
        line["boundary_relaxation"] = boundary_bench(args, peaks)
    if rank == 0 and ws == 1 and not args.no_diffusion:
        line["diffusion"] = diffusion_bench(args, results)
        line["default_physics"] = diffusion_bench(args, results, surface=True)
    if rank == 0 and ws == 1 and not args.no_emulator:
        line["emulator"] = emulator_bench(peaks)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(CPU_SAMPLE)
    if rank == 0:
        print(json.dumps(line), flush=True)
    barrier(dist)
    return 0


DIFF_DEFAULT = dict(lmom_diff_h=True, lmom_diff_v=True, ltemp_diff_h=True, ltemp_diff_v=True, lmass_diff_h=True,
                    lmass_diff_v=True, diff_coeff_scheme_h="smag")
SFC_DEFAULT = dict(lprog_soil_temp=True, nsoillays=5, lsfc_sensible_heat_flux=True, lsfc_phase_trans=True, lpbl=True)


def diffusion_bench(args, results: dict, surface: bool = False) -> dict:
    """The workload with the reference's default &diff (mo_diff_nml.F90:38-53: momentum,
    temperature and mass diffusion on, horizontally and vertically, Smagorinsky horizontal
    coefficient, TKE vertical one) and, with `surface`, its default &surface as well
    (mo_surface_nml.F90:30-37: prognostic soil of five layers, sensible heat flux, surface
    phase-transition switch, PBL): the split and the FP64 step (CUDA events on the library's
    stream), their cost against the same steps without these, and the closure's (and surface
    kernels') share of the split step."""
    import cases
    import lgame_gpu as L
    n = cases.namelist(WORKLOAD, **DIFF_DEFAULT, **(SFC_DEFAULT if surface else {}), **size_overrides(args))
    hm = L.HostModel(n)
    out = {"config": "reference default &diff: all six switches on, smag/tke" +
           ("; reference default &surface: soil (5 layers), sensible heat flux, PBL" if surface else "")}
    runs = [(L.PRECISION_SPLIT, "split", args.steps), (L.PRECISION_FP64, "fp64", min(args.steps, 3))]
    if args.split_only or args.fp64_only:
        runs = [r for r in runs if (r[1] == "split") == args.split_only]
    for prec, name, steps in runs:
        cfg = L.config_from_namelist(n)
        cfg.precision = prec
        g = L.GpuModel(cfg, hm.grid)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(hm.diag)
        for k in range(3):
            g.pchevi(k % 2, (k + 1) % 2, k)
        el = time_steps(L, g, steps, 3) / steps
        e = {"value": 1.0 / el, "ms_per_step": el * 1e3, "kernels_per_step": g.kernels_per_step()}
        base = results.get(prec)
        if base is not None:
            e["ms_per_step_without"] = base["s_per_step"] * 1e3
            e["cost_of_diffusion"] = el / base["s_per_step"] - 1.0
        if prec == L.PRECISION_SPLIT:
            g.set_profiling(True)
            for k in range(3 + steps, 5 + steps):
                g.pchevi(k % 2, (k + 1) % 2, k)
            rep = g.profile_report()
            g.set_profiling(False)
            tot = sum(v["ms"] for v in rep.values())
            e["closure_kernel_shares"] = {k: round(v["ms"] / tot, 4) for k, v in rep.items()
                                          if k.startswith(("ks_diff", "ks_mom_diff", "ks_diss", "ks_sfc", "ks_pbl"))}
        st = g.get_state((3 + steps) % 2)
        e["finite"] = all(bool(np.isfinite(v).all()) for v in st.values())
        g.close()
        out[name] = e
    return out


def boundary_bench(args, peaks, n_swamp: int = 5, reps: int = 20) -> dict:
    """Lateral boundary relaxation (mo_boundaries.F90:19-97) on the workload made non-periodic,
    split precision, swamp layer n_swamp points wide (the reference's default), both boundary
    levels equal to the initial state: the step with the relaxation at its end, and
    lgame_gpu_update_boundaries alone (CUDA events on the library's stream; its two kernels,
    ks_bc_rim over the swamp layer and ks_bc_thermo over all scalar points).  Algorithmic
    bytes: at every scalar point rho_gas, rhotheta_v, theta_v_bg, the background rhotheta_v
    and exner_bg read and theta_v_pert, exner_pert written in FP64 and FP32 (64 B); in the
    swamp layer also both levels, the state and the relaxed FP64 value and FP32 mirror of
    every field (36 B each)."""
    import torch
    import cases
    import lgame_gpu as L
    n = cases.namelist(WORKLOAD, lperiodic=False, **size_overrides(args))
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    cfg.precision = L.PRECISION_SPLIT
    g = L.GpuModel(cfg, hm.grid)
    g.set_state(0, hm.state)
    g.set_state(1, hm.state)
    g.set_diag(hm.diag)
    lev = {f: hm.state[f] for f in L.BC_FIELDS}
    g.bc_setup(n_swamp, 10800, 0.0, None)
    g.set_bc(1, lev)
    g.set_bc(2, lev)
    del hm, lev
    for k in range(args.warmup):
        g.pchevi(k % 2, (k + 1) % 2, k)
    el = time_steps(L, g, args.steps, args.warmup)
    s = torch.cuda.ExternalStream(g.stream_handle())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g.synchronize()
    t_now = (args.warmup + args.steps) * n.dtime
    e0.record(s)
    for r in range(reps):
        g.update_boundaries(r % 2, t_now)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    st = g.get_state(0)
    finite = all(bool(np.isfinite(v).all()) for v in st.values())
    g.close()
    cells = n.nx * n.ny * n.n_layers
    rim = 1.0 - max(n.ny - 2 * n_swamp, 0) * max(n.nx - 2 * n_swamp, 0) / (n.ny * n.nx)
    per_cell = 64.0 + rim * 36.0 * (n.n_constituents + 4)
    gbs = per_cell * cells / (ms * 1e-3) / 1e9
    return {"kernel": "ks_bc_rim + ks_bc_thermo", "n_swamp": n_swamp, "ms_per_step_with_relaxation": el / args.steps * 1e3,
            "avg_launch_ms": ms, "alg_bytes_per_cell": per_cell, "swamp_fraction": rim,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": gbs / peaks["hbm_gbs"], "peak_src": peaks["src"]},
            "finite": finite}


def measure_output(L, g, n, peaks, reps: int = 5) -> dict:
    """The output fields of the time loop (lgame_gpu_output: linear_combine_two_states and
    write_output's variables as floats) for the two state slots.  Kernel: CUDA events on the
    library's stream around calls that fetch no field (the kernel and the crash flag);
    algorithmic bytes per cell: both states' rho (n_constituents), rhotheta_v, exner_pert,
    u, v, w in FP64, theta_v_bg, exner_bg, z_scalar, z_w in FP64, n_constituents + 5 float
    fields written.  End to end: every field copied into page-locked host arrays."""
    import torch
    ncons, cells = n.n_constituents, n.nx * n.ny * n.n_layers
    per_cell = 2 * 8.0 * (ncons + 5) + 4 * 8.0 + 4.0 * (ncons + 5)
    s = torch.cuda.ExternalStream(g.stream_handle())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g.output(0, 1, 0.5, 0.5, fields=[])
    e0.record(s)
    for _ in range(reps):
        g.output(0, 1, 0.5, 0.5, fields=[])
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    fp = []
    host = {}
    for f in L.OUTPUT_FIELDS:
        if f == "rel_humidity" and ncons == 1:
            continue
        shape = (n.ny, n.nx, n.n_layers, ncons) if f == "rho" else (n.ny, n.nx, n.n_layers)
        t = torch.empty(shape[::-1], dtype=torch.float32, pin_memory=True)
        fp.append(t)
        host[f] = t.numpy().T
    import ctypes as C
    ptrs = (C.POINTER(C.c_float) * len(L.OUTPUT_FIELDS))(
        *[host[f].ctypes.data_as(C.POINTER(C.c_float)) if f in host else C.POINTER(C.c_float)()
          for f in L.OUTPUT_FIELDS])
    crashed = C.c_int()
    t0 = time.perf_counter()
    for _ in range(reps):
        L.check(g.lib.lgame_gpu_output(g.h, 0, 1, 0.5, 0.5, ptrs, len(L.OUTPUT_FIELDS), C.byref(crashed)),
                "lgame_gpu_output")
    e2e_s = (time.perf_counter() - t0) / reps
    d2h = sum(v.nbytes for v in host.values())
    gbs = per_cell * cells / (ms * 1e-3) / 1e9
    return {"kernel": "k_output", "avg_launch_ms": ms, "alg_bytes_per_cell": per_cell,
            "roofline": {"bound": "fp64", "achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": gbs / peaks["hbm_gbs"], "peak_src": peaks["src"],
                         "note": "FP64-pipe bound (the reference's FP64 combination, divisions, exp and log "
                                 "per point; ncu: FP64 pipe 86 % busy); frac is of HBM bandwidth"},
            "e2e_ms": e2e_s * 1e3, "d2h_bytes": d2h, "e2e_note": "all fields into page-locked host arrays",
            "crashed": bool(crashed.value)}


def measure_e2e(L, g, hm, args) -> dict:
    """Steps through lgame_gpu_pchevi_host: every step copies the state in from pinned host
    memory and the new state back."""
    import torch

    def pinned_like(a: np.ndarray) -> np.ndarray:
        t = torch.empty(a.shape[::-1], dtype=torch.float64, pin_memory=True)
        v = t.numpy().T  # Fortran-ordered view of the pinned buffer
        v[...] = a
        return v, t

    keep = []
    old, new = {}, {}
    # the soil temperature is part of the state only with the prognostic soil or the sensible
    # heat flux on
    soil = g.cfg.lprog_soil_temp or g.cfg.lsfc_sensible_heat_flux
    for f in (L.STATE_FIELDS if soil else L.ATMOS_FIELDS):
        a, t = pinned_like(hm.state[f])
        b, t2 = pinned_like(np.zeros_like(hm.state[f], order="F"))
        keep += [t, t2]
        old[f], new[f] = a, b
    h2d = sum(v.nbytes for v in old.values())
    d2h = sum(v.nbytes for v in new.values())
    k_e2e = max(2, min(args.steps, 5))
    g.pchevi_host(old, new, 1)  # warm-up
    g.synchronize()
    t0 = time.perf_counter()
    for k in range(k_e2e):
        g.pchevi_host(old, new, k + 1)
    el = time.perf_counter() - t0
    link = link_rates()
    link["numa"] = {"state_in": host_numa_pages(keep[0].data_ptr()), "state_out": host_numa_pages(keep[1].data_ptr()),
                    "gpu_pci_node": gpu_numa_node(), "process_cpu_nodes": cpu_numa_nodes()}
    floor_ms = (h2d / link["h2d_gbs"] + d2h / link["d2h_gbs"]) / 1e6
    return {"value": k_e2e / el, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": k_e2e, "note": "lgame_gpu_pchevi_host: pinned host state in, new state out, every step",
            "ms_per_step": el / k_e2e * 1e3, "link": link, "transfer_floor_ms": floor_ms}


def host_numa_pages(addr: int):
    """{NUMA node: resident pages} of the mapping that holds host address `addr`, from
    /proc/self/numa_maps (None where the kernel does not provide it)."""
    try:
        maps = open("/proc/self/maps").read().splitlines()
        start = None
        for ln in maps:
            a, b = (int(x, 16) for x in ln.split()[0].split("-"))
            if a <= addr < b:
                start = a
                break
        if start is None:
            return None
        for ln in open("/proc/self/numa_maps").read().splitlines():
            f = ln.split()
            if int(f[0], 16) == start:
                return {k[1:]: int(v) for k, v in (x.split("=") for x in f[1:] if x[:1] == "N" and "=" in x)}
    except (OSError, ValueError):
        return None
    return None


def gpu_numa_node():
    """NUMA node the GPU's PCI function reports (sysfs), or None."""
    import subprocess
    try:
        bus = subprocess.run(["nvidia-smi", "--query-gpu=pci.bus_id", "--format=csv,noheader", "-i",
                              str(__import__("torch").cuda.current_device())],
                             capture_output=True, text=True, timeout=20).stdout.strip()
        dom, rest = bus.split(":", 1)
        path = f"/sys/bus/pci/devices/{int(dom, 16):04x}:{rest.lower()}/numa_node"
        return int(open(path).read().strip())
    except (OSError, ValueError, RuntimeError, subprocess.SubprocessError):
        return None


def cpu_numa_nodes():
    """NUMA nodes whose CPUs this process may run on."""
    import glob
    cpus = os.sched_getaffinity(0)
    nodes = []
    for d in sorted(glob.glob("/sys/devices/system/node/node[0-9]*")):
        try:
            lst = open(d + "/cpulist").read().strip()
        except OSError:
            continue
        ids = set()
        for part in filter(None, lst.split(",")):
            a, _, b = part.partition("-")
            ids.update(range(int(a), int(b or a) + 1))
        if ids & cpus:
            nodes.append(int(d.rsplit("node", 1)[1]))
    return nodes


def link_rates(nbytes: int = 1 << 31, reps: int = 3) -> dict:
    """Copy-engine rates of the CPU-GPU link between page-locked host memory and the device
    (CUDA events around torch copies of nbytes, each direction alone).  In + out at these
    rates is the floor of lgame_gpu_pchevi_host's state transfer, which moves one direction at
    a time; part of the copy-out runs while the step still computes."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            dst.copy_(src, non_blocking=True)
        e1.record()
        e1.synchronize()
        out[name] = reps * nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9
    del h, d
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-only", action="store_true")
    ap.add_argument("--split-only", action="store_true", help="measure the split step alone (profiling runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-emulator", action="store_true")
    ap.add_argument("--no-boundaries", action="store_true", help="skip the non-periodic boundary-relaxation run")
    ap.add_argument("--no-diffusion", action="store_true", help="skip the run with the default diffusion closure")
    ap.add_argument("--nx", type=int, default=0, help="override nx=ny (smaller runs for testing)")
    ap.add_argument("--ny", type=int, default=0)
    ap.add_argument("--nl", type=int, default=0, help="override n_layers (profiling captures of column kernels)")
    args = ap.parse_args()
    if args.nx and not args.ny:
        args.ny = args.nx
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    import __graft_entry__
    __graft_entry__.build()
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
