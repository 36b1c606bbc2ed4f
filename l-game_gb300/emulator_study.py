"""Radiation emulator study: training data from the model's own runs, GPU training, accuracy
against the stand-in teacher, inference and coupled-run timings.

    python l-game_gb300/emulator_study.py [--nx 512] [--snapshots 8] [--epochs 20] [--batch 8192]
                                          [--couple-hours 1]

1. Runs the moist jet workload (configs/jet_1024x1024x80.nml at nx = ny = --nx, split
   precision) and takes the emulator features of every column every 15 simulated minutes,
   with surface albedo drawn from U[0.05, 0.8] and cos(zenith) from U[0, 1] per column
   (seeded), and heating-rate targets from the teacher (lgame_rad_teacher, CPU).
2. Trains the MLP (322 -> 512 x 3 -> 160) on 90 % of the columns with Adam on the GPU and
   reports per epoch the loss, the time and the tensor-core GEMM rate; then the RMS error
   (K/day) on the held-out 10 % against the teacher, and that of the best state-independent
   predictor (the mean training profile) for comparison.
3. Times the inference of every column of a snapshot (features, MLP and radiation tendency
   on the GPU) against the teacher on the host cores for the same columns.
4. Runs two coupled copies of the model for --couple-hours with a radiation update every
   15 minutes: one with the emulator (10 % of the columns checked against the teacher,
   fallback above 0.3 K/day), one with the teacher for every column; reports the wall time
   of the radiation updates and the temperature difference between the two runs.
One JSON line per section.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent / "tests"))

import lgame_gpu as L  # noqa: E402
from lgame_gpu import emulator as E  # noqa: E402

T0 = 1576843200.0 + 9 * 3600.0  # a time of day with sun over part of the domain


def model(n, prec=L.PRECISION_SPLIT):
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    cfg.precision = prec
    g = L.GpuModel(cfg, hm.grid)
    g.set_state(0, hm.state)
    g.set_state(1, hm.state)
    g.set_diag(hm.diag)
    E.rad_set_surface(g, hm.surface["sfc_albedo"], hm.surface["lat_geo_scalar"], hm.surface["lon_geo_scalar"])
    return hm, g


def main():
    import cases
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--snapshots", type=int, default=8)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--couple-hours", type=float, default=1.0)
    args = ap.parse_args()
    n = cases.namelist("jet_1024x1024x80", nx=args.nx, ny=args.nx)
    nl = n.n_layers
    steps_15 = int(round(900.0 / n.dtime))

    # 1. data from the model's own run
    hm, g = model(n)
    rng = np.random.default_rng(2024)
    xs, step = [], 0
    t_run = time.time()
    for k in range(args.snapshots):
        for _ in range(steps_15):
            g.pchevi(step % 2, (step + 1) % 2, step)
            step += 1
        x = E.rad_features(g, step % 2, T0 + step * n.dtime)
        x[:, -2] = rng.uniform(0.05, 0.8, x.shape[0])
        x[:, -1] = rng.uniform(0.0, 1.0, x.shape[0])
        xs.append(x)
    t_run = time.time() - t_run
    x = np.concatenate(xs)
    t_teach = time.time()
    y = E.teacher(x, nl)
    t_teach = time.time() - t_teach
    perm = rng.permutation(x.shape[0])
    nva = x.shape[0] // 10
    va, tr = perm[:nva], perm[nva:]
    ntr = (tr.size // args.batch) * args.batch
    tr = tr[:ntr]
    print(json.dumps({"section": "data", "columns": int(x.shape[0]), "train": int(ntr), "validation": int(nva),
                      "features": int(x.shape[1]), "outputs": int(y.shape[1]), "model_steps": step,
                      "model_run_s": round(t_run, 1), "teacher_s": round(t_teach, 2),
                      "teacher_cores": os.cpu_count()}), flush=True)

    # 2. training
    emu = E.Emulator(nlev=nl, hidden=512, batch_max=args.batch, seed=11)
    emu.set_normalization(*E.normalization_from(x[tr], y[tr]))
    emu.set_dataset(x[tr], y[tr])
    emu.stats()
    hist = []
    for ep in range(args.epochs):
        lr = args.lr if ep < int(0.7 * args.epochs) else args.lr * 0.2
        t = time.time()
        loss = emu.train_epoch(args.batch, lr, ep + 1)
        dt = time.time() - t
        nlaunch, flop = emu.stats()
        hist.append({"epoch": ep + 1, "loss": loss, "s": round(dt, 3), "gemm_tflops": flop / dt / 1e12,
                     "columns_per_s": ntr / dt})
    yp = emu.infer(x[va])
    err = yp - y[va]
    rms = lambda a: float(np.sqrt(np.mean(a * a)))
    base = y[tr].mean(0) - y[va]
    print(json.dumps({"section": "training", "epochs": args.epochs, "batch": args.batch,
                      "first": hist[0], "last": hist[-1],
                      "val_rms_k_per_day": {"all": rms(err), "sw": rms(err[:, :nl]), "lw": rms(err[:, nl:])},
                      "no_network_rms_k_per_day": {"all": rms(base), "sw": rms(base[:, :nl]), "lw": rms(base[:, nl:])},
                      "val_max_abs_k_per_day": float(np.abs(err).max())}), flush=True)

    # 3. inference of one snapshot: GPU (features + MLP + tendency) vs teacher (CPU)
    slot = step % 2
    emu.stats()
    t = time.time()
    rep = E.rad_update(g, emu, slot, T0 + step * n.dtime, 0, 1e30)
    t_gpu = time.time() - t
    nlaunch, flop = emu.stats()
    xf = E.rad_features(g, slot, T0 + step * n.dtime)
    t = time.time()
    E.teacher(xf, nl)
    t_cpu = time.time() - t
    ncol = xf.shape[0]
    print(json.dumps({"section": "inference", "columns": ncol, "gpu_update_s": round(t_gpu, 4),
                      "gpu_columns_per_s": ncol / t_gpu, "gemm_tflop": flop / 1e12, "gemm_launches": nlaunch,
                      "teacher_cpu_s": round(t_cpu, 3), "teacher_columns_per_s": ncol / t_cpu,
                      "speedup": t_cpu / t_gpu}), flush=True)

    # 4. coupled runs: emulator (10 % sampled, fallback 0.3 K/day) vs teacher every call
    nsteps = int(round(args.couple_hours * 3600.0 / n.dtime))
    runs = {}
    for kind in ("emulator", "teacher"):
        hm2, g2 = model(n)
        t_rad, fallbacks, rmss = 0.0, 0, []
        t_all = time.time()
        for s in range(nsteps):
            if s % steps_15 == 0:
                g2.synchronize()  # the queued model steps are not radiation time
                t = time.time()
                tt = T0 + s * n.dtime
                if kind == "emulator":
                    r = E.rad_update(g2, emu, s % 2, tt, 10, 0.3)
                    fallbacks += int(r["fallback"])
                    rmss.append(r["rms_k_per_day"])
                else:
                    xf = E.rad_features(g2, s % 2, tt)
                    E.rad_apply_heating(g2, s % 2, E.teacher(xf, nl))
                g2.synchronize()
                t_rad += time.time() - t
            g2.pchevi(s % 2, (s + 1) % 2, s)
        g2.synchronize()
        runs[kind] = {"model": g2, "host": hm2, "rad_s": t_rad, "total_s": time.time() - t_all,
                      "fallbacks": fallbacks, "sample_rms": rmss}
    sa = runs["emulator"]["model"].get_state(nsteps % 2)
    sb = runs["teacher"]["model"].get_state(nsteps % 2)
    hmx = runs["teacher"]["host"]

    def temp(s):
        tb, eb = hmx.grid["theta_v_bg"], hmx.grid["exner_bg"]
        t = (tb + s["theta_v_pert"]) * (eb + s["exner_pert"])
        rv, rd = s["rho"][..., -1], s["rho"][..., -2]
        return t / (1.0 + rv / rd * (0.028965653 / 0.018012 - 1.0))  # M_d / M_v

    dT = temp(sa) - temp(sb)
    print(json.dumps({"section": "coupled", "hours": args.couple_hours, "steps": nsteps,
                      "radiation_calls": (nsteps + steps_15 - 1) // steps_15,
                      "emulator": {k: runs["emulator"][k] for k in ("rad_s", "total_s", "fallbacks", "sample_rms")},
                      "teacher": {k: runs["teacher"][k] for k in ("rad_s", "total_s")},
                      "radiation_speedup": runs["teacher"]["rad_s"] / max(runs["emulator"]["rad_s"], 1e-9),
                      "temperature_diff_k": {"max": float(np.abs(dT).max()), "rms": float(np.sqrt(np.mean(dT * dT)))}}),
          flush=True)


if __name__ == "__main__":
    main()
