"""Split-precision error study: the FP32/FP64 split step against the FP64 step.

    python l-game_gb300/error_study.py [--config jet_1024x1024x80] [--nx 256] [--hours 1,6]
                                       [--every H] [--set key=value ...]

Runs both precision paths from the same initial state for the requested simulated
times and prints, per prognostic field, the max-norm and RMS relative error
    max|split - fp64| / max|fp64|,   rms(split - fp64) / rms(fp64)
as one JSON line per output time, together with the absolute max/RMS of each wind component
in both runs (for a fluid at rest those are the spurious winds) and whether each run is
still finite.  --set overrides namelist items of the configuration (any group).

--twin EPS replaces the split run by a second FP64 run whose initial u wind is multiplied
by (1 + EPS*r), r uniform in [-1, 1] (seeded): the growth of that difference is the
sensitivity of the flow itself to a perturbation of relative size EPS, against which the
split-precision error (FP32 rounding, relative size ~6e-8 per operation) is to be read.

The FP64 GPU step equals the oracle (the CPU FP64 restatement of the reference) to
<= 1e-12 per field per step (tests/test_gpu_parity.py), so it stands in for the oracle
at hour scale, where the oracle itself would need hours of CPU time per simulated hour.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent / "tests"))

import lgame_gpu as L  # noqa: E402


def field_errors(a: dict, b: dict) -> dict:
    out = {}
    for f in L.STATE_FIELDS:
        x, y = a[f], b[f]
        if f == "rho":
            for c in range(x.shape[3]):
                out[f"rho[{c + 1}]"] = _err(x[..., c], y[..., c])
        else:
            out[f] = _err(x, y)
    return out


def _err(x, y):
    d = x - y
    my = float(np.abs(y).max())
    ry = float(np.sqrt(np.mean(y * y)))
    return {"max": float(np.abs(d).max()) / my if my > 0 else float(np.abs(d).max()),
            "rms": float(np.sqrt(np.mean(d * d))) / ry if ry > 0 else float(np.sqrt(np.mean(d * d)))}


def _value(text: str):
    for conv in (int, float):
        try:
            return conv(text)
        except ValueError:
            pass
    return {"true": True, "false": False}.get(text.lower(), text)


def winds(s: dict) -> dict:
    return {f: {"max": float(np.abs(s[f]).max()), "rms": float(np.sqrt(np.mean(s[f] * s[f])))}
            for f in ("wind_u", "wind_v", "wind_w")}


def main():
    import cases
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="jet_1024x1024x80")
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--hours", default="1,6")
    ap.add_argument("--every", type=float, default=0.0, help="extra output interval in hours (0: none)")
    ap.add_argument("--set", action="append", default=[], metavar="KEY=VALUE")
    ap.add_argument("--twin", type=float, default=0.0, metavar="EPS",
                    help="compare FP64 with FP64 from a u wind perturbed by relative EPS")
    ap.add_argument("--variants", default="1",
                    help="split precision modes to compare with FP64: 1 (FP32 column-solve coefficients), "
                         "2 (FP64 vertical acoustic solve), or 1,2")
    args = ap.parse_args()
    over = {"nx": args.nx, "ny": args.nx} if args.nx else {}
    for kv in args.set:
        k, v = kv.split("=", 1)
        over[k] = _value(v)
    n = cases.namelist(args.config, **over)
    hm = L.HostModel(n)
    models = []
    others = [L.PRECISION_FP64] if args.twin else [int(v) for v in args.variants.split(",")]
    names = {L.PRECISION_SPLIT: "split", L.PRECISION_SPLIT_FP64_COLUMN: "split_fp64_column"}
    for idx, prec in enumerate([L.PRECISION_FP64] + others):
        cfg = L.config_from_namelist(n)
        cfg.precision = prec
        g = L.GpuModel(cfg, hm.grid)
        state = hm.state
        if idx >= 1 and args.twin:
            state = dict(hm.state)
            r = np.random.default_rng(12345).uniform(-1.0, 1.0, size=state["wind_u"].shape)
            state["wind_u"] = np.asfortranarray(state["wind_u"] * (1.0 + args.twin * r))
        g.set_state(0, state)
        g.set_state(1, state)
        g.set_diag(hm.diag)
        models.append(g)
    hours = sorted(float(h) for h in args.hours.split(","))
    marks = set(int(round(h * 3600.0 / n.dtime)) for h in hours)
    if args.every > 0:
        k = int(round(args.every * 3600.0 / n.dtime))
        marks |= set(range(k, max(marks) + 1, k))
    last = max(marks)
    t0 = time.time()
    for step in range(last):
        for g in models:
            g.pchevi(step % 2, (step + 1) % 2, step)
        if step + 1 in marks:
            s64 = models[0].get_state((step + 1) % 2)
            stop = False
            for prec, m in zip(others, models[1:]):
                ssp = m.get_state((step + 1) % 2)
                fin = {k: all(bool(np.isfinite(v).all()) for v in s.values()) for k, s in (("fp64", s64), ("split", ssp))}
                line = {"config": args.config, "overrides": {k: v for k, v in over.items() if k not in ("nx", "ny")},
                        "compare": f"fp64 twin eps={args.twin:g}" if args.twin else f"{names[prec]} vs fp64",
                        "nx": n.nx, "ny": n.ny, "n_layers": n.n_layers, "dtime": n.dtime,
                        "steps": step + 1, "hours": (step + 1) * n.dtime / 3600.0, "finite": fin,
                        "errors": field_errors(ssp, s64), "winds_fp64": winds(s64), "winds_split": winds(ssp),
                        "wall_s": round(time.time() - t0, 1)}
                line["worst_max"] = max(v["max"] for v in line["errors"].values())
                print(json.dumps(line), flush=True)
                stop = stop or not all(fin.values())
            if stop:
                break


if __name__ == "__main__":
    main()
