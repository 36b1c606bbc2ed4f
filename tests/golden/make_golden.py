"""Generates the golden vectors of tests/golden/*.npz: the oracle's state after a few
steps of small cases (inputs from the library's host set-up).  Regenerate only when the
oracle is deliberately changed:  python tests/golden/make_golden.py"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path[:0] = [str(HERE.parent), str(HERE.parent.parent / "l-game_gb300"), str(HERE.parent.parent / "oracle")]

import test_oracle  # noqa: E402

CASES = {"schaer_odd": 6, "mountain_rest": 6, "jet": 3}

if __name__ == "__main__":
    for key, nsteps in CASES.items():
        hm, o, b0, b1, st = test_oracle._run(key, nsteps)
        np.savez_compressed(HERE / f"{key}.npz", nsteps=nsteps, budgets=b1, **st)
        print(key, {k: v.shape for k, v in st.items()})
