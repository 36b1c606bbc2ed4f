"""Generates the golden vectors of tests/golden/*.npz: the oracle's state after a few
steps of small cases (inputs from the library's host set-up).  Regenerate only when the
oracle is deliberately changed:  python tests/golden/make_golden.py"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path[:0] = [str(HERE.parent), str(HERE.parent.parent / "l-game_gb300"), str(HERE.parent.parent / "oracle")]

import test_boundaries  # noqa: E402
import test_oracle  # noqa: E402

CASES = {"schaer_odd": 6, "mountain_rest": 6, "jet": 3}


def boundary_output_case(nsteps: int = 5):
    """The non-periodic hills case with the lateral relaxation (swamp layer 3, dtime_bc 15 s,
    seeded boundary levels; two level swaps in five steps), then the output fields of
    0.3*slot 0 + 0.7*slot 1."""
    hm, cfg, o = test_boundaries._oracle("hills_nonperiodic")
    for k in range(nsteps):
        o.pchevi(k % 2, (k + 1) % 2, k)
    st = o.get_state(nsteps % 2)
    out, crashed = o.output(0, 1, 0.3, 0.7)
    io, inew, t_latest = o.bc_state()
    o.close()
    return st, out, np.array([io, inew, t_latest])


if __name__ == "__main__":
    for key, nsteps in CASES.items():
        hm, o, b0, b1, st = test_oracle._run(key, nsteps)
        np.savez_compressed(HERE / f"{key}.npz", nsteps=nsteps, budgets=b1, **st)
        print(key, {k: v.shape for k, v in st.items()})
    st, out, bc = boundary_output_case()
    np.savez_compressed(HERE / "hills_nonperiodic_bc.npz", bc_state=bc, **st,
                        **{"out_" + k: v for k, v in out.items()})
    print("hills_nonperiodic_bc", bc)
