"""Generate the golden fixture of the solver tests from the reference itself.

The reference's simple_solver + cgstep (Born/lin_solver.cpp, Born/cgstep.cpp,
compiled from their sources into oracle/_ref by oracle/build_oracle.py) solve
a seeded dense least-squares problem A m = d (the harness's dense operator)
for 1, 2, ..., K iterations from m = 0; the model and the residual energy
rr.rr after each are stored in cgstep_dense.npz next to this script.  Needs
the reference tree, so it runs in the build container, not on the GPU machine:
python tests/golden/make_solver_golden.py
"""
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.bindings import RefHost  # noqa: E402

NR, NC, K = 48, 24, 24


def problem():
    rng = np.random.default_rng(20261207)
    A = (rng.standard_normal((NR, NC)) / np.sqrt(NR) + 0.5 * np.eye(NR, NC)).astype(np.float32)
    d = rng.standard_normal(NR).astype(np.float32)
    return A, d


def main():
    A, d = problem()
    host = RefHost()
    ms, rrs = [], []
    # the reference's solver writes progress lines on stderr: silence them
    saved = os.dup(2)
    with open(os.devnull, "w") as null:
        os.dup2(null.fileno(), 2)
        try:
            for k in range(1, K + 1):
                m, rr, rc = host.cg_solve(A, d, k)
                if rc != 0:
                    raise RuntimeError(f"reference solve({k}) stopped early")
                ms.append(m)
                rrs.append(rr)
        finally:
            os.dup2(saved, 2)
            os.close(saved)
    np.savez_compressed(Path(__file__).parent / "cgstep_dense.npz", A=A, d=d, models=np.array(ms),
                        rr=np.array(rrs))
    print("cgstep_dense", A.shape, rrs[0], rrs[-1])


if __name__ == "__main__":
    main()
