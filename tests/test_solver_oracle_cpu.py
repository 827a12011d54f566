"""The CPU restatement of simple_solver + cgstep (oracle/solver_oracle.py)
against the reference's own solver: the golden fixture written by the
reference (tests/golden/make_solver_golden.py) and, where the reference tree
is present, a fresh run of it.  After as many iterations as unknowns the
model is the FP64 least-squares solution."""
from pathlib import Path

import numpy as np

from oracle import solver_oracle as SO

GOLDEN = Path(__file__).parent / "golden" / "cgstep_dense.npz"


def test_oracle_cgstep_matches_reference_golden():
    g = np.load(GOLDEN)
    ms, rrs, alphas, betas = SO.cg_solve(g["A"], g["d"], len(g["rr"]))
    assert len(rrs) == len(g["rr"])
    # same arithmetic in the same order: identical bits
    assert np.array_equal(rrs, g["rr"]), np.abs(rrs / g["rr"] - 1).max()
    assert np.array_equal(ms, g["models"])
    # monotone down to the float noise of the converged residual
    assert np.all(rrs[1:] <= rrs[:-1] * (1 + 1e-6))
    assert betas[0] == 0.0 and np.all(np.isfinite(alphas))


def test_oracle_cgstep_converges_to_lstsq():
    g = np.load(GOLDEN)
    ms, _, _, _ = SO.cg_solve(g["A"], g["d"], len(g["rr"]))
    want = SO.lstsq(g["A"], g["d"])
    assert np.linalg.norm(ms[-1] - want) / np.linalg.norm(want) <= 1e-5


def test_golden_is_the_reference(refhost):
    """the fixture equals a fresh run of the reference compiled here"""
    import os
    g = np.load(GOLDEN)
    saved = os.dup(2)
    with open(os.devnull, "w") as null:
        os.dup2(null.fileno(), 2)
        try:
            for k in (1, 2, 7, len(g["rr"])):
                m, rr, rc = refhost.cg_solve(g["A"], g["d"], k)
                assert rc == 0 and rr == g["rr"][k - 1] and np.array_equal(m, g["models"][k - 1])
        finally:
            os.dup2(saved, 2)
            os.close(saved)
