"""The solver layer on the GPU (tests/cpp/solver_driver.cpp over device
vectors) against the reference and against FP64 least squares.

* simple_solver + cgstep (Born/lin_solver.cpp:7-17, :115-143;
  Born/cgstep.cpp:14-58): the model after each of 24 iterations and the
  residual energy rr.rr against the reference's own solver (golden fixture
  tests/golden/cgstep_dense.npz, written by the reference compiled from its
  sources).  The device sums its FP64 dot products in another order than the
  reference's index-order loop, so agreement is to round-off: rr.rr relative
  1e-9, models relative L2 1e-6.  After as many iterations as unknowns the
  model is the FP64 least-squares solution (relative L2 1e-5).
* prec_solver ([L P; eps I], model P x, Born/lin_solver.cpp:21-38) and
  reg_solver ([L; eps R], :39-53, with the scaled identity i_op and with a
  dense R) against the FP64 solutions of their normal equations, after 40
  iterations: the objective |L m - d|^2 + |eps R m|^2 within 1e-7 of its
  minimum (relative), the model within 1e-3 relative L2.  Float vectors set
  the floor: the recursively updated residual reaches the minimum to ~1e-8
  while the model stops 1e-4 to 1e-7 from the FP64 solution, depending on
  rounding (measured 1.3e-4 for the identity regulariser).
  The reference's own prec_solver and reg_solver cannot pin these: compiled
  here and run on the same dense problem they end in a segmentation fault.
* row_op (B A) and col_op ([A; C], Born/combo_oper.cpp) forward, adjoint and
  dot-product test against numpy (relative 1e-6).
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import solver_oracle as SO

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden" / "cgstep_dense.npz"


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def run(tmp_path_factory):
    from sep_code_gb300 import LIB_PATH
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    tmp = tmp_path_factory.mktemp("solvers")
    exe = tmp / "solver_driver"
    subprocess.run([cxx, "-std=c++17", "-O1", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "solver_driver.cpp"), str(LIB_PATH),
                    f"-Wl,-rpath,{Path(LIB_PATH).parent}", "-o", str(exe)], check=True)
    g = np.load(GOLDEN)
    A, d = g["A"], g["d"]
    nr, nc = A.shape
    rng = np.random.default_rng(31)
    nq, nb, nc2 = 20, 30, 16
    inp = {
        "A": A, "d": d,
        "P": np.diag(rng.uniform(0.5, 2.0, nc)) + 0.05 * rng.standard_normal((nc, nc)),
        "R": np.eye(nq, nc, 1) - np.eye(nq, nc),   # first differences
        "B": rng.standard_normal((nb, nr)) / np.sqrt(nr), "C": rng.standard_normal((nc2, nc)),
        "x": rng.standard_normal(nc), "yb": rng.standard_normal(nb), "yr": rng.standard_normal(nr),
        "yc": rng.standard_normal(nc2),
    }
    K, K2, eps = len(g["rr"]), 40, 0.3
    inp["dims"] = np.array([nr, nc, nq, nb, nc2, K, K2, eps])
    inp = {k: np.ascontiguousarray(v, np.float32) for k, v in inp.items()}
    for k, v in inp.items():
        v.tofile(tmp / f"{k}.bin")
    r = subprocess.run([str(exe), str(tmp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr

    def out(name, dtype=np.float32):
        return np.fromfile(tmp / f"{name}.bin", dtype)

    return inp, g, out, (K, eps)


def test_cgstep_matches_reference(run):
    inp, g, out, (K, _) = run
    models = out("simple_models").reshape(K, -1)
    resid = out("simple_resid", np.float64)
    assert len(resid) == K
    rr_rel = np.abs(resid / g["rr"] - 1)
    m_rel = [_rel(models[k], g["models"][k]) for k in range(K)]
    print(f"CGSTEP max rr.rr relative difference {rr_rel.max():.2e}, max model relative L2 "
          f"{max(m_rel):.2e}, bit-identical models {sum(np.array_equal(models[k], g['models'][k]) for k in range(K))}/{K}")
    assert rr_rel.max() <= 1e-9
    assert max(m_rel) <= 1e-6
    assert _rel(models[-1], SO.lstsq(inp["A"], inp["d"])) <= 1e-5


def _objective(A, m, d, R=None, eps=0.0, x=None):
    A = np.asarray(A, np.float64)
    m = np.asarray(m, np.float64)
    r = A @ m - np.asarray(d, np.float64)
    reg = eps * (np.asarray(R, np.float64) @ (m if x is None else x))
    return float(r @ r + reg @ reg)


def test_prec_solver_lstsq(run):
    inp, _, out, (_, eps) = run
    e = float(np.float32(eps))
    want = SO.prec_lstsq(inp["A"], inp["P"], e, inp["d"])
    got = out("prec_model")
    nc = inp["A"].shape[1]
    P = inp["P"].astype(np.float64)
    f_got = _objective(inp["A"], got, inp["d"], np.eye(nc), e, x=np.linalg.solve(P, got))
    f_min = _objective(inp["A"], want, inp["d"], np.eye(nc), e, x=np.linalg.solve(P, want))
    assert f_got - f_min <= 1e-7 * f_min
    assert _rel(got, want) <= 1e-3


def test_reg_solver_identity_lstsq(run):
    inp, _, out, (_, eps) = run
    e = float(np.float32(eps))
    nc = inp["A"].shape[1]
    want = SO.reg_lstsq(inp["A"], np.eye(nc), e, inp["d"])
    got = out("reg_i_model")
    for name in ("prec", "reg_i", "reg_r"):
        r = out(f"{name}_resid", np.float64)
        print(f"SOLVER {name}: {len(r)} iterations, rr.rr {r[0]:.6e} -> {r[-1]:.10e}")
    f_got = _objective(inp["A"], got, inp["d"], np.eye(nc), e)
    f_min = _objective(inp["A"], want, inp["d"], np.eye(nc), e)
    print(f"SOLVER reg_i objective above minimum {(f_got - f_min) / f_min:.2e}, model {_rel(got, want):.2e}")
    assert f_got - f_min <= 1e-7 * f_min
    assert _rel(got, want) <= 1e-3


def test_reg_solver_dense_lstsq(run):
    inp, _, out, (_, eps) = run
    e = float(np.float32(eps))
    want = SO.reg_lstsq(inp["A"], inp["R"], e, inp["d"])
    got = out("reg_r_model")
    f_got = _objective(inp["A"], got, inp["d"], inp["R"], e)
    f_min = _objective(inp["A"], want, inp["d"], inp["R"], e)
    assert f_got - f_min <= 1e-7 * f_min
    assert _rel(got, want) <= 1e-3


def test_row_col_ops(run):
    inp, _, out, _ = run
    A, B, C = (inp[k].astype(np.float64) for k in ("A", "B", "C"))
    x = inp["x"].astype(np.float64)
    assert _rel(out("row_fwd"), B @ (A @ x)) <= 1e-6
    assert _rel(out("row_adj"), A.T @ (B.T @ inp["yb"].astype(np.float64))) <= 1e-6
    assert _rel(out("col_fwd"), np.concatenate([A @ x, C @ x])) <= 1e-6
    assert _rel(out("col_adj"), A.T @ inp["yr"].astype(np.float64) + C.T @ inp["yc"].astype(np.float64)) <= 1e-6
    for name in ("row_dot", "col_dot"):
        d1, d2, d3, d4 = out(name, np.float64)
        assert abs(d1) > 0 and abs(d1 - d2) / abs(d1) <= 1e-6 and abs(d3 - d4) / abs(d3) <= 1e-6, name
