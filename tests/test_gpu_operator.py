"""The C++ operator layer (rtm_zero_op on device vectors) against the
reference's own rtm_zero_op (golden fixtures from tests/golden/make_golden.py),
its dot-product test, and least-squares RTM with cgstep."""
from pathlib import Path

import numpy as np
import pytest

from sep_code_gb300 import model as M
from tests.golden.make_golden import CASES, HASHED_OBS, hashed_traces
from tests.harness import rel_l2

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).parent / "golden"


@pytest.mark.parametrize("case", list(CASES))
def test_reference_mode_matches_reference_operator(case):
    """small: 24x20x28 model, 60 steps; jt2: data sampled every 2 FD steps;
    medium: 48x40x44 model, 600 FD steps (300 samples, jt 2)."""
    from sep_code_gb300.operator import RtmOperator
    g = np.load(GOLDEN / f"rtm_zero_op_{case}.npz")
    s = M.small_survey(**CASES[case])
    op = RtmOperator(s, "reference")
    data = op.forward(s.refl)[0]
    assert rel_l2(data, g["data"]) <= 1e-5
    assert np.array_equal(data, g["data"])
    rnx, rny = s.rec[0], s.rec[1]
    obs = hashed_traces((rny, rnx, s.data_nt), HASHED_OBS[case]) if case in HASHED_OBS else g["obs"]
    image = op.adjoint(obs[None])
    assert rel_l2(image, g["image"]) <= 1e-5
    assert np.array_equal(image, g["image"])


@pytest.mark.parametrize("prec", ["f32", "f16"])
def test_linear_operator_dot_test(prec):
    """my_operator::dot_test on the whole operator (extract / laplac / Born
    pair / map_data / deriv), add=false and add=true, 1e-6 relative"""
    from sep_code_gb300.operator import RtmOperator
    s = M.small_survey(m1=32, m2=28, m3=28, nt=120, seed=5, nbound=6, data_dt=0.001)
    op = RtmOperator(s, "linear", 1, prec)
    d1, d2, d3, d4 = op.dot_test(seed=3)
    assert abs(d1) > 0 and abs(d3) > 0
    assert abs(d1 - d2) / abs(d1) <= 1e-6, (d1, d2)
    assert abs(d3 - d4) / abs(d3) <= 1e-6, (d3, d4)


def test_reference_mode_is_not_an_exact_adjoint():
    """the reference's rtm_forward / rtm_adjoint pair (sponge twice forward,
    once adjoint; source rebuilt backwards) fails a tight dot test; measured
    and reported, which is why least-squares RTM uses the linear mode"""
    from sep_code_gb300.operator import RtmOperator
    s = M.small_survey(m1=32, m2=28, m3=28, nt=120, seed=5, nbound=6, data_dt=0.001)
    d1, d2, _, _ = RtmOperator(s, "reference").dot_test(seed=3)
    assert np.isfinite(d1) and np.isfinite(d2)
    assert abs(d1 - d2) / abs(d1) > 1e-6


def test_lsrtm_reduces_the_residual():
    from sep_code_gb300.operator import RtmOperator
    s = M.small_survey(m1=32, m2=28, m3=28, nt=120, seed=6, nbound=6, data_dt=0.001)
    op = RtmOperator(s, "linear", 2, "f32")
    d = op.forward(s.refl)
    model, resid, secs = op.lsrtm(d, 6)
    r0 = float(np.sum(d.astype(np.float64) ** 2))
    assert np.all(resid > 0) and np.all(np.diff(resid) <= 1e-9 * r0)
    assert resid[-1] < 0.5 * r0
    # the reported residual is |L m - d|^2
    rr = float(np.sum((op.forward(model).astype(np.float64) - d) ** 2))
    assert abs(rr - resid[-1]) <= 1e-3 * r0
    assert np.all(np.diff(secs) > 0)
