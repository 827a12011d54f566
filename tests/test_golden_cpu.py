"""The operator fixtures in tests/golden/ are what the reference's own
rtm_zero_op (compiled from its sources into oracle/_ref, the oracle's loops
standing in for the GPU C ABI) produces with the current oracle, bit for bit,
and the hashed observed traces of the larger case are fixed values."""
from pathlib import Path

import numpy as np
import pytest

from sep_code_gb300 import model as M
from tests.golden.make_golden import CASES, HASHED_OBS, hashed_traces

GOLDEN = Path(__file__).parent / "golden"


def test_hashed_traces_are_fixed_values():
    a = hashed_traces((3, 4, 5), 12).astype(np.float64)
    k = (a + 0.5) * float(1 << 24)
    assert np.array_equal(k, np.round(k))          # k / 2^24 - 1/2 exactly
    assert k.ravel()[:6].astype(np.int64).tolist() == KNOWN
    b = hashed_traces((1000, 1000), 1)
    assert abs(float(b.mean())) < 1e-3 and abs(float(b.std()) - 12 ** -0.5) < 1e-3


KNOWN = [12768038, 8790432, 9314165, 11881999, 8698687, 8202626]


@pytest.mark.parametrize("case", list(CASES))
def test_fixture_is_the_reference_operator_output(case, refhost):
    from oracle.bindings import RefOperator
    g = np.load(GOLDEN / f"rtm_zero_op_{case}.npz")
    s = M.small_survey(**CASES[case])
    ref = RefOperator(refhost)
    data = ref.born_forward(s)
    assert np.abs(data).max() > 0
    assert data.tobytes() == g["data"].tobytes()
    rnx, rny = s.rec[0], s.rec[1]
    obs = hashed_traces((rny, rnx, s.data_nt), HASHED_OBS[case]) if case in HASHED_OBS else g["obs"]
    image = ref.rtm_adjoint(s, obs)
    assert np.abs(image).max() > 0
    assert image.tobytes() == g["image"].tobytes()
