"""The shot-parallel solver on the GPU (one rank): its Python plane search
over the C-API operator reproduces the C++ simple_solver + cgstep
(sepx_lsrtm) on the same multi-shot survey to round-off (the two sum their
FP64 inner products in different orders): models relative L2 1e-5,
residuals relative 1e-6.  And a survey split into two shards, imaged shard by
shard and summed, gives the image of the whole survey (what the image
reduction of two ranks computes)."""
import numpy as np
import pytest

from sep_code_gb300 import shot_parallel as SP
from sep_code_gb300 import surveys as S

pytestmark = pytest.mark.gpu


def _survey():
    s = S.small_survey(m1=24, m2=20, m3=24, nt=80, seed=23)
    s.shots = [(60.0 + 60.0 * i, 50.0 + 50.0 * j, 0.0) for j in range(2) for i in range(2)]
    return s


def test_python_plane_search_matches_cpp_solver():
    from sep_code_gb300.operator import RtmOperator
    s = _survey()
    op = RtmOperator(s, "reference")
    data = op.forward(s.refl)
    m_c, r_c, _ = op.lsrtm(data, 5)
    m_p, r_p, _ = SP.lsrtm(op, data, 5, SP.Comm())
    op.close()
    assert np.linalg.norm(m_p - m_c) / np.linalg.norm(m_c) <= 1e-5
    assert np.max(np.abs(r_p / r_c - 1)) <= 1e-6


def test_shards_sum_to_the_whole_image():
    from sep_code_gb300.operator import RtmOperator
    s = _survey()
    op = RtmOperator(s, "reference")
    data = op.forward(s.refl)
    whole = op.adjoint(data)
    op.close()
    parts = []
    for r in range(2):
        sh = SP.shard_survey(s, r, 2)
        o = RtmOperator(sh, "reference")
        parts.append(o.adjoint(data[r::2]))
        o.close()
    summed = (parts[0].astype(np.float64) + parts[1]).astype(np.float32)
    assert np.linalg.norm(summed - whole) / np.linalg.norm(whole) <= 1e-6
