"""The linearised Born pair (least-squares RTM operator): GPU vs oracle with
FP32 / BF16 / FP16 source snapshots, and the adjoint dot-product test
<L m, d> = <m, L' d> to 1e-6 relative, FP64 sums."""
import numpy as np
import pytest

from sep_code_gb300 import model as M
from tests.harness import LinCase, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    s = M.small_survey(m1=28, m2=24, m3=24, nt=50, seed=12)
    st = M.prepare_shot(s)
    return LinCase(s, st)


@pytest.mark.parametrize("prec", ["f32", "bf16", "f16"])
@pytest.mark.parametrize("js", [1, 3])
def test_lin_parity(case, oracle, prec, js):
    st = case.st
    rng = np.random.default_rng(js)
    m = np.zeros((st.n[2], st.n[1], st.n[0]), np.float32)
    m[4:-8, 4:-16, 4:-16] = rng.standard_normal(m[4:-8, 4:-16, 4:-16].shape)
    d_g = case.gpu_forward(m, js, prec)
    d_o = case.orc_forward(oracle, m, js, prec)
    assert np.abs(d_o).max() > 0
    assert rel_l2(d_g, d_o) <= 1e-5
    assert np.array_equal(d_g, d_o)
    d = rng.standard_normal(d_o.shape).astype(np.float32)
    i_g = case.gpu_adjoint(d, js, prec)
    i_o = case.orc_adjoint(oracle, d, js, prec)
    assert np.abs(i_o).max() > 0
    assert rel_l2(i_g, i_o) <= 1e-5
    assert np.array_equal(i_g, i_o)


def _dot_test(c, js, prec, seed=7):
    st = c.st
    rng = np.random.default_rng(seed)
    m = rng.standard_normal((st.n[2], st.n[1], st.n[0])).astype(np.float32)
    d = rng.standard_normal((st.rnx * st.rny, st.nt_big)).astype(np.float32)
    Lm = c.gpu_forward(m, js, prec)
    Ltd = c.gpu_adjoint(d, js, prec)
    a = float(np.dot(Lm.astype(np.float64).ravel(), d.astype(np.float64).ravel()))
    b = float(np.dot(m.astype(np.float64).ravel(), Ltd.astype(np.float64).ravel()))
    return a, b


@pytest.mark.parametrize("prec", ["f32", "bf16", "f16"])
def test_lin_dot_product(prec):
    """sponge + random boundary, 150 steps at a stable time step; the
    reference's my_operator::dot_test measure |<Lm,d> - <m,L'd>| / |<Lm,d>|,
    tightened from its 1e-4 to 1e-6"""
    s = M.small_survey(m1=40, m2=36, m3=32, nt=150, seed=31, nbound=8, data_dt=0.001)
    st = M.prepare_shot(s)
    a, b = _dot_test(LinCase(s, st), 1, prec)
    assert abs(a) > 0
    assert abs(a - b) / abs(a) <= 1e-6, (a, b)


@pytest.mark.slow
def test_lin_dot_product_128():
    """the 128^3, dx=10 m, dt=1 ms, 1000-step workload (padded 176x176x224)"""
    s = M.anomaly_survey()
    st = M.prepare_shot(s)
    c = LinCase(s, st)
    a, b = _dot_test(c, 1, "f32")
    assert abs(a) > 0
    assert abs(a - b) / abs(a) <= 1e-6, (a, b)


@pytest.mark.slow
def test_lin_forward_repeatable_128():
    """the same forward twice on the 128^3 workload (several CTAs per SM
    sharing tensor memory, 1000 steps): bit-identical traces"""
    s = M.anomaly_survey()
    st = M.prepare_shot(s)
    c = LinCase(s, st)
    m = np.random.default_rng(3).standard_normal((st.n[2], st.n[1], st.n[0])).astype(np.float32)
    d1 = c.gpu_forward(m, 1, "bf16")
    d2 = c.gpu_forward(m, 1, "bf16")
    assert np.abs(d1).max() > 0
    assert np.array_equal(d1.view(np.uint32), d2.view(np.uint32))


def test_snapshot_memory(case):
    from sep_code_gb300 import gpu_funcs as gf
    c = case
    c.gpu_setup()
    b32 = gf.snapshot_bytes(c.st.nt, 4, "f32")
    b16 = gf.snapshot_bytes(c.st.nt, 4, "f16")
    assert 0 < b16 < 0.6 * b32
