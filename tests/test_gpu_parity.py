"""CUDA path vs the oracle on the same seeded shots, through the C ABI.

Tolerance: relative L2 <= 1e-5 on FP32 traces and
images after the full time loop.  The kernels and the oracle share one
floating-point contract (explicit fused multiply-adds in the reference's term
order, shared sponge table), so the results are also expected to be
bit-identical; that is asserted separately.
"""
import numpy as np
import pytest

from sep_code_gb300 import gpu_funcs as gf
from sep_code_gb300 import model as M
from tests.harness import GpuShot, OracleShot, rel_l2

TOL = 1e-5
pytestmark = pytest.mark.gpu


def _cases():
    return {
        "small": dict(),
        # x width not a multiple of the 32-cell tile, odd sizes
        "ragged": dict(m1=37, m2=23, m3=21, nt=40, seed=11),
        # data sampled at twice the propagation step: two-row sinc tables
        "jt2": dict(m1=20, m2=20, m3=20, nt=30, seed=3, data_dt=0.004, dtw=0.004),
        # three propagation steps per data sample: three-row sinc tables
        "jt3": dict(m1=20, m2=20, m3=20, nt=20, seed=3, data_dt=0.006, dtw=0.006),
    }


@pytest.fixture(scope="module", params=list(_cases()))
def shot(request):
    s = M.small_survey(**_cases()[request.param])
    st = M.prepare_shot(s)
    return request.param, s, st


def test_source_prop_parity(shot, oracle):
    name, s, st = shot
    g0, g1 = GpuShot(s, st).source_prop()
    o0, o1 = OracleShot(oracle, s, st).source_prop()
    assert np.abs(o1).max() > 0
    assert rel_l2(g0, o0) <= TOL and rel_l2(g1, o1) <= TOL, name
    assert np.array_equal(g0, o0) and np.array_equal(g1, o1), name


def test_rtm_forward_parity(shot, oracle):
    name, s, st = shot
    rng = np.random.default_rng(5)
    rec0 = rng.standard_normal((st.rnx * st.rny, st.nt_big)).astype(np.float32) * 1e-3
    g = GpuShot(s, st).rtm_forward(st.img_lap, rec_init=rec0)
    o = OracleShot(oracle, s, st).rtm_forward(st.img_lap, rec_init=rec0)
    assert np.abs(o - rec0).max() > 0
    assert rel_l2(g, o) <= TOL, name
    assert np.array_equal(g, o), name


def test_rtm_adjoint_parity(shot, oracle):
    name, s, st = shot
    o_sh = OracleShot(oracle, s, st)
    p0, p1 = o_sh.source_prop()
    rng = np.random.default_rng(9)
    traces = rng.standard_normal((st.rnx * st.rny, st.nt_big)).astype(np.float32)
    # the adjoint reads the fields back in swapped order (Born/rtm_zero_op_3d.cpp:254-262)
    g = GpuShot(s, st).rtm_adjoint(p1, p0, traces)
    o = o_sh.rtm_adjoint(p1, p0, traces)
    assert np.abs(o).max() > 0
    assert rel_l2(g, o) <= TOL, name
    assert np.array_equal(g, o), name


def test_zchunk_invariance():
    s = M.small_survey(m1=24, m2=20, m3=40, nt=30, seed=21)
    st = M.prepare_shot(s)
    outs = []
    for zc in (0, 1, 7, 1000):
        gf.setup_cuda(1)
        gf.set_zchunk(zc)
        outs.append(GpuShot(s, st).rtm_forward(st.img_lap))
    gf.set_zchunk(0)
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_duplicate_points(oracle):
    """Two receivers on one cell and a repeated source point add up in order."""
    s = M.small_survey(m1=20, m2=20, m3=20, nt=25, seed=4)
    st = M.prepare_shot(s)
    st.rec_locs[1] = st.rec_locs[0]
    st.src_locs = st.src_locs.copy()
    rng = np.random.default_rng(2)
    traces = rng.standard_normal((st.rnx * st.rny, st.nt_big)).astype(np.float32)
    gs, osh = GpuShot(s, st), OracleShot(oracle, s, st)
    p0, p1 = osh.source_prop()
    g = gs.rtm_adjoint(p1, p0, traces)
    o = osh.rtm_adjoint(p1, p0, traces)
    assert np.array_equal(g, o)
    gfw = gs.rtm_forward(st.img_lap)
    ofw = osh.rtm_forward(st.img_lap)
    assert np.array_equal(gfw, ofw)
    assert np.array_equal(gfw[0], gfw[1])


def test_short_loops(oracle):
    """nt = 1 (only the first adjoint step) and nt = 2."""
    for nt_data in (1, 2):
        s = M.small_survey(m1=20, m2=20, m3=20, nt=nt_data, seed=8)
        st = M.prepare_shot(s)
        rng = np.random.default_rng(1)
        traces = rng.standard_normal((st.rnx * st.rny, st.nt_big)).astype(np.float32)
        p0 = rng.standard_normal((st.n[2], st.n[1], st.n[0])).astype(np.float32)
        p1 = rng.standard_normal((st.n[2], st.n[1], st.n[0])).astype(np.float32)
        g = GpuShot(s, st).rtm_adjoint(p0, p1, traces)
        o = OracleShot(oracle, s, st).rtm_adjoint(p0, p1, traces)
        assert np.array_equal(g, o), nt_data


def test_short_source_prop_and_one_receiver(oracle):
    """source_prop of nt = 1 and 2 data samples (nt+1 steps), and all three
    loops with a single receiver (a 1 x 1 receiver grid), bit for bit."""
    for nt_data in (1, 2):
        s = M.small_survey(m1=20, m2=20, m3=20, nt=nt_data, seed=8)
        st = M.prepare_shot(s)
        g = GpuShot(s, st).source_prop()
        o = OracleShot(oracle, s, st).source_prop()
        for a, b in zip(g, o):
            assert np.array_equal(a, b), nt_data
    s = M.small_survey(m1=24, m2=20, m3=28, nt=30, seed=4, rnx=1, rny=1)
    st = M.prepare_shot(s)
    gs, os_ = GpuShot(s, st), OracleShot(oracle, s, st)
    gp, op = gs.source_prop(), os_.source_prop()
    assert all(np.array_equal(a, b) for a, b in zip(gp, op))
    gt, ot = gs.rtm_forward(st.img_lap), os_.rtm_forward(st.img_lap)
    assert gt.shape == (1, st.nt_big) and np.abs(ot).max() > 0
    assert np.array_equal(gt, ot)
    gi = gs.rtm_adjoint(op[1], op[0], ot)
    oi = os_.rtm_adjoint(op[1], op[0], ot)
    assert np.abs(oi).max() > 0
    assert np.array_equal(gi, oi)


def test_errors_are_reported():
    gf.setup_cuda(1)
    with pytest.raises(gf.SepxError):
        gf.setup_cuda(2)
    s = M.small_survey()
    st = M.prepare_shot(s)
    gs = GpuShot(s, st)
    bad = st.src_locs.copy()
    bad[0] = 0   # a corner cell the kernels never update
    with pytest.raises(gf.SepxError, match="outside the propagated interior"):
        gf.transfer_source_func(bad, np.zeros((9, 10), np.float32))
    assert gf.device_error() == 0


@pytest.mark.parametrize("rows", [1, 2])
@pytest.mark.parametrize("case", [
    dict(m1=37, m2=23, m3=21, nt=40, seed=11),
    # y interior 48 cells (padded n2 = 64): one and a half 32-row tiles
    dict(m1=24, m2=40, m3=20, nt=30, seed=13),
    dict(m1=20, m2=20, m3=20, nt=30, seed=3, data_dt=0.004, dtw=0.004),
], ids=["ragged", "halfy", "jt2"])
def test_tile_rows_parity(rows, case, oracle):
    """source_prop, Born forward and RTM adjoint with every step kernel on
    one row (32 x 16 tile) or two rows (32 x 32 tile) per thread: both equal
    the oracle bit for bit."""
    s = M.small_survey(**case)
    st = M.prepare_shot(s)
    gf.setup_cuda(1)
    try:
        for mode in (0, 1, 2):
            gf.set_tile_rows(mode, rows)
        g, o = GpuShot(s, st), OracleShot(oracle, s, st)
        g0, g1 = g.source_prop()
        o0, o1 = o.source_prop()
        assert np.array_equal(g0, o0) and np.array_equal(g1, o1)
        rng = np.random.default_rng(5)
        rec0 = rng.standard_normal((st.rnx * st.rny, st.nt_big)).astype(np.float32) * 1e-3
        assert np.array_equal(g.rtm_forward(st.img_lap, rec_init=rec0),
                              o.rtm_forward(st.img_lap, rec_init=rec0))
        traces = rng.standard_normal((st.rnx * st.rny, st.nt_big)).astype(np.float32)
        assert np.array_equal(g.rtm_adjoint(o1, o0, traces), o.rtm_adjoint(o1, o0, traces))
    finally:
        for mode in (0, 1, 2):
            gf.set_tile_rows(mode, 1)


def test_tile_rows_rejects_other_modes():
    gf.setup_cuda(1)
    with pytest.raises(gf.SepxError):
        gf.set_tile_rows(3, 2)
    with pytest.raises(gf.SepxError):
        gf.set_tile_rows(1, 3)
