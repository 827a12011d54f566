"""Batched Born forward: every shot of a batch through one persistent launch
per step (and the same launches captured into a CUDA graph) against the
shot-after-shot loop of the reference's rtm_zero_op (Born/rtm_zero_op_3d.cpp:
123) and against the single-context C ABI.  The arithmetic per cell is the
same kernel code, so the traces must agree bit for bit."""
import numpy as np
import pytest

from sep_code_gb300 import batch as Bt
from sep_code_gb300 import gpu_funcs as gf
from sep_code_gb300 import model as M
from tests.harness import GpuShot

pytestmark = pytest.mark.gpu


def _surveys(nt=60):
    rng = np.random.default_rng(5)
    n3, n2, n1 = 64, 96, 112
    d = 10.0
    z = np.arange(n3)[:, None, None] * d
    vel = np.broadcast_to(1700.0 + 1.5 * z + 40 * rng.standard_normal((n3, 1, 1)), (n3, n2, n1))
    vel = vel.astype(np.float32).copy()
    refl = (rng.standard_normal((n3, n2, n1)) * (rng.random((n3, n2, n1)) < 0.05)).astype(np.float32)
    centers = [(300.0, 300.0), (700.0, 500.0), (520.0, 610.0)]
    windows = [(32, 32, 32), (48, 40, 40), (64, 48, 48)]
    return Bt.window_surveys(vel, refl, d, centers, windows, nt, f0=25.0)


@pytest.fixture(scope="module")
def batch():
    b = Bt.BatchRTM(_surveys())
    yield b
    b.close()


def _run(b, how):
    b.zero_traces()
    b.forward(how)
    return [b.traces(i) for i in range(len(b.setups))]


@pytest.mark.parametrize("style", [0, 1])
def test_batched_equals_sequential(batch, style):
    seq = _run(batch, "sequential")
    assert all(np.abs(t).max() > 0 for t in seq)
    batch.set_tuning(0, 3, style)
    for how in ("persistent", "graph", "graph"):   # the second graph run replays the capture
        got = _run(batch, how)
        for a, b in zip(got, seq):
            assert np.array_equal(a, b), (how, style)
    batch.set_tuning(0, 3, 0)


def test_autotuned_batch_equals_sequential(batch):
    seq = _run(batch, "sequential")
    z, s, sty, ms = batch.autotune(nsteps=4)
    assert z in (16, 24, 32, 48, 64, 96) and s in (2, 3, 4) and sty in (0, 1) and ms > 0
    got = _run(batch, "graph")
    for a, b in zip(got, seq):
        assert np.array_equal(a, b)
    batch.set_tuning(0, 3, 0)


def test_batch_shot_equals_single_context():
    surveys = _surveys()
    b = Bt.BatchRTM(surveys)
    try:
        got = _run(b, "persistent")
    finally:
        b.close()
    for s, t in zip(surveys, got):
        st = M.prepare_shot(s)
        single = GpuShot(s, st).rtm_forward(st.img_lap)
        assert np.array_equal(single, t)


@pytest.mark.parametrize("style", [0, 1])
def test_batched_full_rtm_equals_sequential(style):
    """source_prop + Born forward + RTM adjoint of every shot: batched (one
    launch per step, plain and captured) against the shot loop, images and
    traces bit for bit"""
    b = Bt.BatchRTM(_surveys())
    try:
        b.set_tuning(0, 3, style)
        b.set_images()
        b.rtm("sequential")
        want_img = [b.image(i) for i in range(len(b.setups))]
        want_trc = [b.traces(i) for i in range(len(b.setups))]
        assert all(np.abs(im).max() > 0 for im in want_img)
        for how in ("persistent", "graph", "graph"):
            b.set_images()   # the adjoint overwrote each shot's image buffer
            b.rtm(how)
            for i in range(len(b.setups)):
                assert np.array_equal(b.traces(i), want_trc[i]), (how, i)
                assert np.array_equal(b.image(i), want_img[i]), (how, i)
    finally:
        b.close()
