"""The oracle's checkpointed adjoint of the linearised pair (source wavefield
recomputed segment by segment from checkpoints) gives the image of the stored
snapshots bit for bit, in FP32 with each snapshot codec and in FP64, for
segment lengths that do and do not divide the step count or the snapshot
interval."""
import ctypes as C

import numpy as np
import pytest

from oracle.bindings import damp_ntab
from oracle.shot_setup import make_ctx, prepare_shot, source_vals
from sep_code_gb300 import surveys as S

JS = 3


@pytest.fixture(scope="module")
def case(oracle):
    s = S.small_survey(m1=20, m2=20, m3=24, nt=45, seed=5)
    st = prepare_shot(oracle, s)
    locs, vals = source_vals(oracle, s, st, 8)
    keep = []
    ctx = make_ctx(oracle, s, st, locs, vals, keep)
    rng = np.random.default_rng(2)
    d = rng.standard_normal((st.rnx * st.rny, st.nt_big)).astype(np.float32)
    return s, st, ctx, keep, vals, d


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_ckpt_f32(case, oracle, prec):
    s, st, ctx, keep, vals, d = case
    L = oracle.lib
    shape = (st.n[2], st.n[1], st.n[0])
    snaps = np.zeros(((st.nt + JS - 1) // JS,) + shape, np.float32)
    assert L.orc_lin_source_f32(C.byref(ctx), st.vel2dt2, st.jtd, 9, st.nt, JS, prec, snaps) == 0
    want = np.zeros(shape, np.float32)
    assert L.orc_lin_adjoint_f32(C.byref(ctx), st.vel2dt2, st.jtd, st.nt, JS, snaps, d, want) == 0
    assert np.abs(want).max() > 0
    for seg in (1, 7, 9, st.nt, st.nt + 5):
        img = np.zeros(shape, np.float32)
        assert L.orc_lin_adjoint_ckpt_f32(C.byref(ctx), st.vel2dt2, st.jtd, 9, st.nt, JS, prec, seg,
                                          d, img) == 0
        assert np.array_equal(img, want), seg


def test_ckpt_f64(case, oracle):
    s, st, ctx, keep, vals, d = case
    L = oracle.lib
    tab64 = oracle.damp_table(s.bc_a, s.bc_b, damp_ntab(*st.n), f64=True)
    c64 = oracle.make_ctx64(ctx, st.d, tab64, st.sinc_s.astype(np.float64), st.sinc_d.astype(np.float64),
                            vals.astype(np.float64), keep)
    vel = st.vel2dt2.astype(np.float64)
    d64 = d.astype(np.float64)
    shape = (st.n[2], st.n[1], st.n[0])
    snaps = np.zeros(((st.nt + JS - 1) // JS,) + shape, np.float64)
    assert L.orc_lin_source_f64(C.byref(c64), vel, st.jtd, 9, st.nt, JS, snaps) == 0
    want = np.zeros(shape, np.float64)
    assert L.orc_lin_adjoint_f64(C.byref(c64), vel, st.jtd, st.nt, JS, snaps, d64, want) == 0
    for seg in (4, 10, st.nt):
        img = np.zeros(shape, np.float64)
        assert L.orc_lin_adjoint_ckpt_f64(C.byref(c64), vel, st.jtd, 9, st.nt, JS, seg, d64, img) == 0
        assert np.array_equal(img, want), seg
