"""The image / data vector operations that the reference runs on its
out-of-core SEP datasets -- image_rtm_3d::add_image / extract_sub /
write_volume, data_rtm_3d::add_data, tmute::forward / adjoint -- restated in
oracle/dataimg_oracle.py, pinned bit for bit against the reference's own
classes (compiled from their sources, datasets in memory).

Two reference behaviours are not restated and so are not compared:
* tmute::forward reads one whole cube per axis-3 index and writes back only
  the last (Born/tmute.cpp:58-71), so for n3 > 1 its output is not the masked
  model; the restatement (and the device kernel) masks every cube, which is
  what tmute::adjoint (n3 > 1 included) is the adjoint of;
* a mute start before the first sample makes the reference index before the
  trace (out of bounds); the restatement starts at sample 0.  The pins use
  starts >= 0.
"""
import numpy as np
import pytest

from oracle import dataimg_oracle as O

ORIG = ((0.0, 0.0, 0.0), (10.0, 12.5, 5.0))


@pytest.mark.parametrize("so", [(25.0, -12.5, 31.0), (-40.0, 100.0, -20.0), (0.0, 0.0, 0.0),
                                (900.0, 0.0, 0.0), (13.0, 37.4, 6.0)])
def test_add_image_and_extract_sub_match_reference(refhost, so):
    rng = np.random.default_rng(int(abs(so[0]) + 7))
    o, d = ORIG
    img = rng.standard_normal((6, 7, 9)).astype(np.float32)
    sub = rng.standard_normal((4, 5, 6)).astype(np.float32)
    mute = rng.random((6, 7, 9)).astype(np.float32)
    f = [O.window_offset(so[k], o[k], d[k]) for k in range(3)]
    want = refhost.image_add(img, o, d, sub, so, d)
    got = O.add_image(img, sub, f)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    rs, rmuted = refhost.image_extract(img, mute, o, d, sub.shape, so, d)
    assert np.array_equal(O.extract_sub(img, mute, sub.shape, f).view(np.uint32), rs.view(np.uint32))
    assert np.array_equal(O.write_volume(img, mute).view(np.uint32), rmuted.view(np.uint32))


def test_window_offset_truncates_like_the_reference():
    # (int) of a single-precision quotient, toward zero
    assert O.window_offset(-12.5, 0.0, 10.0) == -1
    assert O.window_offset(37.4, 0.0, 12.5) == 2
    assert O.window_offset(0.3, 0.1, 0.1) == int(np.trunc((np.float32(0.3) - np.float32(0.1)) / np.float32(0.1)))


def test_add_data_matches_reference(refhost):
    rng = np.random.default_rng(5)
    alld = rng.standard_normal((3, 2, 4, 50)).astype(np.float32)
    shot = rng.standard_normal((2, 4, 50)).astype(np.float32)
    for ishot in range(3):
        want = refhost.add_data(alld, ishot, shot)
        assert np.array_equal(O.add_data(alld, ishot, shot).view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("adj", [False, True])
@pytest.mark.parametrize("add", [False, True])
def test_tmute_matches_reference(refhost, adj, add):
    rng = np.random.default_rng(11 + 2 * adj + add)
    # forward: one cube per shot (n3 = 1); adjoint: several cubes and shots
    shape = (2, 3, 1, 6, 64) if not adj else (2, 2, 3, 6, 64)
    m = rng.standard_normal(shape).astype(np.float32)
    d = rng.standard_normal(shape).astype(np.float32)
    t0, vm, o1, d1, o2, d2 = 0.04, 1800.0, 0.0, 0.004, 50.0, 25.0
    rm, rd = refhost.tmute(not adj, add, t0, vm, o1, d1, o2, d2, m, d)
    om, od = O.tmute(adj, add, t0, vm, o1, d1, o2, d2, m, d)
    assert np.array_equal(om.view(np.uint32), rm.view(np.uint32))
    assert np.array_equal(od.view(np.uint32), rd.view(np.uint32))
    st = O.mute_starts(t0, vm, 64, o1, d1, 6, o2, d2)
    assert st.min() > 0 and st.max() < 64 and len(set(st.tolist())) > 1


def test_tmute_restatement_is_a_mask_pair():
    """<T m, d> = <m, T' d> with the forward applied to every cube"""
    rng = np.random.default_rng(3)
    m = rng.standard_normal((2, 3, 6, 40)).astype(np.float32)
    d = rng.standard_normal((2, 3, 6, 40)).astype(np.float32)
    _, tm = O.tmute(False, False, 0.02, 1500.0, 0.0, 0.004, -30.0, 20.0, m, np.zeros_like(d))
    ta, _ = O.tmute(True, False, 0.02, 1500.0, 0.0, 0.004, -30.0, 20.0, np.zeros_like(m), d)
    a = float(np.dot(tm.ravel().astype(np.float64), d.ravel()))
    b = float(np.dot(m.ravel().astype(np.float64), ta.ravel()))
    assert abs(a - b) <= 1e-12 * max(abs(a), 1.0)
    st = O.mute_starts(0.02, 1500.0, 40, 0.0, 0.004, 6, -30.0, 20.0)
    assert st[0] == 0   # a start before the first sample is clamped
