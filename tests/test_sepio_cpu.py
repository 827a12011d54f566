"""SEP regular datasets (the reference's on-disk format, read and written
through SEPlib in Born/sreg.cpp / sregf.cpp) through the library's own reader
and writer, host buffers, on the CPU:

* the hand-made fixture tests/golden/sep_tiny.H (appended history, quoting,
  a word without '=', relative in=, big-endian data; written without the
  library by tests/golden/make_sep_fixture.py) reads to the values it holds;
* written datasets read back bit for bit by numpy as big-endian ('>f4',
  xdr_float) or little-endian ('<f4', native_float) and by the library;
* windows (first / step / size per axis) equal numpy slicing;
* bad headers, short data and out-of-range windows are errors, not crashes.
SEPlib itself is not available here, so the format is pinned by its
published conventions (no reference-written dataset exists to compare to).
"""
from pathlib import Path

import numpy as np
import pytest

from sep_code_gb300 import sepio as S
from sep_code_gb300._lib import SepxError

GOLD = Path(__file__).resolve().parent / "golden"


def test_fixture_header_and_values():
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", GOLD / "make_sep_fixture.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    h = GOLD / "sep_tiny.H"
    nd, n, o, d = S.info(h)
    assert nd == 3 and n[:3] == [4, 3, 2] and n[3:] == [1] * 5
    assert o[:3] == [0.0, -25.0, 100.0]
    assert d[:3] == [np.float32(0.004), 12.5, 25.0]
    assert S.par(h, "label1") == "time (s)" and S.par(h, "label2") == "offset"
    assert S.par(h, "label3") == "y" and S.par(h, "label4") is None
    got = S.read(h)
    assert got.shape == (2, 3, 4)
    assert np.array_equal(got.view(np.uint32), mk.values().view(np.uint32))
    assert np.array_equal(S.read(h, 5, 7), mk.values().ravel()[5:12])


@pytest.mark.parametrize("xdr", [True, False])
def test_write_read_round_trip(tmp_path, xdr):
    rng = np.random.default_rng(4)
    a = rng.standard_normal((3, 5, 7, 11)).astype(np.float32)
    a[0, 0, 0, :4] = [np.inf, -0.0, 1e-45, np.nan]
    p = tmp_path / "cube.H"
    S.write(p, a, o=[0.0, 1.5, -2.0, 3.0], d=[0.004, 10.0, 12.5, 1.0], labels=["t", "x", "y", "s"],
            xdr=xdr)
    raw = np.fromfile(str(p) + "@", ">f4" if xdr else "<f4").reshape(a.shape)
    assert np.array_equal(raw.astype(np.float32).view(np.uint32), a.view(np.uint32))
    nd, n, o, d = S.info(p)
    assert nd == 4 and n[:4] == [11, 7, 5, 3]
    assert o[:4] == [0.0, 1.5, -2.0, 3.0] and d[:4] == [np.float32(0.004), 10.0, 12.5, 1.0]
    assert S.par(p, "data_format") == ("xdr_float" if xdr else "native_float")
    assert np.array_equal(S.read(p).view(np.uint32), a.view(np.uint32))


def test_windows_match_numpy_slicing(tmp_path):
    a = np.arange(6 * 7 * 9, dtype=np.float32).reshape(6, 7, 9)
    p = tmp_path / "w.H"
    S.write(p, a)
    for nw, fw, jw in [([9, 7, 6], None, None), ([3, 2, 2], [1, 2, 3], [3, 4, 2]),
                       ([1, 7, 1], [8, 0, 5], [1, 1, 1]), ([4, 1, 6], [0, 6, 0], [2, 1, 1])]:
        f = fw or [0, 0, 0]
        j = jw or [1, 1, 1]
        want = a[f[2]:f[2] + (nw[2] - 1) * j[2] + 1:j[2], f[1]:f[1] + (nw[1] - 1) * j[1] + 1:j[1],
                 f[0]:f[0] + (nw[0] - 1) * j[0] + 1:j[0]]
        assert np.array_equal(S.read_window(p, nw, fw, jw), want)


def test_errors(tmp_path):
    with pytest.raises(SepxError):
        S.info(tmp_path / "missing.H")
    bad = tmp_path / "bad.H"
    bad.write_text("n1=4 esize=8 in=bad.H@\n")
    with pytest.raises(SepxError):
        S.info(bad)
    bad.write_text("n1=4 data_format=xdr_int in=bad.H@\n")
    with pytest.raises(SepxError):
        S.info(bad)
    bad.write_text("n1=4\n")   # no data file
    with pytest.raises(SepxError):
        S.read(bad)
    short = tmp_path / "short.H"
    short.write_text("n1=8 in=short.H@\n")
    np.zeros(3, ">f4").tofile(str(short) + "@")
    with pytest.raises(SepxError):
        S.read(short)
    a = np.zeros((2, 3), np.float32)
    S.write(tmp_path / "ok.H", a)
    with pytest.raises(SepxError):
        S.read_window(tmp_path / "ok.H", [2, 2], [2, 0], [1, 1])   # 2 + 1 >= 3
    with pytest.raises(SepxError):
        S.read(tmp_path / "ok.H", 4, 3)
    # axis lengths that are not positive ints, or whose product overflows
    for text in ("n1=abc in=x.H@\n", "n1=3000000000 in=x.H@\n",
                 "n1=2000000000 n2=2000000000 n3=2000000000 in=x.H@\n"):
        bad.write_text(text)
        with pytest.raises(SepxError):
            S.info(bad)
