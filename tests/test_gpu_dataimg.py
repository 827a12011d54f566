"""Device image / data vectors against the oracle (oracle/dataimg_oracle.py,
itself pinned to the reference's image_rtm_3d, data_rtm_3d and tmute):

* the C-ABI kernels (sepx_image_add_window, sepx_image_extract_window,
  sepx_tmute) bit for bit on small cases covering windows inside, straddling
  and outside the image, and every add / adjoint combination of the mute;
* the C++ classes (image_rtm_3d, data_rtm_3d, tmute) through a small C++
  program built against the library, bit for bit;
* full size (a 384 x 384 x 320 window of a 512 x 512 x 400 image; the mute of
  512 x 512 receivers x 4000 samples): exact against a masked copy made on
  the device, with the achieved bandwidth of each kernel printed as
  DATAIMG_BW {json} (bytes = what each kernel must read and write).
"""
import json
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import dataimg_oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def gf():
    from sep_code_gb300 import gpu_funcs
    gpu_funcs.setup_cuda(1)
    return gpu_funcs


def _dev(a):
    return torch.tensor(np.ascontiguousarray(a, np.float32)).cuda()


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("f", [(2, -1, 3), (-3, 4, -2), (0, 0, 0), (12, 0, 0), (5, 6, 4),
                               (-6, -5, -4)])
def test_window_add_and_extract_bit_exact(gf, f):
    rng = np.random.default_rng(100 + 7 * f[0] + f[1])
    img = rng.standard_normal((6, 7, 9)).astype(np.float32)
    sub = rng.standard_normal((4, 5, 6)).astype(np.float32)
    mute = rng.random((6, 7, 9)).astype(np.float32)
    ti, ts, tm = _dev(img), _dev(sub), _dev(mute)
    out = torch.full((4, 5, 6), 7.0, device="cuda")
    out1 = torch.full((4, 5, 6), 7.0, device="cuda")
    torch.cuda.synchronize()
    gf.image_add_window(ti.data_ptr(), (9, 7, 6), f, ts.data_ptr(), (6, 5, 4))
    gf.image_extract_window(ti.data_ptr(), tm.data_ptr(), (9, 7, 6), f, out.data_ptr(), (6, 5, 4))
    gf.image_extract_window(ti.data_ptr(), None, (9, 7, 6), f, out1.data_ptr(), (6, 5, 4))
    gf.synchronize()
    want = O.add_image(img, sub, f)
    assert np.array_equal(_bits(ti.cpu().numpy()), _bits(want))
    assert np.array_equal(_bits(out.cpu().numpy()), _bits(O.extract_sub(want, mute, sub.shape, f)))
    assert np.array_equal(_bits(out1.cpu().numpy()), _bits(O.extract_sub(want, None, sub.shape, f)))


@pytest.mark.parametrize("f", [(4, -1, 2), (-4, 3, -1), (12, 0, 0), (-8, 0, 0)])
def test_window_add_and_extract_aligned_bit_exact(gf, f):
    """rows of 16 and 8 floats at offsets that are multiples of 4: the
    16-byte path, windows inside, straddling and outside along x"""
    rng = np.random.default_rng(300 + 7 * f[0] + f[1])
    img = rng.standard_normal((6, 7, 16)).astype(np.float32)
    sub = rng.standard_normal((4, 5, 8)).astype(np.float32)
    mute = rng.random((6, 7, 16)).astype(np.float32)
    ti, ts, tm = _dev(img), _dev(sub), _dev(mute)
    out = torch.full((4, 5, 8), 7.0, device="cuda")
    torch.cuda.synchronize()
    gf.image_add_window(ti.data_ptr(), (16, 7, 6), f, ts.data_ptr(), (8, 5, 4))
    gf.image_extract_window(ti.data_ptr(), tm.data_ptr(), (16, 7, 6), f, out.data_ptr(), (8, 5, 4))
    gf.synchronize()
    want = O.add_image(img, sub, f)
    assert np.array_equal(_bits(ti.cpu().numpy()), _bits(want))
    assert np.array_equal(_bits(out.cpu().numpy()), _bits(O.extract_sub(want, mute, sub.shape, f)))


@pytest.mark.parametrize("adj", [False, True])
@pytest.mark.parametrize("add", [False, True])
def test_tmute_bit_exact(gf, adj, add):
    rng = np.random.default_rng(31 + 2 * adj + add)
    shape = (2, 3, 6, 64)
    m = rng.standard_normal(shape).astype(np.float32)
    d = rng.standard_normal(shape).astype(np.float32)
    # starts before the first sample (clamped), inside, and past the last
    args = (0.04, 1800.0, 0.0, 0.004, -100.0, 150.0)
    tm, td = _dev(m), _dev(d)
    torch.cuda.synchronize()
    gf.tmute(adj, add, args[0], args[1], 64, args[2], args[3], 6, args[4], args[5], 6,
             tm.data_ptr(), td.data_ptr())
    gf.synchronize()
    om, od = O.tmute(adj, add, *args, m, d)
    st = O.mute_starts(args[0], args[1], 64, args[2], args[3], 6, args[4], args[5])
    assert st.min() == 0 and st.max() == 64 and 0 < np.median(st) < 64
    assert np.array_equal(_bits(tm.cpu().numpy()), _bits(om))
    assert np.array_equal(_bits(td.cpu().numpy()), _bits(od))


def test_rejects_bad_arguments(gf):
    from sep_code_gb300._lib import SepxError
    t = torch.zeros(8, device="cuda")
    with pytest.raises(SepxError):
        gf.tmute(False, False, 0.0, 0.0, 8, 0.0, 0.004, 1, 0.0, 1.0, 1, t.data_ptr(), t.data_ptr())
    with pytest.raises(SepxError):
        gf.image_add_window(t.data_ptr(), (0, 1, 1), (0, 0, 0), t.data_ptr(), (1, 1, 1))
    with pytest.raises(SepxError):
        gf.image_extract_window(None, None, (8, 1, 1), (0, 0, 0), t.data_ptr(), (1, 1, 1))


def test_cpp_classes_bit_exact(gf, tmp_path):
    """image_rtm_3d, data_rtm_3d and tmute driven by a C++ caller"""
    from sep_code_gb300 import LIB_PATH
    exe = tmp_path / "dataimg_driver"
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    subprocess.run([cxx, "-std=c++17", "-O1", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "dataimg_driver.cpp"), str(LIB_PATH),
                    f"-Wl,-rpath,{Path(LIB_PATH).parent}", "-o", str(exe)], check=True)
    rng = np.random.default_rng(8)
    so = np.array([13.0, -12.5, 6.0], np.float32)
    inp = {"so": so, "img": rng.standard_normal((6, 7, 9)), "sub": rng.standard_normal((4, 5, 6)),
           "mute": rng.random((6, 7, 9)), "all": rng.standard_normal((3, 2, 4, 50)),
           "shot": rng.standard_normal((2, 4, 50)), "tm_model": rng.standard_normal((2, 3, 6, 64)),
           "tm_data": rng.standard_normal((2, 3, 6, 64))}
    inp = {k: np.ascontiguousarray(v, np.float32) for k, v in inp.items()}
    for k, v in inp.items():
        v.tofile(tmp_path / f"{k}.bin")
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def out(name, shape):
        return np.fromfile(tmp_path / f"{name}.bin", np.float32).reshape(shape)

    o, d = (0.0, 0.0, 0.0), (10.0, 12.5, 5.0)
    f = [O.window_offset(so[k], o[k], d[k]) for k in range(3)]
    added = O.add_image(inp["img"], inp["sub"], f)
    assert np.array_equal(_bits(out("out_add", (6, 7, 9))), _bits(added))
    assert np.array_equal(_bits(out("out_sub", (4, 5, 6))),
                          _bits(O.extract_sub(added, inp["mute"], (4, 5, 6), f)))
    assert np.array_equal(_bits(out("out_muted", (6, 7, 9))), _bits(O.write_volume(added, inp["mute"])))
    want = O.add_data(O.add_data(inp["all"], 1, inp["shot"]), 1, inp["shot"])
    assert np.array_equal(_bits(out("out_data", (3, 2, 4, 50))), _bits(want))
    args = (0.04, 1800.0, 0.0, 0.004, 50.0, 25.0)
    _, fwd = O.tmute(False, False, *args, inp["tm_model"], inp["tm_data"])
    assert np.array_equal(_bits(out("out_tm_fwd", (2, 3, 6, 64))), _bits(fwd))
    adj, _ = O.tmute(True, True, *args, inp["tm_model"], inp["tm_data"])
    assert np.array_equal(_bits(out("out_tm_adj", (2, 3, 6, 64))), _bits(adj))


def _peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _timed(stream, fn, reps=5):
    """mean seconds of fn() over reps launches on the library's stream"""
    fn()
    stream.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        fn()
    b.record(stream)
    b.synchronize()
    return a.elapsed_time(b) / 1e3 / reps


def test_full_size_exact_and_bandwidth(gf):
    """inputs larger than L2 (each volume 419 MB, the traces 4.2 GB)"""
    from sep_code_gb300._lib import lib
    stream = torch.cuda.ExternalStream(lib.sepx_get_stream())
    g = torch.Generator(device="cuda").manual_seed(3)
    n = (512, 512, 400)
    s = (384, 384, 320)
    f = (64, 64, 40)
    img = torch.randn(n[2], n[1], n[0], device="cuda", generator=g)
    sub = torch.randn(s[2], s[1], s[0], device="cuda", generator=g)
    mute = torch.rand(n[2], n[1], n[0], device="cuda", generator=g)
    win = (slice(f[2], f[2] + s[2]), slice(f[1], f[1] + s[1]), slice(f[0], f[0] + s[0]))
    want = img.clone()
    want[win] += sub
    torch.cuda.synchronize()
    gf.image_add_window(img.data_ptr(), n, f, sub.data_ptr(), s)
    gf.synchronize()
    assert torch.equal(img, want)
    out = torch.empty_like(sub)
    torch.cuda.synchronize()
    gf.image_extract_window(img.data_ptr(), mute.data_ptr(), n, f, out.data_ptr(), s)
    gf.synchronize()
    assert torch.equal(out, img[win] * mute[win])
    cells = s[0] * s[1] * s[2]
    t_add = _timed(stream, lambda: gf.image_add_window(img.data_ptr(), n, f, sub.data_ptr(), s))
    t_ext = _timed(stream, lambda: gf.image_extract_window(img.data_ptr(), mute.data_ptr(), n, f,
                                                           out.data_ptr(), s))
    del img, sub, mute, out, want
    # mute of one shot of 512 x 512 receivers x 4000 samples (4 ms): starts 40 ms + x / 2000 m/s
    nt, nx, ny = 4000, 512, 512
    model = torch.randn(ny, nx, nt, device="cuda", generator=g)
    data = torch.empty_like(model)
    torch.cuda.synchronize()
    args = (0.04, 2000.0, nt, 0.0, 0.004, nx, 0.0, 12.5, ny)
    gf.tmute(False, False, *args, model.data_ptr(), data.data_ptr())
    gf.synchronize()
    st = torch.tensor(O.mute_starts(0.04, 2000.0, nt, 0.0, 0.004, nx, 0.0, 12.5), device="cuda")
    mask = torch.arange(nt, device="cuda")[None, :] >= st[:, None]
    assert torch.equal(data, torch.where(mask[None], model, torch.zeros((), device="cuda")))
    t_mute = _timed(stream, lambda: gf.tmute(False, False, *args, model.data_ptr(), data.data_ptr()))
    # bytes: every output sample written, the passed input samples read
    passed = int((nt - st).sum().item()) * ny
    peak, kind = _peak()
    rows = {"image_add_window_384x384x320_in_512x512x400": (12 * cells, t_add),
            "image_extract_window_muted": (12 * cells, t_ext),
            "tmute_512x512x4000": (4 * nt * nx * ny + 4 * passed, t_mute)}
    res = {k: {"bytes": b, "us": 1e6 * t, "GB_s": b / t / 1e9, "frac": b / t / 1e9 / peak}
           for k, (b, t) in rows.items()}
    res["peak_GB_s"] = peak
    res["peak_kind"] = kind
    print("DATAIMG_BW " + json.dumps(res))
    for k, (b, t) in rows.items():
        assert b / t / 1e9 > 0.25 * peak, (k, b / t / 1e9)
