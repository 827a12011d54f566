"""Pins of the oracle and of the product's host code against the reference's
own host C++ (compiled from its sources into oracle/_ref), all on the CPU.

* set-up math (sinc tables, glibc-rand random boundary, padded grid, source
  stencil, wavelet derivative, receiver map): bit-identical three ways;
* trace / image helpers (deriv, laplac, map_data): oracle == reference;
* the reference's rtm_zero_op forward and adjoint, run end to end by its own
  classes with the oracle loops behind the C ABI, against the same shot
  orchestrated by sep_code_gb300.model + the oracle: bit-identical data and
  image, and the same C-ABI call sequence.
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from sep_code_gb300 import gpu_funcs as gf
from sep_code_gb300 import model as M
from tests.golden.make_golden import CASES as GOLDEN_CASES

ROOT = Path(__file__).resolve().parent.parent


def same_bits(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


# ------------------------------------------------------------------ library surface
def _declared(header):
    txt = (ROOT / "include" / header).read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    # C++ classes follow the extern "C" block in sepx_ops.h: only the C ABI counts
    cut = txt.find('#ifdef __cplusplus\n}')
    if cut > 0:
        txt = txt[:cut]
    return sorted(set(re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt)) -
                  {"if", "for", "while", "sizeof", "return", "int", "void"})


@pytest.mark.parametrize("header", ["sepx.h", "sepx_host.h", "sepx_ops.h", "sepx_batch.h",
                                    "sepx_unet.h", "sepx_sepio.h"])
def test_library_exports_every_declared_symbol(header):
    from sep_code_gb300 import LIB_PATH
    lib = C.CDLL(str(LIB_PATH))
    names = _declared(header)
    assert len(names) >= 5 or (header == "sepx_sepio.h" and len(names) == 5)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_named_abi_matches_reference_header():
    """the eleven Born/gpu_funcs_3d.h entry points, by name"""
    names = set(_declared("sepx.h"))
    for n in ["setup_cuda", "source_prop", "rtm_adjoint", "rtm_forward", "transfer_sinc_table_s",
              "transfer_sinc_table_d", "transfer_source_func", "transfer_receiver_func",
              "transfer_vel_func1", "transfer_vel_func2", "create_gpu_space"]:
        assert n in names


def test_calls_without_a_gpu_fail_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gf.SepxError):
        gf.setup_cuda(1)


# ------------------------------------------------------------------ set-up math
@pytest.mark.parametrize("jt", [1, 2, 3, 5, 8])
def test_sinc_tables(jt, oracle, refhost):
    r = refhost.sinc_table(jt)
    assert same_bits(oracle.sinc_table(jt), r)
    assert same_bits(gf.sinc_table(jt), r)
    # row 0 is (numerically) a unit spike at tap 3: interpolation at d = 0
    assert abs(r[0, 3] - 1) < 1e-5 and np.abs(np.delete(r[0], 3)).max() < 1e-5


@pytest.mark.parametrize("seed", [0, 1, 17, 9999, 123456])
def test_glibc_rand(seed, oracle):
    libc = C.CDLL("libc.so.6")
    libc.srand(seed)
    want = np.array([libc.rand() for _ in range(1000)], np.int32)
    oracle.lib.orc_glibc_srand(seed)
    got_o = np.array([oracle.lib.orc_glibc_rand() for _ in range(1000)], np.int32)
    assert np.array_equal(want, got_o)
    assert np.array_equal(want, gf.glibc_rand(seed, 1000))


@pytest.mark.parametrize("nb", [0, 3, 6, 20])
def test_rand_subspace(nb, oracle, refhost):
    rng = np.random.default_rng(nb)
    model = (1500 + rng.random((10, 12, 14)) * 1000).astype(np.float32)
    sn = (14 + 2 * (nb + 4) + 5, 12 + 2 * (nb + 4) + 3, 10 + 3 * nb + 12)
    args = (4321, nb, nb, nb, 0.001, model, (0, 0, 0), (10, 10, 10), sn, (-10.0 * (nb + 4),) * 3,
            (10, 10, 10))
    r = refhost.rand_subspace(*args)
    assert same_bits(oracle.rand_subspace(*args), r)
    assert same_bits(gf.rand_subspace(*args), r)
    if nb:
        assert np.unique(r).size > np.unique(model).size // 2   # boundary randomised


@pytest.mark.parametrize("m", [(128, 128, 128), (512, 512, 400), (37, 23, 21), (192, 192, 256)])
def test_padded_grid(m, oracle, refhost):
    n_ref, o_ref = refhost.compute_domain(*m, (10.0, 10.0, 10.0), 20, 20, 20)
    assert oracle.compute_size(*m, 20, 20, 20) == n_ref
    assert gf.compute_size(*m, 20, 20, 20) == n_ref
    assert all(v % 16 == 0 for v in n_ref)
    assert o_ref == (-240.0, -240.0, -240.0)


def test_wavelet_and_source_stencil(oracle, refhost):
    w = M.ricker(15.0, 0.001, 300)
    wr = refhost.wavelet_deriv(w, 0.001)
    assert same_bits(oracle.wavelet_deriv(w, 0.001), wr)
    assert same_bits(gf.wavelet_deriv(w, 0.001), wr)
    n, o, d = (176, 176, 224), (-240.0, -240.0, -240.0), (10.0, 10.0, 10.0)
    for sx, sy, sz in [(640.0, 640.0, 0.0), (633.3, 12.5, 7.0)]:
        lr, vr = refhost.source_func(wr, 0.001, sx, sy, sz, n, o, d, 308)
        lo, vo = oracle.source_func(wr, sx, sy, sz, n[0], n[1], o, d, 308)
        lp, vp = gf.source_func(wr, sx, sy, sz, n[0], n[1], o, d, 308)
        assert np.array_equal(lr, lo) and np.array_equal(lr, lp)
        assert same_bits(vr, vo) and same_bits(vr, vp)


@pytest.mark.parametrize("fwd", [1, 0])
@pytest.mark.parametrize("add", [0, 1])
def test_trace_and_image_helpers(fwd, add, oracle, refhost):
    rng = np.random.default_rng(10 * fwd + add)
    m = rng.standard_normal((3, 4, 20)).astype(np.float32)
    d = rng.standard_normal((3, 4, 20)).astype(np.float32)
    mr, dr = refhost.deriv(fwd, add, m, d, 0.004)
    mo, do = m.copy(), d.copy()
    (oracle.lib.orc_deriv_forward if fwd else oracle.lib.orc_deriv_adjoint)(add, 20, 4, 3, 0.004, mo, do)
    assert same_bits(mr, mo) and same_bits(dr, do)
    mr, dr = refhost.laplac(fwd, add, m, d)
    mo, do = m.copy(), d.copy()
    (oracle.lib.orc_laplac_forward if fwd else oracle.lib.orc_laplac_adjoint)(add, 20, 4, 3, mo, do)
    assert same_bits(mr, mo) and same_bits(dr, do)
    mm = rng.standard_normal((3, 4, 28)).astype(np.float32)
    mr, dr = refhost.map_data(fwd, add, mm, d)
    mo, do = mm.copy(), d.copy()
    (oracle.lib.orc_map_data_forward if fwd else oracle.lib.orc_map_data_adjoint)(add, 28, 20, 4, 3, mo, do)
    assert same_bits(mr, mo) and same_bits(dr, do)


def test_laplac_forward_numpy_matches_reference(refhost):
    rng = np.random.default_rng(3)
    m = rng.standard_normal((6, 5, 7)).astype(np.float32)
    _, dr = refhost.laplac(1, 0, m, np.zeros_like(m))
    assert same_bits(M.laplac_forward(m), dr)


# ------------------------------------------------------------------ whole operator
def _python_born_forward(oracle, s):
    """the same shot prepared by sep_code_gb300.model, propagated by the oracle,
    post-processed like rtm_zero_op::forward (map_data, deriv)."""
    from tests.harness import OracleShot
    st = M.prepare_shot(s)
    rec = OracleShot(oracle, s, st).rtm_forward(st.img_lap)
    rnx, rny = st.rnx, st.rny
    m = np.ascontiguousarray(rec.reshape(rny, rnx, st.nt_big))
    shot_deriv = np.zeros((rny, rnx, s.data_nt), np.float32)
    oracle.lib.orc_map_data_forward(0, st.nt_big, s.data_nt, rnx, rny, m, shot_deriv)
    data = np.zeros_like(shot_deriv)
    oracle.lib.orc_deriv_forward(0, s.data_nt, rnx, rny, np.float32(s.data_dt), shot_deriv, data)
    return st, data


@pytest.mark.parametrize("case", list(GOLDEN_CASES))
def test_reference_operator_forward(case, oracle, refhost):
    from oracle.bindings import RefOperator
    s = M.small_survey(**GOLDEN_CASES[case])
    ref = RefOperator(refhost)
    d_ref = ref.born_forward(s)
    st, d_py = _python_born_forward(oracle, s)
    assert np.abs(d_ref).max() > 0
    assert same_bits(d_ref, d_py)
    # the C-ABI inputs the reference operator produced are the ones prepare_shot builds
    assert same_bits(ref.last_array("vel1").reshape(st.vel2dt2.shape), st.vel2dt2)
    assert np.array_equal(ref.last_array("rec_loc", np.int32), st.rec_locs)
    assert np.array_equal(ref.last_array("src_loc", np.int32), st.src_locs)
    names = [c[0] for c in ref.log()]
    assert names == ["setup_cuda", "transfer_sinc_table_s", "create_gpu_space",
                     "transfer_sinc_table_d", "transfer_source_func", "transfer_vel_func1",
                     "transfer_vel_func2", "transfer_receiver_func", "rtm_forward"]
    fwd = [c for c in ref.log() if c[0] == "rtm_forward"][0][1]
    assert fwd == [st.n[0], st.n[1], st.n[2], st.jtd, 9, st.nt, st.nt_big, st.rnx, st.rny]


def test_reference_operator_adjoint(oracle, refhost):
    """rtm_zero_op::adjoint: source fields from create_source_fields (+9
    samples), read back swapped, deriv/map_data adjoints, laplac adjoint."""
    from oracle.bindings import RefOperator
    from tests.harness import OracleShot
    s = M.small_survey()
    rng = np.random.default_rng(4)
    rnx, rny = s.rec[0], s.rec[1]
    data = rng.standard_normal((rny, rnx, s.data_nt)).astype(np.float32)
    ref = RefOperator(refhost)
    img_ref = ref.rtm_adjoint(s, data)
    # the same in Python + oracle
    st = M.prepare_shot(s)
    osh = OracleShot(oracle, s, st)
    p0, p1 = osh.source_prop()
    shot_deriv = np.zeros_like(data)
    oracle.lib.orc_deriv_adjoint(0, s.data_nt, rnx, rny, np.float32(s.data_dt), shot_deriv,
                                 np.ascontiguousarray(data))
    rec = np.zeros((rny, rnx, st.nt_big), np.float32)
    oracle.lib.orc_map_data_adjoint(0, st.nt_big, s.data_nt, rnx, rny, rec, shot_deriv)
    img = osh.rtm_adjoint(p1, p0, rec.reshape(rny * rnx, st.nt_big))
    img_lap = np.zeros_like(img)
    n1, n2, n3 = st.n
    oracle.lib.orc_laplac_adjoint(0, n1, n2, n3, img_lap, img)
    # image_rtm_3d::add_image: padded image back onto the model grid
    f = [int(np.float32(st.o[k]) / np.float32(s.spacing[k])) for k in range(3)]
    m3, m2, m1 = s.vel.shape
    want = img_lap[-f[2]:-f[2] + m3, -f[1]:-f[1] + m2, -f[0]:-f[0] + m1]
    assert np.abs(img_ref).max() > 0
    assert same_bits(img_ref, want)
    names = [c[0] for c in ref.log()]
    assert names.count("source_prop") == 1 and names.count("rtm_adjoint") == 1


def test_oracle_born_forward_doubling(oracle):
    """The FP32 restatement is linear in the image up to subnormal rounding:
    doubling the image doubles the traces to relative L2 ~1e-7..1e-6, not exactly
    (the bar the full-size GPU property test uses is 1e-5)."""
    from tests.harness import OracleShot, rel_l2
    s = M.anomaly_survey(n=32, nt=250)
    st = M.prepare_shot(s)
    o = OracleShot(oracle, s, st)
    d1 = o.rtm_forward(st.img_lap)
    d2 = o.rtm_forward(2 * st.img_lap)
    e = rel_l2(d2, 2 * d1)
    assert np.abs(d1).max() > 0
    assert 0 < e <= 1e-5, e
