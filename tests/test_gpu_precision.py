"""Precision study of the source-wavefield store (the snapshot codec).

The linearised Born pair saves the source wavefield every 4 steps as FP32,
BF16 or FP16 (power-of-two max-abs scale per 32x16 block and z plane), and
the adjoint accumulates the zero-lag image in FP32.  The image L'd of each
store is compared with the FP64 oracle of the same algorithm (every quantity
in double, snapshots unquantised); memory of the store and time per step are
reported beside it.

Model family of the 128^3 plain-Born workload (v(z) = 1500 + 0.6 z plus a
Gaussian anomaly, horizons plus spikes, 15 Hz Ricker, dx = 10 m, dt = 1 ms).
Default size: 80^3 and 500 steps (the FP64 oracle's snapshots must fit in host
memory).  SEPX_STUDY_N / SEPX_STUDY_NT override it.  SEPX_PRECISION_FULL=1
adds the 256^3, 2500-step run, against an FP64 oracle that recomputes the
source wavefield from checkpoints (an FP64 snapshot store of that size would
need 160 GB of host memory).
Each test prints one ``PRECISION_STUDY {json}`` line.
"""
import ctypes as C
import json
import os
import time

import numpy as np
import pytest

from sep_code_gb300 import gpu_funcs as gf
from sep_code_gb300 import model as M
from tests.harness import LinCase, rel_l2

pytestmark = pytest.mark.gpu

JS = 4
PRECS = ("f32", "bf16", "f16")
# image relative L2 error against the FP64 oracle: FP32 arithmetic sets the
# floor; the 8-bit (BF16) and 11-bit (FP16) significands of the store add to it
TOL = {"f32": 1e-4, "bf16": 2e-2, "f16": 2e-3}


def _data(case, s, st):
    """Born data of the survey's reflectivity (FP32 store, every step)."""
    m = np.zeros((st.n[2], st.n[1], st.n[0]), np.float32)
    m[:] = st.img_lap
    return case.gpu_forward(m, 1, "f32")


def _gpu_image(case, st, d, prec):
    case.gpu_setup(traces=d)
    gf.synchronize()
    t0 = time.perf_counter()
    gf.lin_source_pass(st.jtd, 9, st.nt, JS, prec)
    gf.synchronize()
    t1 = time.perf_counter()
    gf.lin_adjoint(st.jtd, st.nt, JS, prec)
    gf.synchronize()
    t2 = time.perf_counter()
    img = gf.get_image((st.n[2], st.n[1], st.n[0]))
    return img, (t1 - t0) / st.nt, (t2 - t1) / st.nt


def _oracle_image_f64(oracle, case, s, st, d):
    from oracle.bindings import damp_ntab
    ctx, keep = case.orc_ctx(oracle)
    tab64 = oracle.damp_table(s.bc_a, s.bc_b, damp_ntab(*st.n), f64=True)
    c64 = oracle.make_ctx64(ctx, st.d, tab64, st.sinc_s.astype(np.float64),
                            st.sinc_d.astype(np.float64), case.vals.astype(np.float64), keep)
    vel = st.vel2dt2.astype(np.float64)
    nsnap = (st.nt + JS - 1) // JS
    snaps = np.zeros((nsnap, st.n[2], st.n[1], st.n[0]), np.float64)
    assert oracle.lib.orc_lin_source_f64(C.byref(c64), vel, st.jtd, 9, st.nt, JS, snaps) == 0
    img = np.zeros((st.n[2], st.n[1], st.n[0]), np.float64)
    assert oracle.lib.orc_lin_adjoint_f64(C.byref(c64), vel, st.jtd, st.nt, JS, snaps,
                                          np.ascontiguousarray(d, np.float64), img) == 0
    return img


def test_snapshot_precision_vs_fp64(oracle):
    n = int(os.environ.get("SEPX_STUDY_N", "80"))
    nt = int(os.environ.get("SEPX_STUDY_NT", "500"))
    s = M.anomaly_survey(n=n, nt=nt)
    st = M.prepare_shot(s)
    case = LinCase(s, st)
    d = _data(case, s, st)
    assert np.abs(d).max() > 0
    ref = _oracle_image_f64(oracle, case, s, st, d)
    out = {"grid": f"{n}^3", "padded": "x".join(map(str, st.n)), "steps": st.nt,
           "snapshot_every": JS, "reference": "FP64 oracle (double everywhere, unquantised store)"}
    for prec in PRECS:
        img, t_src, t_adj = _gpu_image(case, st, d, prec)
        err = rel_l2(img, ref)
        out[prec] = {"image_rel_l2_vs_fp64": err,
                     "store_bytes": gf.snapshot_bytes(st.nt, JS, prec),
                     "ms_per_step_source_pass": 1e3 * t_src,
                     "ms_per_step_adjoint": 1e3 * t_adj}
    print("PRECISION_STUDY " + json.dumps(out))
    for prec in PRECS:
        assert out[prec]["image_rel_l2_vs_fp64"] <= TOL[prec], (prec, out[prec])
    assert out["bf16"]["store_bytes"] < 0.55 * out["f32"]["store_bytes"]
    # the FP32 store is the exact FP32 algorithm: the 16-bit stores cost accuracy
    assert out["f32"]["image_rel_l2_vs_fp64"] < out["f16"]["image_rel_l2_vs_fp64"]


def _oracle_image_f64_ckpt(oracle, case, s, st, d, seg):
    """FP64 image with the source wavefield recomputed from checkpoints every
    ``seg`` steps (no full snapshot store; same image as the stored one)."""
    from oracle.bindings import damp_ntab
    ctx, keep = case.orc_ctx(oracle)
    tab64 = oracle.damp_table(s.bc_a, s.bc_b, damp_ntab(*st.n), f64=True)
    c64 = oracle.make_ctx64(ctx, st.d, tab64, st.sinc_s.astype(np.float64),
                            st.sinc_d.astype(np.float64), case.vals.astype(np.float64), keep)
    img = np.zeros((st.n[2], st.n[1], st.n[0]), np.float64)
    assert oracle.lib.orc_lin_adjoint_ckpt_f64(C.byref(c64), st.vel2dt2.astype(np.float64), st.jtd, 9,
                                               st.nt, JS, seg, np.ascontiguousarray(d, np.float64),
                                               img) == 0
    return img


@pytest.mark.skipif(os.environ.get("SEPX_PRECISION_FULL") != "1",
                    reason="256^3 x 2500-step study (about 7 minutes): set SEPX_PRECISION_FULL=1")
def test_snapshot_precision_full_size(oracle):
    """256^3, 2500 steps: every store against the FP64 oracle, whose source
    wavefield is recomputed from checkpoints every 140 steps (an FP64 store of
    625 snapshots would need 160 GB of host memory; the checkpoints and one
    segment's snapshots need about 19 GB)."""
    s = M.anomaly_survey(n=256, nt=2500, seed=20261206)
    st = M.prepare_shot(s)
    case = LinCase(s, st)
    d = _data(case, s, st)
    imgs, out = {}, {"grid": "256^3", "padded": "x".join(map(str, st.n)), "steps": st.nt,
                     "snapshot_every": JS,
                     "reference": "FP64 oracle, source wavefield recomputed from checkpoints"}
    for prec in PRECS:
        img, t_src, t_adj = _gpu_image(case, st, d, prec)
        imgs[prec] = img
        out[prec] = {"store_bytes": gf.snapshot_bytes(st.nt, JS, prec),
                     "ms_per_step_source_pass": 1e3 * t_src,
                     "ms_per_step_adjoint": 1e3 * t_adj}
    t0 = time.perf_counter()
    ref = _oracle_image_f64_ckpt(oracle, case, s, st, d, 140)
    out["oracle_seconds"] = time.perf_counter() - t0
    out["oracle_threads"] = oracle.num_threads()
    for prec in PRECS:
        out[prec]["image_rel_l2_vs_fp64"] = rel_l2(imgs[prec], ref)
    for prec in ("bf16", "f16"):
        out[prec]["image_rel_l2_vs_f32_store"] = rel_l2(imgs[prec], imgs["f32"])
    print("PRECISION_STUDY " + json.dumps(out))
    for prec in PRECS:
        assert out[prec]["image_rel_l2_vs_fp64"] <= TOL[prec], (prec, out[prec])
    assert out["f32"]["image_rel_l2_vs_fp64"] < out["f16"]["image_rel_l2_vs_fp64"]
