"""Full-loop parity: the CUDA path against the oracle after whole time loops.

* The 128^3 anomaly model (padded 176 x 176 x 224, dx 10 m, dt 1 ms, 1000
  steps, 128 x 128 surface receivers): ``source_prop`` (both returned
  fields), ``rtm_forward`` (traces) and ``rtm_adjoint`` (image).
* A 100-step window of the same three loops on the 512 x 512 x 400 layered
  model (padded 560 x 560 x 496, 262,144 receivers), with a random
  reflectivity (100 steps reach no interface of the model and back).

Each side prepares its inputs with its own set-up code: the GPU side with the
product's host math (``sep_code_gb300.model.prepare_shot``), the oracle side
with the oracle's restatement of the reference's host math
(``oracle.shot_setup``).  Each loop is compared twice: fed the oracle's own
inputs (so one loop's difference cannot hide in the next) and chained on the
GPU (its own source fields and traces feed its adjoint).

Tolerance: relative L2 <= 1e-5 on FP32 traces, fields and images (the
parity bar for this path).  Whether the results are also bit-identical is
reported on stdout (``pytest -s``) and asserted nowhere: it is a finding, not
a requirement.  Loops: Born/gpu_funcs_3d.cu:133-315 (source_prop),
:317-505 (rtm_forward), :509-712 (rtm_adjoint).
"""
import numpy as np
import pytest

from oracle.shot_setup import make_ctx
from oracle.shot_setup import prepare_shot as orc_prepare
from oracle.shot_setup import source_vals as orc_source_vals
from sep_code_gb300 import model as M
from sep_code_gb300 import surveys as S
from tests.harness import GpuShot, rel_l2

TOL = 1e-5
pytestmark = pytest.mark.gpu


def _oracle_loops(orc, s):
    st = orc_prepare(orc, s)
    keep = []
    locs9, vals9 = orc_source_vals(orc, s, st, 9)
    ctx9 = make_ctx(orc, s, st, locs9, vals9, keep)
    p0, p1 = orc.source_prop(ctx9, st.vel2dt2, st.jts, 9, st.nt)
    locs8, vals8 = orc_source_vals(orc, s, st, 8)
    ctx8 = make_ctx(orc, s, st, locs8, vals8, keep)
    dat = np.zeros((st.rnx * st.rny, st.nt_big), np.float32)
    traces = orc.rtm_forward(ctx8, st.vel2dt2, st.jtd, np.ascontiguousarray(st.img_lap), dat, 9,
                             st.nt)
    img = orc.rtm_adjoint(ctx8, st.vel2dt2, st.jtd, p1, p0, traces, 9, st.nt)
    return dict(p0=p0, p1=p1, traces=traces, image=img)


def _gpu_loops(s, ref):
    st = M.prepare_shot(s)
    g = GpuShot(s, st)
    p0, p1 = g.source_prop()
    traces = g.rtm_forward(st.img_lap)
    img_fed = g.rtm_adjoint(ref["p1"], ref["p0"], ref["traces"])
    img_chain = g.rtm_adjoint(p1, p0, traces)
    return dict(p0=p0, p1=p1, traces=traces, image=img_fed, image_chained=img_chain)


def _compare(name, gpu, ref):
    rows = []
    for key, want in (("p0", "p0"), ("p1", "p1"), ("traces", "traces"), ("image", "image"),
                      ("image_chained", "image")):
        e = rel_l2(gpu[key], ref[want])
        same = bool(np.array_equal(gpu[key], ref[want]))
        rows.append((key, e, same))
        print(f"PARITY {name} {key}: rel-L2 {e:.3e}, bit-exact {same}, "
              f"max |ref| {np.abs(ref[want]).max():.3e}")
    for key, e, _ in rows:
        assert e <= TOL, (name, key, e)
    for key in ("p1", "traces", "image"):
        assert np.abs(ref[key]).max() > 0, (name, key)


@pytest.fixture(scope="module")
def anomaly(oracle):
    s = S.anomaly_survey()
    return s, _oracle_loops(oracle, s)


def test_anomaly_128_full_loops(anomaly):
    s, ref = anomaly
    st = M.prepare_shot(s)
    assert st.n == (176, 176, 224) and st.nt == 1000 and st.rnx * st.rny == 128 * 128
    _compare("anomaly_128_nt1000", _gpu_loops(s, ref), ref)


def test_layered_full_grid_100_steps(oracle):
    s = S.layered_survey(nt=100)
    # 100 steps reach no interface of the layered model and back: a seeded
    # random reflectivity everywhere makes the Born traces and the image
    # non-zero within the window
    rng = np.random.default_rng(20261206)
    s.refl = (0.01 * rng.standard_normal(s.refl.shape)).astype(np.float32)
    ref = _oracle_loops(oracle, s)
    st = M.prepare_shot(s, with_image=False)
    assert st.n == (560, 560, 496) and st.nt == 100
    _compare("layered_560x560x496_nt100", _gpu_loops(s, ref), ref)
