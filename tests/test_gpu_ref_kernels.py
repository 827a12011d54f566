"""The CUDA path against the reference's own GPU kernels, run on the GB300.

oracle/ref_gpu.py loads the reference's kernels (compiled from
Born/wave_fkernel.3d8o.cu and Born/gpu_funcs_3d.cu into a cubin by
oracle/build_oracle.py) and drives them with the reference's one-GPU loops.
This pins the kernel half of the parity chain on the reference itself: the
CPU oracle is a restatement of those kernels, and here the kernels run.

Tolerance: relative L2 <= 1e-5 on fields, traces and images after the whole
loop.  The two are not bit-identical: the reference is built with -ftz=true
(subnormals flushed), lets nvcc contract its sums into fused multiply-adds
in its own order, evaluates the sponge with expf per cell and forms 1e-6 a b
in double; the measured differences are printed (``pytest -s``).

One exception, measured rather than assumed: the adjoint loop runs the
source wavefield backwards in time from its last two states, and on some
models that reversal amplifies rounding-level differences (on the 24 x 20 x
28, 60-step case a 5e-7 relative perturbation of the two states the CPU
oracle starts from moves its image by 1.1e-3).  Where the image differs from
the reference kernels' by more than 1e-5, the test measures that
sensitivity on the oracle and requires the difference to stay below twice
it: a difference the algorithm's own conditioning explains, not a defect.
"""
import numpy as np
import pytest

from sep_code_gb300 import model as M
from sep_code_gb300 import surveys as S
from tests.harness import GpuShot, rel_l2, source_vals

from oracle.shot_setup import make_ctx
from oracle.shot_setup import prepare_shot as orc_prepare
from oracle.shot_setup import source_vals as orc_source_vals

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def ref():
    from oracle.ref_gpu import RefKernels
    try:
        r = RefKernels()
    except FileNotFoundError as e:
        pytest.skip(str(e))
    yield r
    r.close()


def _ref_loops(ref, s, st):
    n1, n2, n3 = st.n
    ref.create_gpu_space(st.d[0], st.d[1], st.d[2], s.bc_a, s.bc_b, n1, n2, n3)
    ref.transfer_sinc_tables(st.sinc_s, st.sinc_d)
    locs9, vals9 = source_vals(s, st, 9)
    ref.transfer_source_func(locs9, vals9)
    ref.transfer_vel_func1(st.vel2dt2)
    p0, p1 = ref.source_prop(st.jts, 9, st.nt)
    locs8, vals8 = source_vals(s, st, 8)
    ref.transfer_source_func(locs8, vals8)
    ref.transfer_vel_func1(st.vel2dt2)
    nrec = st.rnx * st.rny
    ref.transfer_receiver_func(st.rnx, st.rny, st.rec_locs, np.zeros((nrec, st.nt_big), np.float32))
    traces = ref.rtm_forward(st.jtd, 9, st.nt, st.img_lap)
    ref.transfer_source_func(locs8, vals8)
    ref.transfer_vel_func1(st.vel2dt2)
    ref.transfer_receiver_func(st.rnx, st.rny, st.rec_locs, traces)
    image = ref.rtm_adjoint(st.jtd, 9, st.nt, p1, p0)   # read back swapped, as rtm_zero_op does
    return dict(p0=p0, p1=p1, traces=traces, image=image)


def _our_loops(s, st, ref_out):
    g = GpuShot(s, st)
    p0, p1 = g.source_prop()
    traces = g.rtm_forward(st.img_lap)
    image = g.rtm_adjoint(ref_out["p1"], ref_out["p0"], ref_out["traces"])
    return dict(p0=p0, p1=p1, traces=traces, image=image)


def _image_sensitivity(orc, s, ref_out, rel=5e-7, seed=0):
    """relative change of the oracle's adjoint image when the two source
    states it starts from are perturbed by `rel` (relative, Gaussian)"""
    st = orc_prepare(orc, s)
    keep = []
    locs8, vals8 = orc_source_vals(orc, s, st, 8)
    ctx8 = make_ctx(orc, s, st, locs8, vals8, keep)
    p0, p1, tr = ref_out["p0"], ref_out["p1"], ref_out["traces"]
    base = orc.rtm_adjoint(ctx8, st.vel2dt2, st.jtd, p1, p0, tr, 9, st.nt)
    rng = np.random.default_rng(seed)
    q0 = (p0 * (1 + rel * rng.standard_normal(p0.shape))).astype(np.float32)
    q1 = (p1 * (1 + rel * rng.standard_normal(p1.shape))).astype(np.float32)
    moved = orc.rtm_adjoint(ctx8, st.vel2dt2, st.jtd, q1, q0, tr, 9, st.nt)
    return rel_l2(moved, base)


CASES = {
    "small": lambda: S.small_survey(),
    "ragged": lambda: S.small_survey(m1=37, m2=23, m3=21, nt=40, seed=11),
    "jt2": lambda: S.small_survey(m1=20, m2=20, m3=20, nt=30, seed=3, data_dt=0.004, dtw=0.004),
    "anomaly_128_nt1000": lambda: S.anomaly_survey(),
}


@pytest.mark.parametrize("case", list(CASES))
def test_against_reference_kernels(ref, oracle, case):
    s = CASES[case]()
    st = M.prepare_shot(s)
    want = _ref_loops(ref, s, st)
    got = _our_loops(s, st, want)
    for key in ("p0", "p1", "traces", "image"):
        e = rel_l2(got[key], want[key])
        print(f"REFKERNELS {case} {key}: rel-L2 {e:.3e}, bit-exact {np.array_equal(got[key], want[key])}, "
              f"max |ref| {np.abs(want[key]).max():.3e}")
        assert np.abs(want[key]).max() > 0, (case, key)
        if key == "image" and e > TOL:
            sens = _image_sensitivity(oracle, s, want)
            print(f"REFKERNELS {case} image: oracle sensitivity to 5e-7 in its start states {sens:.3e}")
            assert e <= 2 * sens, (case, key, e, sens)
        else:
            assert e <= TOL, (case, key, e)
