"""Generate the golden fixtures of the operator tests from the reference itself.

The reference's rtm_zero_op forward and adjoint are run by its own host C++
(compiled from its sources into oracle/_ref by oracle/build_oracle.py, SEPlib
replaced by in-memory files, the GPU C ABI by the oracle's loops) on three
seeded surveys; the results are stored as float32 .npz next to this script.
Needs the reference tree, so it runs in the build container, not on the GPU
box:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]

CASES = {
    "small": dict(),
    "jt2": dict(m1=20, m2=20, m3=20, nt=30, seed=3, data_dt=0.004, dtw=0.004),
    # 300 steps on a 48 x 40 x 44 model, a 20 x 16 receiver patch
    "medium": dict(m1=48, m2=40, m3=44, nt=300, seed=9, rnx=20, rny=16, nbound=8),
}
# cases whose observed traces come from hashed_traces instead of the fixture
HASHED_OBS = {"medium": 12}


def hashed_traces(shape, seed):
    """Observed traces from an integer hash (splitmix64 of the sample index):
    the same float32 values on every machine and numpy version, so the fixture
    need not store them.  Values k / 2^24 - 1/2, exact in float32."""
    m = (1 << 64) - 1
    off = np.uint64((seed * 0x9E3779B97F4A7C15) & m)
    z = np.arange(int(np.prod(shape)), dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15) + off
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(40)).astype(np.float64) / float(1 << 24) - 0.5
    return u.astype(np.float32).reshape(shape)


def main():
    sys.path.insert(0, str(ROOT))
    from oracle.bindings import RefHost, RefOperator
    from sep_code_gb300 import model as M
    ref = RefOperator(RefHost())
    for name, kw in CASES.items():
        s = M.small_survey(**kw)
        data = ref.born_forward(s)
        rnx, rny = s.rec[0], s.rec[1]
        if name in HASHED_OBS:
            obs = hashed_traces((rny, rnx, s.data_nt), HASHED_OBS[name])
        else:
            rng = np.random.default_rng(11)
            obs = rng.standard_normal((rny, rnx, s.data_nt)).astype(np.float32)
        image = ref.rtm_adjoint(s, obs)
        out = dict(data=data, image=image)
        if name not in HASHED_OBS:
            out["obs"] = obs
        np.savez_compressed(Path(__file__).parent / f"rtm_zero_op_{name}.npz", **out)
        print(name, data.shape, image.shape, float(np.abs(data).max()), float(np.abs(image).max()))


if __name__ == "__main__":
    main()
