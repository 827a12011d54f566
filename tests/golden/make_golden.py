"""Generate the golden fixtures of the operator tests from the reference itself.

The reference's rtm_zero_op forward and adjoint are run by its own host C++
(compiled from its sources into oracle/_ref by oracle/build_oracle.py, SEPlib
replaced by in-memory files, the GPU C ABI by the oracle's loops) on two small
seeded surveys; the results are stored as float32 .npz next to this script.
Needs the reference tree, so it runs in the build container, not on the GPU
box:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.bindings import RefHost, RefOperator  # noqa: E402
from sep_code_gb300 import model as M  # noqa: E402

CASES = {
    "small": dict(),
    "jt2": dict(m1=20, m2=20, m3=20, nt=30, seed=3, data_dt=0.004, dtw=0.004),
}


def main():
    ref = RefOperator(RefHost())
    for name, kw in CASES.items():
        s = M.small_survey(**kw)
        data = ref.born_forward(s)
        rng = np.random.default_rng(11)
        rnx, rny = s.rec[0], s.rec[1]
        obs = rng.standard_normal((rny, rnx, s.data_nt)).astype(np.float32)
        image = ref.rtm_adjoint(s, obs)
        np.savez_compressed(Path(__file__).parent / f"rtm_zero_op_{name}.npz", data=data, obs=obs,
                            image=image)
        print(name, data.shape, image.shape, float(np.abs(data).max()), float(np.abs(image).max()))


if __name__ == "__main__":
    main()
