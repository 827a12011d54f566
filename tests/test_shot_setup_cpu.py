"""The oracle-side shot preparation (used by the CPU arm of the benchmark)
equals the product's own, bit for bit, on every survey family."""
import numpy as np
import pytest

from oracle.shot_setup import prepare_shot as orc_prepare
from oracle.shot_setup import source_vals as orc_source_vals
from sep_code_gb300 import model as M
from sep_code_gb300 import surveys as S
from tests.harness import source_vals


@pytest.mark.parametrize("make", [
    lambda: S.small_survey(),
    lambda: S.small_survey(m1=37, m2=23, m3=21, nt=40, seed=11),
    lambda: S.small_survey(m1=20, m2=20, m3=20, nt=30, seed=3, data_dt=0.004, dtw=0.004),
    lambda: S.anomaly_survey(n=40, nt=50),
    lambda: S.layered_survey(48, 40, 36, nt=30),
], ids=["small", "ragged", "jt2", "anomaly40", "layered48"])
def test_oracle_setup_matches_product(make, oracle):
    s = make()
    a = M.prepare_shot(s)
    b = orc_prepare(oracle, s)
    for f in ("n", "o", "d", "nt", "jts", "jtd", "nt_big", "rnx", "rny"):
        assert getattr(a, f) == getattr(b, f), f
    assert np.float32(a.dt) == np.float32(b.dt)
    for f in ("sinc_s", "sinc_d", "src_locs", "src_vals", "vel2dt2", "rec_locs", "img_lap"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f
    for extra in (8, 9):
        la, va = source_vals(s, a, extra)
        lb, vb = orc_source_vals(oracle, s, b, extra)
        assert np.array_equal(la, lb) and np.array_equal(va, vb)


def test_surveys_module_loads_no_library():
    import subprocess
    import sys
    code = ("import sys; import sep_code_gb300.surveys, oracle.shot_setup; "
            "bad = [m for m in sys.modules if m.startswith('sep_code_gb300.') and "
            "m not in ('sep_code_gb300.surveys',)]; print(bad); sys.exit(1 if bad else 0)")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                       cwd=str(__import__("pathlib").Path(__file__).resolve().parent.parent))
    assert r.returncode == 0, r.stdout + r.stderr
