"""A compiled C++ program that drives the operator the way the reference's
least-squares RTM program does (tests/cpp/rtm_inv_driver.cpp, after
Born/RTM_inv.cpp:14-68: rtm_zero_op through the reference's constructor,
simple_solver + cgstep, solve, return_model) gives the same image and the
same residual sequence, bit for bit, as the C API path (sepx_rtm_op_create +
sepx_lsrtm) on the same survey."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from sep_code_gb300 import surveys as S

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_rtm_inv_driver_matches_c_api(tmp_path):
    from sep_code_gb300 import LIB_PATH
    from sep_code_gb300.operator import RtmOperator
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "rtm_inv_driver"
    subprocess.run([cxx, "-std=c++17", "-O1", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "rtm_inv_driver.cpp"), str(LIB_PATH),
                    f"-Wl,-rpath,{Path(LIB_PATH).parent}", "-o", str(exe)], check=True)
    s = S.small_survey(m1=24, m2=20, m3=24, nt=80, seed=17)
    # 2 x 2 shots on the shot axes 4 and 5 of the data (x fastest)
    nsx, osx, dsx, nsy, osy, dsy = 2, 70.0, 100.0, 2, 60.0, 80.0
    s.shots = [(osx + dsx * i, osy + dsy * j, 0.0) for j in range(nsy) for i in range(nsx)]
    niter = 4
    op = RtmOperator(s, "reference")
    data = op.forward(s.refl)
    assert np.abs(data).max() > 0
    model_c, resid_c, _ = op.lsrtm(data, niter)
    op.close()

    m3, m2, m1 = s.vel.shape
    rnx, rny, ro2, rd2, ro3, rd3 = s.rec
    dims = [m1, m2, m3, s.spacing[0], s.data_nt, s.data_dt, rnx, rny, ro2, rd2, ro3, rd3,
            nsx, osx, dsx, nsy, osy, dsy, 0.0, s.nbound, s.bc_a, s.bc_b, niter, len(s.wavelet), s.dtw]
    for name, arr in (("dims", dims), ("vel", s.vel), ("wavelet", s.wavelet), ("data", data)):
        np.ascontiguousarray(arr, np.float32).tofile(tmp_path / f"{name}.bin")
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    model_d = np.fromfile(tmp_path / "model.bin", np.float32).reshape(model_c.shape)
    resid_d = np.fromfile(tmp_path / "resid.bin", np.float64)
    assert len(resid_d) == niter and np.all(np.diff(resid_d) < 0), resid_d
    assert np.array_equal(resid_d, resid_c), (resid_d, resid_c)
    assert np.abs(model_c).max() > 0
    assert np.array_equal(model_d, model_c)


def test_drop_in_constructor_checks_its_inputs(tmp_path):
    """Shot positions that do not match the data's shot axes are an error
    from the constructor (C++ exception), not a wrong image."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    from sep_code_gb300 import LIB_PATH
    src = tmp_path / "bad.cpp"
    src.write_text(r'''
#include <cstdio>
#include <stdexcept>
#include "sepx.h"
#include "sepx_ops.h"
int main() {
  sepx_setup_cuda(1);
  float v[8 * 8 * 8], w[16] = {0, 1, 0};
  for (float &x : v) x = 1500.f;
  param_func par;
  par.set("nbound", 4).set("bc_a", 20.0);
  vel_fd_3d vel({axis(8, 0.f, 10.f), axis(8, 0.f, 10.f), axis(8, 0.f, 10.f)}, v);
  image_rtm_3d img("image", &vel);
  source_func src(axis(16, 0.f, 0.002f), w);
  src.set_sources_3d(0.f, axis(1, 30.f, 10.f), axis(1, 30.f, 10.f));
  data_rtm_3d dat({axis(16, 0.f, 0.002f), axis(4, 20.f, 10.f), axis(4, 20.f, 10.f), axis(2), axis(1)}, &par);
  try {
    rtm_zero_op op(&par, &vel, &src, &dat, &img, 8.f, false, false, nullptr);
  } catch (const std::exception &e) {
    printf("%s\n", e.what());
    return 0;
  }
  return 1;
}
''')
    exe = tmp_path / "bad"
    subprocess.run([cxx, "-std=c++17", "-O1", f"-I{ROOT / 'include'}", str(src), str(LIB_PATH),
                    f"-Wl,-rpath,{Path(LIB_PATH).parent}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "source positions" in r.stdout
