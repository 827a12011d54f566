"""Argument checks of the least-squares entry points, on the CPU (they fail
before any device work): a NULL operator, a negative iteration count and an
unknown direction policy are errors with a message, not memory overruns."""
import ctypes as C

import numpy as np


def test_lsrtm_rejects_bad_arguments():
    from sep_code_gb300._lib import lib
    from sep_code_gb300.operator import LsrtmOpts
    d = np.zeros(8, np.float32)
    m = np.zeros(8, np.float32)
    r = np.zeros(4)
    s = np.zeros(4)
    u = np.zeros(4, np.int32)
    fb = C.c_int(-1)
    done = C.c_int(-1)
    assert lib.sepx_lsrtm(None, d, 4, m, r, s, None, None, 0.0, C.byref(fb)) != 0
    assert b"NULL" in lib.sepx_last_error()
    assert lib.sepx_lsrtm(C.c_void_p(1), d, -3, m, r, s, None, None, 0.0, C.byref(fb)) != 0
    assert b"niter" in lib.sepx_last_error()
    opts = LsrtmOpts(None, None, 0, 0.0, 8, 0.0)
    assert lib.sepx_lsrtm_ex(C.c_void_p(1), d, -1, C.byref(opts), m, r, s, u, C.byref(done)) != 0
    assert b"niter" in lib.sepx_last_error()
    opts.policy = 7
    assert lib.sepx_lsrtm_ex(C.c_void_p(1), d, 2, C.byref(opts), m, r, s, u, C.byref(done)) != 0
    assert b"policy" in lib.sepx_last_error()
    assert lib.sepx_lsrtm_ex(C.c_void_p(1), d, 2, None, m, r, s, u, C.byref(done)) != 0
    assert done.value == -1   # nothing ran
