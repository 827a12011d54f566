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


def test_operator_calls_reject_null_arguments():
    from sep_code_gb300 import build
    from sep_code_gb300._lib import lib  # noqa: F401  (builds the library if needed)
    L = C.CDLL(str(build.LIB))
    L.sepx_last_error.restype = C.c_char_p
    L.sepx_rtm_op_create.restype = C.c_void_p
    L.sepx_rtm_op_model_size.restype = C.c_longlong
    L.sepx_rtm_op_data_size.restype = C.c_longlong
    buf = np.zeros(8, np.float32)
    bp = C.c_void_p(buf.ctypes.data)
    assert L.sepx_rtm_op_create(None) is None
    assert b"NULL" in L.sepx_last_error()
    assert L.sepx_rtm_op_model_size(None) == -1
    assert L.sepx_rtm_op_data_size(None) == -1
    assert L.sepx_rtm_op_forward(None, 0, bp, bp) != 0
    assert L.sepx_rtm_op_adjoint(C.c_void_p(1), 0, None, bp) != 0
    assert L.sepx_rtm_op_dot_test(None, C.c_ulonglong(1), None) != 0
    assert b"NULL" in L.sepx_last_error()
