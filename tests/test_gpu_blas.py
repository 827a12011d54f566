"""Device BLAS-1 of the operator layer: FP64-accumulated dot against numpy."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dot(lib, a, b, n):
    out = C.c_double()
    rc = lib.sepx_dot_f32(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr() if b is not None else 0),
                          C.c_longlong(n), C.byref(out))
    assert rc == 0, lib.sepx_last_error()
    return out.value


@pytest.mark.parametrize("n", [0, 1, 1000, 1 << 20, 12345677])
def test_dot_fp64(n):
    import torch
    from sep_code_gb300._lib import lib
    from sep_code_gb300 import gpu_funcs as gf
    gf.setup_cuda(1)
    lib.sepx_dot_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.POINTER(C.c_double)]
    g = torch.Generator().manual_seed(n)
    a = torch.randn(n, generator=g)
    b = torch.randn(n, generator=g)
    want = float(np.dot(a.numpy().astype(np.float64), b.numpy().astype(np.float64)))
    da, db = a.cuda(), b.cuda()
    torch.cuda.synchronize()
    got = _dot(lib, da, db, n)
    assert abs(got - want) <= 1e-12 * max(1.0, float(np.sum(np.abs(a.numpy() * b.numpy()))))
    s = _dot(lib, da, None, n)
    assert abs(s - float(a.numpy().astype(np.float64).sum())) <= 1e-9 * max(1.0, n)
