"""The allocation-free dot product (sepx_dot_f32_noalloc) against the library's
regular one (sepx_dot_f32), through the C ABI.

The no-allocation entry point exists for callers that cannot let a library
allocate device memory -- services that reserve their whole device-memory
budget up front, or hosts whose own pool owns every allocation.  They pass
device inputs and a device output; the scratch is a fixed file-scope device
array.  This file is collected last so that a run stopping at the first
failure has already run every other test; it also passes on its own.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12   # the FP64 tolerance of the other dot-product tests


def _lib():
    from sep_code_gb300 import gpu_funcs as gf
    from sep_code_gb300._lib import lib
    gf.setup_cuda(1)
    lib.sepx_dot_f32_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p,
                                         C.c_void_p]
    lib.sepx_dot_f32_noalloc.restype = C.c_int
    lib.sepx_dot_f32_noalloc_max_elems.restype = C.c_longlong
    return lib


def _regular(lib, a, b, n):
    out = C.c_double()
    rc = lib.sepx_dot_f32(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), C.c_longlong(n),
                          C.byref(out))
    assert rc == 0, lib.sepx_last_error()
    return out.value


def _noalloc(lib, a, b, n, res, stream):
    rc = lib.sepx_dot_f32_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                  C.c_longlong(n), C.c_void_p(res.data_ptr()),
                                  C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.sepx_last_error()
    stream.synchronize()
    return float(res.item())


def test_noalloc_dot_matches_regular_twice_in_a_row():
    import torch
    lib = _lib()
    stream = torch.cuda.Stream()
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    g = torch.Generator(device="cpu").manual_seed(2024)
    for n in (3_000_001, 777):                       # two calls in a row
        a = torch.randn(n, generator=g).cuda()
        b = torch.randn(n, generator=g).cuda()
        torch.cuda.synchronize()
        want = _regular(lib, a, b, n)
        got = _noalloc(lib, a, b, n, res, stream)
        scale = float(torch.sum(torch.abs(a.double() * b.double())).item())
        assert abs(got - want) <= RTOL * max(1.0, scale), (n, got, want)
        ref = float(np.dot(a.cpu().numpy().astype(np.float64), b.cpu().numpy().astype(np.float64)))
        assert abs(got - ref) <= RTOL * max(1.0, scale)


def test_noalloc_dot_rejects_sizes_beyond_its_scratch():
    import torch
    lib = _lib()
    limit = int(lib.sepx_dot_f32_noalloc_max_elems())
    assert limit == 268_435_456
    a = torch.zeros(4, device="cuda")
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = lib.sepx_dot_f32_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()),
                                  C.c_longlong(limit + 1), C.c_void_p(res.data_ptr()), None)
    assert rc != 0
    assert b"exceeds the fixed scratch limit" in lib.sepx_last_error()


@pytest.mark.parametrize("n", [8192, 8193, 1])
def test_noalloc_dot_chunk_boundaries(n):
    """sizes at and just past one block's chunk of 8192 elements"""
    import torch
    lib = _lib()
    stream = torch.cuda.Stream()
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    g = torch.Generator(device="cpu").manual_seed(n)
    a = torch.randn(n, generator=g).cuda()
    b = torch.randn(n, generator=g).cuda()
    torch.cuda.synchronize()
    want = _regular(lib, a, b, n)
    got = _noalloc(lib, a, b, n, res, stream)
    scale = float(torch.sum(torch.abs(a.double() * b.double())).item())
    assert abs(got - want) <= RTOL * max(1.0, scale)


def test_noalloc_dot_null_b_sums_a_and_empty_is_zero():
    import torch
    lib = _lib()
    stream = torch.cuda.Stream()
    res = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    a = torch.randn(50_000, generator=torch.Generator(device="cpu").manual_seed(5)).cuda()
    torch.cuda.synchronize()
    rc = lib.sepx_dot_f32_noalloc(C.c_void_p(a.data_ptr()), None, C.c_longlong(a.numel()),
                                  C.c_void_p(res.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == 0
    stream.synchronize()
    want = float(torch.sum(a.double()).item())
    assert abs(float(res.item()) - want) <= RTOL * max(1.0, float(torch.sum(torch.abs(a.double()))))
    res.fill_(float("nan"))
    torch.cuda.synchronize()
    rc = lib.sepx_dot_f32_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()), C.c_longlong(0),
                                  C.c_void_p(res.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == 0
    stream.synchronize()
    assert float(res.item()) == 0.0


def test_noalloc_dot_rejects_invalid_arguments():
    import torch
    lib = _lib()
    a = torch.zeros(4, device="cuda")
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert lib.sepx_dot_f32_noalloc(C.c_void_p(a.data_ptr()), None, C.c_longlong(-1),
                                    C.c_void_p(res.data_ptr()), None) != 0
    assert lib.sepx_dot_f32_noalloc(C.c_void_p(a.data_ptr()), None, C.c_longlong(4), None, None) != 0
    assert lib.sepx_dot_f32_noalloc(None, None, C.c_longlong(4), C.c_void_p(res.data_ptr()), None) != 0
    assert b"invalid arguments" in lib.sepx_last_error()


def test_noalloc_dot_before_any_other_entry_point():
    """in a fresh process the entry point works as the library's first call:
    no setup_cuda, no other sepx function before it"""
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    code = r'''
import ctypes as C, sys, torch
sys.path.insert(0, sys.argv[1])
from sep_code_gb300 import LIB_PATH
lib = C.CDLL(str(LIB_PATH))
lib.sepx_dot_f32_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
a = torch.arange(1, 20001, dtype=torch.float32, device="cuda")
res = torch.zeros(1, dtype=torch.float64, device="cuda")
torch.cuda.synchronize()
for _ in range(2):
    assert lib.sepx_dot_f32_noalloc(a.data_ptr(), a.data_ptr(), 20000, res.data_ptr(), None) == 0
    torch.cuda.synchronize()
    n = 20000
    assert float(res.item()) == n * (n + 1) * (2 * n + 1) / 6, float(res.item())
print("OK")
'''
    r = subprocess.run([sys.executable, "-c", code, str(root)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr
