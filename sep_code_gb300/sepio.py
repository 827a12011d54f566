"""SEP regular datasets (``name.H`` header + binary data) to and from numpy
arrays or device buffers, through the library's reader / writer
(include/sepx_sepio.h; the reference uses SEPlib, Born/sreg.cpp, sregf.cpp).

Arrays are indexed [n_ndim, ..., n2, n1] (axis 1 fastest), float32.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib

MAX_AXES = 8
_I8 = C.c_int * MAX_AXES
_F8 = C.c_float * MAX_AXES
lib.sepx_sep_info.argtypes = [C.c_char_p, C.POINTER(C.c_int), _I8, _F8, _F8]
lib.sepx_sep_par.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]
lib.sepx_sep_read.argtypes = [C.c_char_p, C.c_longlong, C.c_longlong, C.c_void_p, C.c_int]
lib.sepx_sep_read_window.argtypes = [C.c_char_p, _I8, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
lib.sepx_sep_write.argtypes = [C.c_char_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p,
                               C.c_void_p, C.c_int, C.c_int]
for _f in ("sepx_sep_info", "sepx_sep_par", "sepx_sep_read", "sepx_sep_read_window", "sepx_sep_write"):
    getattr(lib, _f).restype = C.c_int


def _b(path) -> bytes:
    return str(path).encode()


def info(path):
    """(ndim, n[8], o[8], d[8]) of a dataset"""
    nd = C.c_int()
    n, o, d = _I8(), _F8(), _F8()
    check(lib.sepx_sep_info(_b(path), C.byref(nd), n, o, d), "sep_info")
    return nd.value, list(n), list(o), list(d)


def par(path, key, default=None):
    """a header value as a string (default when the header does not set it)"""
    buf = C.create_string_buffer(4096)
    rc = lib.sepx_sep_par(_b(path), key.encode(), buf, len(buf))
    if rc == 1:
        return default
    check(rc, "sep_par")
    return buf.value.decode()


def shape_of(path):
    nd, n, _, _ = info(path)
    return tuple(n[:nd][::-1])


def read(path, first: int = 0, count: int | None = None) -> np.ndarray:
    """the data (or `count` elements from element `first`, flat) into host memory"""
    shp = shape_of(path)
    total = int(np.prod(shp))
    whole = first == 0 and count is None
    count = total - first if count is None else count
    out = np.empty(count, np.float32)
    check(lib.sepx_sep_read(_b(path), first, count, out.ctypes.data, 0), "sep_read")
    return out.reshape(shp) if whole else out


def _window(path, nw, fw, jw):
    nd, n, _, _ = info(path)
    N = _I8(*([*nw] + n[len(nw):]))
    F = _I8(*([*(fw or [0] * len(nw))] + [0] * (MAX_AXES - len(nw))))
    J = _I8(*([*(jw or [1] * len(nw))] + [1] * (MAX_AXES - len(nw))))
    return nd, N, F, J


def read_window(path, nw, fw=None, jw=None) -> np.ndarray:
    """sregf::read_slice: nw / fw / jw per axis (axis 1 first)"""
    nd, N, F, J = _window(path, nw, fw, jw)
    out = np.empty(int(np.prod(list(N))), np.float32)
    check(lib.sepx_sep_read_window(_b(path), N, F, J, out.ctypes.data, 0), "sep_read_window")
    return out.reshape([N[i] for i in range(max(nd, len(nw)))][::-1])


def read_window_to_device(path, dst_ptr: int, nw, fw=None, jw=None) -> None:
    """read_window into a device buffer of prod(nw) elements"""
    _, N, F, J = _window(path, nw, fw, jw)
    check(lib.sepx_sep_read_window(_b(path), N, F, J, dst_ptr, 1), "sep_read_window")


def write(path, a, o=None, d=None, labels=None, xdr: bool = True) -> None:
    """a [.., n2, n1] float32 -> path (header) + path@ (data)"""
    a = np.ascontiguousarray(a, np.float32)
    n = list(a.shape[::-1]) or [1]
    nd = len(n)
    N = (C.c_int * nd)(*n)
    O = (C.c_float * nd)(*(o or [0.0] * nd))
    D = (C.c_float * nd)(*(d or [1.0] * nd))
    lab = "\n".join(labels).encode() if labels else None
    check(lib.sepx_sep_write(_b(path), nd, N, O, D, lab, a.ctypes.data, 0, int(xdr)), "sep_write")


def read_to_device(path, dst_ptr: int, first: int = 0, count: int | None = None) -> None:
    """read into a device buffer (float32, `count` elements)"""
    if count is None:
        count = int(np.prod(shape_of(path))) - first
    check(lib.sepx_sep_read(_b(path), first, count, dst_ptr, 1), "sep_read")


def write_from_device(path, src_ptr: int, n, o=None, d=None, labels=None, xdr: bool = True) -> None:
    """write a device buffer of axes n (axis 1 first)"""
    nd = len(n)
    N = (C.c_int * nd)(*n)
    O = (C.c_float * nd)(*(o or [0.0] * nd))
    D = (C.c_float * nd)(*(d or [1.0] * nd))
    lab = "\n".join(labels).encode() if labels else None
    check(lib.sepx_sep_write(_b(path), nd, N, O, D, lab, src_ptr, 1, int(xdr)), "sep_write")
