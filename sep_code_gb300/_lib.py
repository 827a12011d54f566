"""ctypes binding of the native library (``_build/libsepx.so``).

The library is the product: every propagation runs in its sm_103a kernels.
There is no fallback -- if the library is missing, importing this module raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "libsepx.so"

F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
PP = C.POINTER(C.POINTER(C.c_float))


class SepxError(RuntimeError):
    pass


def _load() -> C.CDLL:
    if not _LIB_PATH.exists():
        raise ImportError(f"{_LIB_PATH} is not built: run `python -m sep_code_gb300.build` "
                          "(or __graft_entry__.build()) first")
    L = C.CDLL(str(_LIB_PATH))
    i, f, b = C.c_int, C.c_float, C.c_bool
    sig = {
        "sepx_setup_cuda": [i],
        "sepx_create_gpu_space": [f, f, f, f, f, f, i, i, i],
        "sepx_transfer_sinc_table_s": [i, i, PP],
        "sepx_transfer_sinc_table_d": [i, i, PP],
        "sepx_transfer_source_func": [i, i, I32P, F32P],
        "sepx_transfer_receiver_func": [i, i, i, I32P, F32P],
        "sepx_transfer_vel_func1": [i, i, i, F32P],
        "sepx_transfer_vel_func2": [i, i, i, F32P],
        "sepx_source_prop": [i, i, i, b, b, F32P, F32P, i, i, i],
        "sepx_rtm_forward": [i, i, i, i, F32P, F32P, i, i, i, i, i],
        "sepx_rtm_adjoint": [i, i, i, i, F32P, F32P, F32P, i, i],
        "sepx_source_prop_resident": [i, i, i],
        "sepx_rtm_forward_resident": [i, i, i],
        "sepx_rtm_adjoint_resident": [i, i, i, i],
        "sepx_set_image": [F32P],
        "sepx_get_image": [F32P],
        "sepx_set_source_fields": [F32P, F32P],
        "sepx_get_source_fields": [F32P, F32P],
        "sepx_set_traces": [F32P],
        "sepx_get_traces": [F32P],
        "sepx_synchronize": [],
        "sepx_zero_traces": [],
        "sepx_device_error": [],
        "sepx_set_zchunk": [i],
        "sepx_set_tile_rows": [i, i],
        "sepx_reset": [],
        "sepx_lin_source_pass": [i, i, i, i, i],
        "sepx_lin_forward_resident": [i, i, i, i, i],
        "sepx_lin_adjoint_resident": [i, i, i, i],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    L.sepx_last_error.restype = C.c_char_p
    L.sepx_kernel_launches.restype = C.c_longlong
    L.sepx_get_stream.restype = C.c_void_p
    L.sepx_snapshot_bytes.argtypes = [i, i, i]
    L.sepx_snapshot_bytes.restype = C.c_longlong
    L.sepx_dot_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.POINTER(C.c_double)]
    L.sepx_dot_f32.restype = C.c_int
    # image / data vectors on the device (device pointers)
    vp = C.c_void_p
    L.sepx_image_add_window.argtypes = [vp, i, i, i, i, i, i, vp, i, i, i]
    L.sepx_image_extract_window.argtypes = [vp, vp, i, i, i, i, i, i, vp, i, i, i]
    L.sepx_tmute.argtypes = [i, i, f, f, i, f, f, i, f, f, C.c_longlong, vp, vp]
    for name in ("sepx_image_add_window", "sepx_image_extract_window", "sepx_tmute"):
        getattr(L, name).restype = C.c_int
    # host set-up math
    L.sepx_host_sinc_table.argtypes = [i, i, F32P]
    L.sepx_host_glibc_rand_sequence.argtypes = [C.c_uint, i, I32P]
    L.sepx_host_rand_subspace.argtypes = [i, i, i, i, f, F32P, i, i, i, f, f, f, f, f, f, i, i, i,
                                          f, f, f, f, f, f, F32P]
    L.sepx_host_compute_size.argtypes = [i] * 7 + [C.POINTER(C.c_int)] * 3
    L.sepx_host_wavelet_deriv.argtypes = [F32P, i, f, F32P]
    L.sepx_host_source_func.argtypes = [F32P, i, f, f, f, i, i, f, f, f, f, f, f, i, I32P, F32P]
    L.sepx_host_calc_stability.argtypes = [f, f, f, i, C.POINTER(C.c_int)]
    L.sepx_host_calc_stability.restype = f
    L.sepx_host_receiver_map.argtypes = [i, i, f, f, f, f, f, i, i, f, f, f, f, f, f, I32P]
    return L


lib = _load()


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        msg = lib.sepx_last_error().decode(errors="replace")
        raise SepxError(f"{what}: {msg}" if what else msg)


def table_ptrs(tab: np.ndarray):
    """float** view of the rows of a C-contiguous float32 2-D array."""
    tab = np.ascontiguousarray(tab, np.float32)
    rows = (C.POINTER(C.c_float) * tab.shape[0])()
    base = tab.ctypes.data
    for r in range(tab.shape[0]):
        rows[r] = C.cast(base + r * tab.strides[0], C.POINTER(C.c_float))
    return rows, tab
