"""Python face of the C ABI (include/sepx.h): the reference's
``Born/gpu_funcs_3d.h`` entry points with numpy buffers, plus the host set-up
math (include/sepx_host.h).  Volumes are ``float32[n3, n2, n1]``, traces
``float32[nrec, ntrace]``.  Every call raises ``SepxError`` on failure."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import SepxError, check, lib, table_ptrs

__all__ = [
    "SepxError", "setup_cuda", "create_gpu_space", "transfer_sinc_table_s", "transfer_sinc_table_d",
    "transfer_source_func", "transfer_receiver_func", "transfer_vel_func1", "transfer_vel_func2",
    "source_prop", "rtm_forward", "rtm_adjoint", "kernel_launches", "device_error", "set_zchunk",
    "sinc_table", "glibc_rand", "rand_subspace", "compute_size", "wavelet_deriv", "source_func",
    "calc_stability", "receiver_map", "synchronize", "reset", "set_tile_rows",
]


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


# ---------------------------------------------------------------- C ABI
def setup_cuda(ngpus: int = 1) -> None:
    check(lib.sepx_setup_cuda(ngpus), "setup_cuda")


def create_gpu_space(d1, d2, d3, bc_a, bc_b, bc_b_y, n1, n2, n3) -> None:
    check(lib.sepx_create_gpu_space(d1, d2, d3, bc_a, bc_b, bc_b_y, n1, n2, n3), "create_gpu_space")


def transfer_sinc_table_s(table) -> None:
    rows, keep = table_ptrs(table)
    check(lib.sepx_transfer_sinc_table_s(keep.shape[1], keep.shape[0], rows), "transfer_sinc_table_s")


def transfer_sinc_table_d(table) -> None:
    rows, keep = table_ptrs(table)
    check(lib.sepx_transfer_sinc_table_d(keep.shape[1], keep.shape[0], rows), "transfer_sinc_table_d")


def transfer_source_func(locs, vals) -> None:
    vals = _f32(vals)
    check(lib.sepx_transfer_source_func(vals.shape[0], vals.shape[1], _i32(locs), vals),
          "transfer_source_func")


def transfer_receiver_func(nx, ny, locs, vals) -> None:
    vals = _f32(vals)
    check(lib.sepx_transfer_receiver_func(nx, ny, vals.shape[1], _i32(locs), vals),
          "transfer_receiver_func")


def transfer_vel_func1(vel) -> None:
    vel = _f32(vel)
    n3, n2, n1 = vel.shape
    check(lib.sepx_transfer_vel_func1(n1, n2, n3, vel), "transfer_vel_func1")


def transfer_vel_func2(vel) -> None:
    vel = _f32(vel)
    n3, n2, n1 = vel.shape
    check(lib.sepx_transfer_vel_func2(n1, n2, n3, vel), "transfer_vel_func2")


def source_prop(shape, jt, npts, nt, get_last=True, damp=False):
    """Returns (p0, p1): the last two source wavefields (older, newest)."""
    n3, n2, n1 = shape
    p0 = np.zeros(shape, np.float32)
    p1 = np.zeros(shape, np.float32)
    check(lib.sepx_source_prop(n1, n2, n3, damp, get_last, p0, p1, jt, npts, nt), "source_prop")
    return p0, p1


def rtm_forward(img, jt, npts_src, nt, nt_big, nx, ny):
    """Born modelling over ``img``; returns the traces float32[nx*ny, nt_big]."""
    img = _f32(img)
    n3, n2, n1 = img.shape
    dat = np.zeros((nx * ny, nt_big), np.float32)
    check(lib.sepx_rtm_forward(n1, n2, n3, jt, img, dat, npts_src, nt, nt_big, nx, ny), "rtm_forward")
    return dat


def rtm_adjoint(p0_s, p1_s, jt, npts, nt):
    """Zero-lag RTM image from the traces given to transfer_receiver_func."""
    p0_s, p1_s = _f32(p0_s), _f32(p1_s)
    n3, n2, n1 = p0_s.shape
    img = np.zeros(p0_s.shape, np.float32)
    check(lib.sepx_rtm_adjoint(n1, n2, n3, jt, p0_s, p1_s, img, npts, nt), "rtm_adjoint")
    return img


# ---------------------------------------------------------------- linearised pair
SNAP_PREC = {"f32": 0, "bf16": 1, "f16": 2}


def set_image(img) -> None:
    check(lib.sepx_set_image(_f32(img)), "set_image")


def get_image(shape):
    out = np.zeros(shape, np.float32)
    check(lib.sepx_get_image(out), "get_image")
    return out


def set_traces(vals) -> None:
    check(lib.sepx_set_traces(_f32(vals)), "set_traces")


def zero_traces() -> None:
    check(lib.sepx_zero_traces(), "zero_traces")


def get_traces(nrec, ntrace):
    out = np.zeros((nrec, ntrace), np.float32)
    check(lib.sepx_get_traces(out), "get_traces")
    return out


def lin_source_pass(jt, npts, nt, js=1, prec="f32") -> None:
    check(lib.sepx_lin_source_pass(jt, npts, nt, js, SNAP_PREC[prec]), "lin_source_pass")


def lin_forward(jt, npts, nt, js=1, prec="f32") -> None:
    """traces (device receiver buffer) += L m, m = the image buffer"""
    check(lib.sepx_lin_forward_resident(jt, npts, nt, js, SNAP_PREC[prec]), "lin_forward")


def lin_adjoint(jt, nt, js=1, prec="f32") -> None:
    """image buffer := L' d, d = the device receiver buffer"""
    check(lib.sepx_lin_adjoint_resident(jt, nt, js, SNAP_PREC[prec]), "lin_adjoint")


def snapshot_bytes(nt, js, prec) -> int:
    return int(lib.sepx_snapshot_bytes(nt, js, SNAP_PREC[prec]))


# ---- image / data vectors kept on the device (device pointers, context stream) ----
def image_add_window(img_ptr, n, f, sub_ptr, s) -> None:
    """image_rtm_3d::add_image: img (n1, n2, n3) cell j + f += sub (s1, s2, s3) cell j"""
    check(lib.sepx_image_add_window(img_ptr, *n, *f, sub_ptr, *s), "image_add_window")


def image_extract_window(img_ptr, mute_ptr, n, f, sub_ptr, s) -> None:
    """image_rtm_3d::extract_sub: sub cell j = (img * mute) cell j + f, 0 outside"""
    check(lib.sepx_image_extract_window(img_ptr, mute_ptr, *n, *f, sub_ptr, *s), "image_extract_window")


def tmute(adj, add, t0, vmute, n1, o1, d1, n2, o2, d2, nrep, model_ptr, data_ptr) -> None:
    """tmute::forward (adj=False) / adjoint on [nrep][n2][n1] traces"""
    check(lib.sepx_tmute(int(adj), int(add), t0, vmute, n1, o1, d1, n2, o2, d2, nrep, model_ptr,
                         data_ptr), "tmute")


def synchronize() -> None:
    check(lib.sepx_synchronize(), "synchronize")


def kernel_launches() -> int:
    return int(lib.sepx_kernel_launches())


def device_error() -> int:
    return int(lib.sepx_device_error())


def set_zchunk(planes: int) -> None:
    check(lib.sepx_set_zchunk(planes), "set_zchunk")


def set_tile_rows(mode: int, rows: int) -> None:
    """Rows per consumer thread of a step kernel: mode 0 source_prop, 1 Born
    forward, 2 RTM adjoint; rows 1 (32 x 16 tile) or 2 (32 x 32 tile)."""
    check(lib.sepx_set_tile_rows(mode, rows), "set_tile_rows")


def reset() -> None:
    check(lib.sepx_reset(), "reset")


# ---------------------------------------------------------------- host set-up math
def sinc_table(ntab: int, nsinc: int = 8) -> np.ndarray:
    out = np.zeros((ntab, nsinc), np.float32)
    lib.sepx_host_sinc_table(ntab, nsinc, out)
    return out


def glibc_rand(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.int32)
    lib.sepx_host_glibc_rand_sequence(seed, n, out)
    return out


def rand_subspace(irand, nr1, nr2, nr3, dt, model, mo, md, sn, so, sd) -> np.ndarray:
    """v^2 dt^2 on the padded grid ``sn`` (n1, n2, n3) with a random boundary."""
    model = _f32(model)
    m3, m2, m1 = model.shape
    out = np.zeros((sn[2], sn[1], sn[0]), np.float32)
    lib.sepx_host_rand_subspace(irand, nr1, nr2, nr3, dt, model, m1, m2, m3, *mo, *md, *sn, *so,
                                *sd, out)
    return out


def compute_size(m1, m2, m3, nbt, nb, nby, fat=4):
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    lib.sepx_host_compute_size(m1, m2, m3, nbt, nb, nby, fat, C.byref(a), C.byref(b), C.byref(c))
    return a.value, b.value, c.value


def wavelet_deriv(w, dt):
    w = _f32(w)
    out = np.zeros_like(w)
    lib.sepx_host_wavelet_deriv(w, len(w), dt, out)
    return out


def source_func(wav_deriv, sx, sy, sz, n1, n2, o, d, nts):
    locs = np.zeros(9, np.int32)
    vals = np.zeros((9, nts), np.float32)
    w = _f32(wav_deriv)
    lib.sepx_host_source_func(w, len(w), sx, sy, sz, n1, n2, *o, *d, nts, locs, vals)
    return locs, vals


def calc_stability(vmax, dmin, data_dt, n_data):
    nt = C.c_int()
    dt = lib.sepx_host_calc_stability(vmax, dmin, data_dt, n_data, C.byref(nt))
    return dt, nt.value


def receiver_map(rnx, rny, ro2, rd2, ro3, rd3, rec_depth, n1, n2, o, d):
    locs = np.zeros(rnx * rny, np.int32)
    lib.sepx_host_receiver_map(rnx, rny, ro2, rd2, ro3, rd3, rec_depth, n1, n2, *o, *d, locs)
    return locs
