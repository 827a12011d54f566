"""CPU restatement of the image / data vector operations that the reference
runs on its out-of-core SEP datasets (test infrastructure only: tests/ use it
to check the device kernels of sepx_image_add_window,
sepx_image_extract_window, sepx_tmute and data_rtm_3d::add_data).

Every value is computed in float32 with the reference's operation order, so
results are compared bit for bit.  The restatement itself is pinned against
the reference's own classes (image_rtm_3d, data_rtm_3d, tmute compiled from
their sources with in-memory datasets, oracle/ref_stubs/ref_shim.cpp).

Layouts: volumes [n3][n2][n1] (axis 1 fastest); traces [..., n2][n1].
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def window_offset(o_in: float, o_out: float, d_out: float) -> int:
    """(int)((o_in - o_out) / d_out) in single precision
    (Born/image_rtm_3d.cpp:33-35, :65-67)"""
    q = (f32(o_in) - f32(o_out)) / f32(d_out)
    return int(np.trunc(q))


def _overlap(n_out: int, n_in: int, f: int):
    """in-index range [a, b) with 0 <= i + f < n_out"""
    a = max(0, -f)
    b = min(n_in, n_out - f)
    return a, max(a, b)


def add_image(img, sub, f):
    """image_rtm_3d::add_image (Born/image_rtm_3d.cpp:24-49): img[j + f] +=
    sub[j] where j + f lies inside img; returns the new img"""
    out = np.array(img, f32, copy=True)
    (a3, b3), (a2, b2), (a1, b1) = (_overlap(out.shape[k], sub.shape[k], f[2 - k]) for k in range(3))
    if a3 < b3 and a2 < b2 and a1 < b1:
        out[a3 + f[2]:b3 + f[2], a2 + f[1]:b2 + f[1], a1 + f[0]:b1 + f[0]] += \
            np.asarray(sub, f32)[a3:b3, a2:b2, a1:b1]
    return out


def extract_sub(img, mute, sub_shape, f):
    """image_rtm_3d::extract_sub (Born/image_rtm_3d.cpp:52-90): sub[j] =
    (img * mute)[j + f], 0 where j + f lies outside img (mute None: 1)"""
    src = np.asarray(img, f32)
    if mute is not None:
        src = src * np.asarray(mute, f32)
    sub = np.zeros(sub_shape, f32)
    (a3, b3), (a2, b2), (a1, b1) = (_overlap(src.shape[k], sub_shape[k], f[2 - k]) for k in range(3))
    if a3 < b3 and a2 < b2 and a1 < b1:
        sub[a3:b3, a2:b2, a1:b1] = src[a3 + f[2]:b3 + f[2], a2 + f[1]:b2 + f[1], a1 + f[0]:b1 + f[0]]
    return sub


def write_volume(img, mute):
    """image_rtm_3d::write_volume (Born/image_rtm_3d.cpp:92-104): img * mute"""
    return np.asarray(img, f32) * np.asarray(mute, f32)


def add_data(all_data, ishot, shot):
    """data_rtm_3d::add_data (Born/data_rtm_3d.cpp:37-51): shot slab ishot +=
    shot; all_data [nshots][n3][n2][n1]"""
    out = np.array(all_data, f32, copy=True)
    out[ishot] += np.asarray(shot, f32).reshape(out.shape[1:])
    return out


def mute_starts(t0, vmute, n1, o1, d1, n2, o2, d2):
    """first passed sample of every trace i2 (Born/tmute.cpp:23-24, :58-59):
    (int)((t_0 + (o2 + d2 i2) / vmute - o1) / d1) in single precision; a start
    before the first sample is taken as 0"""
    i2 = np.arange(n2, dtype=f32)
    tr = f32(t0) + (f32(o2) + f32(d2) * i2) / f32(vmute)
    sf = (tr - f32(o1)) / f32(d1)
    st = np.where(sf >= f32(n1), n1, np.trunc(np.maximum(sf, f32(-1.0)))).astype(np.int64)
    return np.maximum(st, 0)


def tmute(adj: bool, add: bool, t0, vmute, o1, d1, o2, d2, model, data):
    """tmute::forward (data (+)= mask * model) and ::adjoint (model (+)= mask
    * data) (Born/tmute.cpp:4-76) on traces [..., n2][n1]; returns the updated
    (model, data)"""
    model = np.array(model, f32, copy=True)
    data = np.array(data, f32, copy=True)
    n2, n1 = data.shape[-2:]
    st = mute_starts(t0, vmute, n1, o1, d1, n2, o2, d2)
    mask = np.arange(n1)[None, :] >= st[:, None]
    src, dst = (data, model) if adj else (model, data)
    if not add:
        dst[...] = 0.0
    dst[...] = np.where(mask, dst + src, dst)
    return model, data
