"""Synthetic surveys and the per-shot set-up of the Born/RTM operator.

The surveys themselves (``Survey`` and the seeded generators) live in
``surveys.py``, which loads no native code.  ``prepare_shot`` performs
the host-side preparation that ``rtm_zero_op`` does for one shot before each C
ABI call (Born/rtm_zero_op_3d.cpp:8-36, :126-157, :228-262).
"""
from __future__ import annotations

import numpy as np

from . import gpu_funcs as gf
from .surveys import (FAT, ShotSetup, Survey, anomaly_survey, extract_sub,  # noqa: F401
                      laplac_forward, layered_survey, padded_origins, ricker, small_survey)


def padded_grid(s: Survey):
    m3, m2, m1 = s.vel.shape
    n = gf.compute_size(m1, m2, m3, s.nbound, s.nbound, s.nbound, FAT)
    o, d = padded_origins(s)
    return n, o, d


def prepare_shot(s: Survey, ishot: int = 0, nt_big_extra: int = 8, with_image: bool = True) -> ShotSetup:
    n, o, d = padded_grid(s)
    vmax = float(np.float32(s.vel.max()))
    dmin = min(d)   # dx = dy = dz in every workload here (vel_fd_3d::get_min_samp)
    dt, nt = gf.calc_stability(vmax, dmin, s.data_dt, s.data_nt)
    jts = int(np.float32(s.dtw) / np.float32(dt))
    jtd = int(np.float32(s.data_dt) / np.float32(dt))
    sinc_s = gf.sinc_table(jts)
    sinc_d = gf.sinc_table(jtd)
    nt_big = nt_big_extra + s.data_nt
    wd = gf.wavelet_deriv(s.wavelet, s.dtw)
    sx, sy, sz = s.shots[ishot]
    locs, vals = gf.source_func(wd, sx, sy, sz, n[0], n[1], o, d, nt_big)
    seed = int(locs[3]) - (int(locs[3]) // 10000) * 10000
    m3, m2, m1 = s.vel.shape
    vrand = gf.rand_subspace(seed, s.nbound, s.nbound, s.nbound, dt, s.vel, (0.0, 0.0, 0.0), d, n, o, d)
    rnx, rny, ro2, rd2, ro3, rd3 = s.rec
    rec_locs = gf.receiver_map(rnx, rny, ro2, rd2, ro3, rd3, s.rec_depth, n[0], n[1], o, d)
    img_lap = laplac_forward(extract_sub(s, n, o)) if with_image else None
    return ShotSetup(n=n, o=o, d=d, dt=dt, nt=nt, jts=jts, jtd=jtd, sinc_s=sinc_s, sinc_d=sinc_d,
                     src_locs=locs, src_vals=vals, nt_big=nt_big, vel2dt2=vrand, rec_locs=rec_locs,
                     rnx=rnx, rny=rny, img_lap=img_lap)
