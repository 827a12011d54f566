"""Per-shot set-up built from the oracle alone (test infrastructure).

The same preparation ``rtm_zero_op`` performs before each C ABI call
(Born/rtm_zero_op_3d.cpp:8-36 padded domain and stability, :52-77 source
fields with ``nt_big = nt + 9``, :126-157 forward with ``nt + 8``), computed
by the oracle's restatement of the reference's host math
(``orc_compute_size``, ``orc_calc_stability``, ``orc_sinc_table``,
``orc_wavelet_deriv``, ``orc_source_func``, ``orc_rand_subspace``,
``orc_receiver_map`` in ``sepx_oracle.c``).  The CPU side of the benchmark
(its reference arm and its ``cpu_baseline`` leg) uses this, so it loads no
product library; a CPU test checks that it equals the product's own
``sep_code_gb300.model.prepare_shot`` bit for bit.
"""
from __future__ import annotations

import numpy as np

from sep_code_gb300.surveys import (FAT, ShotSetup, Survey, extract_sub, laplac_forward,
                                    padded_origins)

from .bindings import Oracle, damp_ntab


def prepare_shot(orc: Oracle, s: Survey, ishot: int = 0, nt_big_extra: int = 8,
                 with_image: bool = True) -> ShotSetup:
    m3, m2, m1 = s.vel.shape
    n = orc.compute_size(m1, m2, m3, s.nbound, s.nbound, s.nbound, FAT)
    o, d = padded_origins(s)
    vmax = float(np.float32(s.vel.max()))
    dt, nt = orc.calc_stability(vmax, min(d), s.data_dt, s.data_nt)
    jts = int(np.float32(s.dtw) / np.float32(dt))
    jtd = int(np.float32(s.data_dt) / np.float32(dt))
    nt_big = nt_big_extra + s.data_nt
    wd = orc.wavelet_deriv(s.wavelet, s.dtw)
    sx, sy, sz = s.shots[ishot]
    locs, vals = orc.source_func(wd, sx, sy, sz, n[0], n[1], o, d, nt_big)
    # seed = locs[3] % 10000 (Born/rtm_zero_op_3d.cpp:61)
    seed = int(locs[3]) - (int(locs[3]) // 10000) * 10000
    vrand = orc.rand_subspace(seed, s.nbound, s.nbound, s.nbound, dt, s.vel, (0.0, 0.0, 0.0), d,
                              n, o, d)
    rnx, rny, ro2, rd2, ro3, rd3 = s.rec
    rec_locs = orc.receiver_map(rnx, rny, ro2, rd2, ro3, rd3, s.rec_depth, n[0], n[1], o, d)
    img_lap = laplac_forward(extract_sub(s, n, o)) if with_image else None
    return ShotSetup(n=n, o=o, d=d, dt=dt, nt=nt, jts=jts, jtd=jtd, sinc_s=orc.sinc_table(jts),
                     sinc_d=orc.sinc_table(jtd), src_locs=locs, src_vals=vals, nt_big=nt_big,
                     vel2dt2=vrand, rec_locs=rec_locs, rnx=rnx, rny=rny, img_lap=img_lap)


def source_vals(orc: Oracle, s: Survey, st: ShotSetup, extra: int, ishot: int = 0):
    """Source stencil and traces of length data_nt + extra (the source pass
    uses +9, the Born forward and the adjoint +8)."""
    wd = orc.wavelet_deriv(s.wavelet, s.dtw)
    sx, sy, sz = s.shots[ishot]
    return orc.source_func(wd, sx, sy, sz, st.n[0], st.n[1], st.o, st.d, s.data_nt + extra)


def make_ctx(orc: Oracle, s: Survey, st: ShotSetup, locs, vals, keep: list):
    """The oracle's propagation context for one shot (coefficients, sponge
    table, sinc tables, source and receiver maps)."""
    n1, n2, n3 = st.n
    return orc.make_ctx(st.n, orc.fd_coeffs(*st.d), orc.damp_table(s.bc_a, s.bc_b, damp_ntab(n1, n2, n3)),
                        vals.shape[1], st.sinc_s, st.sinc_d, np.ascontiguousarray(locs, np.int32),
                        np.ascontiguousarray(vals, np.float32),
                        np.ascontiguousarray(st.rec_locs, np.int32), st.rnx, st.rny, keep)
