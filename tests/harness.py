"""Shared drivers for the parity tests: the same shot through the CUDA path
(via the C ABI) and through the oracle (CPU restatement of the reference)."""
from __future__ import annotations

import numpy as np

from oracle.bindings import Oracle, damp_ntab
from sep_code_gb300 import gpu_funcs as gf
from sep_code_gb300 import model as M


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def oracle_ctx(orc: Oracle, s: M.Survey, st: M.ShotSetup, src_vals, rec_locs=None, keep=None):
    keep = [] if keep is None else keep
    n1, n2, n3 = st.n
    coeffs = orc.fd_coeffs(*st.d)
    tab = orc.damp_table(s.bc_a, s.bc_b, damp_ntab(n1, n2, n3))
    rec = st.rec_locs if rec_locs is None else rec_locs
    ctx = orc.make_ctx((n1, n2, n3), coeffs, tab, src_vals.shape[1], st.sinc_s, st.sinc_d,
                       np.ascontiguousarray(st.src_locs, np.int32),
                       np.ascontiguousarray(src_vals, np.float32),
                       np.ascontiguousarray(rec, np.int32), st.rnx, st.rny, keep)
    return ctx, keep


def source_vals(s: M.Survey, st: M.ShotSetup, extra: int):
    """source traces of length data_nt + extra (create_source_fields uses +9,
    forward / adjoint use +8)."""
    wd = gf.wavelet_deriv(s.wavelet, s.dtw)
    sx, sy, sz = s.shots[0]
    locs, vals = gf.source_func(wd, sx, sy, sz, st.n[0], st.n[1], st.o, st.d, s.data_nt + extra)
    return locs, vals


class GpuShot:
    """Drives one shot through the C ABI exactly as rtm_zero_op does."""

    def __init__(self, s: M.Survey, st: M.ShotSetup):
        self.s, self.st = s, st
        gf.setup_cuda(1)
        n1, n2, n3 = st.n
        gf.create_gpu_space(st.d[0], st.d[1], st.d[2], s.bc_a, s.bc_b, s.bc_b, n1, n2, n3)
        gf.transfer_sinc_table_s(st.sinc_s)
        gf.transfer_sinc_table_d(st.sinc_d)

    def source_prop(self):
        s, st = self.s, self.st
        locs, vals = source_vals(s, st, 9)
        gf.transfer_source_func(locs, vals)
        gf.transfer_vel_func1(st.vel2dt2)
        return gf.source_prop((st.n[2], st.n[1], st.n[0]), st.jts, 9, st.nt)

    def rtm_forward(self, img, rec_init=None):
        s, st = self.s, self.st
        locs, vals = source_vals(s, st, 8)
        gf.transfer_source_func(locs, vals)
        gf.transfer_vel_func1(st.vel2dt2)
        nrec = st.rnx * st.rny
        rv = np.zeros((nrec, st.nt_big), np.float32) if rec_init is None else rec_init
        gf.transfer_receiver_func(st.rnx, st.rny, st.rec_locs, rv)
        return gf.rtm_forward(img, st.jtd, 9, st.nt, st.nt_big, st.rnx, st.rny)

    def rtm_adjoint(self, p0_s, p1_s, traces):
        s, st = self.s, self.st
        locs, vals = source_vals(s, st, 8)
        gf.transfer_source_func(locs, vals)
        gf.transfer_vel_func1(st.vel2dt2)
        gf.transfer_receiver_func(st.rnx, st.rny, st.rec_locs, traces)
        return gf.rtm_adjoint(p0_s, p1_s, st.jtd, 9, st.nt)


class OracleShot:
    def __init__(self, orc: Oracle, s: M.Survey, st: M.ShotSetup):
        self.orc, self.s, self.st = orc, s, st

    def source_prop(self):
        _, vals = source_vals(self.s, self.st, 9)
        ctx, keep = oracle_ctx(self.orc, self.s, self.st, vals)
        return self.orc.source_prop(ctx, self.st.vel2dt2, self.st.jts, 9, self.st.nt)

    def rtm_forward(self, img, rec_init=None):
        st = self.st
        _, vals = source_vals(self.s, st, 8)
        ctx, keep = oracle_ctx(self.orc, self.s, st, vals)
        nrec = st.rnx * st.rny
        dat = np.zeros((nrec, st.nt_big), np.float32) if rec_init is None else rec_init.copy()
        return self.orc.rtm_forward(ctx, st.vel2dt2, st.jtd, np.ascontiguousarray(img, np.float32),
                                    dat, 9, st.nt)

    def rtm_adjoint(self, p0_s, p1_s, traces):
        st = self.st
        _, vals = source_vals(self.s, st, 8)
        ctx, keep = oracle_ctx(self.orc, self.s, st, vals)
        return self.orc.rtm_adjoint(ctx, st.vel2dt2, st.jtd, np.ascontiguousarray(p0_s, np.float32),
                                    np.ascontiguousarray(p1_s, np.float32),
                                    np.ascontiguousarray(traces, np.float32), 9, st.nt)


PREC = {"f32": 0, "bf16": 1, "f16": 2}


class LinCase:
    """One shot of the linearised Born pair through the GPU and the oracle.
    Model m lives on the padded grid (the image buffer); data d are receiver
    traces [nrec][nt_big]."""

    def __init__(self, s: M.Survey, st: M.ShotSetup):
        self.s, self.st = s, st
        _, self.vals = source_vals(s, st, 8)

    # ---- GPU
    def gpu_setup(self, traces=None):
        st = self.st
        g = GpuShot(self.s, st)
        locs, _ = source_vals(self.s, st, 8)
        gf.transfer_source_func(locs, self.vals)
        gf.transfer_vel_func1(st.vel2dt2)
        nrec = st.rnx * st.rny
        tr = np.zeros((nrec, st.nt_big), np.float32) if traces is None else traces
        gf.transfer_receiver_func(st.rnx, st.rny, st.rec_locs, tr)
        return g

    def gpu_forward(self, m, js, prec):
        st = self.st
        self.gpu_setup()
        gf.set_image(m)
        gf.zero_traces()
        gf.lin_forward(st.jtd, 9, st.nt, js, prec)
        return gf.get_traces(st.rnx * st.rny, st.nt_big)

    def gpu_adjoint(self, d, js, prec, source_pass=True):
        st = self.st
        self.gpu_setup(traces=d)
        if source_pass:
            gf.lin_source_pass(st.jtd, 9, st.nt, js, prec)
        gf.lin_adjoint(st.jtd, st.nt, js, prec)
        return gf.get_image((st.n[2], st.n[1], st.n[0]))

    # ---- oracle
    def orc_ctx(self, orc):
        return oracle_ctx(orc, self.s, self.st, self.vals)

    def orc_forward(self, orc, m, js, prec):
        import ctypes as C
        st = self.st
        ctx, keep = self.orc_ctx(orc)
        dat = np.zeros((st.rnx * st.rny, st.nt_big), np.float32)
        rc = orc.lib.orc_lin_forward_f32(C.byref(ctx), st.vel2dt2, st.jtd, 9, st.nt, js, PREC[prec],
                                         np.ascontiguousarray(m, np.float32), dat)
        assert rc == 0
        return dat

    def orc_adjoint(self, orc, d, js, prec):
        import ctypes as C
        st = self.st
        ctx, keep = self.orc_ctx(orc)
        nsnap = (st.nt + js - 1) // js
        snaps = np.zeros((nsnap, st.n[2], st.n[1], st.n[0]), np.float32)
        rc = orc.lib.orc_lin_source_f32(C.byref(ctx), st.vel2dt2, st.jtd, 9, st.nt, js, PREC[prec], snaps)
        assert rc == 0
        img = np.zeros((st.n[2], st.n[1], st.n[0]), np.float32)
        rc = orc.lib.orc_lin_adjoint_f32(C.byref(ctx), st.vel2dt2, st.jtd, st.nt, js, snaps,
                                         np.ascontiguousarray(d, np.float32), img)
        assert rc == 0
        return img
