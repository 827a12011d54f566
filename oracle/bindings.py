"""ctypes bindings for the oracle libraries (test infrastructure only).

``Oracle`` wraps oracle/_build/libsepx_oracle.so (the CPU restatement);
``RefHost`` wraps oracle/_ref/libsepref.so (the reference's own host C++).
Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build_oracle as _b

F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class OrcCtx(C.Structure):
    _fields_ = [
        ("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int),
        ("coeffs", C.c_float * 13),
        ("damp_tab", C.c_void_p), ("ntab", C.c_int),
        ("ntrace", C.c_int), ("nsinc", C.c_int),
        ("sinc_s", C.c_void_p), ("ns", C.c_int),
        ("sinc_d", C.c_void_p), ("nd", C.c_int),
        ("nsrc", C.c_int), ("src_loc", C.c_void_p), ("src_vals", C.c_void_p),
        ("nrec_x", C.c_int), ("nrec_y", C.c_int), ("rec_loc", C.c_void_p),
    ]


class OrcCtx64(C.Structure):
    _fields_ = [("base", OrcCtx), ("d1", C.c_double), ("d2", C.c_double), ("d3", C.c_double),
                ("damp_tab", C.c_void_p), ("sinc_s", C.c_void_p), ("sinc_d", C.c_void_p),
                ("src_vals", C.c_void_p)]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def damp_ntab(n1: int, n2: int, n3: int) -> int:
    """Largest sponge edge distance a cell can have, plus one."""
    return max(n1, n2, n3) // 2 + 1


class Oracle:
    """CPU restatement of the reference path (FP32 parity, FP64 precision)."""

    def __init__(self, path: Path | None = None):
        path = path or _b.build_oracle()
        L = self.lib = C.CDLL(str(path))
        L.orc_fd_coeffs.argtypes = [C.c_float, C.c_float, C.c_float, F32P]
        L.orc_damp_table_f32.argtypes = [C.c_float, C.c_float, C.c_int, F32P]
        L.orc_damp_table_f64.argtypes = [C.c_float, C.c_float, C.c_int, F64P]
        L.orc_sinc_table.argtypes = [C.c_int, C.c_int, F32P]
        L.orc_glibc_srand.argtypes = [C.c_uint]
        L.orc_glibc_rand.restype = C.c_int
        L.orc_rand_subspace.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, F32P,
                                        C.c_int, C.c_int, C.c_int] + [C.c_float] * 6 + \
            [C.c_int] * 3 + [C.c_float] * 6 + [F32P]
        L.orc_compute_size.argtypes = [C.c_int] * 7 + [C.POINTER(C.c_int)] * 3
        L.orc_source_func.argtypes = [F32P, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                                      C.c_int] + [C.c_float] * 6 + [C.c_int, I32P, F32P]
        L.orc_wavelet_deriv.argtypes = [F32P, C.c_int, C.c_float, F32P]
        L.orc_calc_stability.argtypes = [C.c_float, C.c_float, C.c_float, C.c_int,
                                         C.POINTER(C.c_int)]
        L.orc_calc_stability.restype = C.c_float
        L.orc_receiver_map.argtypes = [C.c_int, C.c_int] + [C.c_float] * 5 + [C.c_int, C.c_int] + \
            [C.c_float] * 6 + [I32P]
        for nm in ("orc_deriv_forward", "orc_deriv_adjoint"):
            getattr(L, nm).argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, F32P, F32P]
        for nm in ("orc_laplac_forward", "orc_laplac_adjoint"):
            getattr(L, nm).argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, F32P, F32P]
        for nm in ("orc_map_data_forward", "orc_map_data_adjoint"):
            getattr(L, nm).argtypes = [C.c_int] * 5 + [F32P, F32P]
        L.orc_wave_step_f32.argtypes = [C.POINTER(OrcCtx), C.c_int, F32P, F32P, F32P]
        L.orc_damp_f32.argtypes = [C.POINTER(OrcCtx), F32P, F32P]
        L.orc_source_prop_f32.argtypes = [C.POINTER(OrcCtx), F32P, F32P, F32P, C.c_int, C.c_int,
                                          C.c_int]
        L.orc_rtm_forward_f32.argtypes = [C.POINTER(OrcCtx), F32P, C.c_int, F32P, F32P, C.c_int,
                                          C.c_int]
        L.orc_rtm_adjoint_f32.argtypes = [C.POINTER(OrcCtx), F32P, C.c_int, F32P, F32P, F32P, F32P,
                                          C.c_int, C.c_int]
        L.orc_source_prop_f64.argtypes = [C.POINTER(OrcCtx64), F64P, F64P, F64P, C.c_int, C.c_int,
                                          C.c_int]
        L.orc_rtm_forward_f64.argtypes = [C.POINTER(OrcCtx64), F64P, C.c_int, F64P, F64P, C.c_int,
                                          C.c_int]
        L.orc_rtm_adjoint_f64.argtypes = [C.POINTER(OrcCtx64), F64P, C.c_int, F64P, F64P, F64P,
                                          F64P, C.c_int, C.c_int]
        L.orc_lin_source_f32.argtypes = [C.POINTER(OrcCtx), F32P, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_int, F32P]
        L.orc_lin_forward_f32.argtypes = [C.POINTER(OrcCtx), F32P, C.c_int, C.c_int, C.c_int,
                                          C.c_int, C.c_int, F32P, F32P]
        L.orc_lin_adjoint_f32.argtypes = [C.POINTER(OrcCtx), F32P, C.c_int, C.c_int, C.c_int, F32P,
                                          F32P, F32P]
        L.orc_lin_source_f64.argtypes = [C.POINTER(OrcCtx64), F64P, C.c_int, C.c_int, C.c_int,
                                         C.c_int, F64P]
        L.orc_lin_adjoint_f64.argtypes = [C.POINTER(OrcCtx64), F64P, C.c_int, C.c_int, C.c_int,
                                          F64P, F64P, F64P]
        L.orc_lin_forward_f64.argtypes = [C.POINTER(OrcCtx64), F64P, C.c_int, C.c_int, C.c_int,
                                          C.c_int, F64P, F64P]
        L.orc_lin_adjoint_ckpt_f32.argtypes = [C.POINTER(OrcCtx), F32P, C.c_int, C.c_int, C.c_int,
                                               C.c_int, C.c_int, C.c_int, F32P, F32P]
        L.orc_lin_adjoint_ckpt_f64.argtypes = [C.POINTER(OrcCtx64), F64P, C.c_int, C.c_int, C.c_int,
                                               C.c_int, C.c_int, F64P, F64P]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_num_threads.argtypes = [C.c_int]

    # ---- helpers ----
    def fd_coeffs(self, d1, d2, d3):
        out = np.zeros(13, np.float32)
        self.lib.orc_fd_coeffs(d1, d2, d3, out)
        return out

    def damp_table(self, bc_a, bc_b, ntab, f64=False):
        out = np.zeros(ntab, np.float64 if f64 else np.float32)
        (self.lib.orc_damp_table_f64 if f64 else self.lib.orc_damp_table_f32)(bc_a, bc_b, ntab, out)
        return out

    def sinc_table(self, ntab, nsinc=8):
        out = np.zeros((ntab, nsinc), np.float32)
        self.lib.orc_sinc_table(ntab, nsinc, out)
        return out

    def rand_subspace(self, irand, nr1, nr2, nr3, dt, model, mo, md, sn, so, sd):
        m3, m2, m1 = model.shape
        out = np.zeros((sn[2], sn[1], sn[0]), np.float32)
        self.lib.orc_rand_subspace(irand, nr1, nr2, nr3, dt, np.ascontiguousarray(model, np.float32),
                                   m1, m2, m3, *mo, *md, *sn, *so, *sd, out)
        return out

    def compute_size(self, m1, m2, m3, nbt, nb, nby, fat=4):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self.lib.orc_compute_size(m1, m2, m3, nbt, nb, nby, fat, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def source_func(self, wav_deriv, sx, sy, sz, n1, n2, o, d, nts):
        locs = np.zeros(9, np.int32)
        vals = np.zeros((9, nts), np.float32)
        w = np.ascontiguousarray(wav_deriv, np.float32)
        self.lib.orc_source_func(w, len(w), sx, sy, sz, n1, n2, *o, *d, nts, locs, vals)
        return locs, vals

    def wavelet_deriv(self, w, dt):
        w = np.ascontiguousarray(w, np.float32)
        out = np.zeros_like(w)
        self.lib.orc_wavelet_deriv(w, len(w), dt, out)
        return out

    def calc_stability(self, vmax, dmin, data_dt, n_data):
        nt = C.c_int()
        dt = self.lib.orc_calc_stability(vmax, dmin, data_dt, n_data, C.byref(nt))
        return dt, nt.value

    def receiver_map(self, rnx, rny, ro2, rd2, ro3, rd3, rec_depth, n1, n2, o, d):
        locs = np.zeros(rnx * rny, np.int32)
        self.lib.orc_receiver_map(rnx, rny, ro2, rd2, ro3, rd3, rec_depth, n1, n2, *o, *d, locs)
        return locs

    # ---- kernels / loops ----
    @staticmethod
    def make_ctx(n, coeffs, damp_tab, ntrace, sinc_s, sinc_d, src_loc, src_vals, rec_loc, rnx, rny,
                 keep):
        """Build an OrcCtx; ``keep`` (a list) holds references to the arrays."""
        c = OrcCtx()
        c.n1, c.n2, c.n3 = n
        for k in range(13):
            c.coeffs[k] = float(coeffs[k])
        arrs = [damp_tab, sinc_s, sinc_d, src_loc, src_vals, rec_loc]
        keep.extend(a for a in arrs if a is not None)
        c.damp_tab = _ptr(damp_tab)
        c.ntab = 0 if damp_tab is None else len(damp_tab)
        c.ntrace = ntrace
        c.nsinc = 8 if sinc_s is None else sinc_s.shape[1]
        c.sinc_s = _ptr(sinc_s)
        c.ns = 0 if sinc_s is None else sinc_s.shape[0]
        c.sinc_d = _ptr(sinc_d)
        c.nd = 0 if sinc_d is None else sinc_d.shape[0]
        c.nsrc = 0 if src_loc is None else len(src_loc)
        c.src_loc = _ptr(src_loc)
        c.src_vals = _ptr(src_vals)
        c.nrec_x, c.nrec_y = rnx, rny
        c.rec_loc = _ptr(rec_loc)
        return c

    def source_prop(self, ctx, vel, jt, npts, nt):
        n = (ctx.n3, ctx.n2, ctx.n1)
        p0 = np.zeros(n, np.float32)
        p1 = np.zeros(n, np.float32)
        rc = self.lib.orc_source_prop_f32(C.byref(ctx), vel, p0, p1, jt, npts, nt)
        if rc:
            raise RuntimeError(f"orc_source_prop_f32 failed ({rc})")
        return p0, p1

    def rtm_forward(self, ctx, vel, jt, img, dat, npts, nt):
        rc = self.lib.orc_rtm_forward_f32(C.byref(ctx), vel, jt, img, dat, npts, nt)
        if rc:
            raise RuntimeError(f"orc_rtm_forward_f32 failed ({rc})")
        return dat

    def rtm_adjoint(self, ctx, vel, jt, p0_s, p1_s, dat, npts, nt):
        img = np.zeros((ctx.n3, ctx.n2, ctx.n1), np.float32)
        rc = self.lib.orc_rtm_adjoint_f32(C.byref(ctx), vel, jt, p0_s, p1_s, img, dat, npts, nt)
        if rc:
            raise RuntimeError(f"orc_rtm_adjoint_f32 failed ({rc})")
        return img

    @staticmethod
    def make_ctx64(ctx, spacing, damp64, sinc_s64, sinc_d64, src_vals64, keep):
        c = OrcCtx64()
        c.base = ctx
        c.d1, c.d2, c.d3 = (float(s) for s in spacing)
        keep.extend([damp64, sinc_s64, sinc_d64, src_vals64])
        c.damp_tab = _ptr(damp64)
        c.sinc_s = _ptr(sinc_s64)
        c.sinc_d = _ptr(sinc_d64)
        c.src_vals = _ptr(src_vals64)
        return c

    def num_threads(self):
        return self.lib.orc_num_threads()

    def set_num_threads(self, n):
        self.lib.orc_set_num_threads(n)


class RefHost:
    """The reference's host C++ compiled from its own sources (oracle/_ref)."""

    def __init__(self, path: Path | None = None):
        path = path or _b.build_ref()
        if path is None or not Path(path).exists():
            raise FileNotFoundError("reference host library is not built (reference tree absent)")
        L = self.lib = C.CDLL(str(path))
        L.ref_sinc_table.argtypes = [C.c_int, C.c_int, F32P]
        L.ref_rand_subspace.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, F32P,
                                        C.c_int, C.c_int, C.c_int] + [C.c_float] * 6 + \
            [C.c_int] * 3 + [C.c_float] * 6 + [F32P]
        L.ref_compute_domain.argtypes = [C.c_int] * 3 + [C.c_float] * 3 + [C.c_int] * 4 + [I32P, F32P]
        L.ref_wavelet_deriv.argtypes = [F32P, C.c_int, C.c_float, C.c_float, F32P]
        L.ref_source_func.argtypes = [F32P, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                      C.c_int, C.c_int, C.c_int] + [C.c_float] * 6 + [C.c_int, I32P, F32P]
        L.ref_deriv.argtypes = [C.c_int] * 5 + [C.c_float, F32P, F32P]
        L.ref_laplac.argtypes = [C.c_int] * 5 + [F32P, F32P]
        L.ref_map_data.argtypes = [C.c_int] * 6 + [F32P, F32P]
        L.ref_cg_solve.argtypes = [F32P, C.c_int, C.c_int, F32P, C.c_int, F32P, C.POINTER(C.c_double)]
        L.ref_cg_solve.restype = C.c_int
        L.ref_dense_dot_test.argtypes = [F32P, C.c_int, C.c_int, C.c_uint]
        L.ref_dense_dot_test.restype = C.c_int

    def sinc_table(self, ntab, nsinc=8):
        out = np.zeros((ntab, nsinc), np.float32)
        self.lib.ref_sinc_table(ntab, nsinc, out)
        return out

    def rand_subspace(self, irand, nr1, nr2, nr3, dt, model, mo, md, sn, so, sd):
        m3, m2, m1 = model.shape
        out = np.zeros((sn[2], sn[1], sn[0]), np.float32)
        self.lib.ref_rand_subspace(irand, nr1, nr2, nr3, dt, np.ascontiguousarray(model, np.float32),
                                   m1, m2, m3, *mo, *md, *sn, *so, *sd, out)
        return out

    def compute_domain(self, m1, m2, m3, md, nbt, nb, nby, fat=4):
        n = np.zeros(3, np.int32)
        o = np.zeros(3, np.float32)
        self.lib.ref_compute_domain(m1, m2, m3, *md, nbt, nb, nby, fat, n, o)
        return tuple(int(x) for x in n), tuple(float(x) for x in o)

    def wavelet_deriv(self, w, dt):
        w = np.ascontiguousarray(w, np.float32)
        out = np.zeros_like(w)
        self.lib.ref_wavelet_deriv(w, len(w), 0.0, dt, out)
        return out

    def source_func(self, wav_deriv, dtw, sx, sy, sz, n, o, d, nts):
        locs = np.zeros(9, np.int32)
        vals = np.zeros((9, nts), np.float32)
        w = np.ascontiguousarray(wav_deriv, np.float32)
        self.lib.ref_source_func(w, len(w), dtw, sx, sy, sz, *n, *o, *d, nts, locs, vals)
        return locs, vals

    def deriv(self, fwd, add, m, d, dt):
        n3, n2, nt = m.shape
        m = np.ascontiguousarray(m, np.float32).copy()
        d = np.ascontiguousarray(d, np.float32).copy()
        self.lib.ref_deriv(int(fwd), int(add), nt, n2, n3, dt, m, d)
        return m, d

    def laplac(self, fwd, add, m, d):
        n3, n2, n1 = m.shape
        m = np.ascontiguousarray(m, np.float32).copy()
        d = np.ascontiguousarray(d, np.float32).copy()
        self.lib.ref_laplac(int(fwd), int(add), n1, n2, n3, m, d)
        return m, d

    def map_data(self, fwd, add, m, d):
        n3, n2, ntb = m.shape
        nt = d.shape[2]
        m = np.ascontiguousarray(m, np.float32).copy()
        d = np.ascontiguousarray(d, np.float32).copy()
        self.lib.ref_map_data(int(fwd), int(add), ntb, nt, n2, n3, m, d)
        return m, d

    # ---- image / data vectors (Born/image_rtm_3d.cpp, data_rtm_3d.cpp, tmute.cpp) ----
    def _dataimg_sigs(self):
        L = self.lib
        if getattr(self, "_di", False):
            return L
        I3 = np.ctypeslib.ndpointer(np.int32, shape=(3,), flags="C_CONTIGUOUS")
        F3 = np.ctypeslib.ndpointer(np.float32, shape=(3,), flags="C_CONTIGUOUS")
        L.ref_image_add.argtypes = [I3, F3, F3, F32P, I3, F3, F3, F32P]
        L.ref_image_extract.argtypes = [I3, F3, F3, F32P, F32P, I3, F3, F3, F32P, F32P]
        L.ref_add_data.argtypes = [C.c_int] * 4 + [F32P, C.c_int, F32P]
        L.ref_tmute.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, C.c_float, C.c_float,
                                C.c_int, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, F32P, F32P]
        self._di = True
        return L

    @staticmethod
    def _grid(shape, o, d):
        return (np.array(shape[::-1], np.int32), np.array(o, np.float32), np.array(d, np.float32))

    def image_add(self, img, o, d, sub, so, sd):
        """image_rtm_3d::add_image; img/sub [n3][n2][n1], o/d per axis (1, 2, 3)"""
        L = self._dataimg_sigs()
        out = np.ascontiguousarray(img, np.float32).copy()
        L.ref_image_add(*self._grid(out.shape, o, d), out, *self._grid(sub.shape, so, sd),
                        np.ascontiguousarray(sub, np.float32))
        return out

    def image_extract(self, img, mute, o, d, sub_shape, so, sd):
        """image_rtm_3d::extract_sub and write_volume: (sub, img * mute)"""
        L = self._dataimg_sigs()
        img = np.ascontiguousarray(img, np.float32)
        sub = np.zeros(sub_shape, np.float32)
        muted = np.zeros_like(img)
        L.ref_image_extract(*self._grid(img.shape, o, d), img, np.ascontiguousarray(mute, np.float32),
                            *self._grid(sub_shape, so, sd), sub, muted)
        return sub, muted

    def add_data(self, all_data, ishot, shot):
        """data_rtm_3d::add_data; all_data [nshots][n3][n2][n1]"""
        L = self._dataimg_sigs()
        out = np.ascontiguousarray(all_data, np.float32).copy()
        ns, n3, n2, n1 = out.shape
        L.ref_add_data(n1, n2, n3, ns, out, ishot, np.ascontiguousarray(shot, np.float32))
        return out

    def tmute(self, fwd, add, t0, vmute, o1, d1, o2, d2, model, data):
        """tmute::forward / adjoint on [n5][n4][n3][n2][n1] datasets: (model, data)"""
        L = self._dataimg_sigs()
        m = np.ascontiguousarray(model, np.float32).copy()
        dd = np.ascontiguousarray(data, np.float32).copy()
        n5, n4, n3, n2, n1 = dd.shape
        L.ref_tmute(int(fwd), int(add), t0, vmute, n1, o1, d1, n2, o2, d2, n3, n4, n5, m, dd)
        return m, dd

    def cg_solve(self, A, d, niter):
        A = np.ascontiguousarray(A, np.float32)
        m = np.zeros(A.shape[1], np.float32)
        rr = C.c_double()
        rc = self.lib.ref_cg_solve(A, A.shape[0], A.shape[1], np.ascontiguousarray(d, np.float32),
                                   niter, m, C.byref(rr))
        return m, rr.value, rc


class RefOperator:
    """The reference's rtm_zero_op driven end to end on the CPU: its own host
    classes (SEP files replaced by in-memory buffers) with the oracle loops
    standing in for the GPU C ABI (oracle/ref_stubs/ref_gpu_stubs.cpp)."""

    def __init__(self, host: "RefHost"):
        L = self.lib = host.lib
        L.ref_file_put.argtypes = [C.c_char_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_long]
        L.ref_param_put.argtypes = [C.c_char_p, C.c_char_p]
        L.ref_file_size.argtypes = [C.c_char_p]
        L.ref_file_size.restype = C.c_long
        L.ref_file_get.argtypes = [C.c_char_p, C.c_void_p, C.c_long]
        L.ref_file_get.restype = C.c_long
        L.ref_log_count.restype = C.c_int
        L.ref_log_entry.argtypes = [C.c_int, C.c_char_p, C.POINTER(C.c_long),
                                    C.POINTER(C.c_double)]
        L.ref_log_entry.restype = C.c_int
        L.ref_last_array.argtypes = [C.c_char_p, C.c_void_p, C.c_long]
        L.ref_last_array.restype = C.c_long

    def put(self, tag, arr, n, o, d):
        n = np.asarray(n, np.int32)
        o = np.asarray(o, np.float32)
        d = np.asarray(d, np.float32)
        a = np.ascontiguousarray(arr, np.float32)
        self._keep = (n, o, d, a)
        self.lib.ref_file_put(tag.encode(), len(n), n.ctypes.data, o.ctypes.data, d.ctypes.data,
                              a.ctypes.data, a.nbytes)

    def param(self, name, value):
        self.lib.ref_param_put(name.encode(), str(value).encode())

    def get(self, tag):
        n = self.lib.ref_file_size(tag.encode())
        out = np.zeros(max(n, 0) // 4, np.float32)
        if n > 0:
            self.lib.ref_file_get(tag.encode(), out.ctypes.data, n)
        return out

    def setup(self, s, data=None):
        """In-memory SEP files and parameters for a Survey-like object ``s``."""
        self.lib.ref_reset()
        self.lib.ref_log_clear()
        rnx, rny, ro2, rd2, ro3, rd3 = s.rec
        sx, sy, sz = s.shots[0]
        for k, v in dict(bc_a=s.bc_a, bc_b=s.bc_b, nbound=s.nbound, src_depth=sz,
                         rec_depth=s.rec_depth, n_gpus=1, aper=8.0).items():
            self.param(k, repr(float(v)) if isinstance(v, float) else v)
        m3, m2, m1 = s.vel.shape
        dd = [float(v) for v in s.spacing]
        if data is None:
            data = np.zeros((rny, rnx, s.data_nt), np.float32)
        self.put("data", data, [s.data_nt, rnx, rny, 1, 1], [0.0, ro2, ro3, sx, sy],
                 [s.data_dt, rd2, rd3, 1.0, 1.0])
        self.put("wavelet", s.wavelet, [len(s.wavelet)], [0.0], [s.dtw])
        self.put("velocity", s.vel, [m1, m2, m3], [0, 0, 0], dd)
        self.put("image", s.refl, [m1, m2, m3], [0, 0, 0], dd)
        self.put("mute", np.ones_like(s.refl), [m1, m2, m3], [0, 0, 0], dd)

    def born_forward(self, s):
        import os
        import tempfile
        self.setup(s)
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as td:   # oc_float::make_temp writes files
            os.chdir(td)
            try:
                self.lib.ref_run_born_forward()
            finally:
                os.chdir(cwd)
        rnx, rny = s.rec[0], s.rec[1]
        return self.get("dataout").reshape(rny, rnx, s.data_nt)

    def rtm_adjoint(self, s, data):
        import os
        import tempfile
        self.setup(s, data=data)
        cwd = os.getcwd()
        with tempfile.TemporaryDirectory() as td:
            os.chdir(td)
            try:
                self.lib.ref_run_rtm_adjoint()
            finally:
                os.chdir(cwd)
        m3, m2, m1 = s.vel.shape
        return self.get("image").reshape(m3, m2, m1)

    def log(self):
        out = []
        name = C.create_string_buffer(64)
        ia = (C.c_long * 16)()
        fa = (C.c_double * 8)()
        for i in range(self.lib.ref_log_count()):
            k = self.lib.ref_log_entry(i, name, ia, fa)
            out.append((name.value.decode(), list(ia)[:k]))
        return out

    def last_array(self, which, dtype=np.float32):
        n = self.lib.ref_last_array(which.encode(), None, 0)
        out = np.zeros(n // 4, dtype)
        self.lib.ref_last_array(which.encode(), out.ctypes.data, n)
        return out
