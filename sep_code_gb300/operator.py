"""rtm_zero_op, dot_test and least-squares RTM through the C API of
include/sepx_ops.h (the C++ operator layer on device-resident vectors)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import SepxError, lib
from .model import Survey


class RtmProblem(C.Structure):
    _fields_ = [
        ("vel", C.c_void_p), ("m1", C.c_int), ("m2", C.c_int), ("m3", C.c_int),
        ("d1", C.c_float), ("d2", C.c_float), ("d3", C.c_float),
        ("wavelet", C.c_void_p), ("nwav", C.c_int), ("dtw", C.c_float),
        ("data_nt", C.c_int), ("data_dt", C.c_float),
        ("rnx", C.c_int), ("rny", C.c_int),
        ("ro2", C.c_float), ("rd2", C.c_float), ("ro3", C.c_float), ("rd3", C.c_float),
        ("rec_depth", C.c_float),
        ("nshots", C.c_int), ("shot_xyz", C.c_void_p),
        ("nbound", C.c_int), ("bc_a", C.c_float), ("bc_b", C.c_float),
        ("mode", C.c_int), ("snap_js", C.c_int), ("snap_prec", C.c_int),
        ("mo1", C.c_float), ("mo2", C.c_float), ("mo3", C.c_float),
    ]


DIRECTION_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_longlong)

_F32P = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_F64P = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
lib.sepx_rtm_op_create.argtypes = [C.POINTER(RtmProblem)]
lib.sepx_rtm_op_create.restype = C.c_void_p
lib.sepx_rtm_op_destroy.argtypes = [C.c_void_p]
lib.sepx_rtm_op_model_size.argtypes = [C.c_void_p]
lib.sepx_rtm_op_model_size.restype = C.c_longlong
lib.sepx_rtm_op_data_size.argtypes = [C.c_void_p]
lib.sepx_rtm_op_data_size.restype = C.c_longlong
lib.sepx_rtm_op_forward.argtypes = [C.c_void_p, C.c_int, _F32P, _F32P]
lib.sepx_rtm_op_adjoint.argtypes = [C.c_void_p, C.c_int, _F32P, _F32P]
lib.sepx_rtm_op_dot_test.argtypes = [C.c_void_p, C.c_ulonglong, _F64P]
lib.sepx_lsrtm.argtypes = [C.c_void_p, _F32P, C.c_int, _F32P, _F64P, _F64P, C.c_void_p, C.c_void_p,
                           C.c_double, C.POINTER(C.c_int)]


class LsrtmOpts(C.Structure):
    """sepx_lsrtm_opts (include/sepx_ops.h)"""
    _fields_ = [("dir", C.c_void_p), ("dir_ctx", C.c_void_p), ("policy", C.c_int),
                ("fallback_ratio", C.c_double), ("probe_every", C.c_int), ("target", C.c_double)]


_I32P = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
lib.sepx_lsrtm_ex.argtypes = [C.c_void_p, _F32P, C.c_int, C.POINTER(LsrtmOpts), _F32P, _F64P, _F64P,
                              _I32P, C.POINTER(C.c_int)]
POLICIES = {"fallback": 0, "adaptive": 1}

MODES = {"reference": 0, "linear": 1}
PREC = {"f32": 0, "bf16": 1, "f16": 2}


class RtmOperator:
    """rtm_zero_op over one Survey.  mode "reference": the reference's
    rtm_forward / rtm_adjoint (random-boundary source reconstruction);
    mode "linear": the exact-adjoint linearised pair with source snapshots."""

    def __init__(self, s: Survey, mode: str = "reference", snap_js: int = 1, snap_prec: str = "f32"):
        self.s = s
        self._keep = [np.ascontiguousarray(s.vel, np.float32),
                      np.ascontiguousarray(s.wavelet, np.float32),
                      np.ascontiguousarray(np.asarray(s.shots, np.float32).reshape(-1, 3))]
        m3, m2, m1 = s.vel.shape
        rnx, rny, ro2, rd2, ro3, rd3 = s.rec
        p = RtmProblem(self._keep[0].ctypes.data, m1, m2, m3, *s.spacing, self._keep[1].ctypes.data,
                       len(s.wavelet), s.dtw, s.data_nt, s.data_dt, rnx, rny, ro2, rd2, ro3, rd3,
                       s.rec_depth, len(s.shots), self._keep[2].ctypes.data, s.nbound, s.bc_a,
                       s.bc_b, MODES[mode], snap_js, PREC[snap_prec])
        h = lib.sepx_rtm_op_create(C.byref(p))
        if not h:
            raise SepxError(lib.sepx_last_error().decode())
        self.h = h
        self.model_shape = (m3, m2, m1)
        self.data_shape = (len(s.shots), rny, rnx, s.data_nt)

    def close(self):
        if self.h:
            lib.sepx_rtm_op_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _chk(self, rc):
        if rc != 0:
            raise SepxError(lib.sepx_last_error().decode())

    def forward(self, model, data=None, add=False):
        out = np.zeros(self.data_shape, np.float32) if data is None else data
        self._chk(lib.sepx_rtm_op_forward(self.h, int(add), np.ascontiguousarray(model, np.float32), out))
        return out

    def adjoint(self, data, model=None, add=False):
        out = np.zeros(self.model_shape, np.float32) if model is None else model
        self._chk(lib.sepx_rtm_op_adjoint(self.h, int(add), out, np.ascontiguousarray(data, np.float32)))
        return out

    def dot_test(self, seed: int = 1):
        out = np.zeros(4, np.float64)
        self._chk(lib.sepx_rtm_op_dot_test(self.h, seed, out))
        return out

    def lsrtm(self, data, niter: int, direction=None, fallback_ratio: float = 0.0,
              policy: str = "fallback", probe_every: int = 8, target: float = 0.0):
        """simple_solver + cgstep; ``direction(g_ptr, n)`` may precondition the
        search direction in place (device pointer).  policy "fallback": with
        fallback_ratio > 0 the solver returns to plain g once a preconditioned
        step lowers rr.rr by less than that ratio (``self.fallback_iter``
        records where); "adaptive": the preconditioned direction is kept while
        its steps remove at least the fraction of rr.rr the latest plain step
        removed, and retried every ``probe_every`` plain iterations.  target >
        0 stops once the residual falls to that fraction of the initial one.
        Returns (model, rr.rr per iteration, seconds per iteration) for the
        iterations run; ``self.used_dir`` marks the preconditioned ones."""
        model = np.zeros(self.model_shape, np.float32)
        resid = np.zeros(niter, np.float64)
        secs = np.zeros(niter, np.float64)
        used = np.zeros(niter, np.int32)
        cb = None
        if direction is not None:
            cb = DIRECTION_FN(lambda ctx, g, n: int(direction(g, n) or 0))
        done = C.c_int(0)
        if policy == "fallback" and target <= 0:
            fb = C.c_int(-1)
            self._chk(lib.sepx_lsrtm(self.h, np.ascontiguousarray(data, np.float32), niter, model, resid,
                                     secs, C.cast(cb, C.c_void_p) if cb else None, None, fallback_ratio,
                                     C.byref(fb)))
            self.fallback_iter = fb.value
            self.used_dir = None
            return model, resid, secs
        opts = LsrtmOpts(C.cast(cb, C.c_void_p) if cb else None, None, POLICIES[policy], fallback_ratio,
                         probe_every, target)
        self._chk(lib.sepx_lsrtm_ex(self.h, np.ascontiguousarray(data, np.float32), niter, C.byref(opts),
                                    model, resid, secs, used, C.byref(done)))
        k = done.value
        self.used_dir = used[:k].copy()
        off = np.nonzero(self.used_dir == 0)[0] if cb else []
        self.fallback_iter = int(off[0]) - 1 if len(off) else -1
        return model, resid[:k], secs[:k]
