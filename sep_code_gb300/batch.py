"""Many shots per time step (include/sepx_batch.h).

``windowed_surveys`` builds the batched workload: a 1024 x 1024 x 400 model
(the layered generator of the 512 x 512 x 400 workload), 16 shots on a
jittered surface grid, each with its own aperture window from 192 x 192 x 256
to 384 x 384 x 320 cells, receivers at every surface node of its window.
``BatchRTM`` sets every shot up through the reference-named C ABI (one device
context per shot, as rtm_zero_op's shot loop does per shot,
Born/rtm_zero_op_3d.cpp:123-157) and runs the Born forward of all shots:
shot after shot, in one persistent launch per step, or as a captured graph.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import gpu_funcs as gf
from . import model as M
from ._lib import SepxError, lib

lib.sepx_batch_begin.argtypes = [C.c_int]
lib.sepx_batch_select.argtypes = [C.c_int]
lib.sepx_batch_rtm_forward.argtypes = [C.c_int] * 4
lib.sepx_batch_source_prop.argtypes = [C.c_int] * 4
lib.sepx_batch_rtm_adjoint.argtypes = [C.c_int] * 4
lib.sepx_batch_autotune.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int), C.POINTER(C.c_float)]
lib.sepx_batch_set_tuning.argtypes = [C.c_int, C.c_int, C.c_int]
lib.sepx_batch_get_tuning.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
for _n in ("sepx_batch_begin", "sepx_batch_select", "sepx_batch_size", "sepx_batch_end",
           "sepx_batch_rtm_forward", "sepx_batch_source_prop", "sepx_batch_rtm_adjoint",
           "sepx_batch_autotune", "sepx_batch_set_tuning",
           "sepx_batch_get_tuning"):
    getattr(lib, _n).restype = C.c_int

HOW = {"sequential": 0, "persistent": 1, "graph": 2}


def _chk(rc):
    if rc != 0:
        raise SepxError(lib.sepx_last_error().decode())


def window_surveys(vel, refl, d, centers, windows, nt, f0=20.0):
    """one Survey per shot: the model window (nx, ny, nz) around (cx, cy),
    clipped to the model; source at the window's surface point of the shot"""
    m3, m2, m1 = vel.shape
    w = M.ricker(f0, 0.001, nt)
    out = []
    for (cx, cy), (wx, wy, wz) in zip(centers, windows):
        x0 = int(np.clip(round(cx / d) - wx // 2, 0, m1 - wx))
        y0 = int(np.clip(round(cy / d) - wy // 2, 0, m2 - wy))
        sub_v = np.ascontiguousarray(vel[:wz, y0:y0 + wy, x0:x0 + wx])
        sub_r = np.ascontiguousarray(refl[:wz, y0:y0 + wy, x0:x0 + wx])
        sx, sy = cx - x0 * d, cy - y0 * d
        out.append(M.Survey(vel=sub_v, spacing=(d, d, d), refl=sub_r, wavelet=w, dtw=0.001,
                            data_nt=nt, data_dt=0.001, rec=(wx, wy, 0.0, d, 0.0, d),
                            shots=[(sx, sy, 0.0)], nbound=20, name=f"window_{wx}x{wy}x{wz}"))
    return out


def windowed_surveys(nt: int = 1000, nshots: int = 16, model=(1024, 1024, 400), seed: int = 20261209):
    """16 shots, uneven windows 192^2 x 256 .. 384^2 x 320, jittered 4 x 4 grid"""
    n1, n2, n3 = model
    big = M.layered_survey(n1, n2, n3, nt=8, seed=seed)
    d = big.spacing[0]
    rng = np.random.default_rng(seed + 1)
    k = int(np.ceil(np.sqrt(nshots)))
    centers, windows = [], []
    sides = np.linspace(192, 384, nshots).astype(int) // 16 * 16
    depths = np.linspace(256, 320, nshots).astype(int) // 16 * 16
    order = rng.permutation(nshots)
    for i in range(nshots):
        gx, gy = i % k, i // k
        cx = ((gx + 0.5) / k + rng.uniform(-0.08, 0.08)) * (n1 - 1) * d
        cy = ((gy + 0.5) / k + rng.uniform(-0.08, 0.08)) * (n2 - 1) * d
        centers.append((cx, cy))
        s = int(sides[order[i]])
        windows.append((s, s, int(depths[order[i]])))
    return window_surveys(big.vel, big.refl, d, centers, windows, nt)


class BatchRTM:
    """The shots of one batch on the device (one context per shot)."""

    def __init__(self, surveys):
        gf.setup_cuda(1)
        self.surveys = list(surveys)
        self.setups = [M.prepare_shot(s) for s in self.surveys]
        jt = {st.jtd for st in self.setups}
        nt = {st.nt for st in self.setups}
        if len(jt) != 1 or len(nt) != 1:
            raise ValueError("every shot of a batch needs the same jt and nt")
        self.jt, self.nt = jt.pop(), nt.pop()
        _chk(lib.sepx_batch_begin(len(self.surveys)))
        try:
            for i, (s, st) in enumerate(zip(self.surveys, self.setups)):
                _chk(lib.sepx_batch_select(i))
                n1, n2, n3 = st.n
                gf.create_gpu_space(st.d[0], st.d[1], st.d[2], s.bc_a, s.bc_b, s.bc_b, n1, n2, n3)
                gf.transfer_sinc_table_s(st.sinc_s)
                gf.transfer_sinc_table_d(st.sinc_d)
                gf.transfer_source_func(st.src_locs, st.src_vals)
                gf.transfer_vel_func1(st.vel2dt2)
                gf.transfer_receiver_func(st.rnx, st.rny, st.rec_locs,
                                          np.zeros((st.rnx * st.rny, st.nt_big), np.float32))
                gf.set_image(st.img_lap)
        finally:
            lib.sepx_batch_select(-1)
        self.cells = [(16 * ((st.n[0] - 8) // 16)) * (16 * ((st.n[1] - 8) // 16)) * (st.n[2] - 12)
                      for st in self.setups]

    def close(self):
        lib.sepx_batch_end()

    def zero_traces(self):
        for i in range(len(self.setups)):
            _chk(lib.sepx_batch_select(i))
            gf.zero_traces()
        lib.sepx_batch_select(-1)

    def _each(self, fn):
        try:
            for i in range(len(self.setups)):
                _chk(lib.sepx_batch_select(i))
                fn(i)
        finally:
            lib.sepx_batch_select(-1)

    def source_prop(self, how: str = "graph"):
        """create_source_fields for every shot: source traces of nt+9 samples"""
        def up(i):
            s, st = self.surveys[i], self.setups[i]
            wd = gf.wavelet_deriv(s.wavelet, s.dtw)
            sx, sy, sz = s.shots[0]
            locs, vals = gf.source_func(wd, sx, sy, sz, st.n[0], st.n[1], st.o, st.d, s.data_nt + 9)
            gf.transfer_source_func(locs, vals)
        self._each(up)
        _chk(lib.sepx_batch_source_prop(self.setups[0].jts, 9, self.nt, HOW[how]))

    def _forward_sources(self):
        self._each(lambda i: gf.transfer_source_func(self.setups[i].src_locs, self.setups[i].src_vals))

    def forward(self, how: str = "graph"):
        """Born forward of every shot (source traces of nt+8 samples)"""
        self._forward_sources()
        _chk(lib.sepx_batch_rtm_forward(self.jt, 9, self.nt, HOW[how]))

    def adjoint(self, how: str = "graph"):
        """RTM adjoint of every shot from its receiver traces and last source_prop"""
        self._forward_sources()
        _chk(lib.sepx_batch_rtm_adjoint(self.jt, 9, self.nt, HOW[how]))

    def set_images(self):
        """upload every shot's reflectivity image (the Born forward's input;
        the adjoint writes its RTM image into the same device buffer)"""
        self._each(lambda i: gf.set_image(self.setups[i].img_lap))

    def image(self, i):
        st = self.setups[i]
        _chk(lib.sepx_batch_select(i))
        try:
            return gf.get_image((st.n[2], st.n[1], st.n[0]))
        finally:
            lib.sepx_batch_select(-1)

    def rtm(self, how: str = "graph"):
        """the bench step of every shot: source_prop, Born forward, adjoint"""
        self.source_prop(how)
        self.zero_traces()
        self.forward(how)
        self.adjoint(how)

    def traces(self, i):
        st = self.setups[i]
        _chk(lib.sepx_batch_select(i))
        try:
            return gf.get_traces(st.rnx * st.rny, st.nt_big)
        finally:
            lib.sepx_batch_select(-1)

    def autotune(self, nsteps: int = 8):
        """returns (z-chunk, ring depth, launch style, ms per step) of the fastest candidate"""
        z, s, sty, ms = C.c_int(), C.c_int(), C.c_int(), C.c_float()
        _chk(lib.sepx_batch_autotune(self.jt, 9, nsteps, C.byref(z), C.byref(s), C.byref(sty),
                                     C.byref(ms)))
        return z.value, s.value, sty.value, ms.value

    def set_tuning(self, zchunk: int, stages: int, style: int = 0):
        _chk(lib.sepx_batch_set_tuning(zchunk, stages, style))

    def cell_updates(self, loops=("forward",)):
        """updated cells x fields x steps of the given loops over the batch"""
        per = {"source_prop": self.nt + 1, "forward": 2 * self.nt, "adjoint": 2 * self.nt - 1}
        return sum(per[k] for k in loops) * sum(self.cells)
