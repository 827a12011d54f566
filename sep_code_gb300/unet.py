"""The learned preconditioner: a 3-D U-Net (4 levels, 16/32/48/64 channels,
3x3x3 convolutions) trained on (m, L'L m) pairs of the Born operator, applied
to the least-squares RTM search direction (g <- N(g) before the forward
product; Born/lin_solver.cpp:127-128 is where the reference forms it).

Every convolution -- forward, data gradient and weight gradient -- runs in the
library's BF16 tcgen05 kernels (include/sepx_unet.h) with FP32 accumulation;
pooling, upsampling, ReLU masks, the loss and Adam are the library's own
memory-bound kernels.  PyTorch only holds device buffers and orders them on
the library's stream.

Structure (channel-last BF16 activations; concatenations are buffers whose
channel slices the layers read and write):

    x (1 ch, stored as 8) -> e1a 16 -> e1b 16 ----------------------------+
      pool -> e2a 32 -> e2b 32 ---------------------------------------+   |
        pool -> e3a 48 -> e3b 48 ------------------------------+      |   |
          pool -> b4a 64 -> b4b 64 -> up -> [64 | 48] d3a 48 -> d3b 48 |   |
                              up -> [48 | 32] d2a 32 -> d2b 32 <------+   |
                              up -> [32 | 16] d1a 16 -> d1b 16 <----------+
    out = x + conv1x1(d1b)      (ReLU after every 3x3x3 convolution)
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import SepxError, lib

_vp = C.c_void_p
_i = C.c_int
_ll = C.c_longlong
_f = C.c_float

_SIGS = {
    "sepx_unet_packed_elems": [_i, _i, _i, _i],
    "sepx_unet_pack_weights": [_vp, _i, _i, _i, _i, _vp, _vp],
    "sepx_unet_pack_weights_many": [_i, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "sepx_unet_conv_fwd": [_vp, _i, _i, _i, _i, _i, _i, _i, _i, _vp, _vp, _i, _i, _vp, _i, _i, _vp,
                           _vp, _vp],
    "sepx_unet_conv_fwd_masked": [_vp, _i, _i, _i, _i, _i, _i, _i, _i, _vp, _vp, _i, _i, _vp, _i, _i,
                                  _vp, _vp, _vp, _i, _i, _vp],
    "sepx_unet_conv_wgrad": [_vp, _i, _i, _i, _i, _i, _i, _i, _i, _vp, _i, _i, _i, _vp, _vp],
    "sepx_unet_conv_wgrad_bias": [_vp, _i, _i, _i, _i, _i, _i, _i, _i, _vp, _i, _i, _i, _vp, _vp, _vp],
    "sepx_unet_avgpool": [_vp, _i, _i, _i, _i, _i, _i, _i, _vp, _i, _i, _vp],
    "sepx_unet_avgpool_bwd": [_vp, _i, _i, _i, _i, _i, _i, _i, _vp, _i, _i, _i, _vp],
    "sepx_unet_upsample": [_vp, _i, _i, _i, _i, _i, _i, _i, _vp, _i, _i, _vp],
    "sepx_unet_upsample_bwd": [_vp, _i, _i, _i, _i, _i, _i, _i, _vp, _i, _i, _vp],
    "sepx_unet_upsample_bwd_masked": [_vp, _i, _i, _i, _i, _i, _i, _i, _vp, _i, _i, _vp, _i, _i, _vp],
    "sepx_unet_avgpool_bwd_masked": [_vp, _i, _i, _i, _i, _i, _i, _i, _vp, _i, _i, _i, _vp, _i, _i, _vp],
    "sepx_unet_relu_mask": [_vp, _i, _i, _vp, _i, _i, _ll, _i, _vp],
    "sepx_unet_bias_grad": [_vp, _i, _i, _ll, _i, _vp, _vp],
    "sepx_unet_to_bf16": [_vp, _ll, _f, _vp, _i, _i, _vp],
    "sepx_unet_mse": [_vp, _vp, _ll, _vp, _i, _vp, _vp],
    "sepx_unet_adam": [_vp, _vp, _vp, _vp, _ll, _f, _f, _f, _f, _i, _vp],
    "sepx_unet_adam_dev": [_vp, _vp, _vp, _vp, _ll, _vp, _vp],
    "sepx_unet_capture_begin": [_vp],
    "sepx_unet_capture_end": [_vp, C.POINTER(C.c_void_p)],
    "sepx_unet_graph_launch": [_vp, _vp],
    "sepx_unet_graph_free": [_vp],
    "sepx_unet_status": [],
    "sepx_unet_set_halo": [_i],
    "sepx_unet_set_wgrad_form": [_i],
}
for _n, _a in _SIGS.items():
    getattr(lib, _n).argtypes = _a
    getattr(lib, _n).restype = C.c_int


def _chk(rc):
    if rc != 0:
        raise SepxError(lib.sepx_last_error().decode())


def _p(t):
    return C.c_void_p(t.data_ptr())


def _r8(c):
    return (c + 7) // 8 * 8


@dataclass(frozen=True)
class Layer:
    name: str
    cin: int          # true input channels
    cout: int
    ntap: int = 27
    relu: bool = True

    @property
    def cin_p(self):
        return _r8(self.cin)


CH = (16, 32, 48, 64)
LAYERS = (
    Layer("e1a", 1, CH[0]), Layer("e1b", CH[0], CH[0]),
    Layer("e2a", CH[0], CH[1]), Layer("e2b", CH[1], CH[1]),
    Layer("e3a", CH[1], CH[2]), Layer("e3b", CH[2], CH[2]),
    Layer("b4a", CH[2], CH[3]), Layer("b4b", CH[3], CH[3]),
    Layer("d3a", CH[3] + CH[2], CH[2]), Layer("d3b", CH[2], CH[2]),
    Layer("d2a", CH[2] + CH[1], CH[1]), Layer("d2b", CH[1], CH[1]),
    Layer("d1a", CH[1] + CH[0], CH[0]), Layer("d1b", CH[0], CH[0]),
    Layer("out", CH[0], 1, ntap=1, relu=False),
)


def init_params(seed: int = 0) -> dict:
    """He-initialised FP32 master weights [ntap][cin_p][cout] and zero biases;
    the output layer starts at zero (the network starts as the identity)."""
    rng = np.random.default_rng(seed)
    out = {}
    for L in LAYERS:
        w = np.zeros((L.ntap, L.cin_p, L.cout), np.float32)
        if L.name != "out":
            std = np.sqrt(2.0 / (L.ntap * L.cin))
            w[:, :L.cin, :] = rng.normal(0.0, std, (L.ntap, L.cin, L.cout))
        out[L.name] = (w, np.zeros(L.cout, np.float32))
    return out


class UNet3D:
    """Device-resident network: parameters, Adam state and activation buffers
    (allocated per input shape).  All work is enqueued on the library stream."""

    def __init__(self, params: dict | None = None, seed: int = 0, grad_streams: int = 2):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda")
        lib.sepx_setup_cuda(1)
        self.stream_ptr = lib.sepx_get_stream()
        self.stream = torch.cuda.ExternalStream(self.stream_ptr)
        params = init_params(seed) if params is None else params
        self.w, self.b, self.gw, self.gb, self.mw, self.vw, self.mb, self.vb = ({} for _ in range(8))
        self.pk, self.pkt = {}, {}
        # parameters, gradients and the two Adam moments each live in one flat
        # FP32 buffer (per-layer views), so that zeroing the gradients and the
        # Adam step are one launch each
        shapes = [(L, (L.ntap, L.cin_p, L.cout), (L.cout,)) for L in LAYERS]
        total = sum(int(np.prod(ws)) + int(np.prod(bs)) for _, ws, bs in shapes)
        with torch.cuda.stream(self.stream):
            self.flat = {k: torch.zeros(total, dtype=torch.float32, device=self.dev)
                         for k in ("p", "g", "m", "v")}
            # Adam hyper-parameters {lr, b1, b2, eps, step}, read by the kernel
            self.hp = torch.zeros(5, dtype=torch.float32, device=self.dev)
            o = 0
            for L, ws, bs in shapes:
                nw, nbias = int(np.prod(ws)), int(np.prod(bs))
                for d, k in ((self.w, "p"), (self.gw, "g"), (self.mw, "m"), (self.vw, "v")):
                    d[L.name] = self.flat[k][o:o + nw].view(ws)
                for d, k in ((self.b, "p"), (self.gb, "g"), (self.mb, "m"), (self.vb, "v")):
                    d[L.name] = self.flat[k][o + nw:o + nw + nbias].view(bs)
                o += nw + nbias
                w, b = params[L.name]
                self.w[L.name].copy_(torch.tensor(np.ascontiguousarray(w, np.float32).reshape(ws)))
                self.b[L.name].copy_(torch.tensor(np.ascontiguousarray(b, np.float32).reshape(bs)))
            for L in LAYERS:
                n = lib.sepx_unet_packed_elems(L.cout, L.cin_p, L.ntap, 0)
                self.pk[L.name] = torch.zeros(n, dtype=torch.bfloat16, device=self.dev)
                n = lib.sepx_unet_packed_elems(L.cout, L.cin_p, L.ntap, 1)
                self.pkt[L.name] = torch.zeros(n, dtype=torch.bfloat16, device=self.dev)
            self.loss = torch.zeros(1, dtype=torch.float64, device=self.dev)
        self.step_count = 0
        self.shape = None
        self.graph, self.graph_io = None, None
        # the weight gradients run on side streams beside the data gradients,
        # taken in turn (each forks from the main stream once its dy is ready;
        # the main stream joins them at the end of the backward pass)
        self.grad_streams = [torch.cuda.Stream(device=self.dev) for _ in range(grad_streams)]
        self._events = [torch.cuda.Event() for _ in range(len(LAYERS) + grad_streams)]
        self._nev = 0
        self._ngs = 0
        self.pack()

    # ---------------------------------------------------------------- params
    def pack(self):
        """BF16 forward and data-gradient operands of every layer, one launch"""
        if getattr(self, "_pack_jobs", None) is None:
            n = 2 * len(LAYERS)
            P, I = C.c_void_p * n, C.c_int * n
            w, out, co, ci, nt, tr = P(), P(), I(), I(), I(), I()
            for i, L in enumerate(LAYERS):
                for k, dst in enumerate((self.pk, self.pkt)):
                    j = 2 * i + k
                    w[j], out[j] = self.w[L.name].data_ptr(), dst[L.name].data_ptr()
                    co[j], ci[j], nt[j], tr[j] = L.cout, L.cin_p, L.ntap, k
            self._pack_jobs = (n, w, out, co, ci, nt, tr)
        n, w, out, co, ci, nt, tr = self._pack_jobs
        _chk(lib.sepx_unet_pack_weights_many(n, w, out, co, ci, nt, tr, self.stream_ptr))

    def params(self) -> dict:
        self.stream.synchronize()
        return {L.name: (self.w[L.name].cpu().numpy().copy(), self.b[L.name].cpu().numpy().copy())
                for L in LAYERS}

    def save(self, path):
        p = self.params()
        np.savez(path, **{f"{k}_w": v[0] for k, v in p.items()}, **{f"{k}_b": v[1] for k, v in p.items()})

    @staticmethod
    def load_params(path) -> dict:
        z = np.load(path)
        return {L.name: (z[f"{L.name}_w"], z[f"{L.name}_b"]) for L in LAYERS}

    # ---------------------------------------------------------------- buffers
    def _alloc(self, nb, D, H, W):
        torch = self.torch
        if D % 8 or H % 8 or W % 8:
            raise ValueError("U-Net volumes must be multiples of 8 along every axis")
        if self.shape == (nb, D, H, W):
            return
        self.shape = (nb, D, H, W)
        dims = [(D >> k, H >> k, W >> k) for k in range(4)]
        V = [nb * d * h * w for d, h, w in dims]
        self.V = V
        self.dims = dims

        def buf(v, c):
            return torch.zeros((v, c), dtype=torch.bfloat16, device=self.dev)

        with torch.cuda.stream(self.stream):
            a = {}
            a["x0"] = buf(V[0], 8)
            a["xf"] = torch.zeros(V[0], dtype=torch.float32, device=self.dev)
            a["e1a"] = buf(V[0], 16); a["cat1"] = buf(V[0], 48)
            a["p1"] = buf(V[1], 16); a["e2a"] = buf(V[1], 32); a["cat2"] = buf(V[1], 80)
            a["p2"] = buf(V[2], 32); a["e3a"] = buf(V[2], 48); a["cat3"] = buf(V[2], 112)
            a["p3"] = buf(V[3], 48); a["b4a"] = buf(V[3], 64); a["b4b"] = buf(V[3], 64)
            a["d3a"] = buf(V[2], 48); a["d3b"] = buf(V[2], 48)
            a["d2a"] = buf(V[1], 32); a["d2b"] = buf(V[1], 32)
            a["d1a"] = buf(V[0], 16); a["d1b"] = buf(V[0], 16)
            a["out"] = torch.zeros(V[0], dtype=torch.float32, device=self.dev)
        self.a, self.g = a, None

    def _alloc_grads(self):
        """gradient buffers, the shapes of the activations (training only)"""
        if self.g is not None:
            return
        torch = self.torch
        with torch.cuda.stream(self.stream):
            g = {k: torch.zeros_like(v) for k, v in self.a.items() if k not in ("xf", "out")}
            g["out"] = torch.zeros((self.V[0], 8), dtype=torch.bfloat16, device=self.dev)
        self.g = g

    # ---------------------------------------------------------------- ops
    def _conv(self, L, x, xcs, xco, lvl, y=None, ycs=0, yco=0, yf=None, resid=None, cin=None):
        nb = self.shape[0]
        D, H, W = self.dims[lvl]
        _chk(lib.sepx_unet_conv_fwd(_p(x), xcs, xco, nb, D, H, W, L.cin_p if cin is None else cin,
                                    L.ntap, _p(self.pk[L.name]), _p(self.b[L.name]), L.cout,
                                    1 if L.relu else 0, _p(y) if y is not None else None, ycs, yco,
                                    _p(yf) if yf is not None else None,
                                    _p(resid) if resid is not None else None, self.stream_ptr))

    def _dgrad(self, L, dy, dycs, dyco, lvl, dx, dxcs, dxco, mask=None):
        """dx = conv^T(dy): the forward kernel with the transposed, flipped
        operand; mask = (y, ycs, yco): the ReLU backward of the layer below,
        fused (dx = 0 where y <= 0)."""
        nb = self.shape[0]
        D, H, W = self.dims[lvl]
        m, mcs, mco = (None, 0, 0) if mask is None else (_p(mask[0]), mask[1], mask[2])
        _chk(lib.sepx_unet_conv_fwd_masked(_p(dy), dycs, dyco, nb, D, H, W, _r8(L.cout), L.ntap,
                                           _p(self.pkt[L.name]), None, L.cin_p, 0, _p(dx), dxcs, dxco,
                                           None, None, m, mcs, mco, self.stream_ptr))

    def _event(self):
        e = self._events[self._nev % len(self._events)]
        self._nev += 1
        return e

    def _wgrad(self, L, x, xcs, xco, dy, dycs, dyco, lvl):
        """weight and bias gradient on the second stream, after everything the
        main stream has enqueued so far (dy is ready there)"""
        nb = self.shape[0]
        D, H, W = self.dims[lvl]
        gs = self.grad_streams[self._ngs % len(self.grad_streams)]
        self._ngs += 1
        e = self._event()
        e.record(self.stream)
        gs.wait_event(e)
        _chk(lib.sepx_unet_conv_wgrad_bias(_p(x), xcs, xco, nb, D, H, W, L.cin_p, L.ntap, _p(dy), dycs,
                                           dyco, L.cout, _p(self.gw[L.name]), _p(self.gb[L.name]),
                                           C.c_void_p(gs.cuda_stream)))

    def _relu_mask(self, y, ycs, yco, dy, dycs, dyco, lvl, c):
        _chk(lib.sepx_unet_relu_mask(_p(y), ycs, yco, _p(dy), dycs, dyco, self.V[lvl], c,
                                     self.stream_ptr))

    def _pool(self, x, xcs, xco, lvl, c, y, ycs, yco):
        nb = self.shape[0]
        D, H, W = self.dims[lvl]
        _chk(lib.sepx_unet_avgpool(_p(x), xcs, xco, nb, D, H, W, c, _p(y), ycs, yco, self.stream_ptr))

    def _pool_bwd(self, dy, dycs, dyco, lvl, c, dx, dxcs, dxco, acc, mask=None):
        nb = self.shape[0]
        D, H, W = self.dims[lvl]
        m, mcs, mco = (None, 0, 0) if mask is None else (_p(mask[0]), mask[1], mask[2])
        _chk(lib.sepx_unet_avgpool_bwd_masked(_p(dy), dycs, dyco, nb, D, H, W, c, _p(dx), dxcs, dxco,
                                              1 if acc else 0, m, mcs, mco, self.stream_ptr))

    def _up(self, x, xcs, xco, lvl, c, y, ycs, yco):
        """nearest x2 upsampling from level lvl to lvl-1"""
        nb = self.shape[0]
        D, H, W = self.dims[lvl]
        _chk(lib.sepx_unet_upsample(_p(x), xcs, xco, nb, D, H, W, c, _p(y), ycs, yco, self.stream_ptr))

    def _up_bwd(self, dy, dycs, dyco, lvl, c, dx, dxcs, dxco, mask=None):
        nb = self.shape[0]
        D, H, W = self.dims[lvl]
        m, mcs, mco = (None, 0, 0) if mask is None else (_p(mask[0]), mask[1], mask[2])
        _chk(lib.sepx_unet_upsample_bwd_masked(_p(dy), dycs, dyco, nb, D, H, W, c, _p(dx), dxcs, dxco,
                                               m, mcs, mco, self.stream_ptr))

    # ---------------------------------------------------------------- network
    def forward_device(self, xf, scale: float = 1.0):
        """xf: FP32 device tensor [nb, D, H, W] (C-contiguous).  Returns the
        FP32 output tensor (x * scale + N(x * scale)), valid on the library stream."""
        nb, D, H, W = xf.shape
        self._alloc(nb, D, H, W)
        a, Ly = self.a, {L.name: L for L in LAYERS}
        V0 = self.V[0]
        _chk(lib.sepx_unet_to_bf16(_p(xf), V0, scale, _p(a["x0"]), 8, 0, self.stream_ptr))
        with self.torch.cuda.stream(self.stream):
            a["xf"].copy_(xf.reshape(-1))
            if scale != 1.0:
                a["xf"].mul_(scale)
        # encoder
        self._conv(Ly["e1a"], a["x0"], 8, 0, 0, a["e1a"], 16, 0)
        self._conv(Ly["e1b"], a["e1a"], 16, 0, 0, a["cat1"], 48, 32)
        self._pool(a["cat1"], 48, 32, 0, 16, a["p1"], 16, 0)
        self._conv(Ly["e2a"], a["p1"], 16, 0, 1, a["e2a"], 32, 0)
        self._conv(Ly["e2b"], a["e2a"], 32, 0, 1, a["cat2"], 80, 48)
        self._pool(a["cat2"], 80, 48, 1, 32, a["p2"], 32, 0)
        self._conv(Ly["e3a"], a["p2"], 32, 0, 2, a["e3a"], 48, 0)
        self._conv(Ly["e3b"], a["e3a"], 48, 0, 2, a["cat3"], 112, 64)
        self._pool(a["cat3"], 112, 64, 2, 48, a["p3"], 48, 0)
        self._conv(Ly["b4a"], a["p3"], 48, 0, 3, a["b4a"], 64, 0)
        self._conv(Ly["b4b"], a["b4a"], 64, 0, 3, a["b4b"], 64, 0)
        # decoder
        self._up(a["b4b"], 64, 0, 3, 64, a["cat3"], 112, 0)
        self._conv(Ly["d3a"], a["cat3"], 112, 0, 2, a["d3a"], 48, 0)
        self._conv(Ly["d3b"], a["d3a"], 48, 0, 2, a["d3b"], 48, 0)
        self._up(a["d3b"], 48, 0, 2, 48, a["cat2"], 80, 0)
        self._conv(Ly["d2a"], a["cat2"], 80, 0, 1, a["d2a"], 32, 0)
        self._conv(Ly["d2b"], a["d2a"], 32, 0, 1, a["d2b"], 32, 0)
        self._up(a["d2b"], 32, 0, 1, 32, a["cat1"], 48, 0)
        self._conv(Ly["d1a"], a["cat1"], 48, 0, 0, a["d1a"], 16, 0)
        self._conv(Ly["d1b"], a["d1a"], 16, 0, 0, a["d1b"], 16, 0)
        self._conv(Ly["out"], a["d1b"], 16, 0, 0, yf=a["out"], resid=a["xf"])
        return a["out"]

    def backward_device(self):
        """Gradients of the loss whose output gradient sits in g['out']
        (accumulated into gw / gb)."""
        self._alloc_grads()
        a, g, Ly = self.a, self.g, {L.name: L for L in LAYERS}
        # output layer (1x1x1, no ReLU)
        self._wgrad(Ly["out"], a["d1b"], 16, 0, g["out"], 8, 0, 0)
        self._dgrad(Ly["out"], g["out"], 8, 0, 0, g["d1b"], 16, 0, mask=(a["d1b"], 16, 0))
        # level 1 decoder
        self._wgrad(Ly["d1b"], a["d1a"], 16, 0, g["d1b"], 16, 0, 0)
        self._dgrad(Ly["d1b"], g["d1b"], 16, 0, 0, g["d1a"], 16, 0, mask=(a["d1a"], 16, 0))
        self._wgrad(Ly["d1a"], a["cat1"], 48, 0, g["d1a"], 16, 0, 0)
        self._dgrad(Ly["d1a"], g["d1a"], 16, 0, 0, g["cat1"], 48, 0)
        self._up_bwd(g["cat1"], 48, 0, 1, 32, g["d2b"], 32, 0, mask=(a["d2b"], 32, 0))
        # level 2 decoder
        self._wgrad(Ly["d2b"], a["d2a"], 32, 0, g["d2b"], 32, 0, 1)
        self._dgrad(Ly["d2b"], g["d2b"], 32, 0, 1, g["d2a"], 32, 0, mask=(a["d2a"], 32, 0))
        self._wgrad(Ly["d2a"], a["cat2"], 80, 0, g["d2a"], 32, 0, 1)
        self._dgrad(Ly["d2a"], g["d2a"], 32, 0, 1, g["cat2"], 80, 0)
        self._up_bwd(g["cat2"], 80, 0, 2, 48, g["d3b"], 48, 0, mask=(a["d3b"], 48, 0))
        # level 3 decoder
        self._wgrad(Ly["d3b"], a["d3a"], 48, 0, g["d3b"], 48, 0, 2)
        self._dgrad(Ly["d3b"], g["d3b"], 48, 0, 2, g["d3a"], 48, 0, mask=(a["d3a"], 48, 0))
        self._wgrad(Ly["d3a"], a["cat3"], 112, 0, g["d3a"], 48, 0, 2)
        self._dgrad(Ly["d3a"], g["d3a"], 48, 0, 2, g["cat3"], 112, 0)
        self._up_bwd(g["cat3"], 112, 0, 3, 64, g["b4b"], 64, 0, mask=(a["b4b"], 64, 0))
        # bottom
        self._wgrad(Ly["b4b"], a["b4a"], 64, 0, g["b4b"], 64, 0, 3)
        self._dgrad(Ly["b4b"], g["b4b"], 64, 0, 3, g["b4a"], 64, 0, mask=(a["b4a"], 64, 0))
        self._wgrad(Ly["b4a"], a["p3"], 48, 0, g["b4a"], 64, 0, 3)
        self._dgrad(Ly["b4a"], g["b4a"], 64, 0, 3, g["p3"], 48, 0)
        # level 3 encoder: skip gradient (cat3[64:112]) + pooling gradient
        self._pool_bwd(g["p3"], 48, 0, 2, 48, g["cat3"], 112, 64, True, mask=(a["cat3"], 112, 64))
        self._wgrad(Ly["e3b"], a["e3a"], 48, 0, g["cat3"], 112, 64, 2)
        self._dgrad(Ly["e3b"], g["cat3"], 112, 64, 2, g["e3a"], 48, 0, mask=(a["e3a"], 48, 0))
        self._wgrad(Ly["e3a"], a["p2"], 32, 0, g["e3a"], 48, 0, 2)
        self._dgrad(Ly["e3a"], g["e3a"], 48, 0, 2, g["p2"], 32, 0)
        # level 2 encoder
        self._pool_bwd(g["p2"], 32, 0, 1, 32, g["cat2"], 80, 48, True, mask=(a["cat2"], 80, 48))
        self._wgrad(Ly["e2b"], a["e2a"], 32, 0, g["cat2"], 80, 48, 1)
        self._dgrad(Ly["e2b"], g["cat2"], 80, 48, 1, g["e2a"], 32, 0, mask=(a["e2a"], 32, 0))
        self._wgrad(Ly["e2a"], a["p1"], 16, 0, g["e2a"], 32, 0, 1)
        self._dgrad(Ly["e2a"], g["e2a"], 32, 0, 1, g["p1"], 16, 0)
        # level 1 encoder
        self._pool_bwd(g["p1"], 16, 0, 0, 16, g["cat1"], 48, 32, True, mask=(a["cat1"], 48, 32))
        self._wgrad(Ly["e1b"], a["e1a"], 16, 0, g["cat1"], 48, 32, 0)
        self._dgrad(Ly["e1b"], g["cat1"], 48, 32, 0, g["e1a"], 16, 0, mask=(a["e1a"], 16, 0))
        self._wgrad(Ly["e1a"], a["x0"], 8, 0, g["e1a"], 16, 0, 0)
        # join: the main stream waits for the weight gradients
        for gs in self.grad_streams:
            e = self._event()
            e.record(gs)
            self.stream.wait_event(e)
        self._ngs = 0

    def zero_grad(self):
        with self.torch.cuda.stream(self.stream):
            self.flat["g"].zero_()
            self.loss.zero_()

    def loss_grad(self, target):
        """MSE against target (FP32 [nb, D, H, W]); gradient into g['out']."""
        self._alloc_grads()
        _chk(lib.sepx_unet_mse(_p(self.a["out"]), _p(target), self.V[0], _p(self.g["out"]), 8,
                               _p(self.loss), self.stream_ptr))

    def _set_hp(self, lr, b1, b2, eps):
        """next step's Adam hyper-parameters into device memory (ordered on
        the library stream; the host values are staged before this returns)"""
        self.step_count += 1
        hp = self.torch.tensor([lr, b1, b2, eps, float(self.step_count)], dtype=self.torch.float32)
        with self.torch.cuda.stream(self.stream):
            self.hp.copy_(hp)

    def _adam_enqueue(self):
        F = self.flat
        _chk(lib.sepx_unet_adam_dev(_p(F["p"]), _p(F["g"]), _p(F["m"]), _p(F["v"]), F["p"].numel(),
                                    _p(self.hp), self.stream_ptr))

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self._set_hp(lr, b1, b2, eps)
        self._adam_enqueue()
        self.pack()

    def _step_body(self, x, target):
        self.zero_grad()
        self.forward_device(x)
        self.loss_grad(target)
        self.backward_device()
        self._adam_enqueue()
        self.pack()

    def train_step(self, x, target, lr=1e-3):
        """one Adam step on a batch x, target (FP32 device tensors [nb, D, H, W]); returns the loss"""
        self._set_hp(lr, 0.9, 0.999, 1e-8)
        if self.graph is not None and self.graph_io == (x.data_ptr(), target.data_ptr(), tuple(x.shape)):
            _chk(lib.sepx_unet_graph_launch(self.graph, self.stream_ptr))
        else:
            self._step_body(x, target)
        self.stream.synchronize()
        return float(self.loss.item())

    def capture_train_step(self, x, target, lr=1e-3):
        """Capture one whole training step (gradient zeroing, forward, loss,
        backward, Adam, weight packing: about 140 launches) into a CUDA graph
        that reads its batch from x and target; train_step on these same
        tensors then replays it with one launch.  Runs one eager step first
        (buffer allocation, kernel attributes), which trains the network on
        this batch once."""
        self.train_step(x, target, lr=lr)
        self.free_graph()
        self.stream.synchronize()
        _chk(lib.sepx_unet_capture_begin(self.stream_ptr))
        try:
            self._step_body(x, target)
        finally:
            h = C.c_void_p()
            rc = lib.sepx_unet_capture_end(self.stream_ptr, C.byref(h))
        _chk(rc)
        self.graph = h
        self.graph_io = (x.data_ptr(), target.data_ptr(), tuple(x.shape))

    def free_graph(self):
        if self.graph is not None:
            lib.sepx_unet_graph_free(self.graph)
        self.graph, self.graph_io = None, None

    def __del__(self):
        try:
            self.free_graph()
        except Exception:
            pass

    def status(self) -> int:
        return lib.sepx_unet_status()


_LEVEL = {"e1": 0, "e2": 1, "e3": 2, "b4": 3, "d3": 2, "d2": 1, "d1": 0, "ou": 0}


def network_flops(nb: int, n: int) -> float:
    """multiply-add FLOPs (x2) of one forward pass of every convolution on nb x n^3"""
    return sum(2.0 * nb * (n >> _LEVEL[L.name[:2]]) ** 3 * L.ntap * L.cin * L.cout for L in LAYERS)


def conv_layer_timing(cin: int, cout: int, nb: int = 4, n: int = 64, reps: int = 2, halo: bool = True,
                      seed: int = 0) -> float:
    """run one 3x3x3 convolution (random BF16 input and weights, ReLU, BF16
    out) on nb volumes of n^3 voxels `reps` times; returns milliseconds per run
    (CUDA events on the library stream)"""
    import torch
    lib.sepx_setup_cuda(1)
    st = lib.sepx_get_stream()
    stream = torch.cuda.ExternalStream(st)
    g = torch.Generator(device="cuda").manual_seed(seed)
    V = nb * n ** 3
    x = torch.randn(V * cin, device="cuda", generator=g).to(torch.bfloat16)
    w = torch.randn(27 * cin * cout, device="cuda", generator=g) * 0.05
    pk = torch.zeros(lib.sepx_unet_packed_elems(cout, cin, 27, 0), dtype=torch.bfloat16, device="cuda")
    y = torch.empty(V * cout, dtype=torch.bfloat16, device="cuda")
    torch.cuda.synchronize()
    _chk(lib.sepx_unet_pack_weights(_p(w), cout, cin, 27, 0, _p(pk), st))
    prev = lib.sepx_unet_set_halo(1 if halo else 0)
    try:
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            _chk(lib.sepx_unet_conv_fwd(_p(x), cin, 0, nb, n, n, n, cin, 27, _p(pk), None, cout, 1, _p(y),
                                        cout, 0, None, None, st))
        b.record(stream)
        b.synchronize()
    finally:
        lib.sepx_unet_set_halo(prev)
    if lib.sepx_unet_status() != 0:
        raise SepxError("convolution kernel reported a device error")
    return a.elapsed_time(b) / reps


def main(argv=None):
    import argparse
    p = argparse.ArgumentParser(description="time single U-Net convolution layers")
    p.add_argument("--layers", default="16:16,48:16", help="comma list of cin:cout")
    p.add_argument("--nb", type=int, default=4)
    p.add_argument("--n", type=int, default=64)
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--gather", action="store_true", help="use the per-tap gather kernel")
    p.add_argument("--train-steps", type=int, default=0,
                   help="instead: time this many Adam training steps on a batch of nb x n^3")
    p.add_argument("--grad-streams", type=int, default=2,
                   help="side streams for the weight gradients of the training step")
    a = p.parse_args(argv)
    if a.train_steps > 0:
        import torch
        model = UNet3D(seed=3, grad_streams=a.grad_streams)
        g = torch.Generator(device="cuda").manual_seed(9)
        x = torch.randn(a.nb, a.n, a.n, a.n, device="cuda", generator=g)
        t = torch.randn(a.nb, a.n, a.n, a.n, device="cuda", generator=g)
        torch.cuda.synchronize()
        model.train_step(x, t)
        s = model.stream
        flops = 3 * network_flops(a.nb, a.n)   # forward + data gradient + weight gradient

        def timed(step):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record(s)
            for _ in range(a.train_steps):
                step()
            ev[1].record(s)
            ev[1].synchronize()
            return ev[0].elapsed_time(ev[1]) / a.train_steps

        def eager():
            model._set_hp(1e-3, 0.9, 0.999, 1e-8)
            model._step_body(x, t)

        def replay():
            model._set_hp(1e-3, 0.9, 0.999, 1e-8)
            _chk(lib.sepx_unet_graph_launch(model.graph, model.stream_ptr))

        ms = timed(eager)
        print(f"train step on {a.nb} x {a.n}^3: {ms:.3f} ms ({flops / ms / 1e9:.1f} TFLOP/s), launched one by one")
        model.capture_train_step(x, t)
        ms = timed(replay)
        print(f"train step on {a.nb} x {a.n}^3: {ms:.3f} ms ({flops / ms / 1e9:.1f} TFLOP/s), one graph")
        return
    for spec in a.layers.split(","):
        cin, cout = (int(v) for v in spec.split(":"))
        ms = conv_layer_timing(cin, cout, a.nb, a.n, a.reps, halo=not a.gather)
        flops = 2.0 * a.nb * a.n ** 3 * 27 * cin * cout
        print(f"conv {cin}->{cout} on {a.nb} x {a.n}^3: {ms:.3f} ms, {flops / ms / 1e9:.1f} TFLOP/s")


if __name__ == "__main__":
    main()
