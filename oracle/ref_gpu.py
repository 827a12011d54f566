"""The reference's own GPU kernels on the GPU (test infrastructure only).

oracle/_ref/ref_kernels.cubin holds wave_kernel, wave_kernel_adj, damp_kernel
(Born/wave_fkernel.3d8o.cu:31-210) and new_src_inject_kernel,
new_data_inject_kernel, new_data_extract_kernel, img_kernel, img_add_kernel
(Born/gpu_funcs_3d.cu:64-131), compiled from their sources by
oracle/build_oracle.py (build_ref_kernels).  This module loads it with the
CUDA driver API and drives the kernels the way the reference's one-GPU time
loops do: the same launch order, grids, arguments, constants, pointer swaps
and offsets (Born/gpu_funcs_3d.cu:133-315 source_prop, :317-505
rtm_forward, :509-712 rtm_adjoint, :714-803 create_gpu_space and the
transfers), with n_gpus = 1, so the multi-GPU halo launches and peer copies
of those loops never run.

Every device buffer is allocated with eight zeroed planes before and after
the region the reference addresses, so an access the reference's indexing
makes just outside its own allocation lands in zeros instead of faulting.

Only tests/ use this module: it is a second oracle, the reference's kernels
themselves, for the GPU parity tests.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build_oracle import REF_CUBIN

RADIUS = 4
FAT = 4
BLOCK = 16


class _Cuda:
    def __init__(self):
        self.lib = C.CDLL("libcuda.so.1")
        self.lib.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        self.lib.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        self.lib.cuModuleGetGlobal_v2.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_size_t), C.c_void_p,
                                                  C.c_char_p]
        self.lib.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        self.lib.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                            C.c_uint, C.c_uint, C.c_void_p, C.POINTER(C.c_void_p),
                                            C.c_void_p]
        self.lib.cuCtxSynchronize.argtypes = []
        self.lib.cuModuleUnload.argtypes = [C.c_void_p]

    def check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUDA driver error {rc}")


class RefKernels:
    """The reference's kernels on the current GPU (torch's primary context)."""

    KERNELS = ("wave_kernel", "wave_kernel_adj", "damp_kernel", "new_src_inject_kernel",
               "new_data_inject_kernel", "new_data_extract_kernel", "img_kernel", "img_add_kernel")

    def __init__(self, path: Path | None = None):
        import torch
        path = Path(path or REF_CUBIN)
        if not path.exists():
            raise FileNotFoundError(f"{path} is not built (the reference tree is needed to build it)")
        torch.zeros(1, device="cuda")   # the primary context, current on this thread
        torch.cuda.synchronize()
        self.torch = torch
        self.cu = _Cuda()
        self.mod = C.c_void_p()
        self.cu.check(self.cu.lib.cuModuleLoad(C.byref(self.mod), str(path).encode()), "cuModuleLoad")
        self.fn = {}
        for k in self.KERNELS:
            f = C.c_void_p()
            self.cu.check(self.cu.lib.cuModuleGetFunction(C.byref(f), self.mod, k.encode()), k)
            self.fn[k] = f
        self._keep = []

    # ---- constants (cudaMemcpyToSymbol of the reference) ----
    def _sym(self, name, value, ctype):
        ptr, size = C.c_uint64(), C.c_size_t()
        self.cu.check(self.cu.lib.cuModuleGetGlobal_v2(C.byref(ptr), C.byref(size), self.mod, name.encode()), name)
        if isinstance(value, np.ndarray):
            buf = np.ascontiguousarray(value)
            nbytes = buf.nbytes
            src = buf.ctypes.data
        else:
            buf = ctype(value)
            nbytes = C.sizeof(buf)
            src = C.addressof(buf)
        if nbytes > size.value:
            raise RuntimeError(f"{name}: {nbytes} bytes for a {size.value}-byte symbol")
        self.cu.check(self.cu.lib.cuMemcpyHtoD_v2(ptr.value, C.c_void_p(src), nbytes), name)

    def _buf(self, n, pad):
        """float device buffer of n floats with pad zeroed floats on each side;
        returns (tensor, device address of element 0)"""
        t = self.torch.zeros(n + 2 * pad, dtype=self.torch.float32, device="cuda")
        return t, t.data_ptr() + 4 * pad

    def _launch(self, name, grid, block, args):
        holders, ptrs = [], []
        for kind, v in args:
            h = {"p": C.c_uint64, "i": C.c_int, "f": C.c_float}[kind](v)
            holders.append(h)
            ptrs.append(C.cast(C.pointer(h), C.c_void_p))
        arr = (C.c_void_p * len(ptrs))(*ptrs)
        self.cu.check(self.cu.lib.cuLaunchKernel(self.fn[name], grid[0], grid[1], 1, block[0], block[1], 1,
                                                 0, None, arr, None), name)

    # ---- create_gpu_space / transfers (Born/gpu_funcs_3d.cu:714-803), one GPU ----
    def create_gpu_space(self, d1, d2, d3, bc_a, bc_b, n1, n2, n3):
        self.n = (n1, n2, n3)
        self.pad = 8 * n1 * n2
        c00 = lambda d: 8.0 / (5.0 * d * d)
        a, b, c = float(d1), float(d2), float(d3)
        coeffs = np.array([-1025.0 / 576.0 * (c00(a) + c00(b) + c00(c)), c00(a), c00(b), c00(c),
                           -c00(a) / 8.0, -c00(b) / 8.0, -c00(c) / 8.0, c00(a) / 63.0, c00(b) / 63.0,
                           c00(c) / 63.0, -c00(a) / 896.0, -c00(b) / 896.0, -c00(c) / 896.0], np.float32)
        self._sym("n1gpu", n1, C.c_int)
        self._sym("n2gpu", n2, C.c_int)
        self._sym("n3gpu", n3, C.c_int)
        self._sym("bc_agpu", bc_a, C.c_float)
        self._sym("bc_bgpu", bc_b, C.c_float)
        self._sym("coeffs", coeffs, None)
        self.vel_t, self.vel = self._buf(n1 * n2 * n3, self.pad)

    def transfer_sinc_tables(self, sinc_s, sinc_d):
        s = np.ascontiguousarray(sinc_s, np.float32)
        d = np.ascontiguousarray(sinc_d, np.float32)
        self.ts = self.torch.tensor(s.ravel()).cuda()
        self.td = self.torch.tensor(d.ravel()).cuda()
        self._sym("sinc_s_table", self.ts.data_ptr(), C.c_uint64)
        self._sym("sinc_d_table", self.td.data_ptr(), C.c_uint64)
        self._sym("nsinc_gpu", s.shape[1], C.c_int)

    def transfer_source_func(self, locs, vals):
        vals = np.ascontiguousarray(vals, np.float32)
        self.npts_s = vals.shape[0]
        self.src_vals = self.torch.tensor(vals.ravel()).cuda()
        self.src_locs = self.torch.tensor(np.ascontiguousarray(locs, np.int32)).cuda()
        self._sym("ntrace_gpu", vals.shape[1], C.c_int)
        self._sym("srcgeom_gpu0", self.src_locs.data_ptr(), C.c_uint64)
        self._sym("source_gpu0", self.src_vals.data_ptr(), C.c_uint64)

    def transfer_receiver_func(self, nx, ny, locs, vals):
        vals = np.ascontiguousarray(vals, np.float32)
        self.rec_shape = vals.shape
        self.data = self.torch.tensor(vals.ravel()).cuda()
        self.rec_locs = self.torch.tensor(np.ascontiguousarray(locs, np.int32)).cuda()
        self._sym("rec_nx_gpu", nx, C.c_int)
        self._sym("rec_ny_gpu", ny, C.c_int)
        self._sym("ntrace_gpu", vals.shape[1], C.c_int)
        self._sym("datageom_gpu0", self.rec_locs.data_ptr(), C.c_uint64)
        self._sym("data_gpu0", self.data.data_ptr(), C.c_uint64)

    def transfer_vel_func1(self, vel):
        self.vel_t[self.pad:self.pad + vel.size] = self.torch.tensor(np.ascontiguousarray(vel, np.float32).ravel()).cuda()

    # ---- geometry of the one-GPU loops ----
    def _geom(self):
        n1, n2, n3 = self.n
        offset = RADIUS * n1 * n2 + RADIUS * n1 + RADIUS
        grid = ((n1 - 2 * FAT) // BLOCK, (n2 - 2 * FAT) // BLOCK)
        gridx = ((n1 + BLOCK - 1) // BLOCK, (n2 + BLOCK - 1) // BLOCK)
        return offset, grid, gridx, RADIUS, n3 - 2 * RADIUS

    def _host(self, t):
        n1, n2, n3 = self.n
        self.cu.check(self.cu.lib.cuCtxSynchronize(), "cuCtxSynchronize")
        return t[self.pad:self.pad + n1 * n2 * n3].cpu().numpy().reshape(n3, n2, n1)

    # ---- the loops ----
    def source_prop(self, jt, npts, nt):
        """Born/gpu_funcs_3d.cu:133-315: nt + 1 steps; returns (p0, p1)"""
        n1, n2, n3 = self.n
        off, grid, _, s3, e3 = self._geom()
        self._sym("dir_gpu", 1, C.c_int)
        (t0, p0), (t1, p1) = self._buf(n1 * n2 * n3, self.pad), self._buf(n1 * n2 * n3, self.pad)
        for it in range(nt + 1):
            idd, ii = it // jt, it % jt
            self._launch("wave_kernel", grid, (16, 16),
                         [("p", p0 + 4 * off), ("p", p1 + 4 * off), ("p", p0 + 4 * off), ("p", self.vel + 4 * off),
                          ("i", s3), ("i", e3)])
            self._launch("new_src_inject_kernel", (1, 1), (npts, 1), [("i", idd), ("i", ii), ("p", p0)])
            (t0, p0), (t1, p1) = (t1, p1), (t0, p0)
        return self._host(t0), self._host(t1)

    def rtm_forward(self, jt, npts_src, nt, img):
        """Born/gpu_funcs_3d.cu:317-505: the Born traces accumulate onto the
        transferred receiver traces; returns them ([nrec][ntrace])"""
        n1, n2, n3 = self.n
        nv = n1 * n2 * n3
        off, grid, gridx, s3, e3 = self._geom()
        self._sym("dir_gpu", 1, C.c_int)
        (ts0, s0), (ts1, s1) = self._buf(nv, self.pad), self._buf(nv, self.pad)
        (td0, d0), (td1, d1) = self._buf(nv, self.pad), self._buf(nv, self.pad)
        ti, im = self._buf(nv, self.pad)
        ti[self.pad:self.pad + nv] = self.torch.tensor(np.ascontiguousarray(img, np.float32).ravel()).cuda()
        for it in range(nt):
            idd, ii = it // jt, it % jt
            damp = lambda a, b: self._launch("damp_kernel", grid, (16, 16),
                                             [("p", a), ("p", b), ("i", s3), ("i", e3), ("i", 0), ("i", 1)])
            damp(d0, d1)
            damp(d0, d1)
            damp(s0, s1)
            self._launch("wave_kernel_adj", grid, (16, 16),
                         [("p", d0 + 4 * off), ("p", d1 + 4 * off), ("p", d0 + 4 * off), ("p", self.vel + 4 * off),
                          ("i", s3), ("i", e3)])
            self._launch("wave_kernel", grid, (16, 16),
                         [("p", s0 + 4 * off), ("p", s1 + 4 * off), ("p", s0 + 4 * off), ("p", self.vel + 4 * off),
                          ("i", s3), ("i", e3)])
            self._launch("new_src_inject_kernel", (1, 1), (npts_src, 1), [("i", idd), ("i", ii), ("p", s0)])
            if it % jt == 0:
                self._launch("img_add_kernel", grid, (16, 16), [("p", im), ("p", d0), ("p", s0)])
            self._launch("new_data_extract_kernel", gridx, (16, 16), [("i", idd), ("i", ii), ("p", d0)])
            (ts0, s0), (ts1, s1) = (ts1, s1), (ts0, s0)
            (td0, d0), (td1, d1) = (td1, d1), (td0, d0)
        self.cu.check(self.cu.lib.cuCtxSynchronize(), "cuCtxSynchronize")
        return self.data.cpu().numpy().reshape(self.rec_shape)

    def rtm_adjoint(self, jt, npts_src, nt, p0_s, p1_s):
        """Born/gpu_funcs_3d.cu:509-712: receiver back-propagation, source
        rebuilt backwards (re-injection into src_p1 at sample it+1, dir = -1),
        zero-lag imaging; returns the image"""
        n1, n2, n3 = self.n
        nv = n1 * n2 * n3
        off, grid, gridx, s3, e3 = self._geom()
        (ts0, s0), (ts1, s1) = self._buf(nv + RADIUS * n1 * n2, self.pad), self._buf(nv + RADIUS * n1 * n2, self.pad)
        (td0, d0), (td1, d1) = self._buf(nv, self.pad), self._buf(nv, self.pad)
        ti, im = self._buf(nv, self.pad)
        ts0[self.pad:self.pad + nv] = self.torch.tensor(np.ascontiguousarray(p0_s, np.float32).ravel()).cuda()
        ts1[self.pad:self.pad + nv] = self.torch.tensor(np.ascontiguousarray(p1_s, np.float32).ravel()).cuda()
        self._sym("dir_gpu", -1, C.c_int)
        for it in range(nt - 1, -1, -1):
            id_s, i_s = (it + 1) // jt, (it + 1) % jt
            idd, ii = it // jt, it % jt
            self._launch("damp_kernel", grid, (16, 16),
                         [("p", d0), ("p", d1), ("i", s3), ("i", e3), ("i", 0), ("i", 1)])
            self._launch("wave_kernel", grid, (16, 16),
                         [("p", d0 + 4 * off), ("p", d1 + 4 * off), ("p", d0 + 4 * off), ("p", self.vel + 4 * off),
                          ("i", s3), ("i", e3)])
            if it < nt - 1:
                self._launch("wave_kernel", grid, (16, 16),
                             [("p", s0 + 4 * off), ("p", s1 + 4 * off), ("p", s0 + 4 * off),
                              ("p", self.vel + 4 * off), ("i", s3), ("i", e3)])
                self._launch("new_src_inject_kernel", (1, 1), (npts_src, 1), [("i", id_s), ("i", i_s), ("p", s1)])
            self._launch("new_data_inject_kernel", gridx, (16, 16), [("i", idd), ("i", ii), ("p", d0)])
            if ii == 0:
                self._launch("img_kernel", grid, (16, 16), [("p", im), ("p", d0), ("p", s0)])
            if it < nt - 1:
                (ts0, s0), (ts1, s1) = (ts1, s1), (ts0, s0)
            (td0, d0), (td1, d1) = (td1, d1), (td0, d0)
        return self._host(ti)

    def close(self):
        if self.mod:
            self.cu.lib.cuModuleUnload(self.mod)
            self.mod = None
