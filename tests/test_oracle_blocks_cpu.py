"""The oracle's loop order: its stencils walk blocks of planes x rows and its
sponge visits only the rows and row ends that can be damped.  Neither may
change a result: the stencils against the same library built as one block
(the plain plane-by-plane walk) on grids whose interior the blocks cut
raggedly, and the sponge against a numpy restatement of damp_kernel
(Born/wave_fkernel.3d8o.cu:183-210), bit for bit."""
import ctypes as C

import numpy as np
import pytest

from oracle.bindings import Oracle, damp_ntab
from oracle.build_oracle import build_oracle


@pytest.fixture(scope="module")
def one_block(tmp_path_factory):
    out = tmp_path_factory.mktemp("orc") / "libsepx_oracle_one_block.so"
    return Oracle(build_oracle(out=out, defines=("OZB=1000000", "OYB=1000000")))


GRIDS = [(48, 40, 64), (37 + 16, 23 + 24, 70), (96, 80, 36)]   # (n1, n2, n3)


def _ctx(orc, n, ntab, keep):
    coeffs = np.zeros(13, np.float32)
    orc.lib.orc_fd_coeffs(10.0, 12.5, 8.0, coeffs)
    tab = np.linspace(0.9, 1.0, ntab).astype(np.float32)
    tab[-3:] = 1.0
    keep.append(tab)
    return orc.make_ctx(n, coeffs, tab, 8, None, None, None, None, None, 0, 0, keep), tab


@pytest.mark.parametrize("n", GRIDS)
def test_stencil_blocks_equal_one_block(oracle, one_block, n):
    rng = np.random.default_rng(sum(n))
    shape = (n[2], n[1], n[0])
    p0 = rng.standard_normal(shape).astype(np.float32)
    p1 = rng.standard_normal(shape).astype(np.float32)
    vel = rng.uniform(0.01, 0.2, shape).astype(np.float32)
    for vel_inside in (0, 1):
        outs = []
        for orc in (oracle, one_block):
            keep = []
            ctx, _ = _ctx(orc, n, damp_ntab(*n), keep)
            o = p0.copy()
            orc.lib.orc_wave_step_f32(C.byref(ctx), vel_inside, o, p1, vel)
            outs.append(o)
        assert not np.array_equal(outs[0], p0)
        assert outs[0].tobytes() == outs[1].tobytes(), (n, vel_inside)


def _damp_numpy(n, tab, p0, p1):
    n1, n2, n3 = n
    xg, yg = 16 * ((n1 - 8) // 16), 16 * ((n2 - 8) // 16)
    z, y, x = np.meshgrid(np.arange(n3), np.arange(yg), np.arange(xg), indexing="ij")
    e = np.minimum.reduce([x - 4, z - 4, n2 - 4 - y, n1 - 4 - x, n3 - 4 - z, y - 4])
    ok = (e >= 0) & (e < len(tab))
    t = np.ones(e.shape, np.float32)
    t[ok] = tab[e[ok]]
    scale = ok & (t < 1)
    a0, a1 = p0.copy(), p1.copy()
    sub0, sub1 = a0[:, :yg, :xg], a1[:, :yg, :xg]
    sub1[scale] = sub1[scale] * t[scale]
    sub0[scale] = sub0[scale] * t[scale]
    return a0, a1


@pytest.mark.parametrize("n", GRIDS)
@pytest.mark.parametrize("ntab", [6, 21, None])
def test_sponge_shell_equals_full_walk(oracle, n, ntab):
    rng = np.random.default_rng(7)
    shape = (n[2], n[1], n[0])
    p0 = rng.standard_normal(shape).astype(np.float32)
    p1 = rng.standard_normal(shape).astype(np.float32)
    keep = []
    ctx, tab = _ctx(oracle, n, ntab or damp_ntab(*n), keep)
    want0, want1 = _damp_numpy(n, tab, p0, p1)
    o0, o1 = p0.copy(), p1.copy()
    oracle.lib.orc_damp_f32(C.byref(ctx), o0, o1)
    assert not np.array_equal(o0, p0)
    assert o0.tobytes() == want0.tobytes() and o1.tobytes() == want1.tobytes()
