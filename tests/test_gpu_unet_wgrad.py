"""The tap-stacked weight gradients (csrc/sepx_unet_wgrad.inc: the z-walk
form and the per-tile form) against the FP64 restatement
(oracle/unet_oracle.py) and the per-tap gather kernel.

Shapes: every (cin, cout) of the U-Net that takes the kernel (cout <= 40,
cin <= 80), ragged planes (H not a multiple of 16, W not a multiple of 8),
an x view and a dy view that are channel slices of wider buffers, volumes
with one plane.  dw and db are added to what they hold.

Tolerance: relative L2 <= 1e-5 against the FP64 sums of the same BF16
operands (FP32 accumulation in a different order).  Every form adds its
CTAs' partial sums in a fixed order, so two runs give identical bits.
"""
import numpy as np
import pytest

from oracle import unet_oracle as U
from tests.harness import rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

CASES = [
    # cin, cout, nb, D, H, W, x channel slice (stride, offset), dy slice (stride, offset)
    (8, 16, 2, 4, 16, 16, (8, 0), (16, 0)),
    (16, 16, 1, 3, 19, 13, (48, 32), (16, 0)),
    (16, 32, 2, 2, 16, 24, (16, 0), (80, 48)),
    (32, 32, 1, 4, 9, 20, (32, 0), (32, 0)),
    (48, 16, 1, 2, 32, 16, (48, 0), (48, 32)),
    (80, 32, 1, 3, 16, 16, (80, 0), (32, 0)),
    (24, 40, 1, 1, 7, 5, (24, 0), (40, 0)),
    # several windows along z per volume
    (16, 16, 2, 40, 16, 16, (16, 0), (16, 0)),
    (48, 16, 1, 33, 16, 24, (48, 0), (16, 0)),
]


def _bf(a):
    return torch.tensor(np.ascontiguousarray(a, np.float32)).to(torch.bfloat16).cuda()


@pytest.fixture(scope="module")
def unet():
    from sep_code_gb300 import unet
    return unet


def _run(unet, xt, xs, dyt, ds, cin, cout, nb, D, H, W, dw0, db0):
    from sep_code_gb300._lib import lib
    st = lib.sepx_get_stream()
    dw = torch.tensor(dw0).cuda()
    db = torch.tensor(db0).cuda()
    torch.cuda.synchronize()
    unet._chk(lib.sepx_unet_conv_wgrad_bias(unet._p(xt), xs[0], xs[1], nb, D, H, W, cin, 27,
                                            unet._p(dyt), ds[0], ds[1], cout, unet._p(dw),
                                            unet._p(db), st))
    lib.sepx_synchronize()
    torch.cuda.synchronize()
    assert lib.sepx_unet_status() == 0
    return dw.cpu().numpy(), db.cpu().numpy()


@pytest.mark.parametrize("cin,cout,nb,D,H,W,xs,ds", CASES)
def test_wgrad_bias_against_fp64_and_gather(unet, cin, cout, nb, D, H, W, xs, ds):
    from sep_code_gb300._lib import lib
    lib.sepx_setup_cuda(1)
    rng = np.random.default_rng(cin * 1000 + cout * 10 + H)
    cout_p = (cout + 7) // 8 * 8
    xbuf = np.zeros((nb, D, H, W, xs[0]))
    x = U.bf16(rng.standard_normal((nb, D, H, W, cin)))
    xbuf[..., xs[1]:xs[1] + cin] = x
    dbuf = np.zeros((nb, D, H, W, ds[0]))
    dy = np.zeros((nb, D, H, W, cout_p))
    dy[..., :cout] = U.bf16(rng.standard_normal((nb, D, H, W, cout)))
    dbuf[..., ds[1]:ds[1] + cout_p] = dy
    # neighbouring channels of the wider buffers hold data the kernel must not read
    xbuf[..., :xs[1]] = 7.0
    xbuf[..., xs[1] + cin:] = -5.0
    dbuf[..., :ds[1]] = 3.0
    dbuf[..., ds[1] + cout_p:] = -2.0
    xt, dyt = _bf(xbuf), _bf(dbuf)
    dw0 = np.full(27 * cin * cout, 0.25, np.float32)
    db0 = np.full(cout, -0.5, np.float32)
    want_dw = U.conv_wgrad(x, dy[..., :cout], 27, cin).ravel() + 0.25
    want_db = dy[..., :cout].sum((0, 1, 2, 3)) - 0.5
    res = {}
    for form in (2, 1, 0):
        prev = lib.sepx_unet_set_wgrad_form(form)
        try:
            dw, db = _run(unet, xt, xs, dyt, ds, cin, cout, nb, D, H, W, dw0, db0)
            dw2, db2 = _run(unet, xt, xs, dyt, ds, cin, cout, nb, D, H, W, dw0, db0)
        finally:
            lib.sepx_unet_set_wgrad_form(prev)
        e_w, e_b = rel_l2(dw, want_dw), rel_l2(db, want_db)
        same = np.array_equal(dw, dw2) and np.array_equal(db, db2)
        res[form] = (e_w, e_b, same)
        assert e_w <= 1e-5 and e_b <= 1e-5, (form, e_w, e_b)
        assert same, form   # every form adds its partial sums in a fixed order
    print(f"WGRAD_TMA cin {cin} cout {cout} {nb}x{D}x{H}x{W}: (dw rel-L2, db rel-L2, repeatable) "
          f"z-walk {res[2]}, per-tile {res[1]}, gather {res[0]}")


def test_bias_grad_kernel(unet):
    """the stand-alone bias gradient (layers the tap-stacked kernel does not
    take): c not a multiple of 8, a channel slice, repeatable bits"""
    from sep_code_gb300._lib import lib
    lib.sepx_setup_cuda(1)
    st = lib.sepx_get_stream()
    rng = np.random.default_rng(5)
    V = 70001
    for c, stride, off in ((1, 8, 0), (48, 112, 64), (64, 64, 0), (13, 24, 8)):
        buf = U.bf16(rng.standard_normal((V, stride)))
        want = buf[:, off:off + c].sum(0) + 1.0
        t = _bf(buf)
        outs = []
        for _ in range(2):
            db = torch.ones(c, dtype=torch.float32).cuda()
            torch.cuda.synchronize()
            unet._chk(lib.sepx_unet_bias_grad(unet._p(t), stride, off, V, c, unet._p(db), st))
            lib.sepx_synchronize()
            torch.cuda.synchronize()
            outs.append(db.cpu().numpy())
        assert rel_l2(outs[0], want) <= 1e-5, (c, rel_l2(outs[0], want))
        assert np.array_equal(outs[0], outs[1])
