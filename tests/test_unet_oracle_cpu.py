"""Pins of the U-Net restatement (oracle/unet_oracle.py) on the CPU: the
network has no counterpart in the reference, so the restatement is checked
against the mathematics itself -- adjoint identities of the convolution,
pooling and upsampling pairs, and central finite differences of the loss
(FP64, no BF16 rounding) against its back-propagated gradient."""
import numpy as np

from oracle import unet_oracle as U
from sep_code_gb300.unet import LAYERS, init_params


def _dot(a, b):
    return float(np.sum(np.asarray(a, np.float64) * np.asarray(b, np.float64)))


def test_convolution_adjoint_pairs():
    rng = np.random.default_rng(0)
    for ntap, cin, cout in ((27, 8, 16), (27, 16, 8), (1, 16, 8)):
        x = rng.standard_normal((1, 4, 6, 8, cin))
        y = rng.standard_normal((1, 4, 6, 8, cout))
        w = rng.standard_normal((ntap, cin, cout))
        a = _dot(U.conv_fwd(x, w, None, False), y)
        assert abs(a - _dot(x, U.conv_dgrad(y, w))) <= 1e-10 * abs(a)
        assert abs(a - _dot(w, U.conv_wgrad(x, y, ntap, cin))) <= 1e-10 * abs(a)


def test_pool_upsample_adjoint_pairs():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2, 4, 6, 8, 8))
    y = rng.standard_normal((2, 2, 3, 4, 8))
    assert abs(_dot(U.avgpool(x), y) - _dot(x, U.avgpool_bwd(y))) <= 1e-10
    assert abs(_dot(U.upsample(y), x) - _dot(y, U.upsample_bwd(x))) <= 1e-10


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0, 1e-30], np.float32)
    r = U.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0            # tie to even
    assert r[2] == 1.0078125                      # above the tie rounds up
    assert abs(r[3] + 3.140625) < 1e-12
    assert r[4] == 65536.0


def test_network_gradient_finite_differences():
    rng = np.random.default_rng(4)
    params = init_params(seed=3)
    w, b = params["out"]
    params["out"] = (rng.standard_normal(w.shape).astype(np.float32) * 0.5, b)
    x = rng.standard_normal((1, 8, 8, 8))
    t = rng.standard_normal((1, 8, 8, 8))
    _, loss, g = U.forward_backward(params, x, t, round_bf16=False)
    h = 1e-6   # small enough that no ReLU changes sides
    for L in LAYERS:
        w, b = params[L.name]
        idx = tuple(int(rng.integers(0, s)) for s in w.shape)
        if L.name == "e1a":
            idx = (idx[0], 0, idx[2])   # only the first input channel is live
        p2 = dict(params)
        wp, wm = w.astype(np.float64).copy(), w.astype(np.float64).copy()
        wp[idx] += h
        wm[idx] -= h
        p2[L.name] = (wp, b)
        lp = U.forward_backward(p2, x, t, round_bf16=False)[1]
        p2[L.name] = (wm, b)
        lm = U.forward_backward(p2, x, t, round_bf16=False)[1]
        fd = (lp - lm) / (2 * h)
        an = g[L.name][0][idx]
        assert abs(fd - an) <= 1e-8 + 1e-5 * abs(an), (L.name, fd, an)
