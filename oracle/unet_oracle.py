"""CPU FP64 restatement of the learned preconditioner's network (test
infrastructure only: tests/ use it to check the GPU kernels and gradients).

The U-Net has no counterpart in the reference; this module restates the
published mathematics -- 3-D cross-correlation with zero padding, its data and
weight gradients (back-propagation), 2x2x2 average pooling, nearest
upsampling, ReLU, mean-squared error -- in float64 numpy, with the network
wiring of sep_code_gb300/unet.py.  Where the GPU stores a tensor in BF16 the
restatement rounds the same tensor to BF16 (round to nearest even), so the two
differ only by the order of FP32 accumulation.

Layouts: activations [nb, D, H, W, C]; weights [ntap][cin_p][cout].
"""
from __future__ import annotations

import numpy as np


def bf16(a):
    """round to the nearest BF16 value (ties to even), returned as float64"""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    if nan.any():
        out[nan] = np.nan
    return out


def taps(ntap):
    if ntap == 1:
        return [(0, 0, 0)]
    return [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]


def _shift(x, dz, dy, dx):
    """s[v] = x[v + (dz, dy, dx)] with zeros outside"""
    nb, D, H, W, C = x.shape
    p = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    return p[:, 1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :]


def conv_fwd(x, w, b, relu):
    ntap, cin_p, cout = w.shape
    y = np.zeros(x.shape[:4] + (cout,))
    for t, (dz, dy, dx) in enumerate(taps(ntap)):
        y += _shift(x[..., :cin_p], dz, dy, dx) @ w[t]
    if b is not None:
        y += b
    return np.maximum(y, 0.0) if relu else y


def conv_dgrad(dy, w):
    """dx[v] = sum_t dy[v - off(t)] w[t]^T"""
    ntap, cin_p, cout = w.shape
    dx = np.zeros(dy.shape[:4] + (cin_p,))
    for t, (dz, dyy, dxx) in enumerate(taps(ntap)):
        dx += _shift(dy[..., :cout] @ w[t].T, -dz, -dyy, -dxx)
    return dx


def conv_wgrad(x, dy, ntap, cin_p):
    cout = dy.shape[-1]
    dw = np.zeros((ntap, cin_p, cout))
    for t, (dz, dyy, dxx) in enumerate(taps(ntap)):
        xs = _shift(x[..., :cin_p], dz, dyy, dxx).reshape(-1, cin_p)
        dw[t] = xs.T @ dy.reshape(-1, cout)
    return dw


def avgpool(x):
    nb, D, H, W, C = x.shape
    return x.reshape(nb, D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4, 6))


def avgpool_bwd(dy):
    return np.repeat(np.repeat(np.repeat(dy, 2, 1), 2, 2), 2, 3) / 8.0


def upsample(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 1), 2, 2), 2, 3)


def upsample_bwd(dy):
    nb, D, H, W, C = dy.shape
    return dy.reshape(nb, D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4, 6))


CH = (16, 32, 48, 64)


def forward_backward(params, x, target, round_bf16=True):
    """Loss and parameter gradients of the network on x, target [nb, D, H, W]
    (FP64 arithmetic, BF16 rounding where the GPU stores BF16 unless
    round_bf16 is False).  params: {name: (w [ntap][cin_p][cout], b [cout])}
    (weights rounded to BF16 here as the GPU packs them).  Returns
    (out, loss, {name: (dw, db)})."""
    bf16 = globals()["bf16"] if round_bf16 else (lambda a: np.asarray(a, np.float64))
    W_ = {k: bf16(v[0]) for k, v in params.items()}
    B_ = {k: np.asarray(v[1], np.float64) for k, v in params.items()}
    x = np.asarray(x, np.float64)[..., None]
    x0 = np.zeros(x.shape[:4] + (8,))
    x0[..., :1] = bf16(x)
    A = {}

    def conv(name, inp, relu=True):
        return bf16(conv_fwd(inp, W_[name], B_[name], relu))

    A["e1a"] = conv("e1a", x0)
    A["e1b"] = conv("e1b", A["e1a"])
    A["p1"] = bf16(avgpool(A["e1b"]))
    A["e2a"] = conv("e2a", A["p1"])
    A["e2b"] = conv("e2b", A["e2a"])
    A["p2"] = bf16(avgpool(A["e2b"]))
    A["e3a"] = conv("e3a", A["p2"])
    A["e3b"] = conv("e3b", A["e3a"])
    A["p3"] = bf16(avgpool(A["e3b"]))
    A["b4a"] = conv("b4a", A["p3"])
    A["b4b"] = conv("b4b", A["b4a"])
    A["cat3"] = np.concatenate([upsample(A["b4b"]), A["e3b"]], -1)
    A["d3a"] = conv("d3a", A["cat3"])
    A["d3b"] = conv("d3b", A["d3a"])
    A["cat2"] = np.concatenate([upsample(A["d3b"]), A["e2b"]], -1)
    A["d2a"] = conv("d2a", A["cat2"])
    A["d2b"] = conv("d2b", A["d2a"])
    A["cat1"] = np.concatenate([upsample(A["d2b"]), A["e1b"]], -1)
    A["d1a"] = conv("d1a", A["cat1"])
    A["d1b"] = conv("d1b", A["d1a"])
    out = conv_fwd(A["d1b"], W_["out"], B_["out"], False)[..., 0] + x[..., 0]
    V = out.size
    r = out - np.asarray(target, np.float64)
    loss = float((r * r).sum() / V)
    G = {}
    g_out = np.zeros(out.shape + (8,))
    g_out[..., 0] = bf16(2.0 * r / V)

    def back(name, dy, inp, ntap=27):
        """weight / bias gradient of layer `name` and the BF16 data gradient"""
        w = W_[name]
        G[name] = (conv_wgrad(inp, dy[..., :w.shape[2]], ntap, w.shape[1]),
                   dy[..., :w.shape[2]].reshape(-1, w.shape[2]).sum(0))
        return bf16(conv_dgrad(dy[..., :w.shape[2]], w))

    def mask(dy, y):
        return np.where(y > 0, dy, 0.0)

    g = back("out", g_out, A["d1b"], ntap=1)
    g = mask(g, A["d1b"]); g = back("d1b", g, A["d1a"])
    g = mask(g, A["d1a"]); g_cat1 = back("d1a", g, A["cat1"])
    g = bf16(upsample_bwd(g_cat1[..., :32]))
    g = mask(g, A["d2b"]); g = back("d2b", g, A["d2a"])
    g = mask(g, A["d2a"]); g_cat2 = back("d2a", g, A["cat2"])
    g = bf16(upsample_bwd(g_cat2[..., :48]))
    g = mask(g, A["d3b"]); g = back("d3b", g, A["d3a"])
    g = mask(g, A["d3a"]); g_cat3 = back("d3a", g, A["cat3"])
    g = bf16(upsample_bwd(g_cat3[..., :64]))
    g = mask(g, A["b4b"]); g = back("b4b", g, A["b4a"])
    g = mask(g, A["b4a"]); g_p3 = back("b4a", g, A["p3"])
    g = bf16(avgpool_bwd(g_p3) + g_cat3[..., 64:])
    g = mask(g, A["e3b"]); g = back("e3b", g, A["e3a"])
    g = mask(g, A["e3a"]); g_p2 = back("e3a", g, A["p2"])
    g = bf16(avgpool_bwd(g_p2) + g_cat2[..., 48:])
    g = mask(g, A["e2b"]); g = back("e2b", g, A["e2a"])
    g = mask(g, A["e2a"]); g_p1 = back("e2a", g, A["p1"])
    g = bf16(avgpool_bwd(g_p1) + g_cat1[..., 32:])
    g = mask(g, A["e1b"]); g = back("e1b", g, A["e1a"])
    g = mask(g, A["e1a"]); back("e1a", g, x0)
    return out, loss, G
