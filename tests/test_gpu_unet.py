"""The learned preconditioner's tensor-core kernels against the CPU FP64
restatement (oracle/unet_oracle.py): convolution forward, data gradient and
weight gradient per layer shape, the memory-bound pieces, and the gradients of
the whole network (back-propagation through all 15 layers).

Tolerances: FP32 outputs of a convolution of BF16 operands differ from the
FP64 sum only by FP32 accumulation order -- relative L2 <= 1e-5.  Outputs
stored in BF16 carry its rounding (2^-9 relative): <= 8e-3.  Network
gradients, where BF16 rounding of every activation can flip near a rounding
boundary and propagate: within 0.08 of the BF16-storage restatement per layer
(measured: at most 0.054, at the 4^3 bottom level, whose sums have fewest
terms; 0.0006-0.03 elsewhere), and no further from the exact FP64 gradient
than twice that restatement.
"""
import numpy as np
import pytest

from oracle import unet_oracle as U
from tests.harness import rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def net():
    from sep_code_gb300 import unet
    return unet


def _bf(a):
    return torch.tensor(np.ascontiguousarray(a, np.float32)).to(torch.bfloat16).cuda()


def _np(t):
    return t.float().cpu().numpy().astype(np.float64)


def _sync(net):
    from sep_code_gb300._lib import lib
    lib.sepx_synchronize()
    torch.cuda.synchronize()


CASES = [(8, 16, 27), (16, 32, 27), (48, 64, 27), (112, 48, 27), (80, 32, 27), (16, 1, 1),
         (64, 112, 27)]


@pytest.mark.parametrize("cin,cout,ntap", CASES)
def test_conv_forward_dgrad_wgrad(net, cin, cout, ntap):
    from sep_code_gb300._lib import lib
    rng = np.random.default_rng(cin * 100 + cout)
    nb, D, H, W = 2, 8, 16, 16
    cin_p = (cin + 7) // 8 * 8
    x = U.bf16(rng.standard_normal((nb, D, H, W, cin_p)))
    w = (rng.standard_normal((ntap, cin_p, cout)) / np.sqrt(ntap * cin)).astype(np.float32)
    b = rng.standard_normal(cout).astype(np.float32)
    lib.sepx_setup_cuda(1)
    st = lib.sepx_get_stream()
    wt = torch.tensor(w, dtype=torch.float32).cuda()
    bt = torch.tensor(b, dtype=torch.float32).cuda()
    pk = torch.zeros(net.lib.sepx_unet_packed_elems(cout, cin_p, ntap, 0), dtype=torch.bfloat16).cuda()
    pkt = torch.zeros(net.lib.sepx_unet_packed_elems(cout, cin_p, ntap, 1), dtype=torch.bfloat16).cuda()
    torch.cuda.synchronize()
    net._chk(net.lib.sepx_unet_pack_weights(net._p(wt), cout, cin_p, ntap, 0, net._p(pk), st))
    net._chk(net.lib.sepx_unet_pack_weights(net._p(wt), cout, cin_p, ntap, 1, net._p(pkt), st))
    xt = _bf(x)
    V = nb * D * H * W
    yf = torch.zeros(V * cout, dtype=torch.float32).cuda()
    torch.cuda.synchronize()
    # forward, FP32 output
    net._chk(net.lib.sepx_unet_conv_fwd(net._p(xt), cin_p, 0, nb, D, H, W, cin_p, ntap, net._p(pk),
                                        net._p(bt), cout, 0, None, 0, 0, net._p(yf), None, st))
    _sync(net)
    want = U.conv_fwd(x, U.bf16(w), b, False)
    got = yf.cpu().numpy().reshape(want.shape)
    assert net.lib.sepx_unet_status() == 0
    assert rel_l2(got, want) <= 1e-5, rel_l2(got, want)
    # forward with ReLU into a BF16 channel slice of a wider buffer
    if cout % 8 == 0:
        ybuf = torch.zeros((V, cout + 16), dtype=torch.bfloat16).cuda()
        torch.cuda.synchronize()
        net._chk(net.lib.sepx_unet_conv_fwd(net._p(xt), cin_p, 0, nb, D, H, W, cin_p, ntap, net._p(pk),
                                            net._p(bt), cout, 1, net._p(ybuf), cout + 16, 8, None,
                                            None, st))
        _sync(net)
        yb = _np(ybuf)
        assert rel_l2(yb[:, 8:8 + cout].reshape(want.shape), np.maximum(want, 0)) <= 8e-3
        assert not yb[:, :8].any() and not yb[:, 8 + cout:].any()
    # data gradient: dx = conv^T(dy), BF16 output
    cout_p = (cout + 7) // 8 * 8
    dy = np.zeros((nb, D, H, W, cout_p))
    dy[..., :cout] = U.bf16(rng.standard_normal((nb, D, H, W, cout)))
    dyt = _bf(dy)
    dx = torch.zeros((V, cin_p), dtype=torch.bfloat16).cuda()
    torch.cuda.synchronize()
    net._chk(net.lib.sepx_unet_conv_fwd(net._p(dyt), cout_p, 0, nb, D, H, W, cout_p, ntap, net._p(pkt),
                                        None, cin_p, 0, net._p(dx), cin_p, 0, None, None, st))
    _sync(net)
    want_dx = U.conv_dgrad(dy[..., :cout], U.bf16(w))
    assert rel_l2(_np(dx).reshape(want_dx.shape), want_dx) <= 8e-3
    # weight gradient, FP32 accumulation (added to what dw holds)
    dw = torch.full((ntap * cin_p * cout,), 0.25, dtype=torch.float32).cuda()
    torch.cuda.synchronize()
    net._chk(net.lib.sepx_unet_conv_wgrad(net._p(xt), cin_p, 0, nb, D, H, W, cin_p, ntap, net._p(dyt),
                                          cout_p, 0, cout, net._p(dw), st))
    _sync(net)
    want_dw = U.conv_wgrad(x, dy[..., :cout], ntap, cin_p) + 0.25
    assert rel_l2(dw.cpu().numpy().reshape(want_dw.shape), want_dw) <= 1e-5
    assert net.lib.sepx_unet_status() == 0


def test_pool_upsample_mask(net):
    from sep_code_gb300._lib import lib
    lib.sepx_setup_cuda(1)
    st = lib.sepx_get_stream()
    rng = np.random.default_rng(3)
    nb, D, H, W, C = 2, 8, 8, 16, 16
    x = U.bf16(rng.standard_normal((nb, D, H, W, C)))
    xt = _bf(x)
    V = nb * D * H * W
    y = torch.zeros((V // 8, C), dtype=torch.bfloat16).cuda()
    torch.cuda.synchronize()
    net._chk(net.lib.sepx_unet_avgpool(net._p(xt), C, 0, nb, D, H, W, C, net._p(y), C, 0, st))
    _sync(net)
    assert rel_l2(_np(y), U.bf16(U.avgpool(x)).reshape(-1, C)) <= 1e-6
    up = torch.zeros((V, C), dtype=torch.bfloat16).cuda()
    torch.cuda.synchronize()
    net._chk(net.lib.sepx_unet_upsample(net._p(y), C, 0, nb, D // 2, H // 2, W // 2, C, net._p(up), C,
                                        0, st))
    _sync(net)
    assert np.array_equal(_np(up), U.upsample(_np(y).reshape(nb, D // 2, H // 2, W // 2, C)).reshape(-1, C))
    ub = torch.zeros((V // 8, C), dtype=torch.bfloat16).cuda()
    torch.cuda.synchronize()
    net._chk(net.lib.sepx_unet_upsample_bwd(net._p(xt), C, 0, nb, D // 2, H // 2, W // 2, C, net._p(ub),
                                            C, 0, st))
    _sync(net)
    assert rel_l2(_np(ub), U.bf16(U.upsample_bwd(x)).reshape(-1, C)) <= 1e-6
    m = _bf(x)
    g = _bf(np.ones_like(x))
    torch.cuda.synchronize()
    net._chk(net.lib.sepx_unet_relu_mask(net._p(m), C, 0, net._p(g), C, 0, V, C, st))
    _sync(net)
    assert np.array_equal(_np(g).reshape(x.shape), (x > 0).astype(np.float64))


def test_network_gradients_match_oracle(net):
    """one forward + backward of the whole U-Net on a 32^3 volume (4^3 at the
    bottom level), every layer's weight and bias gradient against the FP64
    restatement.  The GPU rounds every stored activation and gradient to BF16
    after FP32 sums, the restatement after FP64 sums: where the two roundings
    differ (or a ReLU input sits within a rounding of zero) the difference
    propagates, most at the coarse levels whose sums have fewest terms.  A
    wiring error (a wrong channel slice, skip or pooling gradient) shows as
    an O(1) error instead."""
    rng = np.random.default_rng(11)
    params = net.init_params(seed=5)
    w, b = params["out"]
    params["out"] = (rng.standard_normal(w.shape).astype(np.float32) * 0.3, b + 0.01)
    params = {k: (v[0], v[1] + rng.standard_normal(v[1].shape).astype(np.float32) * 0.05)
              for k, v in params.items()}
    nb, D, H, W = 1, 32, 32, 32
    x = rng.standard_normal((nb, D, H, W)).astype(np.float32)
    tgt = rng.standard_normal((nb, D, H, W)).astype(np.float32)
    model = net.UNet3D(params)
    xt = torch.tensor(x).cuda()
    tt = torch.tensor(tgt).cuda()
    torch.cuda.synchronize()
    model.zero_grad()
    out = model.forward_device(xt)
    model.loss_grad(tt)
    model.backward_device()
    model.stream.synchronize()
    assert model.status() == 0
    o_out, o_loss, o_g = U.forward_backward(params, x, tgt)
    _, _, ex_g = U.forward_backward(params, x, tgt, round_bf16=False)
    # BF16 activations through 15 layers: a rounding that flips between the
    # FP32 and the FP64 sums moves the output at the 1e-3 level
    assert rel_l2(out.cpu().numpy().reshape(o_out.shape), o_out) <= 1e-2
    assert abs(float(model.loss.item()) - o_loss) <= 1e-2 * o_loss
    errs = {}
    for L in net.LAYERS:
        gw = model.gw[L.name].cpu().numpy()
        gb = model.gb[L.name].cpu().numpy()
        ew, eb = o_g[L.name]
        xw, xb = ex_g[L.name]
        assert np.abs(ew).max() > 0, L.name
        # against the BF16-storage restatement, and how far the GPU and that
        # restatement each sit from the exact FP64 gradient
        errs[L.name] = (rel_l2(gw, ew), rel_l2(gb, eb), rel_l2(gw, xw), rel_l2(ew, xw))
    print("UNET_GRAD_REL_L2", errs)
    for name, (ew_, eb_, gx, ox) in errs.items():
        assert ew_ <= 0.08 and eb_ <= 0.08, (name, ew_, eb_)
        assert gx <= 2.0 * ox + 0.01, (name, gx, ox)


def test_training_reduces_loss(net):
    """Adam on a fixed smoothing task: the loss falls by more than half"""
    rng = np.random.default_rng(2)
    model = net.UNet3D(seed=1)
    nb, D, H, W = 2, 16, 16, 16
    x = rng.standard_normal((nb, D, H, W)).astype(np.float32)
    # target: 3-point smoothing along every axis of x (a fixed linear operator)
    t = x.copy()
    for ax in (1, 2, 3):
        t = (np.roll(t, 1, ax) + 2 * t + np.roll(t, -1, ax)) / 4
    xt, tt = torch.tensor(x).cuda(), torch.tensor(t.astype(np.float32)).cuda()
    torch.cuda.synchronize()
    losses = [model.train_step(xt, tt, lr=2e-3) for _ in range(60)]
    assert model.status() == 0
    assert losses[-1] < 0.5 * losses[0], (losses[0], losses[-1])


def test_captured_training_step_matches_eager(net):
    """The whole training step captured once into a CUDA graph and replayed
    (new learning rate and step count each replay, read from device memory)
    trains like the same steps launched one by one: same losses and weights
    to FP32 summation-order noise (some kernels add with atomics)."""
    rng = np.random.default_rng(8)
    nb, D, H, W = 2, 16, 16, 32
    x = rng.standard_normal((nb, D, H, W)).astype(np.float32)
    t = (0.5 * x + 0.1 * rng.standard_normal(x.shape)).astype(np.float32)
    xt, tt = torch.tensor(x).cuda(), torch.tensor(t).cuda()
    lrs = [2e-3, 1.5e-3, 1e-3, 5e-4, 2.5e-4]
    graph, twin = net.UNet3D(seed=4), net.UNet3D(seed=4)
    torch.cuda.synchronize()
    graph.capture_train_step(xt, tt)          # one eager step at lr 1e-3, then the capture
    assert graph.graph is not None
    l0 = twin.train_step(xt, tt, lr=1e-3)     # the same first step on the eager twin
    lg = [graph.train_step(xt, tt, lr=lr) for lr in lrs[1:]]
    le2 = [twin.train_step(xt, tt, lr=lr) for lr in lrs[1:]]
    assert graph.status() == 0 and twin.status() == 0
    assert graph.step_count == twin.step_count == len(lrs)
    print("UNET_GRAPH losses graph", [l0] + lg, "eager", [l0] + le2)
    graph2 = twin
    for a, b in zip(lg, le2):
        assert abs(a - b) <= 1e-4 * abs(b), (a, b)
    for L in net.LAYERS:
        wa = graph.w[L.name].cpu().numpy()
        wb = graph2.w[L.name].cpu().numpy()
        assert rel_l2(wa, wb) <= 1e-4, (L.name, rel_l2(wa, wb))
    graph.free_graph()


HALO_CASES = [(2, 8, 24, 20, 16, 16, 0), (1, 6, 32, 16, 32, 48, 0), (1, 5, 16, 8, 48, 16, 1),
              (1, 4, 17, 9, 16, 32, 1), (2, 3, 16, 24, 32, 32, 0),
              # odd channel-group counts (one zero group in the halo)
              (2, 4, 16, 8, 8, 16, 0), (1, 3, 20, 12, 24, 16, 0), (1, 3, 16, 16, 24, 32, 1),
              # the widest layer that fits (weights 135 KB + one 85 KB halo)
              (1, 3, 16, 16, 80, 32, 0)]


@pytest.mark.parametrize("nb,D,H,W,cin,cout,tr", HALO_CASES)
def test_halo_conv_matches_gather_and_oracle(net, nb, D, H, W, cin, cout, tr):
    """the halo-staged kernel (input halo by TMA, taps as shifted shared-memory
    descriptors) against the per-tap gather kernel and the FP64 restatement:
    partial tiles (H % 16, W % 8), several volumes, forward and data-gradient
    packings, even and odd numbers of 8-channel groups"""
    from sep_code_gb300._lib import lib
    rng = np.random.default_rng(nb * 1000 + D * 100 + H + cin)
    lib.sepx_setup_cuda(1)
    st = lib.sepx_get_stream()
    # forward operand (tr 0): w [27][cin][cout]; data-gradient operand (tr 1):
    # the layer cout -> cin, so its master weights are [27][cout][cin]
    w = (rng.standard_normal((27, cout if tr else cin, cin if tr else cout)) / np.sqrt(27 * cin)).astype(np.float32)
    x = U.bf16(rng.standard_normal((nb, D, H, W, cin)))
    wt = torch.tensor(w).cuda()
    lay_out, lay_in = (cin, cout) if tr else (cout, cin)
    pk = torch.zeros(net.lib.sepx_unet_packed_elems(lay_out, lay_in, 27, tr), dtype=torch.bfloat16).cuda()
    torch.cuda.synchronize()
    net._chk(net.lib.sepx_unet_pack_weights(net._p(wt), lay_out, lay_in, 27, tr, net._p(pk), st))
    xt = _bf(x)
    V = nb * D * H * W
    outs = []
    for halo in (1, 0):
        prev = lib.sepx_unet_set_halo(halo)
        yf = torch.zeros(V * cout, dtype=torch.float32).cuda()
        torch.cuda.synchronize()
        net._chk(net.lib.sepx_unet_conv_fwd(net._p(xt), cin, 0, nb, D, H, W, cin, 27, net._p(pk), None, cout,
                                            0, None, 0, 0, net._p(yf), None, st))
        _sync(net)
        lib.sepx_unet_set_halo(prev)
        outs.append(yf.cpu().numpy())
    assert net.lib.sepx_unet_status() == 0
    if tr:
        want = U.conv_dgrad(x, U.bf16(w))
    else:
        want = U.conv_fwd(x, U.bf16(w), None, False)
    assert rel_l2(outs[0].reshape(want.shape), want) <= 1e-5, rel_l2(outs[0].reshape(want.shape), want)
    # the two kernels sum the same products in different orders (a layer that
    # fits one halo buffer goes channel pair by channel pair over the taps)
    assert rel_l2(outs[0], outs[1]) <= 1e-5


def test_halo_conv_speed_384(net):
    """16 -> 16 channels on a 384^3 volume, both kernels, CUDA events on the
    library stream; prints UNET_HALO {json}"""
    import json
    from sep_code_gb300._lib import lib
    lib.sepx_setup_cuda(1)
    st = lib.sepx_get_stream()
    stream = torch.cuda.ExternalStream(st)
    D = H = W = 384
    res = {}
    for cin, cout in ((8, 16), (16, 16), (32, 32), (48, 16), (80, 32)):
        g = torch.Generator(device="cuda").manual_seed(cin)
        x = torch.randn(D * H * W * cin, device="cuda", generator=g).to(torch.bfloat16)
        wt = torch.randn(27 * cin * cout, device="cuda", generator=g) * 0.05
        pk = torch.zeros(net.lib.sepx_unet_packed_elems(cout, cin, 27, 0), dtype=torch.bfloat16).cuda()
        y = torch.empty(D * H * W * cout, dtype=torch.bfloat16, device="cuda")
        torch.cuda.synchronize()
        net._chk(net.lib.sepx_unet_pack_weights(net._p(wt), cout, cin, 27, 0, net._p(pk), st))
        flops = 2.0 * D * H * W * 27 * cin * cout
        for halo in (1, 0):
            prev = lib.sepx_unet_set_halo(halo)

            def run():
                net._chk(net.lib.sepx_unet_conv_fwd(net._p(x), cin, 0, 1, D, H, W, cin, 27, net._p(pk), None,
                                                    cout, 1, net._p(y), cout, 0, None, None, st))
            run()
            stream.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(3):
                run()
            b.record(stream)
            b.synchronize()
            lib.sepx_unet_set_halo(prev)
            ms = a.elapsed_time(b) / 3
            res[f"{cin}->{cout} {'halo' if halo else 'gather'}"] = {"ms": ms, "TFLOP_s": flops / ms / 1e9}
        del x, y
    assert net.lib.sepx_unet_status() == 0
    print("UNET_HALO " + json.dumps(res))


def test_network_speed(net):
    """whole-network timing, halo-staged and gather convolutions: one Adam
    training step on a batch of 4 x 64^3 and the inference of one 384^3
    search direction; CUDA events on the library stream; prints UNET_NET
    {json} with the convolution FLOPs per second"""
    import json
    from sep_code_gb300._lib import lib
    model = net.UNet3D(seed=3)
    stream = model.stream
    g = torch.Generator(device="cuda").manual_seed(9)

    def conv_flops(nb, n):
        f = 0.0
        lvl = {"e1": 0, "e2": 1, "e3": 2, "b4": 3, "d3": 2, "d2": 1, "d1": 0, "ou": 0}
        for L in net.LAYERS:
            v = nb * (n >> lvl[L.name[:2]]) ** 3
            f += 2.0 * v * L.ntap * L.cin * L.cout
        return f

    def timed(fn, reps):
        fn()
        stream.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / reps

    x = torch.randn(4, 64, 64, 64, device="cuda", generator=g)
    t = torch.randn(4, 64, 64, 64, device="cuda", generator=g)
    big = torch.randn(1, 384, 384, 384, device="cuda", generator=g)
    torch.cuda.synchronize()
    res = {}
    for halo in (1, 0):
        prev = lib.sepx_unet_set_halo(halo)
        tag = "halo" if halo else "gather"
        ms = timed(lambda: model.train_step(x, t, lr=1e-4), 5)
        # forward + data gradient + weight gradient = 3 x the forward FLOPs
        res[f"train_step_4x64^3 {tag}"] = {"ms": ms, "TFLOP_s": 3 * conv_flops(4, 64) / ms / 1e9}
        ms = timed(lambda: model.forward_device(big), 2)
        res[f"inference_384^3 {tag}"] = {"ms": ms, "TFLOP_s": conv_flops(1, 384) / ms / 1e9}
        lib.sepx_unet_set_halo(prev)
    assert model.status() == 0
    print("UNET_NET " + json.dumps(res))


@pytest.mark.parametrize("cin,cout,shape", [(16, 16, (2, 8, 16, 16)), (48, 64, (2, 4, 8, 8)),
                                            (16, 1, (1, 4, 16, 16))])
def test_fused_relu_backward_is_bit_identical(net, cin, cout, shape):
    """The ReLU backward fused into the data gradient, the pooling gradient
    and the upsampling gradient gives the same bits as the separate
    relu_mask pass after them."""
    from sep_code_gb300._lib import lib
    lib.sepx_setup_cuda(1)
    st = lib.sepx_get_stream()
    rng = np.random.default_rng(cin + cout)
    nb, D, H, W = shape
    ntap = 1 if cout == 1 else 27
    cin_p, cout_p = (cin + 7) // 8 * 8, (cout + 7) // 8 * 8
    V = nb * D * H * W
    w = (rng.standard_normal((ntap, cin_p, cout)) / np.sqrt(ntap * cin)).astype(np.float32)
    wt = torch.tensor(w).cuda()
    pkt = torch.zeros(net.lib.sepx_unet_packed_elems(cout, cin_p, ntap, 1), dtype=torch.bfloat16).cuda()
    torch.cuda.synchronize()
    net._chk(net.lib.sepx_unet_pack_weights(net._p(wt), cout, cin_p, ntap, 1, net._p(pkt), st))
    dy = np.zeros((V, cout_p))
    dy[:, :cout] = U.bf16(rng.standard_normal((V, cout)))
    act = U.bf16(rng.standard_normal((V, cin_p + 8)))   # mask view: channels 8 .. 8 + cin_p
    dyt, actt = _bf(dy), _bf(act)
    outs = []
    for fused in (True, False):
        dx = torch.zeros((V, cin_p), dtype=torch.bfloat16).cuda()
        torch.cuda.synchronize()
        m = (net._p(actt), cin_p + 8, 8) if fused else (None, 0, 0)
        net._chk(net.lib.sepx_unet_conv_fwd_masked(net._p(dyt), cout_p, 0, nb, D, H, W, cout_p, ntap,
                                                   net._p(pkt), None, cin_p, 0, net._p(dx), cin_p, 0,
                                                   None, None, *m, st))
        if not fused:
            net._chk(net.lib.sepx_unet_relu_mask(net._p(actt), cin_p + 8, 8, net._p(dx), cin_p, 0, V, cin_p, st))
        _sync(net)
        outs.append(dx.view(torch.int16).cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
    assert (outs[0] == 0).mean() > 0.3   # the mask did zero about half
    # pooling gradient (accumulating into a slice) and upsampling gradient
    C = cin_p
    g2 = _bf(U.bf16(rng.standard_normal((V // 8, C))))
    base = U.bf16(rng.standard_normal((V, 2 * C)))
    res = []
    for fused in (True, False):
        dst = _bf(base)
        torch.cuda.synchronize()
        m = (net._p(actt), cin_p + 8, 8) if fused else (None, 0, 0)
        net._chk(net.lib.sepx_unet_avgpool_bwd_masked(net._p(g2), C, 0, nb, D, H, W, C, net._p(dst), 2 * C, C,
                                                      1, *m, st))
        if not fused:
            net._chk(net.lib.sepx_unet_relu_mask(net._p(actt), cin_p + 8, 8, net._p(dst), 2 * C, C, V, C, st))
        _sync(net)
        res.append(dst.view(torch.int16).cpu().numpy())
    assert np.array_equal(res[0], res[1])
    fine = _bf(U.bf16(rng.standard_normal((V, C))))
    act2 = _bf(U.bf16(rng.standard_normal((V // 8, C))))
    res = []
    for fused in (True, False):
        dx = torch.zeros((V // 8, C), dtype=torch.bfloat16).cuda()
        torch.cuda.synchronize()
        m = (net._p(act2), C, 0) if fused else (None, 0, 0)
        net._chk(net.lib.sepx_unet_upsample_bwd_masked(net._p(fine), C, 0, nb, D // 2, H // 2, W // 2, C,
                                                       net._p(dx), C, 0, *m, st))
        if not fused:
            net._chk(net.lib.sepx_unet_relu_mask(net._p(act2), C, 0, net._p(dx), C, 0, V // 8, C, st))
        _sync(net)
        res.append(dx.view(torch.int16).cpu().numpy())
    assert np.array_equal(res[0], res[1])
    assert net.lib.sepx_unet_status() == 0


def test_learned_train_loop_replays_the_captured_step(net):
    """learned.train: fixed batch buffers, the first step captured into a
    graph and replayed for the others; on a fixed smoothing task the epoch
    losses fall, and the weights equal those of the same steps launched one
    by one to summation-order noise."""
    from sep_code_gb300 import learned
    rng = np.random.default_rng(12)
    n, D = 8, 16
    X = rng.standard_normal((n, D, D, D)).astype(np.float32)
    Y = X.copy()
    for ax in (1, 2, 3):
        Y = (np.roll(Y, 1, ax) + 2 * Y + np.roll(Y, -1, ax)) / 4
    Y = Y.astype(np.float32)
    m1 = net.UNet3D(seed=2)
    hist = learned.train(m1, X, Y, epochs=4, batch=2, lr=2e-3, seed=1)
    assert m1.graph is not None and m1.status() == 0
    assert all(np.isfinite(hist)) and hist[-1] < hist[0], hist
    # the same schedule, every step launched one by one
    m2 = net.UNet3D(seed=2)
    r = np.random.default_rng(1)
    Xd, Yd = torch.tensor(X).cuda(), torch.tensor(Y).cuda()
    for ep in range(4):
        order = r.permutation(n)
        lr_ep = 2e-3 * (0.5 * (1 + np.cos(np.pi * ep / 4)))
        for i in range(0, n - 1, 2):
            idx = torch.tensor(order[i:i + 2], device="cuda")
            xb, yb = Xd.index_select(0, idx).contiguous(), Yd.index_select(0, idx).contiguous()
            torch.cuda.synchronize()
            m2.train_step(xb, yb, lr=max(lr_ep, 2e-3 * 0.02))
    for L in net.LAYERS:
        a, b = m1.w[L.name].cpu().numpy(), m2.w[L.name].cpu().numpy()
        assert rel_l2(a, b) <= 1e-3, (L.name, rel_l2(a, b))
    m1.free_graph()
