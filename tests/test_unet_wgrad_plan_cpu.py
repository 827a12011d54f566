"""CPU check of the tap-stacked weight-gradient schedules in
csrc/sepx_unet_wgrad.inc: a numpy walk through the kernels' index
arithmetic -- tiles (16 y x 8 x, K = 8 y + x), the dY copies moved by -sx in
the A rows, the X copies moved by (dz, sy - 1, -1) in the B columns plus the
ones column, the z-walk's windows and ring of four plane slots (a slot is
refilled only after its plane's last tile), the partial layout -- against
the direct sum dW[t][c][m] = sum_u dY[u][m] X[u + off(t)][c] and db.  Also
the shared-memory and tensor-memory plans of every U-Net layer shape that
takes these kernels, as the host code sizes them (227 KB per CTA, 512
columns per SM, the A view of 64 or 128 rows inside the carve), and the
K-chunk walk of the split-K gather convolution.
"""
import numpy as np
import pytest

KB = 2048
SMEM_MAX = 227 * 1024


def _np_of(ngi):
    return ((8 * (3 * ngi + 1)) + 15) // 16 * 16


def zw_plan(nb, D, H, W, cin, cout, nsm=152, smem_per_sm=233472, reserved=1024):
    """conv_wgrad_zw's host plan (sepx_unet.cu); None where it does not apply"""
    ngi, ngo = cin // 8, (cout + 7) // 8
    if 3 * ngo > 16 or ngi > 6:
        return None
    np_ = _np_of(ngi)
    if 3 * np_ > 512:
        return None
    a_bytes, pl = 3 * ngo * KB, np_ // 8 * KB
    rawb, rawa = 18 * 8 * cin * 2, 16 * 10 * 8 * ngo * 2
    raw = (rawb + rawa + 127) // 128 * 128
    fixed = 2 * a_bytes + 4 * pl + (2 * 4 + 12) * 8 + 16 + 128
    if fixed + 2 * raw > SMEM_MAX:
        return None
    ncols = 32
    while ncols < 3 * np_:
        ncols *= 2

    def per_sm_of(nr):
        sm = fixed + nr * raw
        if sm > SMEM_MAX:
            return 0
        return min(smem_per_sm // (((sm + 127) // 128) * 128 + reserved), 512 // ncols)
    nraw = 2
    for nr in (3, 4):
        if per_sm_of(nr) >= per_sm_of(nraw):
            nraw = nr
    per_sm = per_sm_of(nraw)
    slots = nsm * per_sm
    ty, tx = (H + 15) // 16, (W + 2 + 7) // 8
    cols = nb * ty * tx
    best, zc = 1e300, D
    while True:
        nzc = (D + zc - 1) // zc
        per = (cols * nzc + slots - 1) // slots
        cost = per * (zc + 2 / 3)
        if cost < best:
            best, bz, bnzc = cost, zc, nzc
        if zc <= 4:
            break
        zc = (zc + 1) // 2
    nitems = cols * bnzc
    return dict(ngi=ngi, ngo=ngo, np=np_, a_bytes=a_bytes, pl=pl, raw=raw, nraw=nraw,
                smem=fixed + nraw * raw, ncols=ncols, per_sm=per_sm, grid=min(nitems, slots),
                zc=bz, nzc=bnzc, nitems=nitems, ty=ty, tx=tx,
                mrows=64 if 3 * 8 * ngo <= 64 else 128)


def _box(arr, C, xs, ys, z, n, bx, by):
    """TMA box with zero fill outside the volume: [by][bx][C]"""
    nb, D, H, W, _ = arr.shape
    out = np.zeros((by, bx, C))
    if not 0 <= z < D:
        return out
    ya, yb = max(ys, 0), min(ys + by, H)
    xa, xb = max(xs, 0), min(xs + bx, W)
    if ya < yb and xa < xb:
        out[ya - ys:yb - ys, xa - xs:xb - xs] = arr[n, z, ya:yb, xa:xb, :C]
    return out


def zw_emulate(x, dy, cin, cout, p):
    nb, D, H, W, _ = x.shape
    ngi, ngo, np_ = p["ngi"], p["ngo"], p["np"]
    cp, ci, G = 8 * ngo, 8 * ngi, p["grid"]
    part = np.zeros((G, 27, cin, cout))
    bpart = np.zeros((G, cout))
    for b in range(G):
        nitem = (p["nitems"] - 1 - b) // G + 1 if p["nitems"] > b else 0
        acc = np.zeros((3, 128, np_))
        slot, dead, planes, u = [None] * 4, set(), {}, 0
        for j in range(nitem):
            item = b + j * G
            bx = item % p["tx"]; r = item // p["tx"]
            by = r % p["ty"]; r //= p["ty"]
            zb = r % p["nzc"]; n = r // p["nzc"]
            z0 = zb * p["zc"]; nz = min(p["zc"], D - z0); y0, x0 = by * 16, bx * 8
            ubase = u
            for pp in range(nz + 2):
                s = u % 4
                assert slot[s] is None or slot[s] in dead, "plane slot refilled while in use"
                raw = _box(x, cin, x0 - 1, y0 - 1, z0 - 1 + pp, n, 8, 18)      # [18][8][cin]
                B = np.zeros((128, np_))
                for sy in range(3):
                    for g in range(ngi):
                        jj = sy * ngi + g
                        B[:, 8 * jj:8 * jj + 8] = raw[sy:sy + 16, :, 8 * g:8 * g + 8].reshape(128, 8)
                B[:, 24 * ngi:24 * ngi + 8] = 1.0
                planes[u], slot[s] = B, u
                if pp >= 2:
                    zl = pp - 2
                    rawa = _box(dy, cp, x0 - 2, y0, z0 + zl, n, 10, 16)        # [16][10][cp]
                    A = np.zeros((128, 128))
                    for sx in range(3):
                        for g in range(ngo):
                            jj = sx * ngo + g
                            A[8 * jj:8 * jj + 8] = rawa[:, 2 - sx:10 - sx, 8 * g:8 * g + 8].reshape(128, 8).T
                    u0 = ubase + zl
                    for dzl in range(3):
                        assert slot[(u0 + dzl) % 4] == u0 + dzl
                        acc[dzl] += A @ planes[u0 + dzl]
                    dead.add(u0)
                    if zl == nz - 1:
                        dead.update({u0 + 1, u0 + 2})
                u += 1
        for dzl in range(3):
            for rr in range(3 * cp):
                sx, m = rr // cp, rr % cp
                if m >= cout:
                    continue
                for nn in range(np_):
                    sy, c = nn // ci, nn % ci
                    if sy < 3 and c < cin:
                        part[b, dzl * 9 + sy * 3 + sx, c, m] = acc[dzl, rr, nn]
                    elif sy == 3 and c == 0 and sx == 0 and dzl == 0:
                        bpart[b, m] = acc[dzl, rr, nn]
    return part.sum(0), bpart.sum(0)


def pertile_emulate(x, dy, cin, cout, ndz, groups):
    """conv_wgrad_tma_kernel: every tile, ndz dz blocks per CTA group"""
    nb, D, H, W, _ = x.shape
    ngi, ngo = cin // 8, (cout + 7) // 8
    np_, cp, ci = _np_of(ngi), 8 * ngo, 8 * ngi
    ty, tx = (H + 15) // 16, (W + 2 + 7) // 8
    ntiles = nb * D * ty * tx
    dw = np.zeros((27, cin, cout)); db = np.zeros(cout)
    for gz in range(3 // ndz):
        for gi in range(groups):
            acc = np.zeros((ndz, 128, np_))
            for tile in range(gi, ntiles, groups):
                bx = tile % tx; r = tile // tx; by = r % ty; r //= ty
                z = r % D; n = r // D; x0, y0 = bx * 8, by * 16
                A = np.zeros((128, 128))
                for sx in range(3):
                    for g in range(ngo):
                        jj = sx * ngo + g
                        A[8 * jj:8 * jj + 8] = _box(dy, cp, x0 - sx, y0, z, n, 8, 16)[:, :, 8 * g:8 * g + 8].reshape(128, 8).T
                for dzl in range(ndz):
                    dz = gz * ndz + dzl - 1
                    B = np.zeros((128, np_))
                    for sy in range(3):
                        for g in range(ngi):
                            jj = sy * ngi + g
                            B[:, 8 * jj:8 * jj + 8] = _box(x, cin, x0 - 1, y0 - 1 + sy, z + dz, n, 8, 16)[:, :, 8 * g:8 * g + 8].reshape(128, 8)
                    B[:, 24 * ngi:24 * ngi + 8] = 1.0
                    acc[dzl] += A @ B
            for dzl in range(ndz):
                dzi = gz * ndz + dzl
                for sx in range(3):
                    for sy in range(3):
                        dw[dzi * 9 + sy * 3 + sx] += acc[dzl, sx * cp:sx * cp + cout, sy * ci:sy * ci + cin].T
                if dzi == 0:
                    db += acc[dzl, :cout, 24 * ngi]
    return dw, db


def direct(x, dy, cin, cout):
    nb, D, H, W, _ = x.shape
    xp = np.zeros((nb, D + 2, H + 2, W + 2, cin))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    dw = np.zeros((27, cin, cout))
    for t in range(27):
        dz, dyy, dx = t // 9 - 1, (t % 9) // 3 - 1, t % 3 - 1
        xs = xp[:, 1 + dz:1 + dz + D, 1 + dyy:1 + dyy + H, 1 + dx:1 + dx + W]
        dw[t] = np.einsum("nzyxc,nzyxm->cm", xs, dy[..., :cout])
    return dw, dy[..., :cout].sum((0, 1, 2, 3))


LAYER_SHAPES = [((4, 64, 64, 64), 8, 16), ((4, 64, 64, 64), 16, 16), ((4, 64, 64, 64), 48, 16),
                ((4, 32, 32, 32), 16, 32), ((4, 32, 32, 32), 32, 32)]


@pytest.mark.parametrize("shape,cin,cout", LAYER_SHAPES)
def test_zwalk_plans_fit(shape, cin, cout):
    p = zw_plan(*shape, cin, cout)
    assert p is not None
    total = 2 * p["a_bytes"] + 4 * p["pl"] + p["nraw"] * p["raw"]
    assert p["smem"] <= SMEM_MAX
    assert p["a_bytes"] + (p["mrows"] // 8) * KB <= total       # A view of the second slot
    assert 3 * p["np"] <= p["ncols"] <= 512 and p["per_sm"] * p["ncols"] <= 512
    assert 3 * 8 * p["ngo"] <= p["mrows"]
    assert p["np"] // 8 > 3 * p["ngi"]                              # the ones group exists


@pytest.mark.parametrize("cin,cout,shape,nsm", [(8, 16, (1, 5, 9, 13), 3), (16, 32, (2, 6, 17, 8), 4),
                                                (48, 16, (1, 7, 16, 20), 5), (24, 40, (1, 1, 7, 5), 2)])
def test_zwalk_schedule_gives_the_weight_gradient(cin, cout, shape, nsm):
    rng = np.random.default_rng(cin + cout)
    nb, D, H, W = shape
    p = zw_plan(nb, D, H, W, cin, cout, nsm=nsm)
    ngo = (cout + 7) // 8
    x = rng.standard_normal((nb, D, H, W, cin))
    dy = np.zeros((nb, D, H, W, 8 * ngo))
    dy[..., :cout] = rng.standard_normal((nb, D, H, W, cout))
    dw, db = zw_emulate(x, dy, cin, cout, p)
    w2, b2 = direct(x, dy, cin, cout)
    assert np.abs(dw - w2).max() < 1e-9 and np.abs(db - b2).max() < 1e-9


@pytest.mark.parametrize("cin,cout,ndz", [(16, 16, 3), (80, 32, 1)])
def test_pertile_schedule_gives_the_weight_gradient(cin, cout, ndz):
    rng = np.random.default_rng(cin * cout)
    nb, D, H, W = 1, 3, 17, 10
    x = rng.standard_normal((nb, D, H, W, cin))
    ngo = (cout + 7) // 8
    dy = np.zeros((nb, D, H, W, 8 * ngo))
    dy[..., :cout] = rng.standard_normal((nb, D, H, W, cout))
    dw, db = pertile_emulate(x, dy, cin, cout, ndz, groups=3)
    w2, b2 = direct(x, dy, cin, cout)
    assert np.abs(dw - w2).max() < 1e-9 and np.abs(db - b2).max() < 1e-9


def test_split_k_chunk_positions_cover_every_tap_and_channel_once():
    """conv_fwd_kernel's split K: split k sums K chunks [k*kper, (k+1)*kper)
    of 64 (8 groups of 8 channels), starting at tap (kb*64)/cin and channel
    (kb*64)%cin and stepping 8 channels at a time (next tap at cin).  Every
    (tap, channel group) is visited by exactly one split, in K order."""
    KKC = 64
    for cin in (8, 16, 32, 48, 64, 80, 112):
        for ntap in (1, 27):
            kch = (ntap * cin + KKC - 1) // KKC
            mt = 16
            splits = min((2 * 152 + mt - 1) // mt, kch // 2) if kch >= 4 else 1
            kper = (kch + splits - 1) // splits
            splits = (kch + kper - 1) // kper
            seen = []
            for k in range(splits):
                kb = k * kper
                nk = min(kper, kch - kb)
                tap, c0 = (kb * KKC) // cin, (kb * KKC) % cin
                for _ in range(nk):
                    for _ in range(KKC // 8):
                        if tap < ntap:
                            seen.append((tap, c0))
                        c0 += 8
                        if c0 >= cin:
                            c0 -= cin
                            tap += 1
            want = [(t, c) for t in range(ntap) for c in range(0, cin, 8)]
            assert seen == want, (cin, ntap)
