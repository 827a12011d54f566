"""Learned preconditioning of least-squares RTM.

* ``make_pairs``: training pairs (L'L m, m) generated by the Born operator
  itself (the exact-adjoint linearised pair of rtm_zero_op) from seeded
  random horizon-plus-spike reflectivities on small velocity models.
* ``train``: Adam on the U-Net (sep_code_gb300/unet.py) with the library's
  BF16 tensor-core forward and backward kernels; inputs and targets are
  normalised to unit RMS (the network learns the shape of (L'L)^-1, the CG
  plane search sets the length).
* ``UNetDirection``: the search-direction hook g <- |g| N(g / |g|) that
  ``RtmOperator.lsrtm`` (simple_solver + cgstep, Born/lin_solver.cpp:115-143)
  applies before the forward product.  cgstep's two-term plane search
  (Born/cgstep.cpp:14-58) keeps the data residual non-increasing for any
  direction, so plain CG remains the yardstick of what the network buys.
"""
from __future__ import annotations

import ctypes as C
import time
from pathlib import Path

import numpy as np

from . import model as M
from ._lib import lib
from .operator import RtmOperator
from .unet import UNet3D

WEIGHTS = Path(__file__).resolve().parent / "data" / "unet_precond.npz"


def random_reflectivity(rng, shape, nhor=(3, 7), spike_frac=0.01, amp=0.05):
    """horizons (gently dipping planes) plus sparse spikes, model grid [m3, m2, m1]"""
    m3, m2, m1 = shape
    r = np.zeros(shape, np.float32)
    z = np.arange(m3)[:, None, None]
    y = np.arange(m2)[None, :, None]
    x = np.arange(m1)[None, None, :]
    for _ in range(int(rng.integers(nhor[0], nhor[1] + 1))):
        z0 = rng.uniform(0.15, 0.9) * m3
        dzx, dzy = rng.uniform(-0.15, 0.15, 2)
        surf = z0 + dzx * (x - m1 / 2) + dzy * (y - m2 / 2)
        r += np.where(np.abs(z - surf) < 0.5, rng.normal(0, amp), 0.0).astype(np.float32)
    spikes = rng.random(shape) < spike_frac
    r[spikes] += rng.normal(0, amp, int(spikes.sum())).astype(np.float32)
    r[: max(2, m3 // 16)] = 0.0   # no reflectors at the source / receiver depth
    return r


def velocity_model(rng, shape, d):
    """smooth v(z) with a random gradient and a weak lateral perturbation (m/s)"""
    m3, m2, m1 = shape
    z = np.arange(m3)[:, None, None] * d
    y = np.arange(m2)[None, :, None] * d
    x = np.arange(m1)[None, None, :] * d
    v0 = rng.uniform(1500.0, 2200.0)
    grad = rng.uniform(0.3, 1.0)
    kx, ky = rng.uniform(0.5, 2.0, 2) * 2 * np.pi / (m1 * d)
    v = v0 + grad * z + 80.0 * np.sin(kx * x) * np.cos(ky * y)
    return np.broadcast_to(v, shape).astype(np.float32).copy()


def patch_survey(vel, refl, d, nt, f0=15.0):
    m3, m2, m1 = vel.shape
    c1, c2 = (m1 - 1) * d / 2, (m2 - 1) * d / 2
    return M.Survey(vel=vel, spacing=(d, d, d), refl=refl, wavelet=M.ricker(f0, 0.001, nt), dtw=0.001,
                    data_nt=nt, data_dt=0.001, rec=(m1, m2, 0.0, d, 0.0, d), shots=[(c1, c2, 0.0)],
                    nbound=20, name="patch")


def make_pairs(npairs: int, n: int = 64, nt: int = 1100, d: float = 12.5, nvel: int = 20,
               seed: int = 20261207, snap_js: int = 4, iterates: int = 0, verbose: bool = False):
    """(x, m) pairs, x = L'L m, both [npairs, n, n, n] FP32 numpy, unit RMS each.

    iterates > 0: each random reflectivity m also yields the pairs (g_k, e_k)
    of that many steepest-descent iterates m_k on |L m_k - L m|^2 (exact line
    search): e_k = m - m_k is the remaining error and g_k = L'(L m - L m_k) =
    L'L e_k the gradient there -- the inputs the solver hands the network after
    its first iteration.  Each pair costs one forward and one adjoint."""
    rng = np.random.default_rng(seed)
    X = np.zeros((npairs, n, n, n), np.float32)
    Y = np.zeros((npairs, n, n, n), np.float32)
    per = (npairs + nvel - 1) // nvel
    k = 0
    t0 = time.perf_counter()

    def put(x, m):
        nonlocal k
        X[k] = x / max(np.sqrt(np.mean(x.astype(np.float64) ** 2)), 1e-30)
        Y[k] = m / max(np.sqrt(np.mean(m.astype(np.float64) ** 2)), 1e-30)
        k += 1

    while k < npairs:
        vel = velocity_model(rng, (n, n, n), d)
        s = patch_survey(vel, np.zeros_like(vel), d, nt)
        op = RtmOperator(s, mode="linear", snap_js=snap_js, snap_prec="f32")
        try:
            done = 0
            while done < per and k < npairs:
                m = random_reflectivity(rng, (n, n, n))
                r = op.forward(m)            # residual of m_0 = 0: d - L m_0 = L m
                g = op.adjoint(r)
                put(g, m)
                done += 1
                mk = np.zeros_like(m)
                for _ in range(iterates):
                    if k >= npairs or done >= per:
                        break
                    lg = op.forward(g)
                    gg = float(np.dot(g.ravel().astype(np.float64), g.ravel()))
                    ll = float(np.dot(lg.ravel().astype(np.float64), lg.ravel()))
                    if not (ll > 0):
                        break
                    a = gg / ll
                    mk = (mk + a * g).astype(np.float32)
                    r = (r - a * lg).astype(np.float32)
                    g = op.adjoint(r)
                    put(g, m - mk)
                    done += 1
        finally:
            op.close()
        if verbose:
            print(f"pairs {k}/{npairs}  {time.perf_counter() - t0:.1f} s", flush=True)
    return X, Y


def train(net: UNet3D, X, Y, epochs: int = 10, batch: int = 4, lr: float = 1e-3, seed: int = 0,
          verbose: bool = False):
    """Adam over shuffled mini-batches; returns the mean loss of every epoch."""
    import torch
    rng = np.random.default_rng(seed)
    with torch.cuda.stream(net.stream):
        Xd = torch.tensor(X, device="cuda")
        Yd = torch.tensor(Y, device="cuda")
    net.stream.synchronize()
    hist = []
    n = len(X)
    # fixed batch buffers: the first step is captured into a CUDA graph
    # (UNet3D.capture_train_step) and every later step replays it
    with torch.cuda.stream(net.stream):
        xb = torch.empty((batch,) + tuple(Xd.shape[1:]), dtype=Xd.dtype, device="cuda")
        yb = torch.empty((batch,) + tuple(Yd.shape[1:]), dtype=Yd.dtype, device="cuda")
    captured = False
    for ep in range(epochs):
        order = rng.permutation(n)
        lr_ep = lr * (0.5 * (1 + np.cos(np.pi * ep / max(epochs, 1))))   # cosine decay
        tot = 0.0
        nb = 0
        for i in range(0, n - batch + 1, batch):
            idx = torch.tensor(order[i:i + batch], device="cuda")
            with torch.cuda.stream(net.stream):
                torch.index_select(Xd, 0, idx, out=xb)
                torch.index_select(Yd, 0, idx, out=yb)
            step_lr = max(lr_ep, lr * 0.02)
            if not captured:
                net.capture_train_step(xb, yb, lr=step_lr)   # trains on this batch once
                net.stream.synchronize()
                tot += float(net.loss.item())
                captured = True
            else:
                tot += net.train_step(xb, yb, lr=step_lr)
            nb += 1
        hist.append(tot / max(nb, 1))
        if verbose:
            print(f"epoch {ep}: loss {hist[-1]:.5f}", flush=True)
    return hist


class _CudaView:
    """__cuda_array_interface__ over a raw device pointer (no ownership)."""

    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f4",
                                         "data": (int(ptr), False), "version": 3, "strides": None,
                                         "stream": None}


class UNetDirection:
    """g <- |g| N(g / |g|) on the device, in place (the lsrtm direction hook)."""

    def __init__(self, net: UNet3D, model_shape):
        self.net = net
        self.shape = tuple(model_shape)
        if any(s % 8 for s in self.shape):
            raise ValueError("the model grid must be a multiple of 8 along every axis")
        self.seconds = 0.0
        self.calls = 0

    def __call__(self, g_ptr, n):
        import torch
        t0 = time.perf_counter()
        g = torch.as_tensor(_CudaView(g_ptr, (1,) + self.shape), device="cuda")
        dot = C.c_double()
        if lib.sepx_dot_f32(C.c_void_p(g_ptr), C.c_void_p(g_ptr), C.c_longlong(n), C.byref(dot)):
            return -1
        nrm = float(np.sqrt(max(dot.value / n, 0.0)))
        if nrm == 0.0:
            return 0
        out = self.net.forward_device(g, scale=1.0 / nrm)
        with torch.cuda.stream(self.net.stream):
            g.view(-1).copy_(out).mul_(nrm)
        self.net.stream.synchronize()
        self.seconds += time.perf_counter() - t0
        self.calls += 1
        return 0


def load_network(path: Path | None = None) -> UNet3D:
    path = WEIGHTS if path is None else Path(path)
    return UNet3D(UNet3D.load_params(path))


# ---------------------------------------------------------------------------
# least-squares RTM: plain CG against the learned direction
# ---------------------------------------------------------------------------
def lsrtm_survey(n: int = 384, nt: int = 3000, nshots: int = 4, d: float = 12.5, seed: int = 20261208):
    """The 384^3, dx 12.5 m, 3000-step, 4-shot least-squares RTM workload:
    smooth velocity, random horizon-plus-spike reflectivity, shots on a 2x2
    surface grid, receivers at every surface node."""
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    vel = velocity_model(rng, shape, d)
    refl = random_reflectivity(rng, shape, nhor=(6, 10), spike_frac=0.005)
    s = patch_survey(vel, refl, d, nt)
    q = np.sqrt(nshots)
    k = max(int(round(q)), 1)
    pos = [((i + 0.5) / k * (n - 1) * d, (j + 0.5) / k * (n - 1) * d, 0.0)
           for j in range(k) for i in range(k)][:nshots]
    s.shots = pos
    s.name = f"lsrtm_{n}^3_{nt}_{nshots}shots"
    return s


def lsrtm_compare(s, niter: int = 20, net: UNet3D | None = None, snap_js: int = 4,
                  snap_prec: str = "bf16", fallback_ratio: float = 0.9, verbose: bool = False,
                  policies=("fallback",), probe_every: int = 8, target: float = 0.0,
                  plain_to_learned: bool = False, plain_cap: int = 200) -> dict:
    """Plain simple_solver + cgstep against the same solver with the learned
    direction (one run per direction policy), on data d = L m_true of the
    survey's reflectivity.  target > 0 stops every run at that relative data
    residual (niter caps it).  "learned" holds the first policy's run.

    plain_to_learned: plain CG runs after the learned one, until it reaches the
    learned run's final residual (at most plain_cap iterations), so that both
    are compared at the same data residual: wall time to it, and each image
    against the plain image at that residual and against the true
    reflectivity (key "same_residual")."""
    op = RtmOperator(s, mode="linear", snap_js=snap_js, snap_prec=snap_prec)
    runs = {}
    try:
        t0 = time.perf_counter()
        d = op.forward(s.refl)
        t_fwd = time.perf_counter() - t0
        dd = float(np.dot(d.astype(np.float64).ravel(), d.astype(np.float64).ravel()))
        if not plain_to_learned:
            m_plain, r_plain, s_plain = op.lsrtm(d, niter, target=target)
            if verbose:
                print("plain", np.sqrt(r_plain / dd), s_plain, flush=True)
        net = load_network() if net is None else net
        for pol in policies:
            hook = UNetDirection(net, op.model_shape)
            m_nn, r_nn, s_nn = op.lsrtm(d, niter, direction=hook, fallback_ratio=fallback_ratio,
                                        policy=pol, probe_every=probe_every, target=target)
            used = op.used_dir
            runs[pol] = (m_nn, r_nn, s_nn, hook.seconds, hook.calls, op.fallback_iter,
                         None if used is None else used.tolist())
            if verbose:
                print("learned", pol, np.sqrt(r_nn / dd), s_nn, flush=True)
        if plain_to_learned:
            r_goal = float(np.sqrt(runs[policies[0]][1][-1] / dd)) * (1 + 1e-9)
            m_plain, r_plain, s_plain = op.lsrtm(d, plain_cap, target=r_goal)
            if verbose:
                print("plain", np.sqrt(r_plain / dd), s_plain, flush=True)
    finally:
        op.close()

    def rel(a, b):
        return float(np.linalg.norm((a - b).astype(np.float64)) / max(np.linalg.norm(b.astype(np.float64)), 1e-30))

    def t_to(res, secs, level):
        hit = np.nonzero(res <= level)[0]
        return float(secs[hit[0]]) if len(hit) else None

    rp = np.sqrt(r_plain / dd)
    final_plain = float(rp[-1])
    by_policy = {}
    for pol, (m_nn, r_nn, s_nn, dsec, dcalls, fb_iter, used) in runs.items():
        rn = np.sqrt(r_nn / dd)
        by_policy[pol] = {
            "rel_residual": rn.tolist(), "seconds": s_nn.tolist(),
            "direction_seconds": dsec, "direction_calls": dcalls,
            "fallback_ratio": fallback_ratio, "probe_every": probe_every if pol == "adaptive" else None,
            "plain_g_from_iteration": fb_iter + 1 if fb_iter >= 0 else None,
            "used_direction": used,
            "time_to_1e-2": t_to(rn, s_nn, 1e-2),
            "time_to_plain_final_residual": t_to(rn, s_nn, final_plain),
            "image_rel_l2_vs_plain_cg": rel(m_nn, m_plain),
            "image_rel_l2_vs_true": rel(m_nn, s.refl),
        }
    first = by_policy[policies[0]] if policies else None

    def pick(key):
        return first[key] if first else None

    same = None
    if plain_to_learned and first:
        m_nn = runs[policies[0]][0]
        reached = bool(rp[-1] <= first["rel_residual"][-1] * (1 + 1e-9))
        same = {"residual": first["rel_residual"][-1], "plain_reached": reached,
                "plain_iterations": len(rp), "plain_seconds": float(s_plain[-1]),
                "learned_iterations": len(first["rel_residual"]), "learned_seconds": first["seconds"][-1],
                "speedup": float(s_plain[-1]) / first["seconds"][-1] if reached else None,
                "image_rel_l2_learned_vs_plain": rel(m_nn, m_plain),
                "image_rel_l2_vs_true": {"plain": rel(m_plain, s.refl), "learned": rel(m_nn, s.refl)}}
    return {
        "workload": s.name, "iterations": niter, "target": target or None, "same_residual": same,
        "store": f"{snap_prec} every {snap_js} steps",
        "seconds_data_generation": t_fwd,
        "plain": {"rel_residual": rp.tolist(), "seconds": s_plain.tolist()},
        "learned": first,
        "learned_by_policy": by_policy,
        "time_to_1e-2": {"plain": t_to(rp, s_plain, 1e-2), "learned": pick("time_to_1e-2")},
        "time_to_plain_final_residual": {"plain": float(s_plain[-1]),
                                         "learned": pick("time_to_plain_final_residual")},
        "image_rel_l2_vs_plain_cg": {"learned_final": pick("image_rel_l2_vs_plain_cg")},
        "image_rel_l2_vs_true": {"plain": rel(m_plain, s.refl), "learned": pick("image_rel_l2_vs_true")},
    }


def main(argv=None):
    import argparse
    import json
    p = argparse.ArgumentParser(description="train the U-Net preconditioner / compare LSRTM")
    sub = p.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--pairs", type=int, default=4000)
    t.add_argument("--n", type=int, default=64)
    t.add_argument("--nt", type=int, default=1100)
    t.add_argument("--epochs", type=int, default=24)
    t.add_argument("--batch", type=int, default=4)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--out", default=str(WEIGHTS))
    t.add_argument("--iterates", type=int, default=0,
                   help="also train on this many steepest-descent iterates per reflectivity")
    c = sub.add_parser("lsrtm")
    c.add_argument("--n", type=int, default=384)
    c.add_argument("--nt", type=int, default=3000)
    c.add_argument("--shots", type=int, default=4)
    c.add_argument("--iters", type=int, default=20)
    c.add_argument("--weights", default=str(WEIGHTS))
    c.add_argument("--out", default=None)
    c.add_argument("--policies", default="fallback",
                   help="comma list of fallback,adaptive (empty: plain CG only)")
    c.add_argument("--probe-every", type=int, default=8)
    c.add_argument("--target", type=float, default=0.0)
    c.add_argument("--plain-to-learned", action="store_true",
                   help="run plain CG until it reaches the learned run's final residual")
    c.add_argument("--plain-cap", type=int, default=200)
    a = p.parse_args(argv)
    if a.cmd == "train":
        t0 = time.perf_counter()
        X, Y = make_pairs(a.pairs, n=a.n, nt=a.nt, iterates=a.iterates, verbose=True)
        t1 = time.perf_counter()
        net = UNet3D(seed=0)
        hist = train(net, X, Y, epochs=a.epochs, batch=a.batch, lr=a.lr, verbose=True)
        t2 = time.perf_counter()
        Path(a.out).parent.mkdir(parents=True, exist_ok=True)
        net.save(a.out)
        print(json.dumps({"pairs": a.pairs, "iterates": a.iterates, "patch": a.n, "nt": a.nt,
                          "seconds_pairs": t1 - t0,
                          "seconds_training": t2 - t1, "epochs": a.epochs, "loss": hist}))
    else:
        s = lsrtm_survey(a.n, a.nt, a.shots)
        res = lsrtm_compare(s, a.iters, net=load_network(a.weights), verbose=True,
                            policies=tuple(x for x in a.policies.split(",") if x), probe_every=a.probe_every,
                            target=a.target, plain_to_learned=a.plain_to_learned, plain_cap=a.plain_cap)
        txt = json.dumps(res)
        print(txt)
        if a.out:
            Path(a.out).write_text(txt)


if __name__ == "__main__":
    main()
