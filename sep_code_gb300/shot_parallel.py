"""Shot-parallel least-squares RTM: one GPU per rank, the shots of a survey
dealt round-robin to the ranks.

The reference runs its shots one after the other inside rtm_zero_op::forward
and ::adjoint (Born/rtm_zero_op_3d.cpp:123, :226) and solves with
simple_solver + cgstep (Born/lin_solver.cpp:115-143, Born/cgstep.cpp:14-58).
Shots are independent, so here each rank owns an operator over its own
shots, the data are sharded by shot and the model (the image) is replicated:

* forward ``L m``: every rank models its shots; no communication;
* adjoint ``L' d``: every rank images its shots, then one sum-reduce of the
  image (FP32, the model size) gives every rank the same gradient;
* the conjugate-direction step needs the data-space inner products gg.gg,
  gg.rr (first iteration) or gg.gg, ss.ss, gg.ss, gg.rr, ss.rr (later ones)
  and the residual energy rr.rr: each rank's FP64 partial sums, summed in one
  all-reduce of a few doubles each.

So one iteration costs one image reduction and two reductions of at most
five doubles.  Every rank performs the same model-space updates on identical
values and ends with the same image.  The step is the plane search of
cgstep with its arithmetic (FP64 inner products and step lengths, vector
updates evaluated in FP64 and rounded to float).  No cluster multicast and no
peer loads are used: the reductions go through torch.distributed (NCCL
between GPUs, gloo on the CPU).
"""
from __future__ import annotations

import time

import numpy as np

F32 = np.float32


class Comm:
    """Sum-reductions over the ranks of the default torch.distributed group
    (a single process needs none)."""

    def __init__(self):
        try:
            import torch.distributed as dist
            self.dist = dist if dist.is_available() and dist.is_initialized() else None
        except ImportError:
            self.dist = None
        self.rank = self.dist.get_rank() if self.dist else 0
        self.size = self.dist.get_world_size() if self.dist else 1
        self.calls = {"image": 0, "scalars": 0}

    def _sum(self, arr: np.ndarray) -> np.ndarray:
        if self.dist is None:
            return arr
        import torch
        t = torch.from_numpy(np.ascontiguousarray(arr))
        if self.dist.get_backend() == "nccl":
            t = t.cuda()
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return t.cpu().numpy().astype(arr.dtype, copy=False)

    def sum_image(self, img: np.ndarray) -> np.ndarray:
        self.calls["image"] += 1
        return self._sum(np.asarray(img, F32))

    def sum_scalars(self, vals) -> np.ndarray:
        self.calls["scalars"] += 1
        return self._sum(np.asarray(vals, np.float64))


def shard(items, rank: int, size: int):
    """The items of rank ``rank``: every size-th one, from position rank."""
    return list(items)[rank::size]


def shard_survey(s, rank: int, size: int):
    """A copy of survey ``s`` holding only this rank's shots."""
    import copy
    t = copy.copy(s)
    t.shots = shard(s.shots, rank, size)
    return t


def _dot(a, b) -> float:
    return float(np.dot(a.astype(np.float64).ravel(), b.astype(np.float64).ravel()))


def _step(y, a, x, b):
    """y * a + b * x evaluated in FP64, rounded to float (cgstep's updates)"""
    return (y.astype(np.float64) * a + b * x.astype(np.float64)).astype(F32)


def lsrtm(op, data_local: np.ndarray, niter: int, comm: Comm | None = None, small: float = 1e-20):
    """simple_solver + cgstep from m = 0 over sharded data.

    op: this rank's operator, ``forward(m) -> data of its shots`` and
    ``adjoint(d) -> image of its shots`` (e.g. ``RtmOperator`` of the rank's
    shard of the survey).  data_local: this rank's observed data.  Returns
    (model, rr.rr after each iteration, seconds at each iteration); the model
    and the residuals are the same on every rank."""
    comm = comm or Comm()
    rr = (np.asarray(data_local, F32).astype(np.float64) * -1.0).astype(F32)
    m = s = None
    ss = np.zeros_like(rr)
    forget = True
    resid, secs = [], []
    t0 = time.perf_counter()
    for _ in range(niter):
        g = comm.sum_image(op.adjoint(rr))
        gg = op.forward(g)
        if m is None:
            m = np.zeros_like(g)
            s = np.zeros_like(g)
        if forget:
            gg_gg, gg_rr = comm.sum_scalars([_dot(gg, gg), _dot(gg, rr)])
            if abs(gg_gg) < small:
                break
            beta, alfa = 0.0, -gg_rr / gg_gg
        else:
            gg_gg, ss_ss, gg_ss, gg_rr, ss_rr = comm.sum_scalars(
                [_dot(gg, gg), _dot(ss, ss), _dot(gg, ss), _dot(gg, rr), _dot(ss, rr)])
            if abs(gg_gg) < small or abs(ss_ss) < small:
                break
            determ = gg_gg * ss_ss * (1.0 - gg_ss / gg_gg * gg_ss / ss_ss)
            gg_rr, ss_rr = -gg_rr, -ss_rr
            alfa = (ss_ss * gg_rr - gg_ss * ss_rr) / determ
            beta = (-gg_ss * gg_rr + gg_gg * ss_rr) / determ
        s = _step(s, beta, g, alfa)
        ss = _step(ss, beta, gg, alfa)
        m = (m + s).astype(F32)
        rr = (rr + ss).astype(F32)
        forget = False
        resid.append(float(comm.sum_scalars([_dot(rr, rr)])[0]))
        secs.append(time.perf_counter() - t0)
    return m, np.array(resid), np.array(secs)


def main(argv=None):
    """Least-squares RTM of a multi-shot survey with the shots spread over
    the ranks of a torchrun launch (one GPU each):

        python -m torch.distributed.run --nproc-per-node N \\
            -m sep_code_gb300.shot_parallel [--n 128] [--nt 1000] [--shots 8] [--niter 5]
    """
    import argparse
    import json
    import os

    import torch.distributed as dist

    from . import learned as Lr
    from .operator import RtmOperator

    p = argparse.ArgumentParser()
    p.add_argument("--n", type=int, default=128)
    p.add_argument("--nt", type=int, default=1000)
    p.add_argument("--shots", type=int, default=8)
    p.add_argument("--niter", type=int, default=5)
    a = p.parse_args(argv)
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("LOCAL_RANK", "0")
        dist.init_process_group("nccl")
    comm = Comm()
    s = Lr.lsrtm_survey(n=a.n, nt=a.nt, nshots=a.shots)
    mine = shard_survey(s, comm.rank, comm.size)
    op = RtmOperator(mine, "linear", 4, "bf16")
    data = op.forward(s.refl)
    m, resid, secs = lsrtm(op, data, a.niter, comm)
    if comm.rank == 0:
        print(json.dumps({"ranks": comm.size, "shots": len(s.shots), "residual": (resid / resid[0]).tolist(),
                          "seconds": secs.tolist(), "reductions": comm.calls}))
    op.close()
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
