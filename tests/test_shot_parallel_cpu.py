"""The shot-parallel least-squares solver on the CPU: two gloo ranks, each
with a dense operator over its own shots, give the single-rank solution of
the same problem (all shots on one rank), with one image reduction and two
scalar reductions per iteration."""
import os
import socket

import numpy as np

from sep_code_gb300 import shot_parallel as SP

NSHOT, NM, ND, NITER = 5, 40, 30, 12


class DenseShots:
    """forward: m -> data of the given shots [nshot][ND]; adjoint: their image"""

    def __init__(self, mats):
        self.mats = [np.asarray(a, np.float64) for a in mats]

    def forward(self, m):
        return np.stack([(a @ m.astype(np.float64)).astype(np.float32) for a in self.mats])

    def adjoint(self, d):
        out = np.zeros(self.mats[0].shape[1], np.float64)
        for a, di in zip(self.mats, d):
            out += a.T @ di.astype(np.float64)
        return out.astype(np.float32)


def _problem():
    rng = np.random.default_rng(4)
    mats = [rng.standard_normal((ND, NM)) / np.sqrt(ND) for _ in range(NSHOT)]
    m_true = rng.standard_normal(NM).astype(np.float32)
    data = np.stack([(a @ m_true).astype(np.float32) for a in mats])
    data += 0.01 * rng.standard_normal(data.shape).astype(np.float32)
    return mats, data


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        mats, data = _problem()
        comm = SP.Comm()
        mine = SP.shard(range(NSHOT), comm.rank, comm.size)
        op = DenseShots([mats[i] for i in mine])
        m, resid, _ = SP.lsrtm(op, data[mine], NITER, comm)
        q.put((rank, m, resid, dict(comm.calls), mine))
    finally:
        dist.destroy_process_group()


def test_two_ranks_match_one():
    import torch.multiprocessing as mp
    mats, data = _problem()
    m1, r1, _ = SP.lsrtm(DenseShots(mats), data, NITER, SP.Comm())
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    for _ in procs:
        rank, m, resid, calls, mine = q.get(timeout=300)
        got[rank] = (m, resid, calls, mine)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got[0][3] == [0, 2, 4] and got[1][3] == [1, 3]
    # every rank holds the same model and residuals
    assert np.array_equal(got[0][0], got[1][0]) and np.array_equal(got[0][1], got[1][1])
    m2, r2 = got[0][0], got[0][1]
    assert np.linalg.norm(m2 - m1) / np.linalg.norm(m1) <= 1e-5
    assert np.max(np.abs(r2 / r1 - 1)) <= 1e-5
    assert np.all(r2[1:] < r2[:-1])
    # one image reduction and two scalar reductions per iteration
    assert got[0][2] == {"image": NITER, "scalars": 2 * NITER}


def test_single_rank_is_the_dense_solution():
    """enough iterations reach the FP64 least-squares model"""
    mats, data = _problem()
    m, resid, _ = SP.lsrtm(DenseShots(mats), data, 60, SP.Comm())
    A = np.vstack(mats)
    want = np.linalg.lstsq(A, data.astype(np.float64).ravel(), rcond=None)[0]
    assert np.linalg.norm(m - want) / np.linalg.norm(want) <= 1e-4
