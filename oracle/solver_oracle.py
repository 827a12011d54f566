"""CPU restatement of the reference's least-squares solver on a dense operator
(test infrastructure; only tests/ use it).

``cg_solve`` follows simple_solver + cgstep (Born/lin_solver.cpp:7-17,
:115-143; Born/cgstep.cpp:14-58) with the reference's arithmetic: float32
vectors, FP64 dot products accumulated in index order
(Born/hypercube_float.cpp:123-132), vector updates evaluated in FP64 and
rounded once to float (scale_add, Born/hypercube_float.cpp:212-218), float
additions (``add``, :219-223), and the dense operator of the reference harness
(oracle/ref_stubs/ref_shim.cpp ``dense_op``: each output an FP64 sum in index
order, rounded to float, then added in float).  Pinned against the
reference's own solver compiled here (tests/golden/cgstep_dense.npz).

``lstsq`` and friends are plain FP64 solutions of the normal equations that
prec_solver and reg_solver (Born/lin_solver.cpp:21-53) converge to.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def _dot(a, b) -> float:
    s = 0.0
    for x, y in zip(a.tolist(), b.tolist()):
        s += x * y
    return s


def _matvec(A, x, add_to=None, adjoint=False):
    """dense_op forward (adjoint=False) or adjoint: FP64 sums in index order,
    rounded to float, added in float to add_to (zero when None)."""
    A64 = A.astype(np.float64)
    xs = x.astype(np.float64).tolist()
    rows = A64.T if adjoint else A64
    out = np.zeros(rows.shape[0], F32) if add_to is None else add_to.copy()
    for i, row in enumerate(rows.tolist()):
        s = 0.0
        for a, v in zip(row, xs):
            s += a * v
        out[i] = F32(out[i] + F32(s))
    return out


def _scale_add(y, a, x, b):
    """y = y*a + b*x in FP64, rounded to float (the three-argument scale_add)"""
    return (y.astype(np.float64) * a + b * x.astype(np.float64)).astype(F32)


def cg_solve(A, d, niter, small=1e-20):
    """simple_solver(cgstep, d, A).solve(niter) from m = 0.  Returns (model
    after each iteration [niter][nc], rr.rr after each iteration, alphas,
    betas); stops early where cgstep reports a zero direction."""
    A = np.asarray(A, F32)
    d = np.asarray(d, F32)
    nr, nc = A.shape
    rr = (d.astype(np.float64) * -1.0).astype(F32)   # init_rr: data scaled by -1
    m = np.zeros(nc, F32)
    s = np.zeros(nc, F32)
    ss = np.zeros(nr, F32)
    forget = True
    ms, rrs, alphas, betas = [], [], [], []
    for _ in range(niter):
        g = _matvec(A, rr, adjoint=True)
        gg = _matvec(A, g)
        if forget:
            beta = 0.0
            gg_gg = _dot(gg, gg)
            if abs(gg_gg) < small:
                break
            alfa = -_dot(gg, rr) / gg_gg
        else:
            gg_gg, ss_ss, gg_ss = _dot(gg, gg), _dot(ss, ss), _dot(gg, ss)
            if abs(gg_gg) < small or abs(ss_ss) < small:
                break
            determ = gg_gg * ss_ss * (1.0 - gg_ss / gg_gg * gg_ss / ss_ss)
            gg_rr, ss_rr = -_dot(gg, rr), -_dot(ss, rr)
            alfa = (ss_ss * gg_rr - gg_ss * ss_rr) / determ
            beta = (-gg_ss * gg_rr + gg_gg * ss_rr) / determ
        s = _scale_add(s, beta, g, alfa)
        ss = _scale_add(ss, beta, gg, alfa)
        m = (m + s).astype(F32)
        rr = (rr + ss).astype(F32)
        forget = False
        ms.append(m.copy())
        rrs.append(_dot(rr, rr))
        alphas.append(alfa)
        betas.append(beta)
    return np.array(ms), np.array(rrs), np.array(alphas), np.array(betas)


def lstsq(A, d):
    """min |A m - d|^2 in FP64"""
    A = np.asarray(A, np.float64)
    return np.linalg.solve(A.T @ A, A.T @ np.asarray(d, np.float64))


def prec_lstsq(A, P, eps, d):
    """prec_solver's problem: min |A P x - d|^2 + eps^2 |x|^2; returns m = P x"""
    AP = np.asarray(A, np.float64) @ np.asarray(P, np.float64)
    x = np.linalg.solve(AP.T @ AP + eps * eps * np.eye(AP.shape[1]), AP.T @ np.asarray(d, np.float64))
    return np.asarray(P, np.float64) @ x


def reg_lstsq(A, R, eps, d):
    """reg_solver's problem: min |A m - d|^2 + |eps R m|^2 (the regulariser
    applies its scale eps)"""
    A = np.asarray(A, np.float64)
    R = np.asarray(R, np.float64)
    return np.linalg.solve(A.T @ A + eps * eps * (R.T @ R), A.T @ np.asarray(d, np.float64))
