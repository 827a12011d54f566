"""What the trained U-Net preconditioner buys inside least-squares RTM.

The committed network (sep_code_gb300/data/unet_precond.npz, trained on 2000
64^3 pairs (L'L m, m) of the Born operator) preconditions the search
direction of simple_solver + cgstep; plain CG runs on the same operator and
data.  On an unseen survey the learned direction must reach plain CG's final
data residual in fewer iterations and end lower; the plane search keeps the
residual non-increasing either way.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_learned_direction_beats_plain_cg():
    from sep_code_gb300 import learned as Lr
    s = Lr.lsrtm_survey(n=64, nt=1000, nshots=1, seed=97)
    r = Lr.lsrtm_compare(s, niter=8, snap_prec="f32")
    rp = np.array(r["plain"]["rel_residual"])
    rn = np.array(r["learned"]["rel_residual"])
    print("LSRTM_SMALL", r["plain"]["rel_residual"], r["learned"]["rel_residual"])
    assert np.all(np.diff(rp) <= 1e-12) and np.all(np.diff(rn) <= 1e-12)
    assert rn[-1] < rp[-1]
    hit = np.nonzero(rn <= rp[-1])[0]
    assert len(hit) and hit[0] < len(rp) - 1
    assert r["learned"]["direction_calls"] >= 1


def test_direction_hook_is_finite_and_in_place():
    import torch
    from sep_code_gb300 import learned as Lr
    net = Lr.load_network()
    hook = Lr.UNetDirection(net, (32, 32, 32))
    g = torch.randn(32 * 32 * 32, device="cuda")
    torch.cuda.synchronize()
    before = g.clone()
    assert hook(g.data_ptr(), g.numel()) == 0
    torch.cuda.synchronize()
    assert torch.isfinite(g).all()
    assert not torch.equal(g, before)
