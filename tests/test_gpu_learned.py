"""What the trained U-Net preconditioner buys inside least-squares RTM.

The committed network (sep_code_gb300/data/unet_precond.npz, trained on 4000
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


def test_learned_reaches_a_residual_sooner_at_equal_image_error():
    """Both solvers stopped at the same data residual (the learned run's after
    8 iterations; plain CG runs until it reaches it): the learned direction
    gets there in fewer iterations and less wall time, and its image is at
    least as close to the true reflectivity as the plain image at that
    residual (5% margin).  The two images themselves differ by more than
    either's size (measured 1.8 relative L2): at one data residual they hold
    different parts of what the data do not constrain."""
    from sep_code_gb300 import learned as Lr
    s = Lr.lsrtm_survey(n=64, nt=1000, nshots=1, seed=97)
    r = Lr.lsrtm_compare(s, niter=8, snap_prec="f32", plain_to_learned=True, plain_cap=80)
    same = r["same_residual"]
    print("LSRTM_SAME_RESIDUAL", same)
    assert same["plain_reached"]
    assert same["learned_seconds"] < same["plain_seconds"]
    assert same["learned_iterations"] < same["plain_iterations"]
    err = same["image_rel_l2_vs_true"]
    assert err["learned"] <= 1.05 * err["plain"]


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


def _replay_adaptive(rr, rr0, used, ratio, probe):
    """the SEPX_DIR_ADAPTIVE rule applied to the recorded residual energies"""
    want, cur, gain_plain, run, prev = [], 1, -1.0, 0, rr0
    for v in rr:
        want.append(cur)
        gain = 1.0 - v / prev
        if cur:
            cur = int(not (ratio > 0 and v > ratio * prev)) if gain_plain < 0 else int(gain >= gain_plain)
            run = 0
        else:
            gain_plain = gain
            run += 1
            cur = int(run >= probe)
        prev = v
    return want


def test_adaptive_direction_policy_and_target_stop():
    """SEPX_DIR_ADAPTIVE follows its rule iteration by iteration (checked by
    replaying it on the recorded residuals), keeps the residual
    non-increasing, and a target residual stops the solver at the first
    iteration that reaches it."""
    from sep_code_gb300 import learned as Lr
    from sep_code_gb300.operator import RtmOperator
    s = Lr.lsrtm_survey(n=64, nt=1000, nshots=1, seed=97)
    op = RtmOperator(s, mode="linear", snap_js=4, snap_prec="f32")
    try:
        d = op.forward(s.refl)
        dd = float(np.dot(d.astype(np.float64).ravel(), d.astype(np.float64).ravel()))
        hook = Lr.UNetDirection(Lr.load_network(), op.model_shape)
        _, rr, _ = op.lsrtm(d, 10, direction=hook, fallback_ratio=0.9, policy="adaptive", probe_every=2)
        used = op.used_dir.tolist()
        assert len(rr) == 10 and np.all(np.diff(rr) <= 1e-12 * dd)
        assert used[0] == 1 and 0 in used
        assert used == _replay_adaptive(rr, dd, used, 0.9, 2)
        # the plain run stopped by a target taken from its own 6th iteration
        _, rp, _ = op.lsrtm(d, 10)
        tgt = float(np.sqrt(rp[5] / dd)) * (1 + 1e-9)
        _, rs, _ = op.lsrtm(d, 10, target=tgt)
        assert len(rs) == 6 and np.allclose(rs, rp[:6], rtol=0, atol=0)
    finally:
        op.close()


def test_descent_iterate_pairs_are_normal_equation_pairs():
    """make_pairs(iterates=2): every input is L'L applied to its target (up to
    the unit-RMS normalisation of each): the descent iterates' gradients are
    the normal operator of the remaining error"""
    from sep_code_gb300 import learned as Lr
    from sep_code_gb300.operator import RtmOperator
    X, Y = Lr.make_pairs(3, n=32, nt=400, nvel=1, seed=5, iterates=2)
    assert np.all(np.isfinite(X)) and np.all(np.isfinite(Y))
    # the same velocity model the generator drew (first draw of its rng)
    rng = np.random.default_rng(5)
    vel = Lr.velocity_model(rng, (32, 32, 32), 12.5)
    s = Lr.patch_survey(vel, np.zeros_like(vel), 12.5, 400)
    op = RtmOperator(s, mode="linear", snap_js=4, snap_prec="f32")
    try:
        for k in range(3):
            want = op.adjoint(op.forward(Y[k]))
            want = want / np.sqrt(np.mean(want.astype(np.float64) ** 2))
            err = np.linalg.norm((X[k] - want).astype(np.float64)) / np.linalg.norm(want.astype(np.float64))
            assert err <= 1e-3, (k, err)
        # the iterates are different problems: the error shrinks its low-frequency part
        assert np.linalg.norm(X[1] - X[0]) > 1e-2 * np.linalg.norm(X[0])
    finally:
        op.close()
