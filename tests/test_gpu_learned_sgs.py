"""The learned SGS correction inside the library's step (lexgb_set_sgs_net) against the
differentiable PyTorch path used for training (lex_gb300.autograd step + sgs_cnn.correct), and
training through the solver: a few Adam steps on one coarse-grained sprint lower its loss."""
import pytest

pytestmark = pytest.mark.gpu

DIMS = (32, 16, 16)
SPACING = (600.0, 600.0, 300.0)


def _solver_and_state():
    import numpy as np
    from lex_gb300.solver import Solver
    from lex_gb300.workload import warm_bubble
    from lex_gb300 import autograd as lag
    nx, ny, nz = DIMS
    phys, prof = warm_bubble(nx, ny, nz, *SPACING, amplitude=2.0, radius_h=3000.0, seed=3)
    S = Solver(nx, ny, nz, *SPACING, 3.0, 32, turb_opt=1)
    S.integrate_base_state(prof["theta0"], prof["qv0"])
    S.upload(phys, dtype=np.float32)
    S.step(20)                       # winds and pi' develop
    x0 = lag.get_state(S)
    S.step(10)
    x1 = lag.get_state(S)
    return S, x0, x1


def _net_with_output(seed=3, scale=0.05):
    import torch
    from lex_gb300 import sgs_cnn
    net = sgs_cnn.SGSNet(seed=seed)
    g = torch.Generator(device="cpu").manual_seed(seed + 1)
    w = torch.zeros_like(net.w[3].cpu())
    w[:, :5, :] = torch.randn(27, 5, 32, generator=g) * scale / (27 * 32) ** 0.5
    net.w[3] = w.cuda()
    net.b[3][:5] = torch.randn(5, generator=g).cuda() * 0.1 * scale
    net.refresh()
    return net


def _rel(a, b):
    return float((a - b).norm() / b.norm())


def test_fused_correction_matches_torch_path(built_lib):
    torch = pytest.importorskip("torch")
    from lex_gb300 import autograd as lag, sgs_cnn
    S, x0, x1 = _solver_and_state()
    with S:
        scale = sgs_cnn.make_scale([x0, x1])
        net = _net_with_output()
        with torch.no_grad():
            plain = lag.step(S, x0)
            ref = sgs_cnn.correct(net, plain, scale, DIMS)
        sgs_cnn.attach(S, None, None)
        lag.set_state(S, x0)
        S.step(1)
        y_plain = lag.get_state(S)
        sgs_cnn.attach(S, net, scale)
        lag.set_state(S, x0)
        S.step(1)
        y = lag.get_state(S)
        lag.set_state(S, x0)
        S.step(1, graph=False)                     # the same kernels in plain stream order
        y_eager = lag.get_state(S)
        sgs_cnn.attach(S, None, None)
        lag.set_state(S, x0)
        S.step(1)
        y_off = lag.get_state(S)
    for f, (a, b) in enumerate(zip(y_plain, plain)):
        if f != 3 or b.norm() > 0:
            assert _rel(a, b) <= 1e-5, ("plain step", f, _rel(a, b))
    for f in (0, 1, 2, 3, 5):
        inc, inc_ref = y[f] - y_plain[f], ref[f] - plain[f]
        assert float(inc_ref.norm()) > 0, f
        assert _rel(inc, inc_ref) <= 1e-2, ("correction", f, _rel(inc, inc_ref))
    assert torch.equal(y[4], y_plain[4])            # pi' is not corrected
    assert torch.equal(y[3][0], y_plain[3][0]) and torch.equal(y[3][-1], y_plain[3][-1])   # bottom, lid
    for a, b in zip(y_off, y_plain):                 # turning it off restores the plain step
        assert torch.equal(a, b)
    for a, b in zip(y_eager, y):                     # graph and plain launches agree bit for bit
        assert torch.equal(a, b)


def test_training_through_the_solver_lowers_the_sprint_loss(built_lib):
    torch = pytest.importorskip("torch")
    from lex_gb300 import learned_sgs as L, sgs_cnn
    snaps = L.fine_truth(2.0, 5, t_end=30.0, every=30.0, fine=(96, 96, 48))
    S = L.coarse_solver(dims=(16, 16, 16))
    with S:
        scale = L.field_scale(snaps)
        net = sgs_cnn.SGSNet(seed=0)
        hist = L.train(S, net, [snaps], scale, steps_per_sprint=10, iters=30, lr=1e-5, warmup=5)
        with torch.no_grad():
            out = L.sprint(S, tuple(a.detach() for a in snaps[0]), 10, net, scale, grad=False)
            after = float(L.loss_fn(out, snaps[1], scale))
    assert all(h == h for h in hist)                 # finite
    assert after < hist[0], (hist[0], after)
