"""The learned SGS correction inside the library's step (lexgb_set_sgs_net) against the
differentiable PyTorch path used for training (lex_gb300.autograd step + sgs_cnn.correct);
training through the solver: a few Adam steps on one coarse-grained sprint lower its loss; and
what a trained network (tests/golden/sgs_net_32.npz) gains over Smagorinsky alone on a held-out run."""
import json

import numpy as np
import pytest

from conftest import report_path

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


def _stored_network():
    """The network and packing ranges of tests/golden/sgs_net_32.npz (tests/golden/make_sgs_net.py)."""
    import torch
    from conftest import load_golden
    from lex_gb300 import sgs_cnn
    g = load_golden("sgs_net_32.npz")
    nw = sum(1 for k in g if k[0] == "w" and k[1:].isdigit())
    net = sgs_cnn.SGSNet(seed=0)
    net.load_state_dict({"w": [torch.from_numpy(g["w%d" % i]) for i in range(nw)],
                         "b": [torch.from_numpy(g["b%d" % i]) for i in range(nw)]})
    lo = torch.from_numpy(g["lo"]).cuda()
    rin = torch.from_numpy(g["rin"]).cuda()
    rl = torch.from_numpy(g["rout_level"]).cuda()
    return net, lo, rin, rl, json.loads(str(g["summary"]))


def test_trained_network_beats_smagorinsky_on_the_held_out_run(built_lib):
    """What the learned correction gains (one_sprint_functions.py:118-165 applied after every
    coarse step): on the held-out 600 s run (a bubble the training never saw; 100 m truth
    coarse-grained to 600 m x 600 m x 300 m), the relative L2 error of theta' of the corrected
    coarse run is below that of the run with Smagorinsky alone, by at least 20% on average, and
    a corrected step costs at most 1.3 plain ones."""
    from lex_gb300 import learned_sgs as L
    from lex_gb300.workload import random_bubbles
    net, lo, rin, rl, summary = _stored_network()
    held = L.fine_run(random_bubbles(300, 1, 19200.0, 19200.0, centred=True), 300)
    S = L.coarse_solver()
    with S:
        nz, ny, nx = held[0][0].shape
        scale = {"lo": lo, "rin": rin, "rout": rl.view(5, nz + 1, 1, 1).expand(5, nz + 1, ny, nx).contiguous()}
        base = L.theta_error(S, held)
        learned = L.theta_error(S, held, net, scale)
        plain_ms = L.step_cost(S, held[0])
        corr_ms = L.step_cost(S, held[0], net, scale)
    with open(report_path("learned_sgs_report.json"), "w") as f:
        json.dump({"theta_err_smagorinsky": base, "theta_err_learned": learned,
                   "mean_smagorinsky": float(np.mean(base)), "mean_learned": float(np.mean(learned)),
                   "ms_per_step_plain": plain_ms, "ms_per_step_learned": corr_ms,
                   "training_summary": {k: summary[k] for k in ("chosen", "cost_ratio", "seconds")}}, f, indent=1)
    assert np.mean(learned) <= 0.8 * np.mean(base), (np.mean(learned), np.mean(base))
    assert corr_ms <= 1.3 * plain_ms, (corr_ms, plain_ms)
