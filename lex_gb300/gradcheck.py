"""Gradient of a 600 s warm-bubble rollout with respect to the initial theta' and the Smagorinsky
constant, checked against central finite differences (the differentiable-step case: 64^3 at
300 m x 300 m x 150 m, dt 2 s, 300 big steps).

    loss = mean over the grid of (theta'(600 s) - theta'_target)^2,  theta' = theta - 300 K
    theta'_target: the same run started from a 2.5 K bubble instead of 2 K

The backward runs the library's reverse mode through lex_gb300.autograd with a checkpoint every
`seg` steps (torch.utils.checkpoint over segments: only every seg-th state is kept, a segment
is recomputed in the backward pass).  Finite differences use the library's graph forward
(FP32, theta kept relative to theta_ref) on seeded random directions v of the initial theta (unit
normal per point) and on Cs (tests/test_gpu_gradcheck.py takes them from the FP64 oracle instead):
    <dL/dtheta0, v>  vs  (L(theta0 + eps v) - L(theta0 - eps v)) / (2 eps)
    dL/dCs           vs  (L(Cs + eps) - L(Cs - eps)) / (2 eps)

    python -m lex_gb300.gradcheck [--steps 300] [--dirs 16] [--eps 1e-3] [--out result.json]
"""
import json
import time

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

from . import autograd as lag
from .solver import Solver
from .workload import warm_bubble


def experiment(n=64, spacing=(300.0, 300.0, 150.0), dt=2.0, steps=300, seg=10, ndirs=16, eps=1e-3, cs0=0.18,
               seed=2025, log=print):
    t0 = time.time()
    S = Solver(n, n, n, *spacing, dt, 32, turb_opt=1)
    phys, prof = warm_bubble(n, n, n, *spacing, amplitude=2.0, seed=seed)
    S.integrate_base_state(prof["theta0"], prof["qv0"])
    # theta in the device layout (theta - theta_ref, exact in FP32) throughout: the loss's theta'
    # = theta - 300 K is that plus a constant
    off = float(prof["theta0"][1]) - 300.0
    S.upload(phys, dtype=np.float32)
    x0 = lag.get_state(S, raw=True)
    phys_t, _ = warm_bubble(n, n, n, *spacing, amplitude=2.5, seed=seed)
    S.upload(phys_t, dtype=np.float32)
    S.step(steps)
    target = lag.get_state(S, raw=True)[0].double() + off

    def loss_nograd(theta0, cs):
        if cs != S.cs:
            S.set_cs(cs)
        lag.set_state(S, (theta0,) + tuple(x0[1:]), raw=True)
        S.step(steps)
        th = lag.get_state(S, raw=True)[0]
        return float(((th.double() + off - target) ** 2).mean())

    # gradient by the reverse mode, checkpoint every seg steps
    theta0 = x0[0].clone().requires_grad_(True)
    cs = torch.tensor(cs0, dtype=torch.float64, device="cuda", requires_grad=True)
    state = (theta0,) + tuple(x0[1:])
    for _ in range(steps // seg):
        state = checkpoint(lambda *s: lag.rollout(S, s, seg, cs, raw=True), *state, use_reentrant=False)
    L = ((state[0].double() + off - target) ** 2).mean()
    L.backward()
    g_theta, g_cs = theta0.grad.detach().double(), float(cs.grad)
    t_grad = time.time() - t0
    if log:
        log("loss %.6g, gradient in %.1f s" % (float(L.detach()), t_grad))
    # finite differences with the FP32 graph forward
    gen = torch.Generator(device="cuda").manual_seed(seed)
    dirs = []
    for k in range(ndirs):
        v = torch.randn(theta0.shape, device="cuda", generator=gen)
        lp = loss_nograd(x0[0] + eps * v, cs0)
        lm = loss_nograd(x0[0] - eps * v, cs0)
        fd = (lp - lm) / (2 * eps)
        ad = float((g_theta * v.double()).sum())
        dirs.append({"fd": fd, "adjoint": ad, "rel_err": abs(ad - fd) / max(abs(fd), 1e-300)})
        if log:
            log("direction %2d  fd %.6e  adjoint %.6e  rel. err %.2e" % (k, fd, ad, dirs[-1]["rel_err"]))
    lp = loss_nograd(x0[0], cs0 + eps)
    lm = loss_nograd(x0[0], cs0 - eps)
    S.set_cs(cs0)
    fd_cs = (lp - lm) / (2 * eps)
    S.close()
    rel = [d["rel_err"] for d in dirs]
    return {"case": "%d^3 at %s m, dt %g s, %d steps, checkpoint every %d steps" % (n, spacing, dt, steps, seg),
            "loss": float(L.detach()), "grad_seconds": t_grad, "eps": eps, "directions": dirs,
            "rel_err_median": float(np.median(rel)), "rel_err_max": float(np.max(rel)),
            "dL_dCs": {"fd": fd_cs, "adjoint": g_cs, "rel_err": abs(g_cs - fd_cs) / max(abs(fd_cs), 1e-300)},
            "seconds": time.time() - t0}


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--seg", type=int, default=10)
    ap.add_argument("--dirs", type=int, default=16)
    ap.add_argument("--eps", type=float, default=1e-3)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    r = experiment(steps=a.steps, seg=a.seg, ndirs=a.dirs, eps=a.eps)
    line = json.dumps(r)
    print(line)
    if a.out:
        with open(a.out, "w") as f:
            f.write(line + "\n")


if __name__ == "__main__":
    main()
