"""Learned SGS correction: training data, training through the differentiable solver, evaluation.

Training data (the role of dataset_generation.py:12-194, which reads pre-built 40^3 benchmark
sequences): the library's own fine runs of the warm bubble (100 m) are coarse-grained onto the
coarse grid (600 m x 600 m x 300 m: factors 6, 6, 3) every `every` seconds -
    theta, pi', qv : box means over the fine cells of a coarse cell
    u (v)          : means over the fine faces that make up a coarse x (y) face
    w              : means over the fine faces that make up a coarse z face
Training (lex_dl_train.py:49-131): from a coarse-grained state, a sprint of coarse steps with the
CNN correction after each step (one_sprint_functions.py:128-163) is compared with the
coarse-grained truth at the sprint's end; the loss is the sum over theta, u, v, w, qv of the
squared error normalised by each field's range (the reference adds Laplacian and negative-qv
terms).  Gradients flow through the solver (lex_gb300.autograd) and the CNN (lex_gb300.sgs_cnn);
Adam updates the weights.  Evaluation: coarse runs with and without the correction against the
coarse-grained fine run, error of theta' = theta - 300 K.
"""
import time

import numpy as np
import torch

from . import autograd as lag
from . import sgs_cnn
from .solver import Solver
from .workload import warm_bubble

FACTORS = (6, 6, 3)


def coarse_grain(state, f=FACTORS):
    """Device-layout state (theta, u, v, w, pi', qv) -> the coarse grid (factors fx, fy, fz)."""
    fx, fy, fz = f
    th, u, v, w, p, q = state
    nz, ny, nx = th.shape
    NZ, NY, NX = nz // fz, ny // fy, nx // fx

    def cells(a):
        return a.reshape(NZ, fz, NY, fy, NX, fx).mean(dim=(1, 3, 5))
    uc = u[:, :, ::fx].reshape(NZ, fz, NY, fy, NX).mean(dim=(1, 3))
    vc = v[:, ::fy, :].reshape(NZ, fz, NY, NX, fx).mean(dim=(1, 4))
    wc = w[::fz].reshape(NZ + 1, NY, fy, NX, fx).mean(dim=(2, 4))
    return (cells(th), uc.contiguous(), vc.contiguous(), wc.contiguous(), cells(p), cells(q))


def fine_truth(amplitude=2.0, seed=2025, t_end=600.0, every=30.0, fine=(192, 192, 96), spacing=(100., 100., 100.),
               dt=1.0, f=FACTORS):
    """Coarse-grained snapshots (t = 0, every, ..., t_end) of a fine warm-bubble run."""
    nx, ny, nz = fine
    phys, prof = warm_bubble(nx, ny, nz, *spacing, amplitude=amplitude, seed=seed)
    S = Solver(nx, ny, nz, *spacing, dt, 32, turb_opt=1)
    S.integrate_base_state(prof["theta0"], prof["qv0"])
    S.upload(phys, dtype=np.float32)
    per = int(round(every / dt))
    snaps = [coarse_grain(lag.get_state(S))]
    for _ in range(int(round(t_end / every))):
        S.step(per)
        snaps.append(coarse_grain(lag.get_state(S)))
    torch.cuda.synchronize()
    S.close()
    return snaps


def coarse_solver(dims=(32, 32, 32), spacing=(600., 600., 300.), dt=3.0):
    nx, ny, nz = dims
    _, prof = warm_bubble(nx, ny, nz, *spacing)
    S = Solver(nx, ny, nz, *spacing, dt, 32, turb_opt=1)
    S.integrate_base_state(prof["theta0"], prof["qv0"])
    return S


def field_scale(snapshots):
    """Per-level ranges of the training snapshots (the scaling_params of the reference)."""
    return sgs_cnn.make_scale(snapshots)


def sprint(S, state, nsteps, net=None, scale=None, grad=True):
    """nsteps coarse steps, each followed by the CNN correction when net is given."""
    dims = (S.nx, S.ny, S.nz)
    with torch.set_grad_enabled(grad):
        for _ in range(nsteps):
            state = lag.step(S, state)
            if net is not None:
                state = sgs_cnn.correct(net, state, scale, dims)
    return state


def loss_fn(state, truth, scale):
    """Sum over theta, u, v, w, qv of the squared error, each field divided by its largest
    per-level input range (the normalised L2 loss of lex_dl_train.py:49-99 without its Laplacian
    and negative-qv terms)."""
    total = 0.0
    for f, i in enumerate((0, 1, 2, 3, 5)):
        r = scale["rin"][f].max()
        total = total + ((state[i] - truth[i]) / r).pow(2).sum()
    return total


def train(S, net, series, scale, steps_per_sprint=10, iters=200, lr=1e-4, warmup=50, sprints=1, seed=0, log=None):
    """Adam on rollouts drawn from the coarse-grained series (lists of snapshot tuples): from a
    snapshot, `sprints` sprints of `steps_per_sprint` corrected coarse steps, the loss summed over
    the snapshots they end at.  The learning rate rises linearly over the first `warmup` steps."""
    rng = np.random.default_rng(seed)
    for t in net.params():
        t.requires_grad_(True)
    hist = []
    for it in range(iters):
        s = series[rng.integers(len(series))]
        k = int(rng.integers(len(s) - sprints))
        state = tuple(a.detach() for a in s[k])
        loss = 0.0
        for j in range(1, sprints + 1):
            state = sprint(S, state, steps_per_sprint, net, scale)
            loss = loss + loss_fn(state, s[k + j], scale)
        grads = torch.autograd.grad(loss, net.params())
        n = net.step_count + 1
        sgs_cnn.adam_step(net, [g.detach() for g in grads], lr=lr * min(1.0, n / max(1, warmup)))
        hist.append(float(loss.detach()))
        if log and (it % 20 == 0 or it == iters - 1):
            log("iter %d loss %.4g" % (it, hist[-1]))
    return hist


def theta_error(S, snaps, net=None, scale=None, steps_per_snapshot=10):
    """Relative L2 error of theta' = theta - 300 K along a coarse run from snaps[0] against the
    coarse-grained truth; with `net`, the library applies the correction after every step."""
    sgs_cnn.attach(S, net, scale)
    lag.set_state(S, tuple(a.detach() for a in snaps[0]))
    errs = []
    for k in range(1, len(snaps)):
        S.step(steps_per_snapshot)
        th = lag.get_state(S)[0]
        ref = snaps[k][0] - 300.0
        errs.append(float((th - snaps[k][0]).norm() / ref.norm()))
    sgs_cnn.attach(S, None, None)
    return errs


def step_cost(S, state, net=None, scale=None, n=200):
    """Mean ms per coarse step (with the fused correction when net is given), CUDA events on the
    stream the solver runs on."""
    sgs_cnn.attach(S, net, scale)
    lag.set_state(S, tuple(a.detach() for a in state))
    S.step(3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    S.step(n)
    e1.record()
    e1.synchronize()
    sgs_cnn.attach(S, None, None)
    return e0.elapsed_time(e1) / n


def experiment(train_amplitudes=(1.5, 2.0, 2.5), train_seeds=(1, 2), val=(2.0, 33), test=(2.0, 77), iters=1500,
               chunk=100, lr=3e-5, sprints=1, log=print):
    """Train on fine runs of the given bubble amplitudes and noise seeds; after every `chunk`
    iterations the coarse run of a validation case is scored (mean relative theta' error over its
    snapshots) and the best weights are kept; they are then evaluated on a held-out test case."""
    t0 = time.time()
    series = [fine_truth(a, s) for a in train_amplitudes for s in train_seeds]
    val_snaps = fine_truth(*val)
    held = fine_truth(*test)
    scale = field_scale([x for s in series for x in s])
    S = coarse_solver()
    base_val = theta_error(S, val_snaps)
    base = theta_error(S, held)
    net = sgs_cnn.SGSNet(seed=0)
    best = (float(np.mean(base_val)), None, 0)
    curve = []
    for c in range(max(1, iters // chunk)):
        hist = train(S, net, series, scale, iters=chunk, lr=lr, sprints=sprints, seed=c)
        v = float(np.mean(theta_error(S, val_snaps, net, scale)))
        curve.append({"iters": (c + 1) * chunk, "loss": float(np.mean(hist)), "val_theta_err": v})
        if log:
            log("iters %d  mean loss %.4g  validation theta' error %.4f (Smagorinsky %.4f)"
                % ((c + 1) * chunk, np.mean(hist), v, np.mean(base_val)))
        if v < best[0]:
            best = (v, net.state_dict(), (c + 1) * chunk)
    if best[1] is not None:
        net.load_state_dict(best[1])
    learned = theta_error(S, held, net, scale) if best[1] is not None else list(base)
    cost_plain = step_cost(S, held[0])
    cost_learned = step_cost(S, held[0], net, scale)
    S.close()
    return {"theta_err_smagorinsky": base, "theta_err_learned": learned, "best_iters": best[2],
            "val_theta_err_smagorinsky": float(np.mean(base_val)), "val_theta_err_learned": best[0], "curve": curve,
            "ms_per_step_plain": cost_plain, "ms_per_step_learned": cost_learned,
            "cost_ratio": cost_learned / cost_plain, "lr": lr, "sprints": sprints, "seconds": time.time() - t0,
            "net": net, "scale": scale}


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="train and evaluate the learned SGS correction (warm bubble, "
                                             "100 m fine runs coarse-grained to 600 m x 600 m x 300 m)")
    ap.add_argument("--iters", type=int, default=1500)
    ap.add_argument("--chunk", type=int, default=100)
    ap.add_argument("--lr", type=float, default=3e-5)
    ap.add_argument("--sprints", type=int, default=1)
    ap.add_argument("--out", default=None, help="JSON summary; the weights go beside it (.pt)")
    a = ap.parse_args(argv)
    r = experiment(iters=a.iters, chunk=a.chunk, lr=a.lr, sprints=a.sprints)
    net, scale = r.pop("net"), r.pop("scale")
    line = json.dumps(r)
    print(line)
    if a.out:
        with open(a.out, "w") as f:
            f.write(line + "\n")
        torch.save({"net": net.state_dict(), "scale": {k: v.cpu() for k, v in scale.items()}},
                   a.out.rsplit(".", 1)[0] + ".pt")


if __name__ == "__main__":
    main()
