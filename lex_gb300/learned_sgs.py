"""Learned SGS correction: training data, training through the differentiable solver, evaluation.

Training data (the role of dataset_generation.py:12-194, which reads pre-built benchmark
sequences): the library's own 100 m warm-bubble runs are coarse-grained onto the 600 m x 600 m x
300 m grid (factors 6, 6, 3) every `every` seconds -
    theta, pi', qv : box means over the fine cells of a coarse cell
    u (v)          : means over the fine faces that make up a coarse x (y) face
    w              : means over the fine faces that make up a coarse z face
and, for the a-priori stage, also one coarse step (3 s) later.  Two training stages:
  a priori   the network maps the coarse model's step of a coarse-grained state to the residual
             (coarse-grained truth one step later minus that step), Adam on batches of states;
  through the solver (lex_dl_train.py:49-131)  from a coarse-grained state, sprints of coarse
             steps with the correction after each step (one_sprint_functions.py:128-163) are
             compared with the coarse-grained truth at the sprints' ends; the loss is the sum over
             theta, u, v, w, qv of the squared error over each field's range (its Laplacian and
             negative-qv terms are options).  Gradients flow through the solver
             (lex_gb300.autograd, step-level checkpointing) and the CNN (lex_gb300.sgs_cnn); the
             weights with the best validation score are kept.
Evaluation: coarse runs with and without the correction against the coarse-grained fine run,
relative L2 error of theta' = theta - 300 K, and the cost of a corrected step.
"""
import time

import numpy as np
import torch

from . import autograd as lag
from . import sgs_cnn
from .solver import Solver
from .workload import random_bubbles, warm_bubble, warm_bubbles

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


def fine_run(bubbles, seed, t_end=600.0, every=30.0, fine=(192, 192, 96), spacing=(100., 100., 100.), dt=1.0,
             f=FACTORS, pair_steps=0):
    """Coarse-grained snapshots (t = 0, every, ..., t_end) of a fine run of the given bubbles
    ((amplitude, radius, x centre, y centre) each); with pair_steps > 0 also the coarse-grained
    state pair_steps fine steps after each snapshot but the last -> (snaps, nexts)."""
    nx, ny, nz = fine
    phys, prof = warm_bubbles(nx, ny, nz, *spacing, bubbles, seed=seed)
    S = Solver(nx, ny, nz, *spacing, dt, 32, turb_opt=1)
    S.integrate_base_state(prof["theta0"], prof["qv0"])
    S.upload(phys, dtype=np.float32)
    per = int(round(every / dt))
    snaps, nexts = [coarse_grain(lag.get_state(S), f)], []
    for _ in range(int(round(t_end / every))):
        if pair_steps:
            S.step(pair_steps)
            nexts.append(coarse_grain(lag.get_state(S), f))
            S.step(per - pair_steps)
        else:
            S.step(per)
        snaps.append(coarse_grain(lag.get_state(S), f))
    torch.cuda.synchronize()
    S.close()
    return (snaps, nexts) if pair_steps else snaps


def fine_truth(amplitude=2.0, seed=2025, t_end=600.0, every=30.0, fine=(192, 192, 96), spacing=(100., 100., 100.),
               dt=1.0, f=FACTORS, radius_h=2000.0):
    """Coarse-grained snapshots of a fine run of one bubble at mid-domain."""
    bub = [(amplitude, radius_h, 0.5 * fine[0] * spacing[0], 0.5 * fine[1] * spacing[1])]
    return fine_run(bub, seed, t_end, every, fine, spacing, dt, f)


def coarse_solver(dims=(32, 32, 32), spacing=(600., 600., 300.), dt=3.0):
    nx, ny, nz = dims
    _, prof = warm_bubble(nx, ny, nz, *spacing)
    S = Solver(nx, ny, nz, *spacing, dt, 32, turb_opt=1)
    S.integrate_base_state(prof["theta0"], prof["qv0"])
    return S


def laplacian(a, spacing):
    """7-point Laplacian of a cell field [nz][ny][nx] as the training loss computes it
    (laplace_of_tensor_jnp, dataset_generation.py:320-347): periodic in x and y, the end levels
    copied in z (zero gradient through the bottom and the lid), and no vertical term in the first
    and last x columns - the reference zeroes s_z[:, :, 0] and s_z[:, :, -1] of its
    [sequence][step][x][y][z] arrays (:334-335), whose third index is x."""
    dx, dy, dz = spacing
    lx = (torch.roll(a, -1, 2) - 2.0 * a + torch.roll(a, 1, 2)) / (dx * dx)
    ly = (torch.roll(a, -1, 1) - 2.0 * a + torch.roll(a, 1, 1)) / (dy * dy)
    z = torch.zeros_like(a[:1])
    gz = torch.cat([z, (a[1:] - a[:-1]) / dz, z], 0)
    keep = torch.ones(a.shape[2], dtype=a.dtype, device=a.device)
    keep[0] = 0.0
    keep[-1] = 0.0
    return lx + ly + (gz[1:] - gz[:-1]) / dz * keep


def field_scale(snapshots, spacing=None):
    """Per-level ranges of the training snapshots (the scaling_params of the reference); with
    `spacing`, also the ranges of the theta and qv Laplacians (+1e-7, +1e-10) for the Laplacian
    loss terms."""
    sc = sgs_cnn.make_scale(snapshots)
    if spacing is not None:
        la = []
        for i, margin in ((0, 1.0e-7), (5, 1.0e-10)):
            vals = [laplacian(s[i], spacing) for s in snapshots]
            la.append(float(max(float(v.max()) for v in vals) - min(float(v.min()) for v in vals)) + margin)
        sc["la"] = la
    return sc


def sprint(S, state, nsteps, net=None, scale=None, grad=True):
    """nsteps coarse steps, each followed by the CNN correction when net is given."""
    dims = (S.nx, S.ny, S.nz)
    with torch.set_grad_enabled(grad):
        for _ in range(nsteps):
            state = lag.step(S, state)
            if net is not None:
                state = sgs_cnn.correct(net, state, scale, dims)
    return state


def loss_fn(state, truth, scale, spacing=None, laplacian_terms=False, neg_qv=False):
    """Sum over theta, u, v, w, qv of the squared error, each field divided by its largest
    per-level input range (the normalised L2 loss of lex_dl_train.py:49-99).  Options from the
    same loss: laplacian_terms adds the squared errors of the theta and qv Laplacians over their
    ranges (needs `spacing` and a scale from field_scale(..., spacing)); neg_qv adds the
    negative part of qv over its range (lex_dl_train.py:92-97)."""
    total = 0.0
    for f, i in enumerate((0, 1, 2, 3, 5)):
        r = scale["rin"][f].max()
        total = total + ((state[i] - truth[i]) / r).pow(2).sum()
    if laplacian_terms:
        for k, i in enumerate((0, 5)):
            d = laplacian(state[i], spacing) - laplacian(truth[i], spacing)
            total = total + (d / scale["la"][k]).pow(2).sum()
    if neg_qv:
        total = total + torch.relu(-state[5]).sum() / scale["rin"][4].max()
    return total


def train(S, net, series, scale, steps_per_sprint=10, iters=200, lr=1e-4, warmup=50, sprints=1, seed=0, log=None,
          laplacian_terms=False, neg_qv=False):
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
            loss = loss + loss_fn(state, s[k + j], scale, (S.cfg.dx, S.cfg.dy, S.cfg.dz), laplacian_terms, neg_qv)
        grads = torch.autograd.grad(loss, net.params())
        n = net.step_count + 1
        sgs_cnn.adam_step(net, [g.detach() for g in grads], lr=lr * min(1.0, n / max(1, warmup)))
        hist.append(float(loss.detach()))
        if log and (it % 20 == 0 or it == iters - 1):
            log("iter %d loss %.4g" % (it, hist[-1]))
    return hist


def residual_pairs(S, snaps, nexts, steps=1):
    """(state after `steps` plain coarse steps from a coarse-grained snapshot, residual = the
    coarse-grained truth at that time minus that state) for each snapshot with a successor."""
    out = []
    sgs_cnn.attach(S, None, None)
    for x, y in zip(snaps, nexts):
        lag.set_state(S, tuple(a.detach() for a in x))
        S.step(steps)
        m = lag.get_state(S)
        out.append((m, tuple(b - a for a, b in zip(m, y))))
    return out


def pretrain(net, pairs, scale, dims, iters=500, lr=1e-3, batch=8, warmup=50, seed=0, log=None):
    """A-priori stage: Adam on batches of `batch` pairs; the loss is the squared error between the
    unpacked correction of the stepped state and the residual, each field over its largest
    per-level range (pi' excluded: it is not corrected)."""
    rng = np.random.default_rng(seed)
    for t in net.params():
        t.requires_grad_(True)
    rmax = [float(scale["rin"][f].max()) for f in range(5)]
    hist = []
    for it in range(iters):
        loss = 0.0
        for k in rng.integers(len(pairs), size=batch):
            m, r = pairs[k]
            d = sgs_cnn.unpack(sgs_cnn.net_apply(net, sgs_cnn.pack(m, scale), dims), scale, dims)
            for f, i in enumerate((0, 1, 2, 3, 5)):
                loss = loss + ((d[i] - r[i]) / rmax[f]).pow(2).sum() / batch
        grads = torch.autograd.grad(loss, net.params())
        n = net.step_count + 1
        sgs_cnn.adam_step(net, [g.detach() for g in grads], lr=lr * min(1.0, n / max(1, warmup)))
        hist.append(float(loss.detach()))
        if log and (it % 50 == 0 or it == iters - 1):
            log("a priori iter %d loss %.4g" % (it, hist[-1]))
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


def _select(S, net, series, val, scale, iters, chunk, lr, sprints, log, tag, loss_opts=None):
    """Training through the solver in chunks, scored on the validation case after each chunk.
    Candidates: no correction (Smagorinsky alone, the fallback), the starting weights and every
    chunk; the network is left with the best weights, and `use` is False when no correction
    scored best."""
    base = float(np.mean(theta_error(S, val)))
    best = (base, None, -1)
    v0 = float(np.mean(theta_error(S, val, net, scale)))
    if v0 < best[0]:
        best = (v0, net.state_dict(), 0)
    curve = [{"iters": 0, "val_theta_err": v0}]
    for c in range(max(1, iters // chunk)):
        hist = train(S, net, series, scale, iters=chunk, lr=lr, sprints=sprints, seed=1000 + c, **(loss_opts or {}))
        v = float(np.mean(theta_error(S, val, net, scale)))
        curve.append({"iters": (c + 1) * chunk, "loss": float(np.mean(hist)), "val_theta_err": v})
        if log:
            log("%s iters %d  mean loss %.4g  validation theta' error %.4f (Smagorinsky %.4f)"
                % (tag, (c + 1) * chunk, np.mean(hist), v, base))
        if v == v and v < best[0]:
            best = (v, net.state_dict(), (c + 1) * chunk)
    if best[1] is not None:
        net.load_state_dict(best[1])
    return {"val_theta_err_smagorinsky": base, "val_theta_err_learned": best[0], "best_iters": best[2],
            "use": best[1] is not None, "curve": curve}


def experiment(n_train=8, iters_prior=300, iters=600, chunk=100, lr_prior=1e-3, lr=3e-5, sprints=2, log=print,
               laplacian_terms=False, neg_qv=False):
    """The 32^3 case: 100 m runs of one mid-domain bubble with amplitude U(1, 3) K and horizontal
    radius U(1.5, 3) km (seeded), coarse-grained 6 x 6 x 3.  An a-priori stage on one-step
    residuals, then training through the solver (`sprints` x 10-step unrolls) from the a-priori
    weights and, separately, from an untrained network (last layer zero: no correction); the
    branch and iteration with the best validation score are kept and evaluated on a held-out run
    against Smagorinsky alone."""
    t0 = time.time()
    L = (19200.0, 19200.0)
    bub = lambda seed: random_bubbles(seed, 1, *L, centred=True)
    runs = [fine_run(bub(100 + i), 100 + i, pair_steps=3) for i in range(n_train)]
    series = [r[0] for r in runs]
    val = fine_run(bub(200), 200)
    held = fine_run(bub(300), 300)
    scale = field_scale([x for s in series for x in s], spacing=(600.0, 600.0, 300.0))
    opts = {"laplacian_terms": laplacian_terms, "neg_qv": neg_qv}
    S = coarse_solver()
    dims = (S.nx, S.ny, S.nz)
    base = theta_error(S, held)
    pairs = [p for sn, nx_ in runs for p in residual_pairs(S, sn[:-1], nx_)]
    prior_net = sgs_cnn.SGSNet(seed=0)
    hp = pretrain(prior_net, pairs, scale, dims, iters=iters_prior, lr=lr_prior, log=log)
    prior = theta_error(S, held, prior_net, scale)
    sel_prior = _select(S, prior_net, series, val, scale, iters, chunk, lr, sprints, log, "from a-priori", opts)
    scratch_net = sgs_cnn.SGSNet(seed=0)
    sel_scratch = _select(S, scratch_net, series, val, scale, iters, chunk, lr, sprints, log, "from scratch", opts)
    if sel_prior["val_theta_err_learned"] <= sel_scratch["val_theta_err_learned"]:
        net, sel, branch = prior_net, sel_prior, "a-priori weights"
    else:
        net, sel, branch = scratch_net, sel_scratch, "untrained network"
    if not sel["use"]:
        branch = "no correction (Smagorinsky scored best on validation)"
    learned = theta_error(S, held, net, scale) if sel["use"] else list(base)
    cost_plain = step_cost(S, held[0])
    cost_learned = step_cost(S, held[0], net, scale)
    S.close()
    return {"case": "32^3 at 600 x 600 x 300 m, 600 s; held-out bubble %s" % [tuple(round(v, 3) for v in b)
                                                                              for b in bub(300)],
            "theta_err_smagorinsky": base, "theta_err_a_priori": prior, "theta_err_learned": learned,
            "a_priori_loss_first_last": [hp[0], float(np.mean(hp[-20:]))], "chosen": branch,
            "through_solver_from_a_priori": sel_prior, "through_solver_from_scratch": sel_scratch,
            "ms_per_step_plain": cost_plain, "ms_per_step_learned": cost_learned,
            "cost_ratio": cost_learned / cost_plain, "seconds": time.time() - t0, "net": net, "scale": scale}


def experiment_large(net_state=None, iters=300, chunk=50, lr=3e-5, sprints=2, t_end=1800.0, fine_dt=0.5, log=print,
                     laplacian_terms=False, neg_qv=False):
    """The 128 x 128 x 64 case (76.8 x 76.8 x 19.2 km at 600 x 600 x 300 m, dt 3 s): four
    non-overlapping bubbles with amplitude U(1, 3) K, radius U(1.5, 3) km; 100 m runs (768 x 768 x
    192, dt `fine_dt`) coarse-grained; the network (from `net_state`, else untrained: last layer
    zero) is trained through the solver with `sprints` x 10-step unrolls on one run, selected on a
    second (Smagorinsky alone is a candidate), evaluated on a third over t_end against Smagorinsky
    alone; the cost of a corrected step against a plain one."""
    t0 = time.time()
    L = (76800.0, 76800.0)
    fine, dims = (768, 768, 192), (128, 128, 64)
    # 100 m runs at dt 0.5 s: at dt 1 s a 3 K bubble's 100 m run goes non-finite after about
    # 870 s, once its updraft passes 40 m/s (the 600 m coarse runs stay finite at dt 3 s)
    run = lambda seed: fine_run(random_bubbles(seed, 4, *L), seed, t_end=t_end, fine=fine, dt=fine_dt)
    train_s, val, held = run(400), run(450), run(500)
    if log:
        log("fine runs done (%.0f s)" % (time.time() - t0))
    scale = field_scale(train_s, spacing=(600.0, 600.0, 300.0))
    S = coarse_solver(dims=dims)
    base = theta_error(S, held)
    net = sgs_cnn.SGSNet(seed=0)
    if net_state is not None:
        net.load_state_dict(net_state)
    start = theta_error(S, held, net, scale)
    sel = _select(S, net, [train_s], val, scale, iters, chunk, lr, sprints, log, "128x128x64",
                  {"laplacian_terms": laplacian_terms, "neg_qv": neg_qv})
    learned = theta_error(S, held, net, scale) if sel["use"] else list(base)
    cost_plain = step_cost(S, held[0])
    cost_learned = step_cost(S, held[0], net, scale)
    S.close()
    return {"case": "128x128x64 at 600 x 600 x 300 m, %g s; test bubbles %s" % (
                t_end, [tuple(round(v, 3) for v in b) for b in random_bubbles(500, 4, *L)]),
            "theta_err_smagorinsky": base, "theta_err_start": start, "theta_err_learned": learned, **sel,
            "ms_per_step_plain": cost_plain, "ms_per_step_learned": cost_learned,
            "cost_ratio": cost_learned / cost_plain, "seconds": time.time() - t0, "net": net, "scale": scale}


def _host(scale):
    """A scale dict with its tensors on the host (the Laplacian ranges are plain floats)."""
    return {k: (v.cpu() if torch.is_tensor(v) else v) for k, v in scale.items()}


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="train and evaluate the learned SGS correction (warm bubbles, "
                                             "100 m runs coarse-grained to 600 m x 600 m x 300 m)")
    ap.add_argument("--case", choices=["32", "128", "both"], default="32",
                    help="32: 32^3 single-bubble runs; 128: 128x128x64 four-bubble runs; both: 32 then 128 "
                         "starting from the 32^3 network")
    ap.add_argument("--iters-prior", type=int, default=300)
    ap.add_argument("--iters", type=int, default=600)
    ap.add_argument("--iters-large", type=int, default=300)
    ap.add_argument("--lr", type=float, default=3e-5)
    ap.add_argument("--sprints", type=int, default=2)
    ap.add_argument("--laplacian", action="store_true", help="add the theta / qv Laplacian loss terms")
    ap.add_argument("--neg-qv", action="store_true", help="add the negative-qv loss term")
    ap.add_argument("--init", default=None, help="start the 128 case from the 32^3 network of a previous --out .pt")
    ap.add_argument("--out", default=None, help="JSON summary (one line per case); weights beside it (.pt)")
    a = ap.parse_args(argv)
    lines, nets = [], {}
    state = torch.load(a.init)["32"]["net"] if a.init else None
    if a.case in ("32", "both"):
        r = experiment(iters_prior=a.iters_prior, iters=a.iters, lr=a.lr, sprints=a.sprints,
                       laplacian_terms=a.laplacian, neg_qv=a.neg_qv)
        net, scale = r.pop("net"), r.pop("scale")
        state = net.state_dict()
        nets["32"] = {"net": state, "scale": _host(scale)}
        lines.append(json.dumps(r))
        print(lines[-1], flush=True)
    if a.case in ("128", "both"):
        r = experiment_large(net_state=state, iters=a.iters_large, lr=a.lr, sprints=a.sprints,
                             laplacian_terms=a.laplacian, neg_qv=a.neg_qv)
        net, scale = r.pop("net"), r.pop("scale")
        nets["128"] = {"net": net.state_dict(), "scale": _host(scale)}
        lines.append(json.dumps(r))
        print(lines[-1], flush=True)
    if a.out:
        with open(a.out, "w") as f:
            f.write("\n".join(lines) + "\n")
        torch.save(nets, a.out.rsplit(".", 1)[0] + ".pt")


if __name__ == "__main__":
    main()
