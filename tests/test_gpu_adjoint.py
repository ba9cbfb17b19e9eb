"""Reverse mode of the big step (lexgb_step_vjp) against central finite differences of the FP64
oracle: for random directions v and adjoint seeds ybar,

    <ybar, J v>  (oracle, FP64, (F(x + eps v) - F(x - eps v)) / 2 eps)
    <J^T ybar, v> (GPU reverse mode, FP32)

must agree to 1e-4 relative to ||ybar|| ||J v||.  Seeds restricted to single output fields
check the paths one at a time (theta/qv update, acoustic winds, pi')."""
import json
import os

import numpy as np
import pytest

from conftest import load_golden, report_path
from test_gpu_parity import FIELDS

pytestmark = pytest.mark.gpu

TOL = 1e-4
REPORT = {}


@pytest.fixture(scope="module", autouse=True)
def report():
    yield
    with open(report_path("adjoint_report.json"), "w") as f:
        json.dump(REPORT, f, indent=1, sort_keys=True)


def _setup(nstages, turb=0, cor=0):
    from oracle.ic import Grid
    from oracle.dycore import Dycore
    from lex_gb300.solver import Solver
    g = load_golden("ops_random.npz")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    base = dict(theta0=g["col_theta0"], qv0=g["col_qv0"], pi0=g["col_pi0"], rho0=g["col_rho0"])
    D = Dycore(Grid(nx, ny, nz, float(g["dx"]), float(g["dy"]), float(g["dz"])), base, float(g["dt"]),
               int(g["n_sound"]), turb=bool(turb), cor_opt=cor)
    S = Solver(nx, ny, nz, float(g["dx"]), float(g["dy"]), float(g["dz"]), float(g["dt"]), int(g["n_sound"]),
               turb_opt=turb, cor_opt=cor)
    S.set_base_columns(g["col_theta0"], g["col_qv0"], g["col_pi0"], g["col_rho0"])
    x0 = tuple(g["in_" + f] for f in FIELDS)
    S.upload(x0)

    def forward(x):
        if nstages == 3:
            return D.step(x)[0]
        xs = x
        sgs = D.smagorinsky(x[0], x[1], x[2], x[3], x[5]) if turb else None
        for s, (dts, n) in enumerate(D.stage_plan()[:nstages]):
            xs, _ = D.stage(x, xs, dts, sgs, n)
        return xs
    return g, D, S, x0, forward


def _pad(v):
    from oracle.ic import pad_scalar, pad_u, pad_v
    T, u, v_, w, p, q = v
    return (pad_scalar(T), pad_u(np.concatenate([u, u[:1]], 0)), pad_v(np.concatenate([v_, v_[:, :1]], 1)),
            pad_scalar(w), pad_scalar(p), pad_scalar(q))


def _interior(x, nx, ny):
    T, u, v, w, p, q = x
    c = (slice(3, -3), slice(3, -3), slice(1, -1))
    return (T[c], u[3:3 + nx, 3:-3, 1:-1], v[3:-3, 3:3 + ny, 1:-1], w[c], p[c], q[c])


def _direction(rng, nx, ny, nz):
    w = rng.standard_normal((nx, ny, nz + 1)) * 0.5
    w[:, :, 0] = 0.0
    w[:, :, -1] = 0.0
    return (rng.standard_normal((nx, ny, nz)) * 0.3, rng.standard_normal((nx, ny, nz)), rng.standard_normal((nx, ny, nz)),
            w, rng.standard_normal((nx, ny, nz)) * 1e-4, rng.standard_normal((nx, ny, nz)) * 1e-4)


CASES = [(1, None, 0, 0), (1, "theta", 0, 0), (1, "pip", 0, 0), (1, "u", 0, 0), (1, "w", 0, 0), (3, None, 0, 0),
         (1, None, 1, 0), (1, "theta", 1, 0), (1, "u", 1, 0), (1, "w", 1, 0), (3, None, 1, 0),
         (3, None, 1, 1), (3, "v", 1, 2)]


@pytest.mark.parametrize("nstages,only,turb,cor", CASES,
                         ids=["%s%s%s%s" % ("step" if n == 3 else "stage0", "_" + o if o else "", "_smag" if t else "",
                                            "_cor%d" % c if c else "") for n, o, t, c in CASES])
def test_reverse_mode_matches_oracle_finite_differences(built_lib, nstages, only, turb, cor):
    g, D, S, x0, forward = _setup(nstages, turb, cor)
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    rng = np.random.default_rng(7)
    errs = []
    for trial in range(3):
        v = _direction(rng, nx, ny, nz)
        yb = _direction(rng, nx, ny, nz)
        if only is not None:
            yb = tuple(a if f == only else np.zeros_like(a) for f, a in zip(FIELDS, yb))
        eps = 1e-3
        vp = _pad(v)
        xp = tuple(a + eps * b for a, b in zip(x0, vp))
        xm = tuple(a - eps * b for a, b in zip(x0, vp))
        jv = [(a - b) / (2 * eps) for a, b in zip(_interior(forward(xp), nx, ny), _interior(forward(xm), nx, ny))]
        lhs = sum(float(np.sum(a * b)) for a, b in zip(yb, jv))
        xb = S.step_vjp(yb, nstages=nstages)
        rhs = sum(float(np.sum(np.asarray(a, np.float64) * b)) for a, b in zip(xb, v))
        scale = np.sqrt(sum(float(np.sum(a * a)) for a in yb)) * np.sqrt(sum(float(np.sum(a * a)) for a in jv))
        errs.append((lhs, rhs, abs(lhs - rhs) / scale))
    S.close()
    REPORT["%d_%s_%d_cor%d" % (nstages, only, turb, cor)] = errs
    assert all(e[2] <= TOL for e in errs), errs


def test_kept_step_reverse_equals_recomputed_reverse(built_lib):
    """lexgb_step_keep + lexgb_step_vjp_kept (intermediates from the forward) gives the same adjoint
    as lexgb_step_vjp (recomputed), and the kept forward advances the state like lexgb_step."""
    import ctypes
    from lex_gb300 import _lib
    g, D, S, x0, forward = _setup(3, 1)
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    rng = np.random.default_rng(11)
    yb = _direction(rng, nx, ny, nz)
    ref = S.step_vjp(yb, nstages=3)
    S.step(1)
    stepped = S.download()
    S.upload(x0)
    _lib.check(S.lib.lexgb_step_keep(S.handle))
    kept_state = S.download()
    dev = [np.ascontiguousarray(np.asarray(a, np.float32).transpose(2, 1, 0)) for a in yb]
    out = [np.empty_like(a) for a in dev]
    _lib.check(S.lib.lexgb_step_vjp_kept(S.handle, (ctypes.c_void_p * 6)(*[a.ctypes.data for a in dev]),
                                         (ctypes.c_void_p * 6)(*[a.ctypes.data for a in out]), 0))
    S.close()
    for a, b in zip(kept_state, stepped):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(out, ref):
        np.testing.assert_array_equal(a.transpose(2, 1, 0), b)


@pytest.mark.parametrize("cor,nsteps", [(0, 1), (0, 3), (1, 1), (1, 3)],
                         ids=["step", "rollout3", "step_coriolis", "rollout3_coriolis"])
def test_reverse_mode_matches_reference_autograd(built_lib, cor, nsteps):
    """The library's reverse mode against the reference's own: torch.autograd through the reference's
    unmodified ws_rk3_big_step (one_sprint_functions.py:10-30) under the torch stand-in for jax, FP64,
    Smagorinsky on (tests/golden/adjoint_vjp.npz, the stand-in for jax.vjp of the reference step).
    One big step and a three-step rollout through lex_gb300.autograd (step-level checkpointing), with
    and without Coriolis.  Bar, per field (relative L2 against the FP64 adjoint; w on faces 1..nz-1,
    which are the state's free values): within 1e-5, or no further from it than the reference's own
    reverse mode run in FP32 is (stored in the fixture), whichever is larger."""
    import torch
    from lex_gb300 import autograd as lag
    from lex_gb300.solver import Solver
    g = load_golden("adjoint_vjp.npz")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    S = Solver(nx, ny, nz, float(g["dx"]), float(g["dy"]), float(g["dz"]), float(g["dt"]), int(g["n_sound"]),
               turb_opt=1, cor_opt=cor, f_cor=float(g["f_cor"]))
    S.set_base_columns(g["col_theta0"], g["col_qv0"], g["col_pi0"], g["col_rho0"])
    x = [torch.tensor(g["x_" + f], dtype=torch.float32, device="cuda").requires_grad_(True) for f in FIELDS]
    y = lag.rollout(S, tuple(x), nsteps)
    yb = [torch.tensor(g["ybar_" + f], dtype=torch.float32, device="cuda") for f in FIELDS]
    gx = torch.autograd.grad(y, x, yb)
    S.close()
    errs, bars = {}, {}
    for f, a in zip(FIELDS, gx):
        ref = g["cor%d_n%d_xbar_%s" % (cor, nsteps, f)]
        got = a.double().cpu().numpy()
        if f == "w":
            ref, got = ref[1:-1], got[1:-1]
        errs[f] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        bars[f] = max(1e-5, float(g["cor%d_n%d_fp32err_%s" % (cor, nsteps, f)]))
    REPORT["reference_autograd_cor%d_n%d" % (cor, nsteps)] = {"err": errs, "bar": bars}
    assert all(errs[f] <= bars[f] for f in FIELDS), (errs, bars)
