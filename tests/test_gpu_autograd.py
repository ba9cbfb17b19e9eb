"""torch.autograd through a rollout of big steps (lex_gb300.autograd) against central finite
differences of the FP64 oracle: <dL/dx0, v> == (L(x0 + eps v) - L(x0 - eps v)) / 2 eps for
L = <ybar, x_N>, to 1e-4 relative to ||ybar|| ||J v||."""
import numpy as np
import pytest

from conftest import load_golden
from test_gpu_parity import FIELDS
from test_gpu_adjoint import _direction, _interior, _pad

pytestmark = pytest.mark.gpu
NSTEPS = 2


def _to_dev(a):
    import torch
    return torch.tensor(np.ascontiguousarray(np.asarray(a, np.float32).transpose(2, 1, 0)), device="cuda")


def _from_dev(t):
    return t.detach().cpu().numpy().astype(np.float64).transpose(2, 1, 0)


def test_rollout_gradient_matches_oracle_finite_differences(built_lib):
    torch = pytest.importorskip("torch")
    from oracle.ic import Grid
    from oracle.dycore import Dycore
    from lex_gb300.solver import Solver
    from lex_gb300 import autograd as lag
    g = load_golden("ops_random.npz")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    base = dict(theta0=g["col_theta0"], qv0=g["col_qv0"], pi0=g["col_pi0"], rho0=g["col_rho0"])
    D = Dycore(Grid(nx, ny, nz, float(g["dx"]), float(g["dy"]), float(g["dz"])), base, float(g["dt"]),
               int(g["n_sound"]), turb=True)
    x0 = tuple(g["in_" + f] for f in FIELDS)

    def forward(x):
        for _ in range(NSTEPS):
            x = D.step(x)[0]
        return x

    with Solver(nx, ny, nz, float(g["dx"]), float(g["dy"]), float(g["dz"]), float(g["dt"]), int(g["n_sound"]),
                turb_opt=1) as S:
        S.set_base_columns(g["col_theta0"], g["col_qv0"], g["col_pi0"], g["col_rho0"])
        xi = _interior(x0, nx, ny)
        state = tuple(_to_dev(a).requires_grad_(True) for a in xi)
        out = lag.rollout(S, state, NSTEPS)
        rng = np.random.default_rng(3)
        yb = _direction(rng, nx, ny, nz)
        loss = sum((o * _to_dev(y)).sum() for o, y in zip(out, yb))
        loss.backward()
        grads = [_from_dev(t.grad) for t in state]
        # the forward of the autograd path equals the oracle rollout to the FP32 level: theta is
        # carried in K, so its floor is the FP32 spacing of ~300 K values
        ref = _interior(forward(x0), nx, ny)
        for f, a, r, r0 in zip(FIELDS, out, ref, xi):
            got = _from_dev(a)
            floor = 2.4e-7 * np.linalg.norm(r)
            assert np.linalg.norm(got - r) <= 1e-5 * np.linalg.norm(r - r0) + floor, f
    v = _direction(rng, nx, ny, nz)
    eps = 1e-3
    vp = _pad(v)
    fp = _interior(forward(tuple(a + eps * b for a, b in zip(x0, vp))), nx, ny)
    fm = _interior(forward(tuple(a - eps * b for a, b in zip(x0, vp))), nx, ny)
    jv = [(a - b) / (2 * eps) for a, b in zip(fp, fm)]
    lhs = sum(float(np.sum(a * b)) for a, b in zip(yb, jv))
    rhs = sum(float(np.sum(a * b)) for a, b in zip(grads, v))
    scale = np.sqrt(sum(float(np.sum(a * a)) for a in yb)) * np.sqrt(sum(float(np.sum(a * a)) for a in jv))
    assert abs(lhs - rhs) <= 1e-4 * scale, (lhs, rhs)


def test_rollout_gradient_with_respect_to_cs(built_lib):
    """d<ybar, x_N>/dCs through torch.autograd (the library's accumulation over each step's eddy
    viscosity) against a central difference of the FP64 oracle in Cs, eps = 1e-3."""
    torch = pytest.importorskip("torch")
    from oracle.ic import Grid
    from oracle.dycore import Dycore
    from lex_gb300.solver import Solver
    from lex_gb300 import autograd as lag
    g = load_golden("ops_random.npz")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    base = dict(theta0=g["col_theta0"], qv0=g["col_qv0"], pi0=g["col_pi0"], rho0=g["col_rho0"])
    grid = Grid(nx, ny, nz, float(g["dx"]), float(g["dy"]), float(g["dz"]))
    x0 = tuple(g["in_" + f] for f in FIELDS)
    cs0 = 0.18

    def forward(cs):
        D = Dycore(grid, base, float(g["dt"]), int(g["n_sound"]), turb=True, cs=cs)
        x = x0
        for _ in range(NSTEPS):
            x = D.step(x)[0]
        return _interior(x, nx, ny)

    rng = np.random.default_rng(11)
    yb = _direction(rng, nx, ny, nz)
    with Solver(nx, ny, nz, float(g["dx"]), float(g["dy"]), float(g["dz"]), float(g["dt"]), int(g["n_sound"]),
                turb_opt=1) as S:
        S.set_base_columns(g["col_theta0"], g["col_qv0"], g["col_pi0"], g["col_rho0"])
        state = tuple(_to_dev(a) for a in _interior(x0, nx, ny))
        cs = torch.tensor(cs0, dtype=torch.float64, device="cuda", requires_grad=True)
        out = lag.rollout(S, state, NSTEPS, cs=cs)
        loss = sum((o * _to_dev(y)).sum() for o, y in zip(out, yb))
        loss.backward()
        got = float(cs.grad)
    eps = 1e-3
    jv = [(a - b) / (2 * eps) for a, b in zip(forward(cs0 + eps), forward(cs0 - eps))]
    lhs = sum(float(np.sum(a * b)) for a, b in zip(yb, jv))
    scale = np.sqrt(sum(float(np.sum(a * a)) for a in yb)) * np.sqrt(sum(float(np.sum(a * a)) for a in jv))
    assert abs(lhs) > 1e-3 * scale                     # Cs matters in this case
    assert abs(lhs - got) <= 1e-4 * scale, (lhs, got, scale)


def test_backward_uses_the_cs_of_its_forward(built_lib):
    """A step's backward differentiates the step with the Cs its forward used, even when the solver's
    Cs is changed before backward (the forward's Cs is recorded and restored around the reverse pass)."""
    torch = pytest.importorskip("torch")
    from lex_gb300.solver import Solver
    from lex_gb300 import autograd as lag
    g = load_golden("ops_random.npz")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    x0 = tuple(g["in_" + f] for f in FIELDS)
    yb = _direction(np.random.default_rng(5), nx, ny, nz)
    grads = []
    with Solver(nx, ny, nz, float(g["dx"]), float(g["dy"]), float(g["dz"]), float(g["dt"]), int(g["n_sound"]),
                turb_opt=1) as S:
        S.set_base_columns(g["col_theta0"], g["col_qv0"], g["col_pi0"], g["col_rho0"])
        for change in (False, True):
            S.set_cs(0.18)
            state = tuple(_to_dev(a).requires_grad_(True) for a in _interior(x0, nx, ny))
            out = lag.rollout(S, state, 2)
            if change:
                S.set_cs(0.3)
            loss = sum((o * _to_dev(y)).sum() for o, y in zip(out, yb))
            loss.backward()
            grads.append([_from_dev(t.grad) for t in state])
            assert S.cs == (0.3 if change else 0.18)      # restored after the reverse pass
    for a, b in zip(*grads):
        np.testing.assert_array_equal(a, b)
