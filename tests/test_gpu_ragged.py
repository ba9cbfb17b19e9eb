"""Parity on ragged grids: sizes that leave the kernels' tiles partly outside the grid.

The golden vectors use 16x12x8, 16x16x12 and 32^3 grids.  These cases add nx not a multiple of
4 (the kernels' scalar staging paths), nx not a multiple of the 32-wide tiles, ny smaller than
a tile's halo reach, and nz = 1 and 2 (mod 4), where the last vertical tile holds one or two
levels and the one-sided top extrapolations reach below the tile.  8 x 5 x 7 and the smallest
grid the library accepts, 4 x 4 x 6, put a 32 x 8 tile and its halo across several periods of
the grid (wrapped by full modulo).  The oracle (FP64) is the
reference; it is pinned to the reference's own outputs by tests/test_oracle_golden.py.
"""
import pytest

from conftest import rel_l2
from test_gpu_parity import FIELDS, inner, state_err

pytestmark = pytest.mark.gpu

GRIDS = [(18, 10, 13), (20, 7, 14), (36, 6, 9), (8, 5, 7), (4, 4, 6)]


def _case(nx, ny, nz, seed=5):
    from oracle.ic import Grid, WarmBubble, random_state
    from oracle.dycore import Dycore
    dx, dy, dz, dt = 600.0, 500.0, 300.0, 3.0
    phys, base, _ = WarmBubble(nx, ny, nz, dx, dy, dz).build()
    _, rho0, theta0, pi0, qv0, _ = base
    cols = dict(theta0=theta0[0, 0], qv0=qv0[0, 0], pi0=pi0[0, 0], rho0=rho0[0, 0])
    state = random_state(phys, nx, ny, nz, seed)
    D = Dycore(Grid(nx, ny, nz, dx, dy, dz), cols, dt, 32)
    return (dx, dy, dz, dt), cols, state, D


def _solver(nx, ny, nz, geom, cols, pairs=False):
    from lex_gb300.solver import Solver
    dx, dy, dz, dt = geom
    S = Solver(nx, ny, nz, dx, dy, dz, dt, 32, turb_opt=1, acoustic_pairs=pairs)
    S.set_base_columns(cols["theta0"], cols["qv0"], cols["pi0"], cols["rho0"])
    return S


def _oracle_ops(D, state):
    th, u, v, w, pip, qv = state
    div = D.mass_divergence(u, v, w)
    trho = th * (1.0 + (461.5 / 287.04) * qv) / (1.0 + qv)
    pu, pv, pw = D.pgf(pip, trho)
    s2 = D.deformation(u, v, w)[6]
    n2 = D.brunt_vaisala(th, qv)
    km, _ = D.eddy_coefficients(s2, n2)
    sg = D.smagorinsky(th, u, v, w, qv)
    return {
        "mass_div": (inner(div), 2e-6), "theta_rho": (inner(trho), 2e-7),
        "adv_theta": (D.advect_scalar(th, u, v, w, div, 1e-17), 5e-6),
        "adv_qv": (D.advect_scalar(qv, u, v, w, div, 1e-18), 5e-6),
        "adv_u": (D.advect_u(u, v, w, div), 5e-6), "adv_v": (D.advect_v(u, v, w, div), 5e-6),
        "adv_w": (D.advect_w(u, v, w, div), 5e-6), "buoy_w": (D.buoyancy(th, qv)[1], 2e-6),
        "pgf_u": (pu, 2e-6), "pgf_v": (pv, 2e-6), "pgf_w": (pw, 2e-6),
        "adv_pi": (D.advect_pi(pip, u, v, w), 2e-6),
        "n2": (inner(n2), 5e-6), "km": (inner(km), 5e-6),
        "sgs_u": (sg[0], 5e-6), "sgs_v": (sg[1], 5e-6), "sgs_w": (sg[2], 5e-6),
        "sgs_theta": (sg[3], 5e-6), "sgs_qv": (sg[4], 5e-6),
    }


@pytest.mark.parametrize("nx,ny,nz", GRIDS, ids=["%dx%dx%d" % g for g in GRIDS])
def test_operators_on_ragged_grid(built_lib, nx, ny, nz):
    geom, cols, state, D = _case(nx, ny, nz)
    ref = _oracle_ops(D, state)
    errs = {}
    with _solver(nx, ny, nz, geom, cols) as S:
        S.upload(state)
        for name, (r, tol) in ref.items():
            out = S.diagnose(name)
            assert out.shape == r.shape, name
            errs[name] = (rel_l2(out, r), tol)
    bad = {k: e for k, (e, t) in errs.items() if not e <= t}
    assert not bad, bad


@pytest.mark.parametrize("pairs", [False, True], ids=["one_substep_per_launch", "two_substeps_per_launch"])
@pytest.mark.parametrize("nx,ny,nz", GRIDS, ids=["%dx%dx%d" % g for g in GRIDS])
def test_step_on_ragged_grid(built_lib, nx, ny, nz, pairs):
    geom, cols, state, D = _case(nx, ny, nz)
    nxt, _ = D.step(state)
    with _solver(nx, ny, nz, geom, cols, pairs) as S:
        S.upload(state)
        S.step(1)
        out = S.download()
    for f, a, r, a0 in zip(FIELDS, out, nxt, state):
        err = state_err(a, r, a0, f)
        assert err <= 1e-5, (f, err)
