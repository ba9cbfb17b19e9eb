"""The three forms of the acoustic sub-steps against each other, and the persistent form's bounded
waits: "rows" (one launch per sub-step, float4 rows), "tile" (one launch per sub-step, 32 x 4 x 8
blocks sharing values between warps) and "persistent" (all sub-steps of stages 1 and 2 in one
cooperative launch per stage, pi' of each block's tile kept in shared memory, inputs staged by TMA).

* All forms evaluate the same expressions for every face and cell (sound_rk_step0/1/2,
  one_step_integration.py:519-556, :638-675, :757-794), so a step taken any way agrees to FP32
  rounding; each agrees with the FP64 oracle within the parity bar.
* A barrier wait that gives up makes the step report LEXGB_ERR_TIMEOUT on the host (no trap, no
  hang), and the context stays usable: a new upload and step reproduce an undisturbed run.
"""
import numpy as np
import pytest

from test_gpu_parity import FIELDS, state_err

pytestmark = pytest.mark.gpu


def _case(nx, ny, nz, seed=3):
    from oracle.ic import WarmBubble, random_state
    phys, base, _ = WarmBubble(nx, ny, nz, 400.0, 300.0, 200.0).build()
    cols = dict(theta0=base[2][0, 0], qv0=base[4][0, 0], pi0=base[3][0, 0], rho0=base[1][0, 0])
    return random_state(phys, nx, ny, nz, seed=seed), cols


def _run(x0, cols, nx, ny, nz, nsteps, form, turb=1):
    from lex_gb300.solver import Solver
    with Solver(nx, ny, nz, 400.0, 300.0, 200.0, 2.0, 32, turb_opt=turb, acoustic_kernel=form) as S:
        S.set_base_columns(cols["theta0"], cols["qv0"], cols["pi0"], cols["rho0"])
        S.upload(x0)
        S.step(nsteps)
        out = S.download()
        used = S.acoustic_form
    return out, used


@pytest.mark.parametrize("dims", [(64, 32, 20), (32, 16, 9), (96, 40, 12)], ids=lambda d: "x".join(map(str, d)))
def test_acoustic_forms_agree(built_lib, dims):
    nx, ny, nz = dims
    x0, cols = _case(nx, ny, nz)
    ref, used = _run(x0, cols, nx, ny, nz, 2, "rows")
    assert used == "rows"
    for form in ("tile", "persistent"):
        out, used = _run(x0, cols, nx, ny, nz, 2, form)
        assert used == form
        for f, p, q, r0 in zip(FIELDS, out, ref, x0):
            err = state_err(p, q, r0, f)
            assert err <= 1e-6, (form, f, err)


def test_form_fallback_on_grids_that_do_not_fit(built_lib):
    """A form the grid does not allow falls back: nx = 20 fits neither the tile nor the persistent form."""
    x0, cols = _case(20, 12, 8)
    _, used = _run(x0, cols, 20, 12, 8, 1, "persistent")
    assert used == "rows"


@pytest.mark.parametrize("form", ["tile", "persistent"])
def test_acoustic_form_matches_oracle(built_lib, form):
    from oracle.ic import Grid
    from oracle.dycore import Dycore
    nx, ny, nz = 64, 16, 12
    x0, cols = _case(nx, ny, nz, seed=9)
    out, used = _run(x0, cols, nx, ny, nz, 1, form)
    assert used == form
    ref, _ = Dycore(Grid(nx, ny, nz, 400.0, 300.0, 200.0), cols, 2.0, 32).step(x0)
    for f, a, r, a0 in zip(FIELDS, out, ref, x0):
        err = state_err(a, r, a0, f)
        assert err <= 1e-5, (f, err)


def test_barrier_timeout_is_reported_and_context_recovers(built_lib):
    from lex_gb300.solver import Solver
    from lex_gb300._lib import LexError, LEXGB_ERR_TIMEOUT
    nx, ny, nz = 64, 32, 20
    x0, cols = _case(nx, ny, nz)
    ref, used = _run(x0, cols, nx, ny, nz, 1, "persistent")
    assert used == "persistent"
    with Solver(nx, ny, nz, 400.0, 300.0, 200.0, 2.0, 32, turb_opt=1, acoustic_kernel="persistent") as S:
        S.set_base_columns(cols["theta0"], cols["qv0"], cols["pi0"], cols["rho0"])
        S.upload(x0)
        S.set_barrier_limit(-1000)      # test mode: each barrier waits for an arrival that never comes
        S.step(1)
        with pytest.raises(LexError) as ei:
            S.synchronize()
        assert ei.value.code == LEXGB_ERR_TIMEOUT
        S.synchronize()                 # reported once; the context still works
        S.set_barrier_limit(0)
        S.upload(x0)
        S.step(1)
        again = S.download()
    for f, a, b in zip(FIELDS, again, ref):
        np.testing.assert_array_equal(a, b, err_msg=f)
