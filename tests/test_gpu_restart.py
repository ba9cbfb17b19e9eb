"""Checkpoint / restart: a solver restored from Solver.save continues bit for bit; the non-finite
check raises on a state with a NaN put there on the host (no GPU fault involved)."""
import numpy as np
import pytest

from conftest import load_golden
from test_gpu_parity import FIELDS

pytestmark = pytest.mark.gpu


def _solver(g):
    from lex_gb300.solver import Solver
    S = Solver(int(g["nx"]), int(g["ny"]), int(g["nz"]), float(g["dx"]), float(g["dy"]), float(g["dz"]),
               float(g["dt"]), int(g["n_sound"]), turb_opt=1, cs=0.2)
    S.set_base_columns(g["col_theta0"], g["col_qv0"], g["col_pi0"], g["col_rho0"])
    return S


def test_restart_continues_bit_for_bit(built_lib, tmp_path):
    from lex_gb300.solver import Solver
    g = load_golden("bubble_steps.npz")
    path = str(tmp_path / "ckpt.npz")
    with _solver(g) as S:
        S.upload(tuple(g["in_" + f] for f in FIELDS))
        S.step(2)
        S.save(path)
        S.step(2)
        a = S.download(np.float64)
    with Solver.restore(path) as R:
        assert R.cs == 0.2
        R.step(2)
        b = R.download(np.float64)
    for f, x, y in zip(FIELDS, a, b):
        assert np.array_equal(x, y), f


def test_check_finite_raises_on_a_nan_state(built_lib):
    g = load_golden("bubble_steps.npz")
    with _solver(g) as S:
        st = [g["in_" + f].copy() for f in FIELDS]
        S.upload(tuple(st))
        S.check_finite()
        st[0][5, 5, 3] = np.nan
        S.upload(tuple(st))
        with pytest.raises(FloatingPointError):
            S.check_finite()
