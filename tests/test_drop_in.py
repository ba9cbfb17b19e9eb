"""The drop-in sprint API (lex_gb300/one_sprint_functions.py) mirrors one_sprint_functions.py:
argument checking and the surface tuple on the CPU, the integration itself on the GPU."""
import types

import numpy as np
import pytest

from conftest import load_golden
from test_gpu_parity import FIELDS, state_err

OK = (2, 0, 0, 0, 0, 0, 1)


def namelist(g, sprint_n=1):
    return types.SimpleNamespace(nx=int(g["nx"]), ny=int(g["ny"]), nz=int(g["nz"]), dx=float(g["dx"]),
                                 dy=float(g["dy"]), dz=float(g["dz"]), dt=float(g["dt"]),
                                 n_sound=int(g["n_sound"]), sprint_n=sprint_n, fCor=1.0e-4)


def base_state(g):
    nx, ny = int(g["nx"]) + 6, int(g["ny"]) + 6
    col = lambda c: np.broadcast_to(np.asarray(c, dtype=np.float64), (nx, ny, c.size)).copy()
    rho0, th0 = col(g["col_rho0"]), col(g["col_theta0"])
    return (rho0 * th0, rho0, th0, col(g["col_pi0"]), col(g["col_qv0"]), np.zeros((nx - 6, ny - 6)))


@pytest.mark.parametrize("opt,exc", [((1, 0, 0, 0, 0, 0, 1), NotImplementedError),
                                     ((3, 0, 0, 0, 0, 0, 1), NotImplementedError),
                                     ((2, 1, 0, 0, 0, 0, 1), NotImplementedError),
                                     ((2, 0, 1, 0, 0, 0, 1), NotImplementedError),
                                     ((2, 0, 0, 0, 1, 0, 1), NotImplementedError),
                                     ((2, 0, 0, 0, 0, 0, 2), NotImplementedError),
                                     ((2, 0, 0, 3, 0, 0, 1), ValueError),
                                     ((2, 0, 0, 0, 0, 0), ValueError)])
def test_model_opt_outside_the_gpu_path_is_refused(opt, exc):
    from lex_gb300 import one_sprint_functions as sp
    with pytest.raises(exc):
        sp.check_model_opt(opt)


def test_first_step_flux_is_the_zero_surface_tuple():
    from lex_gb300 import one_sprint_functions as sp
    g = load_golden("bubble_steps.npz")
    sp.configure(namelist(g))
    sfc = sp.get_first_step_flux(None, None, None, OK)
    assert len(sfc) == 9 and sfc[0] == -999 and sfc[1] == -999   # one_step_integration.py:181-186
    for a in sfc[2:]:
        assert a.shape == (int(g["nx"]), int(g["ny"])) and not a.any()


@pytest.mark.gpu
def test_big_step_and_sprint_match_reference(built_lib):
    from lex_gb300 import one_sprint_functions as sp
    g = load_golden("bubble_steps.npz")
    x0 = tuple(g["in_" + f].copy() for f in FIELDS)
    keep = tuple(a.copy() for a in x0)
    base = base_state(g)
    sp.configure(namelist(g, sprint_n=2))
    x1, sfc = sp.ws_rk3_big_step(x0, base, None, OK)
    assert len(sfc) == 9
    for f, a, a0, k in zip(FIELDS, x1, x0, keep):
        np.testing.assert_array_equal(a0, k)            # inputs are not modified
        assert state_err(a, g["f64_step1_" + f], a0, f) <= 1e-5, f
    x3, _ = sp.ws_rk3_sprint(x1, base, None, OK)         # resident state: no upload
    for f, a, a0 in zip(FIELDS, x3, x0):
        assert state_err(a, g["f64_step3_" + f], a0, f) <= 1e-5, f
    sp.configure(namelist(g))                            # releases the solver
