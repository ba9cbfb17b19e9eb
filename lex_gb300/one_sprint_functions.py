"""Drop-in replacement for LEX's sprint API (one_sprint_functions.py) on the GB300 solver.

LEX's driver imports this module's names (``lex_relay.py:11``) and calls

    get_first_step_flux(phys_state, base_state, grids, model_opt)      lex_relay.py:25
    ws_rk3_sprint(phys_state, base_state, grids, model_opt)            lex_relay.py:48
    ws_rk3_big_step(phys_state, base_state, grids, model_opt)          one_sprint_functions.py:10-30

with the tuples of ``setup_lex.setup_grid_n_ic`` (setup_lex.py:66-69):

    phys_state = (theta, u, v, w, pi', qv)                padded [x][y][z], ghosts 3 / 3 / 1
    base_state = (rho0*theta0, rho0, theta0, pi0, qv0, T_sfc)
    grids      = (x3d, y3d, z3d, x3d4u, y3d4v, z3d4w, cc1, cc2, tauh, tauf)
    model_opt  = (solver_opt, damp_opt, rad_opt, cor_opt, sfc_opt, pic_opt, turb_opt)

The grid sizes, spacings, dt, n_sound and sprint_n come from the namelist module, as in the
reference (``namelist_n_constants``, imported on first use, or the object given to
:func:`configure`).  Like the reference, the functions return new padded arrays and never
modify their inputs.  The solver and its device state persist across calls: a state returned
by :func:`ws_rk3_sprint` and passed back unchanged is not uploaded again.

Only solver_opt 2 with damping, radiation and surface fluxes off and turb_opt 0 or 1 is
implemented on the GPU; other options raise ``NotImplementedError`` (no CPU fallback).
"""
import numpy as np

from .solver import Solver

_nl = None
_solver = None
_key = None
_last = None   # (returned tuple, id of its arrays) of the last sprint


def configure(namelist):
    """Use ``namelist`` (any object with nx, ny, nz, dx, dy, dz, dt, n_sound, sprint_n and,
    when cor_opt is on, fCor) instead of importing ``namelist_n_constants``."""
    global _nl, _solver, _key, _last
    _nl = namelist
    if _solver is not None:
        _solver.close()
    _solver, _key, _last = None, None, None


def _namelist():
    global _nl
    if _nl is None:
        import namelist_n_constants as nl  # the caller's LEX namelist
        _nl = nl
    return _nl


def check_model_opt(model_opt):
    """Validate the 7-tuple (one_step_integration.py:22) against what the GPU path implements."""
    if len(model_opt) != 7:
        raise ValueError("model_opt must be (solver_opt, damp_opt, rad_opt, cor_opt, sfc_opt, pic_opt, turb_opt)")
    solver_opt, damp_opt, rad_opt, cor_opt, sfc_opt, pic_opt, turb_opt = model_opt
    if solver_opt != 2:
        raise NotImplementedError("solver_opt=%r: only the split-explicit solver (2) runs on the GPU" % (solver_opt,))
    if damp_opt or rad_opt or sfc_opt or pic_opt:
        raise NotImplementedError("damping, radiation, surface fluxes and pic_opt are not implemented on the GPU")
    if turb_opt not in (0, 1):
        raise NotImplementedError("turb_opt=%r: only 0 (off) and 1 (Smagorinsky) run on the GPU" % (turb_opt,))
    if cor_opt not in (0, 1, 2):
        raise ValueError("cor_opt must be 0, 1 or 2")
    return int(cor_opt), int(turb_opt)


def _ensure(base_state, model_opt):
    global _solver, _key, _last
    nl = _namelist()
    cor_opt, turb_opt = check_model_opt(model_opt)
    key = (int(nl.nx), int(nl.ny), int(nl.nz), float(nl.dx), float(nl.dy), float(nl.dz), float(nl.dt),
           int(nl.n_sound), cor_opt, turb_opt, float(getattr(nl, "fCor", 1.0e-4)))
    if _solver is None or key != _key:
        if _solver is not None:
            _solver.close()
        _solver = Solver(key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7], turb_opt=turb_opt,
                         cor_opt=cor_opt, f_cor=key[10])
        _solver._base_cols = None
        _key, _last = key, None
    # the device stores theta relative to theta0 of the base state: a new base state also
    # invalidates the resident phys_state
    cols = tuple(np.asarray(base_state[i], dtype=np.float64)[0, 0, :].copy() for i in (2, 4, 3, 1))
    if _solver._base_cols is None or not all(np.array_equal(a, b) for a, b in zip(cols, _solver._base_cols)):
        _solver.set_base_state(base_state)
        _solver._base_cols = cols
        _last = None
    return _solver


def _sfc_zeros():
    """sfc_etc with surface fluxes off (one_step_integration.py:48-55, 181-186)."""
    nl = _namelist()
    z = lambda: np.zeros((int(nl.nx), int(nl.ny)))
    return (-999, -999, z(), z(), z(), z(), z(), z(), z())


def _advance(phys_state, base_state, model_opt, nsteps):
    global _last
    s = _ensure(base_state, model_opt)
    resident = _last is not None and len(phys_state) == 6 and all(a is b for a, b in zip(phys_state, _last))
    if not resident:
        s.upload(tuple(np.asarray(a) for a in phys_state))
    s.step(nsteps)
    dtype = np.result_type(*(np.asarray(a).dtype for a in phys_state))
    out = s.download(np.float64 if dtype == np.float64 else np.float32)
    _last = out
    return out


def ws_rk3_big_step(phys_state, base_state, grids, model_opt):
    """One WS-RK3 big step (one_sprint_functions.py:10-30) -> (phys_state, sfc_others)."""
    return _advance(phys_state, base_state, model_opt, 1), _sfc_zeros()


def ws_rk3_sprint(phys_state, base_state, grids, model_opt):
    """nl.sprint_n big steps (one_sprint_functions.py:109-115) -> (phys_state, sfc_others)."""
    return _advance(phys_state, base_state, model_opt, int(_namelist().sprint_n)), _sfc_zeros()


def get_first_step_flux(phys_state, base_state, grids, model_opt):
    """Surface fluxes of the first stage (one_sprint_functions.py:168-174): with sfc_opt off they
    are the zero fields of one_step_integration.py:48-55."""
    check_model_opt(model_opt)
    return _sfc_zeros()
