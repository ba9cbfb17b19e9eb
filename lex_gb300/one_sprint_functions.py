"""Drop-in replacement for LEX's sprint API (one_sprint_functions.py) on the GB300 solver.

LEX's driver imports this module's names (``lex_relay.py:11``) and calls

    get_first_step_flux(phys_state, base_state, grids, model_opt)      lex_relay.py:25
    ws_rk3_sprint(phys_state, base_state, grids, model_opt)            lex_relay.py:48
    ws_rk3_big_step(phys_state, base_state, grids, model_opt)          one_sprint_functions.py:10-30
    ws_rk3_sprint_dl(phys_state, base_state, grids, model_opt,
                     dl_params, scaling_params)                        lex_dl_relay.py:97

with the tuples of ``setup_lex.setup_grid_n_ic`` (setup_lex.py:66-69):

    phys_state = (theta, u, v, w, pi', qv)                padded [x][y][z], ghosts 3 / 3 / 1
    base_state = (rho0*theta0, rho0, theta0, pi0, qv0, T_sfc)
    grids      = (x3d, y3d, z3d, x3d4u, y3d4v, z3d4w, cc1, cc2, tauh, tauf)
    model_opt  = (solver_opt, damp_opt, rad_opt, cor_opt, sfc_opt, pic_opt, turb_opt)

The grid sizes, spacings, dt, n_sound and sprint_n come from the namelist module, as in the
reference (``namelist_n_constants``, imported on first use, or the object given to
:func:`configure`).  Like the reference, the functions return new padded arrays and never
modify their inputs.  The solver and its device state persist across calls: the state a sprint
returns stays on the device (:class:`ResidentField` objects, read like NumPy arrays), a state passed
back unchanged is not uploaded again, and the host copy is made when something reads the arrays -
for ``lex_relay.py`` that is ``write.save2nc`` (write_netcdf.py:56-57), one download of the six
fields per save.

Only solver_opt 2 with damping, radiation and surface fluxes off and turb_opt 0 or 1 is
implemented on the GPU; other options raise ``NotImplementedError`` (no CPU fallback).
"""
import weakref

import numpy as np
from numpy.lib.mixins import NDArrayOperatorsMixin

from .solver import Solver, FIELDS, padded_shape

_nl = None
_solver = None
_key = None
_last = None   # weak reference to the state the last call returned (still on the device)
_sgs = None    # (ids of dl_params and scaling_params, device tensors) of the attached network


def _retire_last():
    """Keep the last returned state readable before the device state it refers to changes."""
    global _last
    prev = _last() if _last is not None else None
    if prev is not None:
        prev.preserve()
    _last = None


def configure(namelist):
    """Use ``namelist`` (any object with nx, ny, nz, dx, dy, dz, dt, n_sound, sprint_n and,
    when cor_opt is on, fCor) instead of importing ``namelist_n_constants``."""
    global _nl, _solver, _key, _last, _sgs
    _retire_last()
    _nl = namelist
    if _solver is not None:
        _solver.close()
    _solver, _key, _last, _sgs = None, None, None, None


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
    global _solver, _key, _last, _sgs
    nl = _namelist()
    cor_opt, turb_opt = check_model_opt(model_opt)
    key = (int(nl.nx), int(nl.ny), int(nl.nz), float(nl.dx), float(nl.dy), float(nl.dz), float(nl.dt),
           int(nl.n_sound), cor_opt, turb_opt, float(getattr(nl, "fCor", 1.0e-4)))
    if _solver is None or key != _key:
        _retire_last()
        if _solver is not None:
            _solver.close()
        _solver = Solver(key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7], turb_opt=turb_opt,
                         cor_opt=cor_opt, f_cor=key[10])
        _solver._base_cols = None
        _key, _last, _sgs = key, None, None
    # the device stores theta relative to theta0 of the base state: a new base state also
    # invalidates the resident phys_state
    cols = tuple(np.asarray(base_state[i], dtype=np.float64)[0, 0, :].copy() for i in (2, 4, 3, 1))
    if _solver._base_cols is None or not all(np.array_equal(a, b) for a, b in zip(cols, _solver._base_cols)):
        _retire_last()
        _solver.set_base_state(base_state)
        _solver._base_cols = cols
    return _solver


def _sfc_zeros():
    """sfc_etc with surface fluxes off (one_step_integration.py:48-55, 181-186)."""
    nl = _namelist()
    z = lambda: np.zeros((int(nl.nx), int(nl.ny)))
    return (-999, -999, z(), z(), z(), z(), z(), z(), z())


class _ResidentState:
    """The six fields a sprint left on the device.  The host copy (padded reference layout, one
    download of all six fields) is made on first read and is read-only, as JAX arrays are
    immutable.  Before the solver advances past this state, an unread state is copied on the
    device (``preserve``), so it can still be read afterwards."""
    downloads = 0   # host copies made (all states), for tests and for tracing IO

    def __init__(self, solver, dtype):
        self.solver = solver
        self.dtype = dtype
        self.host = None
        self.snap = None

    def preserve(self):
        if self.host is None and self.snap is None:
            self.snap = [_device_copy(p, n) for p, n in zip(self.solver.device_ptrs(), _counts(self.solver))]
            self.theta_ref = _theta_ref(self.solver)

    def materialize(self):
        if self.host is None:
            if self.snap is None:
                host = self.solver.download(self.dtype)
            else:
                host = _pad_host(self.snap, self.theta_ref, self.solver, self.dtype)
                self.snap = None
            for a in host:
                a.setflags(write=False)
            self.host = host
            _ResidentState.downloads += 1
        return self.host


class ResidentField(NDArrayOperatorsMixin):
    """One field of a sprint's result on the device, in the reference's padded [x][y][z] layout.

    Reads like a NumPy array (``np.asarray``, slicing, ``np.reshape``, arithmetic); the first read of
    any field of the state copies all six to the host.  Read-only: to change a state, make a new
    array (JAX arrays are immutable too)."""

    def __init__(self, state, index):
        self._state = state
        self._index = index
        nx, ny, nz = state.solver.nx, state.solver.ny, state.solver.nz
        self.shape = padded_shape(nx, ny, nz, FIELDS[index])
        self.dtype = np.dtype(state.dtype)
        self.ndim = 3
        self.size = int(np.prod(self.shape))

    def __array__(self, dtype=None, copy=None):
        a = self._state.materialize()[self._index]
        if dtype is not None and np.dtype(dtype) != a.dtype:
            return a.astype(dtype)
        return a.copy() if copy else a

    def __getitem__(self, idx):
        return np.asarray(self)[idx]

    def __len__(self):
        return self.shape[0]

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        inputs = tuple(np.asarray(x) if isinstance(x, ResidentField) else x for x in inputs)
        return getattr(ufunc, method)(*inputs, **kwargs)

    def __repr__(self):
        where = "host" if self._state.host is not None else "device"
        return "ResidentField(%s, shape=%s, dtype=%s, on %s)" % (FIELDS[self._index], self.shape, self.dtype, where)


class _DeviceArray:
    """A device allocation seen by torch without a copy (``__cuda_array_interface__``)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f4", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def _device_copy(ptr, n):
    """A device-to-device copy of the n FP32 values at ``ptr``, ordered after the solver's work."""
    import torch
    if _solver is not None:
        _solver.synchronize()
    out = torch.as_tensor(_DeviceArray(ptr, n), device="cuda").clone()
    torch.cuda.current_stream().synchronize()   # before the solver writes its state again
    return out


def _counts(solver):
    nx, ny, nz = solver.nx, solver.ny, solver.nz
    return [nx * ny * (nz + 1) if f == 3 else nx * ny * nz for f in range(6)]


def _theta_ref(solver):
    """The constant the device subtracts from theta (lexgb_config.theta_ref, else theta0 at level 1)."""
    return float(solver.cfg.theta_ref) if solver.cfg.theta_ref != 0.0 else float(solver._base[0][1])


def _pad_host(snap, theta_ref, solver, dtype):
    """Device-layout copies -> the padded reference layout on the host, as lexgb_download_state makes it."""
    from .workload import _pad
    nx, ny, nz = solver.nx, solver.ny, solver.nz
    out = []
    for f, t in enumerate(snap):
        a = t.cpu().numpy().astype(np.float64).reshape((nz + 1 if f == 3 else nz), ny, nx).transpose(2, 1, 0)
        if f == 0:
            a = a + theta_ref
        if f == 1:
            a = np.concatenate([a, a[:1]], 0)
        if f == 2:
            a = np.concatenate([a, a[:, :1]], 1)
        out.append(np.ascontiguousarray(_pad(a, "u" if f == 1 else ("v" if f == 2 else "s")), dtype=dtype))
    return tuple(out)


def _advance(phys_state, base_state, model_opt, nsteps, sgs=None):
    global _last
    s = _ensure(base_state, model_opt)
    _attach(s, sgs)
    prev = _last() if _last is not None else None
    resident = prev is not None and len(phys_state) == 6 and all(
        isinstance(a, ResidentField) and a._state is prev for a in phys_state)
    if resident:
        prev.preserve()              # the caller may still read it after this sprint
    else:
        if prev is not None:
            prev.preserve()
        s.upload(tuple(np.asarray(a) for a in phys_state))
    dtype = np.result_type(*(np.dtype(a.dtype) for a in phys_state))
    s.step(nsteps)
    st = _ResidentState(s, np.float64 if dtype == np.float64 else np.float32)
    _last = weakref.ref(st)
    return tuple(ResidentField(st, f) for f in range(6))


def sgs_arrays(dl_params, scaling_params, nx, ny, nz):
    """The reference's simpleCNN parameters and scaling_params in the library's layout (NumPy).

    dl_params: {'Conv_0' .. 'Conv_3': {'kernel': [3, 3, 3, cin, cout] (x, y, z offsets), 'bias':
    [cout]}} (dl_models.py:19-30, flax: cross-correlation, zero padding) -> BF16 [27][cout][cin]
    with the offset (dz+1)*9 + (dy+1)*3 + (dx+1), channels zero-padded to the kernels' widths.
    scaling_params: (theta_min, theta_max, u_min, u_max, v_min, v_max, w_min, w_max, qv_min,
    qv_max, ...) with keepdims shapes on each field's own points (dataset_generation.py:80-105).
    Input: per-level minimum and max - min + 0.01 (1e-5 for qv) over x and y (dl_models.py:128-152),
    per face level for w; output: max - min at every point (one_sprint_functions.py:139-143), u and v
    on their faces 0..nx-1 / 0..ny-1 (the duplicated periodic face nx / ny is not stored), w on faces
    0..nz.  Returns (weights [27][cout][cin] FP32 per layer, biases, {'lo', 'rin': [5][nz+1],
    'rout': [5][nz+1][ny][nx]}), entry / level nz repeating the top level for all but w."""
    from . import sgs_cnn
    ws, bs = [], []
    for li, (cin, cout, _) in enumerate(sgs_cnn.LAYERS):
        p = dl_params["Conv_%d" % li]
        k = np.asarray(p["kernel"], dtype=np.float32)
        if k.ndim != 5 or k.shape[:3] != (3, 3, 3) or k.shape[3] > cin or k.shape[4] > cout:
            raise ValueError("Conv_%d kernel must be [3, 3, 3, cin, cout] of simpleCNN, got %s" % (li, k.shape))
        w = np.zeros((27, cout, cin), np.float32)
        w[:, :k.shape[4], :k.shape[3]] = k.transpose(2, 1, 0, 4, 3).reshape(27, k.shape[4], k.shape[3])
        b = np.zeros(cout, np.float32)
        b[:k.shape[4]] = np.asarray(p["bias"], np.float32)
        ws.append(w)
        bs.append(b)
    if len(scaling_params) < 10:
        raise ValueError("scaling_params must hold (theta, u, v, w, qv) minima and maxima")
    own = ((nx, ny, nz), (nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1), (nx, ny, nz))
    lo, rin, rout = [], [], []
    for f, margin in enumerate((0.01, 0.01, 0.01, 0.01, 1.0e-5)):
        mn = np.asarray(scaling_params[2 * f], np.float64).squeeze()
        mx = np.asarray(scaling_params[2 * f + 1], np.float64).squeeze()
        if mn.shape != own[f] or mx.shape != own[f]:
            raise ValueError("scaling_params[%d:%d] have shape %s, expected %s on the grid"
                             % (2 * f, 2 * f + 2, mn.shape, own[f]))
        l, h = mn.min(axis=(0, 1)), mx.max(axis=(0, 1))
        r = (mx - mn)[:nx, :ny]                       # u, v: faces 0..nx-1 / 0..ny-1
        if f != 3:                                    # repeat the top level as entry nz
            l, h = np.append(l, l[-1]), np.append(h, h[-1])
            r = np.concatenate([r, r[:, :, -1:]], axis=2)
        lo.append(l)
        rin.append(h - l + margin)
        rout.append(r.transpose(2, 1, 0))
    return ws, bs, {"lo": np.stack(lo), "rin": np.stack(rin), "rout": np.ascontiguousarray(np.stack(rout))}


def _sgs_tensors(dl_params, scaling_params, nx, ny, nz):
    """sgs_arrays on the device: BF16 weights, FP32 biases and ranges."""
    import torch
    ws, bs, sc = sgs_arrays(dl_params, scaling_params, nx, ny, nz)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float32).cuda()
    return ([dev(w).to(torch.bfloat16) for w in ws], [dev(b) for b in bs], {k: dev(v) for k, v in sc.items()})


def _attach(solver, sgs):
    """Attach (sgs = (dl_params, scaling_params)) or detach (None) the fused correction."""
    global _sgs
    from . import sgs_cnn
    if sgs is None:
        if _sgs is not None:
            sgs_cnn.attach(solver, None, None)
            _sgs = None
        return
    key = (id(sgs[0]), id(sgs[1]), id(solver))
    if _sgs is not None and _sgs[0] == key:
        return
    nl = _namelist()
    ws, bs, scale = _sgs_tensors(sgs[0], sgs[1], int(nl.nx), int(nl.ny), int(nl.nz))

    class _Net:
        wbf, b = ws, bs
    sgs_cnn.attach(solver, _Net, scale)
    _sgs = (key, ws, bs, scale)


def ws_rk3_big_step(phys_state, base_state, grids, model_opt):
    """One WS-RK3 big step (one_sprint_functions.py:10-30) -> (phys_state, sfc_others)."""
    return _advance(phys_state, base_state, model_opt, 1), _sfc_zeros()


def ws_rk3_sprint(phys_state, base_state, grids, model_opt):
    """nl.sprint_n big steps (one_sprint_functions.py:109-115) -> (phys_state, sfc_others)."""
    return _advance(phys_state, base_state, model_opt, int(_namelist().sprint_n)), _sfc_zeros()


def ws_rk3_sprint_dl(phys_state, base_state, grids, model_opt, dl_params, scaling_params):
    """nl.sprint_n big steps, each followed by the simpleCNN correction of theta, u, v, w, qv
    (one_sprint_functions.py:118-163), applied by the library inside its step graph (BF16
    tensor-core convolutions) -> (phys_state, sfc_others).  Needs nx a multiple of 16.  The
    weights and ranges are uploaded again only when other parameter objects are passed."""
    n = int(_namelist().sprint_n)
    return _advance(phys_state, base_state, model_opt, n, sgs=(dl_params, scaling_params)), _sfc_zeros()


def get_first_step_flux(phys_state, base_state, grids, model_opt):
    """Surface fluxes of the first stage (one_sprint_functions.py:168-174): with sfc_opt off they
    are the zero fields of one_step_integration.py:48-55."""
    check_model_opt(model_opt)
    return _sfc_zeros()
