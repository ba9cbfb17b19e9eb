"""Output writers with the names and arguments of LEX's write_netcdf.py / write_zarr.py, for
lex_relay.py end to end.

    save2nc(phys_state, sfc_others, grids, sprint_i, model_time)     write_netcdf.py:8-120
    save2nc_base(base_state, grids)                                  write_netcdf.py:123-183
    save2zarr(phys_state, sfc_others, sprint_i, model_time)          write_zarr.py:13-62

netCDF4 and zarr are not part of this stack, so every writer stores the variables the reference
writes, with its names, dimensions and dtypes (interior of the padded arrays, a leading time
axis of one where the netCDF file has one), in a NumPy ``.npz`` archive named by the namelist's
``file_name_format % sprint_i`` / ``base_file_name`` with the extension replaced.  The surface
fields are written only with sfc_opt on and pip_const only with pic_opt on, as in the
reference.  The returned value is the file name.
"""
import os

import numpy as np

from . import one_sprint_functions as _sp

NGX, NGY, NGZ = 3, 3, 1
SFC_NAMES = ("tau_x", "tau_y", "sen", "evap", "T_ref", "q_ref", "u10")


def _npz_name(name):
    return os.path.splitext(name)[0] + ".npz"


def _interior(a):
    return np.asarray(a)[NGX:-NGX, NGY:-NGY, NGZ:-NGZ]


def _write(filename, arrays):
    d = os.path.dirname(filename)
    if d:
        os.makedirs(d, exist_ok=True)
    np.savez(filename, **arrays)
    return filename


def _state_arrays(phys_state, sfc_others, model_time, dtype, time_axis):
    nl = _sp._namelist()
    theta, u, v, w, pip, qv = phys_state
    info, pip_const, tau_x, tau_y, sen, evap, t_ref, q_ref, u10n = sfc_others
    shape = lambda a: (1,) + a.shape if time_axis else a.shape
    out = {"time": np.asarray([model_time], dtype=np.float32 if dtype == np.float32 else np.float64)}
    for name, a in (("theta", theta), ("pip", pip), ("qv", qv), ("u", u), ("v", v), ("w", w)):
        x = _interior(a).astype(dtype)
        out[name] = x.reshape(shape(x))
    if time_axis:
        out["info"] = np.asarray([info], dtype=np.float32)
        if getattr(nl, "pic_opt", 0):
            out["pip_const"] = np.asarray([pip_const], dtype=np.float32)
    if getattr(nl, "sfc_opt", 0):
        for name, a in zip(SFC_NAMES, (tau_x, tau_y, sen, evap, t_ref, q_ref, u10n)):
            x = np.asarray(a, dtype=dtype).reshape(int(nl.nx), int(nl.ny))
            out[name] = x.reshape(shape(x))
    return out


def save2nc(phys_state, sfc_others, grids, sprint_i, model_time):
    """FP32 state snapshot with its coordinates (x, y, z, x4u, y4v, z4w) -> file name."""
    nl = _sp._namelist()
    out = _state_arrays(phys_state, sfc_others, model_time, np.float32, True)
    x3d, y3d, z3d, x3d4u, y3d4v, z3d4w = (np.asarray(g) for g in grids[:6])
    out.update(x=x3d[NGX:-NGX, 0, 0].astype(np.float32), y=y3d[0, NGY:-NGY, 0].astype(np.float32),
               z=z3d[0, 0, NGZ:-NGZ].astype(np.float32), x4u=x3d4u[NGX:-NGX, 0, 0].astype(np.float32),
               y4v=y3d4v[0, NGY:-NGY, 0].astype(np.float32), z4w=z3d4w[0, 0, NGZ:-NGZ].astype(np.float32))
    return _write(_npz_name(nl.file_name_format % sprint_i), out)


def save2nc_base(base_state, grids):
    """FP64 base state (rho0*theta0, rho0, theta0, pi0, qv0 on the interior; surface T) -> file name."""
    nl = _sp._namelist()
    rho0_theta0, rho0, theta0, pi0, qv0, surface_t = base_state
    x3d, y3d, z3d = (np.asarray(g) for g in grids[:3])
    out = {"x": x3d[NGX:-NGX, 0, 0].astype(np.float64), "y": y3d[0, NGY:-NGY, 0].astype(np.float64),
           "z": z3d[0, 0, NGZ:-NGZ].astype(np.float64), "time": np.zeros(1)}
    for name, a in (("rho0_theta0", rho0_theta0), ("rho0", rho0), ("theta0", theta0), ("pi0", pi0), ("qv0", qv0)):
        out[name] = _interior(a).astype(np.float64)[None]
    out["T_sfc"] = np.asarray(surface_t, dtype=np.float64).reshape(1, int(nl.nx), int(nl.ny))
    return _write(_npz_name(nl.base_file_name), out)


def save2zarr(phys_state, sfc_others, sprint_i, model_time):
    """FP64 state snapshot (the Zarr store's arrays, no time axis on the fields) -> file name."""
    nl = _sp._namelist()
    out = _state_arrays(phys_state, sfc_others, model_time, np.float64, False)
    return _write(_npz_name(nl.file_name_format % sprint_i), out)
