"""The output writers keep the reference's variable names, shapes and dtypes (write_netcdf.py,
write_zarr.py), stored as .npz because netCDF4 and zarr are not part of this stack."""
import os
import types

import numpy as np


def _namelist(tmp, nx=8, ny=6, nz=4, sfc_opt=0):
    return types.SimpleNamespace(nx=nx, ny=ny, nz=nz, dx=600.0, dy=600.0, dz=300.0, dt=3.0, n_sound=32, sprint_n=1,
                                 file_name_format=os.path.join(str(tmp), "out", "lex_out_%0.4i.nc"),
                                 base_file_name=os.path.join(str(tmp), "out", "lex_base.nc"), sfc_opt=sfc_opt, pic_opt=0)


def _state(nx, ny, nz, seed=0):
    r = np.random.default_rng(seed)
    s = (nx + 6, ny + 6, nz + 2)
    return (r.normal(size=s), r.normal(size=(s[0] + 1, s[1], s[2])), r.normal(size=(s[0], s[1] + 1, s[2])),
            r.normal(size=(s[0], s[1], s[2] + 1)), r.normal(size=s), r.normal(size=s))


def _grids(nx, ny, nz):
    x = np.arange(-3, nx + 3) * 600.0
    y = np.arange(-3, ny + 3) * 600.0
    z = np.arange(-1, nz + 1) * 300.0
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    Xu = np.broadcast_to(np.arange(-3, nx + 4)[:, None, None] * 600.0 - 300.0, (nx + 7, ny + 6, nz + 2))
    Yv = np.broadcast_to(np.arange(-3, ny + 4)[None, :, None] * 600.0 - 300.0, (nx + 6, ny + 7, nz + 2))
    Zw = np.broadcast_to(np.arange(-1, nz + 2)[None, None, :] * 300.0 - 150.0, (nx + 6, ny + 6, nz + 3))
    return (X, Y, Z, Xu, Yv, Zw, None, None, None, None)


def test_writers_store_the_reference_variables(tmp_path):
    from lex_gb300 import one_sprint_functions as sp, write_netcdf, write_zarr
    nx, ny, nz = 8, 6, 4
    sp.configure(_namelist(tmp_path, nx, ny, nz, sfc_opt=1))
    st = _state(nx, ny, nz)
    sfc = (-999, -999) + tuple(np.full((nx, ny), float(i)) for i in range(7))
    f = write_netcdf.save2nc(st, sfc, _grids(nx, ny, nz), 3, 90.0)
    assert f.endswith("lex_out_0003.npz") and os.path.exists(f)
    with np.load(f) as d:
        assert d["theta"].shape == (1, nx, ny, nz) and d["theta"].dtype == np.float32
        assert d["u"].shape == (1, nx + 1, ny, nz) and d["v"].shape == (1, nx, ny + 1, nz)
        assert d["w"].shape == (1, nx, ny, nz + 1)
        assert np.array_equal(d["qv"][0], st[5][3:-3, 3:-3, 1:-1].astype(np.float32))
        assert np.array_equal(d["u"][0], st[1][3:-3, 3:-3, 1:-1].astype(np.float32))
        assert d["x"].shape == (nx,) and d["x4u"].shape == (nx + 1,) and d["z4w"].shape == (nz + 1,)
        assert float(d["time"][0]) == 90.0 and d["info"][0] == -999
        assert d["u10"].shape == (1, nx, ny) and float(d["u10"][0, 0, 0]) == 6.0
    z = write_zarr.save2zarr(st, sfc, 4, 120.0)
    with np.load(z) as d:
        assert d["theta"].shape == (nx, ny, nz) and d["theta"].dtype == np.float64
        assert np.array_equal(d["w"], st[3][3:-3, 3:-3, 1:-1])
    cols = lambda c: np.broadcast_to(np.asarray(c, float)[None, None, :], (nx + 6, ny + 6, nz + 2)).copy()
    base = (cols(np.arange(nz + 2)), cols(np.ones(nz + 2)), cols(300.0 + np.zeros(nz + 2)), cols(np.ones(nz + 2)),
            cols(np.zeros(nz + 2)), np.full((nx, ny), 300.0))
    b = write_netcdf.save2nc_base(base, _grids(nx, ny, nz))
    with np.load(b) as d:
        assert d["theta0"].shape == (1, nx, ny, nz) and d["T_sfc"].shape == (1, nx, ny)
        assert np.array_equal(d["rho0_theta0"][0, 0, 0], np.arange(1, nz + 1, dtype=float))
