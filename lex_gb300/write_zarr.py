"""save2zarr with the name and arguments of LEX's write_zarr.py:13 (lex_relay.py:13 imports
this module by name); the store is written as a NumPy archive (see write_netcdf)."""
from .write_netcdf import save2zarr  # noqa: F401
