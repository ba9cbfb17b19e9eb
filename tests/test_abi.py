"""The C ABI: every entry point declared in include/lexgb.h is exported by liblexgb.so and bound
by the ctypes layer; argument validation that happens before any CUDA call works without a GPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "lexgb.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lexgb_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from lex_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_header_declares_the_expected_surface():
    names = declared_functions()
    for n in ("lexgb_create", "lexgb_destroy", "lexgb_step", "lexgb_upload_state", "lexgb_download_state",
              "lexgb_set_base_columns", "lexgb_budget", "lexgb_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    from lex_gb300 import _lib
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name


def test_invalid_configs_are_rejected_before_touching_the_gpu(lib):
    from lex_gb300 import _lib
    cfg = _lib.Config()
    assert lib.lexgb_default_config(ctypes.byref(cfg)) == 0
    assert (cfg.nx, cfg.ny, cfg.nz, cfg.n_sound) == (240, 240, 120, 32)
    h = ctypes.c_void_p()
    for field, bad in (("nx", 3), ("nz", 5), ("n_sound", 0), ("turb_opt", 2), ("cor_opt", 3), ("dt", 0.0)):
        c = _lib.Config()
        lib.lexgb_default_config(ctypes.byref(c))
        setattr(c, field, bad)
        assert lib.lexgb_create(ctypes.byref(c), ctypes.byref(h)) == _lib.LEXGB_ERR_ARG, field
        assert _lib.last_error()
    assert lib.lexgb_create(None, ctypes.byref(h)) == _lib.LEXGB_ERR_ARG


def test_calls_on_a_null_context_report_errors(lib):
    from lex_gb300 import _lib
    assert lib.lexgb_step(None, 1, 0) == _lib.LEXGB_ERR_ARG
    assert lib.lexgb_synchronize(None) == _lib.LEXGB_ERR_ARG
    assert lib.lexgb_destroy(None) == 0
    buf = ctypes.create_string_buffer(8)
    n = lib.lexgb_last_error(buf, 8)
    assert n >= len(buf.value)
