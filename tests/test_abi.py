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
    for field, bad in (("nx", 3), ("nz", 5), ("n_sound", 0), ("turb_opt", 2), ("cor_opt", 3), ("dt", 0.0),
                       ("cs", -0.1)):
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


def test_new_entry_points_validate_before_touching_the_gpu(lib):
    from lex_gb300 import _lib
    g = ctypes.c_double()
    assert lib.lexgb_set_cs(None, 0.2) == _lib.LEXGB_ERR_ARG
    assert lib.lexgb_get_cs_grad(None, ctypes.byref(g), 0) == _lib.LEXGB_ERR_ARG
    assert lib.lexgb_set_sgs_net(None, None, None, None, None, None, 1) == _lib.LEXGB_ERR_ARG
    # the convolution's shape rules: nx a multiple of 16, cin a multiple of 16, cout 8, 16 or 32
    p = ctypes.c_void_p(1)
    for nx, cin, cout in ((10, 16, 32), (16, 24, 32), (16, 16, 12), (0, 16, 32)):
        assert lib.lexgb_cnn_conv3d(nx, 4, 4, cin, cout, p, p, None, None, p, None, 1, cout, None) == _lib.LEXGB_ERR_ARG
        assert _lib.last_error()
    assert lib.lexgb_cnn_conv3d_dw(16, 4, 4, 48, 32, 32, p, p, p, None, None) == _lib.LEXGB_ERR_ARG
    assert lib.lexgb_cnn_adam(0, p, p, p, p, None, 1e-3, 0.9, 0.999, 1e-8, 1, None) == _lib.LEXGB_ERR_ARG



def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No CPU fallback: without the built library every entry into the package raises."""
    from lex_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "liblexgb.so"))
    with pytest.raises(ImportError):
        _lib.load()
    from lex_gb300.solver import Solver
    with pytest.raises(ImportError):
        Solver(16, 16, 8, 100.0, 100.0, 100.0, 1.0)
