"""A NumPy stand-in for the small part of ``jax`` that LEX's dynamical core uses.

Test infrastructure only.  It lets the reference's own, unmodified Python source
(advection.py, one_step_integration.py, turbulence.py, ...) run on the CPU in
this container, where JAX is not installed, so that golden input/output vectors
can be generated from the reference itself (``make_golden.py``).

What it provides:
  * ``jax.jit``                -> a wrapper that casts every array argument to the
                                  working dtype (FP32 emulates JAX's default with
                                  ``jax_enable_x64`` off, FP64 emulates x64 mode);
  * ``jax.numpy``              -> NumPy functions that return ``JArr`` arrays;
  * ``x.at[idx].set(v)``       -> functional update on ``JArr``;
  * ``jax.lax.select``         -> ``np.where``.
Every ufunc on a ``JArr`` casts its array operands to the working dtype first,
so NumPy float64 placeholders inside the reference (``np.zeros(...)``) do not
promote an FP32 computation to FP64, just as JAX would not.

The flax/optax/zarr imports that the reference's namelist pulls in at import
time are replaced by empty stub modules.
"""
import sys
import types
import functools
import numpy as np

_STATE = {"dtype": np.float64}


def set_dtype(dt):
    _STATE["dtype"] = np.dtype(dt).type


def _wd():
    return _STATE["dtype"]


class _At:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        arr = self._arr

        class _Setter:
            def set(self_inner, val):
                out = np.array(arr, dtype=_wd(), copy=True).view(JArr)
                out[idx] = np.asarray(val, dtype=_wd())
                return out
        return _Setter()


class JArr(np.ndarray):
    """ndarray with JAX's functional ``.at[...].set(...)``."""

    @property
    def at(self):
        return _At(self)

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        wd = _wd()
        conv = []
        for x in inputs:
            if isinstance(x, np.ndarray):
                x = np.asarray(x)
                if x.dtype.kind == "f" and x.dtype != wd:
                    x = x.astype(wd)
                conv.append(x)
            else:
                conv.append(x)
        if "out" in kwargs:
            kwargs["out"] = tuple(np.asarray(o) for o in kwargs["out"])
        res = getattr(ufunc, method)(*conv, **kwargs)
        if isinstance(res, np.ndarray):
            if res.dtype.kind == "f" and res.dtype != wd:
                res = res.astype(wd)
            return res.view(JArr)
        if isinstance(res, tuple):
            return tuple(r.view(JArr) if isinstance(r, np.ndarray) else r for r in res)
        return res


def _wrap(x):
    if isinstance(x, np.ndarray):
        if x.dtype.kind == "f" and x.dtype != _wd():
            x = x.astype(_wd())
        return x.view(JArr)
    if isinstance(x, (float, np.floating)):
        return _wd()(x)
    return x


def _cast_tree(x):
    if isinstance(x, tuple):
        return tuple(_cast_tree(v) for v in x)
    if isinstance(x, list):
        return [_cast_tree(v) for v in x]
    if isinstance(x, np.ndarray):
        return _wrap(x)
    return x


def _fn(npf):
    @functools.wraps(npf)
    def f(*args, **kwargs):
        args = [_cast_tree(a) if isinstance(a, (np.ndarray, list, tuple)) else a for a in args]
        return _wrap(np.asarray(npf(*args, **kwargs))) if not isinstance(npf(*args, **kwargs), tuple) \
            else npf(*args, **kwargs)
    return f


def _zeros(shape, dtype=None):
    return np.zeros(shape, dtype=dtype or _wd()).view(JArr)


def _ones(shape, dtype=None):
    return np.ones(shape, dtype=dtype or _wd()).view(JArr)


def _concat(arrs, axis=0):
    return _wrap(np.concatenate([np.asarray(_wrap(np.asarray(a))) for a in arrs], axis=axis))


def _simple(npf):
    def f(*args, **kwargs):
        args = [_wrap(np.asarray(a)) if isinstance(a, np.ndarray) else a for a in args]
        return _wrap(np.asarray(npf(*args, **kwargs)))
    return f


def _jit(fun=None, static_argnames=None, **_kw):
    if fun is None:
        return lambda f: _jit(f, static_argnames=static_argnames)

    @functools.wraps(fun)
    def wrapper(*args, **kwargs):
        args = tuple(_cast_tree(a) for a in args)
        kwargs = {k: _cast_tree(v) for k, v in kwargs.items()}
        return fun(*args, **kwargs)
    return wrapper


def _select(pred, a, b):
    return _wrap(np.where(np.asarray(pred), np.asarray(a), np.asarray(b)))


def _unavailable(*_a, **_k):
    raise NotImplementedError("not provided by the NumPy stand-in")


def install():
    """Register the stand-in modules in ``sys.modules`` (idempotent)."""
    if "jax" in sys.modules and getattr(sys.modules["jax"], "_is_standin", False):
        return
    jax = types.ModuleType("jax")
    jax._is_standin = True
    jnp = types.ModuleType("jax.numpy")
    for name in ["abs", "fmin", "fmax", "maximum", "minimum", "sqrt", "cbrt", "log", "exp", "cos",
                 "sin", "arctan", "where", "cumsum", "sum", "mean", "reshape", "max", "min"]:
        setattr(jnp, name, _simple(getattr(np, name)))
    jnp.zeros = _zeros
    jnp.ones = _ones
    jnp.concatenate = _concat
    jnp.shape = np.shape
    jnp.pi = np.pi
    jnp.float32 = np.float32
    jnp.float64 = np.float64
    lax = types.ModuleType("jax.lax")
    lax.select = _select
    lax.linalg = types.SimpleNamespace(tridiagonal_solve=_unavailable)
    rnd = types.ModuleType("jax.random")
    rnd.key = _unavailable
    rnd.uniform = _unavailable
    scipy = types.ModuleType("jax.scipy")
    scipy.sparse = types.SimpleNamespace(linalg=types.SimpleNamespace(bicgstab=_unavailable,
                                                                      gmres=_unavailable))
    jax.numpy = jnp
    jax.lax = lax
    jax.random = rnd
    jax.scipy = scipy
    jax.jit = _jit
    jax.vmap = _unavailable
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)
    sys.modules.update({"jax": jax, "jax.numpy": jnp, "jax.lax": lax, "jax.random": rnd,
                        "jax.scipy": scipy})
    # import-time dependencies of namelist_n_constants.py that the dynamical core never calls
    dlm = types.ModuleType("dl_models")
    dlm.AutoEncoder = lambda *a, **k: None
    dlm.simpleCNN = lambda *a, **k: None
    optax = types.ModuleType("optax")
    optax.constant_schedule = lambda v: v
    for name, mod in {"dl_models": dlm, "optax": optax}.items():
        sys.modules.setdefault(name, mod)


def load_reference(ref_dir):
    """Import the reference's dynamical-core modules from ``ref_dir`` under the stand-in."""
    install()
    sys.dont_write_bytecode = True
    if ref_dir not in sys.path:
        sys.path.insert(0, ref_dir)
    import namelist_n_constants as nl
    import advection as adv
    import one_step_integration as one
    import one_sprint_functions as sp
    import turbulence as turb
    import pressure_equations as pres_eqn
    import pressure_gradient_coriolis as pres_grad
    import boundary_conditions as bc
    import setup_lex as setl
    return types.SimpleNamespace(nl=nl, adv=adv, one=one, sp=sp, turb=turb, pres_eqn=pres_eqn,
                                 pres_grad=pres_grad, bc=bc, setl=setl)
