"""A torch stand-in for the small part of ``jax`` that LEX's dynamical core uses.

Test infrastructure only, like ``jax_standin.py`` (its NumPy sibling).  It runs the reference's
own, unmodified Python source on torch tensors, which gives two things the NumPy stand-in cannot:

  * speed: torch's multi-threaded CPU kernels make hundreds of RK3 steps of the 192 x 192 x 96
    workload feasible here (``make_golden.py --long``);
  * reverse mode: every operation is a differentiable torch operation (``x.at[i].set(v)`` is an
    out-of-place index assignment), so ``torch.autograd`` through ``ws_rk3_big_step`` is the
    stand-in for ``jax.vjp`` of the reference.

What it provides: ``jax.jit`` (identity decorator), ``jax.numpy`` functions on tensors, the
``.at[idx].set(v)`` property on ``torch.Tensor`` (added by ``install()``), ``jax.lax.select``,
and a ``numpy`` replacement inside ``one_step_integration`` whose ``zeros`` placeholders are
tensors.  Arithmetic runs in torch's default dtype, set by ``install(dtype)``.
"""
import functools
import sys
import types

import numpy as np
import torch

_STATE = {"dtype": torch.float64}


def _t(x):
    """Array-like -> tensor in the working dtype (tensors of another float dtype are cast)."""
    if isinstance(x, torch.Tensor):
        return x.to(_STATE["dtype"]) if x.is_floating_point() and x.dtype != _STATE["dtype"] else x
    if isinstance(x, (bool, np.bool_)) or (isinstance(x, np.ndarray) and x.dtype == np.bool_):
        return torch.as_tensor(np.asarray(x))
    if isinstance(x, (int, np.integer)) and not isinstance(x, bool):
        return torch.as_tensor(float(x), dtype=_STATE["dtype"])
    return torch.as_tensor(np.asarray(x, dtype=np.float64), dtype=_STATE["dtype"])


class _At:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        arr = self._arr

        class _Setter:
            def set(self_inner, val):
                out = arr.clone()
                out[idx] = _t(val) if not isinstance(val, (int, float)) else val
                return out
        return _Setter()


def _un(f):
    return lambda x, *a, **k: f(_t(x), *a, **k)


def _bin(f):
    return lambda a, b: f(_t(a), _t(b))


def _where(c, a=None, b=None):
    return torch.where(_t(c), _t(a), _t(b))


def _concat(arrs, axis=0):
    return torch.cat([_t(a) for a in arrs], dim=axis)


def _zeros(shape, dtype=None):
    return torch.zeros(tuple(shape) if not isinstance(shape, int) else shape, dtype=_STATE["dtype"])


def _ones(shape, dtype=None):
    return torch.ones(tuple(shape) if not isinstance(shape, int) else shape, dtype=_STATE["dtype"])


def _cbrt(x):
    x = _t(x)
    return torch.sign(x) * torch.abs(x) ** (1.0 / 3.0)


def _reduce(f):
    def g(x, axis=None, **_k):
        x = _t(x)
        return f(x) if axis is None else f(x, dim=axis)
    return g


def _jit(fun=None, static_argnames=None, **_kw):
    if fun is None:
        return lambda f: _jit(f, static_argnames=static_argnames)
    return functools.wraps(fun)(lambda *a, **k: fun(*a, **k))


def _unavailable(*_a, **_k):
    raise NotImplementedError("not provided by the torch stand-in")


def set_dtype(dtype):
    """Switch the working dtype of an installed stand-in (the imported reference modules follow)."""
    _STATE["dtype"] = dtype
    torch.set_default_dtype(dtype)


def install(dtype=torch.float64):
    """Register the stand-in modules in ``sys.modules`` and set the working dtype."""
    _STATE["dtype"] = dtype
    torch.set_default_dtype(dtype)
    torch.Tensor.at = property(lambda self: _At(self))
    jax = types.ModuleType("jax")
    jax._is_standin = True
    jnp = types.ModuleType("jax.numpy")
    for name in ("abs", "sqrt", "log", "exp", "cos", "sin", "arctan"):
        setattr(jnp, name, _un(getattr(torch, name if name != "arctan" else "atan")))
    jnp.cbrt = _cbrt
    jnp.fmin = _bin(torch.fmin)
    jnp.fmax = _bin(torch.fmax)
    jnp.maximum = _bin(torch.maximum)
    jnp.minimum = _bin(torch.minimum)
    jnp.where = _where
    jnp.concatenate = _concat
    jnp.zeros = _zeros
    jnp.ones = _ones
    jnp.reshape = lambda a, shape: torch.reshape(_t(a), tuple(shape))
    jnp.shape = lambda a: tuple(a.shape)
    jnp.sum = _reduce(torch.sum)
    jnp.mean = _reduce(torch.mean)
    jnp.cumsum = lambda x, axis=0: torch.cumsum(_t(x), dim=axis)
    jnp.pi = np.pi
    jnp.float32 = torch.float32
    jnp.float64 = torch.float64
    lax = types.ModuleType("jax.lax")
    lax.select = lambda p, a, b: torch.where(_t(p), _t(a), _t(b))
    lax.linalg = types.SimpleNamespace(tridiagonal_solve=_unavailable)
    rnd = types.ModuleType("jax.random")
    rnd.key = _unavailable
    rnd.uniform = _unavailable
    scipy = types.ModuleType("jax.scipy")
    scipy.sparse = types.SimpleNamespace(linalg=types.SimpleNamespace(bicgstab=_unavailable, gmres=_unavailable))
    jax.numpy, jax.lax, jax.random, jax.scipy = jnp, lax, rnd, scipy
    jax.jit = _jit
    jax.vmap = _unavailable
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)
    sys.modules.update({"jax": jax, "jax.numpy": jnp, "jax.lax": lax, "jax.random": rnd, "jax.scipy": scipy})
    dlm = types.ModuleType("dl_models")
    dlm.AutoEncoder = lambda *a, **k: None
    dlm.simpleCNN = lambda *a, **k: None
    optax = types.ModuleType("optax")
    optax.constant_schedule = lambda v: v
    for name, mod in {"dl_models": dlm, "optax": optax}.items():
        sys.modules.setdefault(name, mod)


def load_reference(ref_dir, dtype=torch.float64):
    """Import the reference's dynamical-core modules from ``ref_dir`` under the torch stand-in."""
    install(dtype)
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
    # the reference's np.zeros placeholders (heating, surface fluxes, Coriolis when off) as tensors
    shim = types.ModuleType("numpy_tensor_zeros")
    shim.__dict__.update({k: getattr(np, k) for k in dir(np) if not k.startswith("__")})
    shim.zeros = _zeros
    one.np = shim
    return types.SimpleNamespace(nl=nl, adv=adv, one=one, sp=sp, turb=turb, pres_eqn=pres_eqn,
                                 pres_grad=pres_grad, bc=bc)


def tree(x):
    """NumPy arrays (nested in tuples) -> tensors in the working dtype."""
    if isinstance(x, (tuple, list)):
        return type(x)(tree(v) for v in x)
    if isinstance(x, np.ndarray):
        return _t(x)
    return x
