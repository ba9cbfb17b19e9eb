"""The big step as a differentiable PyTorch operation on CUDA tensors.

``step(solver, state)`` advances one WS-RK3 big step (one_sprint_functions.py:10-30) and
records it for autograd; its backward is the hand-written reverse mode of the library
(``lexgb_step_vjp``).  Only the step's input state is saved (step-level checkpointing): the
backward pass recomputes the step's stages and acoustic sub-steps from it, so a rollout of N
steps keeps N states alive, not N times the ~50 intermediate fields of a step.  This replaces
``jax.vjp`` / ``jax.grad`` through ``ws_rk3_sprint_dl_train`` (one_sprint_functions.py:33-96,
lex_dl_train.py:114).  The forward keeps the intermediates of the step it ran last
(``lexgb_step_keep``), so the backward of the most recent step reuses them instead of
recomputing (``lexgb_step_vjp_kept``); earlier steps of a rollout are recomputed.  The
Smagorinsky constant can be an input too (``step(solver, state, cs=tensor)``): its gradient is
the library's FP64 accumulation of the derivative through every step's eddy viscosity.

State layout: a tuple of six float32 CUDA tensors in the device layout, x fastest -
theta, u, v, pi', qv of shape (nz, ny, nx) and w of shape (nz+1, ny, nx) (u on west faces,
v on south faces, w on faces 0..nz).  theta is in K, or with ``raw=True`` relative to the
solver's theta_ref as the device stores it (exact: FP32 kelvin rounds theta to about 3e-5 K, so a
rollout in kelvin re-rounds the state at every step boundary).  There is no CPU path: without a GPU
and the built library the calls raise.
"""
import ctypes

import torch

from . import _lib
from .solver import Solver


def _shapes(solver):
    nx, ny, nz = solver.nx, solver.ny, solver.nz
    c = (nz, ny, nx)
    return (c, c, c, (nz + 1, ny, nx), c, c)


def _check(solver, tensors):
    if len(tensors) != 6:
        raise ValueError("state must have 6 tensors (theta, u, v, w, pi', qv)")
    for t, shp in zip(tensors, _shapes(solver)):
        if not t.is_cuda or t.dtype != torch.float32 or tuple(t.shape) != shp:
            raise ValueError("state tensors must be float32 CUDA tensors of shapes %s" % (_shapes(solver),))


def _ptrs(tensors):
    return (ctypes.c_void_p * 6)(*[t.data_ptr() for t in tensors])


def _bind_stream(solver):
    # torch's default stream has the handle 0, which the C ABI reads as "the context's own
    # stream": name the legacy default stream explicitly (cudaStreamLegacy) instead
    h = torch.cuda.current_stream().cuda_stream
    solver.set_stream(h if h else 1)


def set_state(solver, tensors, raw=False):
    """Copy a device-layout state into the solver (ordered on torch's current stream); raw: theta
    relative to theta_ref."""
    tensors = tuple(t.contiguous() for t in tensors)
    _check(solver, tensors)
    _bind_stream(solver)
    _lib.check(solver.lib.lexgb_set_state_interior(solver.handle, _ptrs(tensors), 2 if raw else 1))


def get_state(solver, raw=False):
    """The solver's state as new device-layout tensors; raw: theta relative to theta_ref."""
    out = tuple(torch.empty(s, dtype=torch.float32, device="cuda") for s in _shapes(solver))
    _bind_stream(solver)
    _lib.check(solver.lib.lexgb_get_state_interior(solver.handle, _ptrs(out), 2 if raw else 1))
    return out


class _Step(torch.autograd.Function):
    @staticmethod
    def forward(ctx, solver, cs, raw, *state):
        if cs is not None and float(cs) != solver.cs:
            _bind_stream(solver)
            solver.set_cs(float(cs))
        ctx.with_cs = cs is not None
        ctx.cs = solver.cs      # the backward differentiates the step with this step's Cs
        ctx.raw = raw
        set_state(solver, state, raw)
        _bind_stream(solver)
        _lib.check(solver.lib.lexgb_step_keep(solver.handle))
        solver._keep_count = getattr(solver, "_keep_count", 0) + 1
        solver._kept_token = solver._keep_count
        ctx.token = solver._kept_token
        ctx.solver = solver
        ctx.save_for_backward(*state)
        return get_state(solver, raw)

    @staticmethod
    def backward(ctx, *grads):
        solver = ctx.solver
        gy = tuple((g if g is not None else torch.zeros(s, device="cuda")).contiguous().float()
                   for g, s in zip(grads, _shapes(solver)))
        gx = tuple(torch.empty(s, dtype=torch.float32, device="cuda") for s in _shapes(solver))
        _bind_stream(solver)
        cs_now = solver.cs
        if cs_now != ctx.cs:                                    # Cs changed since this step's forward
            solver.set_cs(ctx.cs)
        if ctx.with_cs:
            solver.cs_grad(reset=True)                          # start this step's accumulation at zero
        if getattr(solver, "_kept_token", None) == ctx.token:   # this step's intermediates are still kept
            _lib.check(solver.lib.lexgb_step_vjp_kept(solver.handle, _ptrs(gy), _ptrs(gx), 1))
        else:                                                   # recompute from the saved input
            set_state(solver, ctx.saved_tensors, ctx.raw)
            _lib.check(solver.lib.lexgb_step_vjp(solver.handle, 3, _ptrs(gy), _ptrs(gx), 1))
        solver._kept_token = None
        if solver.cs != cs_now:
            solver.set_cs(cs_now)
        gcs = torch.tensor(solver.cs_grad(reset=True), dtype=torch.float64, device="cuda") if ctx.with_cs else None
        return (None, gcs, None) + gx


def step(solver, state, cs=None, raw=False):
    """One differentiable big step: state -> next state (tuples of six CUDA tensors); cs: an
    optional scalar tensor, the Smagorinsky constant of the step, differentiable; raw: theta
    relative to the solver's theta_ref (see the module docstring)."""
    if not isinstance(solver, Solver):
        raise TypeError("solver must be a lex_gb300.solver.Solver")
    return _Step.apply(solver, cs, bool(raw), *state)


def rollout(solver, state, nsteps, cs=None, raw=False):
    """nsteps differentiable big steps (the sprint of one_sprint_functions.py:109-115)."""
    for _ in range(int(nsteps)):
        state = step(solver, state, cs, raw)
    return state
