"""Array-namespace dispatch for the oracle: the same restated formulas run on NumPy arrays or on
torch tensors (CPU or CUDA, FP64 or FP32).

TEST INFRASTRUCTURE ONLY (see oracle/dycore.py).  The torch form exists so that the FP64 oracle
can evaluate full-size workloads (192 x 192 x 96, hundreds of steps) in a test's time budget; it
computes the same expressions in the same order as the NumPy form, and tests/test_oracle_golden.py
checks the two against each other.
"""
import numpy as np

try:
    import torch
except ImportError:  # the NumPy form needs nothing else
    torch = None


def is_torch(*arrays):
    return torch is not None and any(isinstance(a, torch.Tensor) for a in arrays)


def where(c, a, b):
    if is_torch(c, a, b):
        return torch.where(c, a, b)
    return np.where(c, a, b)


def fmin(cap, x):
    """np.fmin(cap, x) for a scalar cap."""
    if is_torch(x):
        return torch.clamp_max(x, cap)
    return np.fmin(cap, x)


def concat(seq, axis):
    if is_torch(*seq):
        return torch.cat(list(seq), dim=axis)
    return np.concatenate(seq, axis=axis)


def zeros_like(a):
    return torch.zeros_like(a) if is_torch(a) else np.zeros_like(a)


def zeros(shape, like):
    if is_torch(like):
        return torch.zeros(shape, dtype=like.dtype, device=like.device)
    return np.zeros(shape, dtype=like.dtype)


def arange(lo, hi, like):
    if is_torch(like):
        return torch.arange(lo, hi, device=like.device)
    return np.arange(lo, hi)


def size(a):
    return a.numel() if is_torch(a) else a.size


def log(a):
    return torch.log(a) if is_torch(a) else np.log(a)


def sqrt(a):
    return torch.sqrt(a) if is_torch(a) else np.sqrt(a)


def broadcast_to(a, shape):
    return torch.broadcast_to(a, shape) if is_torch(a) else np.broadcast_to(a, shape)


def to_torch(a, device, dtype=None):
    """A NumPy array (or tensor) as a tensor on ``device`` (FP64 unless ``dtype`` is given)."""
    dtype = dtype or torch.float64
    return torch.as_tensor(np.asarray(a) if not isinstance(a, torch.Tensor) else a, dtype=dtype, device=device)


def to_numpy(a):
    return a.detach().cpu().numpy() if is_torch(a) else np.asarray(a)
