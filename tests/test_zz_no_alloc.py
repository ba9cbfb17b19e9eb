"""lexgb_budget_noalloc: the budget entry point for callers that cannot allocate device memory
(code inside a framework that owns all device memory through its own pool, work being
recorded into a CUDA graph, loops that cannot take cudaMalloc's implicit synchronisation).

It is called through the C ABI on a state held in device memory and must agree with the
allocating entry point lexgb_budget on two calls in a row (both sum the same FP64 per-cell
contributions in a different order: 1e-12 relative).  This file is collected last so that a
run stopping at the first failure has already run every other test; it also passes alone.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("mass", "vapour", "kinetic", "rho_theta")


def test_budget_noalloc_matches_budget_on_two_calls(built_lib):
    import torch
    from lex_gb300 import _lib
    from lex_gb300.solver import Solver
    from lex_gb300.workload import warm_bubble

    nx, ny, nz, dx, dy, dz = 64, 48, 40, 300.0, 300.0, 150.0
    phys, prof = warm_bubble(nx, ny, nz, dx, dy, dz)
    with Solver(nx, ny, nz, dx, dy, dz, 2.0, 32, turb_opt=1) as S:
        pi0, rho0 = S.integrate_base_state(prof["theta0"], prof["qv0"])
        S.upload(phys)
        S.step(2)                 # winds and pi' become non-zero
        S.synchronize()           # the solver's stream does not order with the default stream
        ref = S.budget()
        fields = (ctypes.c_void_p * 6)(*S.device_ptrs())
        # the caller owns the inputs and the output; the entry point allocates nothing
        rho_d = torch.tensor(rho0, dtype=torch.float64, device="cuda")
        pi_d = torch.tensor(pi0, dtype=torch.float64, device="cuda")
        out = torch.empty(4, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        theta_ref = float(prof["theta0"][1])   # the solver's default theta_ref (theta0 at level 1)
        for call in range(2):
            out.fill_(float("nan"))
            torch.cuda.synchronize()
            rc = built_lib.lexgb_budget_noalloc(nx, ny, nz, dx, dy, dz, theta_ref, fields, rho_d.data_ptr(),
                                                pi_d.data_ptr(), out.data_ptr(), None)
            assert rc == 0, _lib.last_error()
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            for k, key in enumerate(KEYS):
                assert np.isfinite(got[k]), (call, key)
                assert abs(got[k] - ref[key]) <= 1e-12 * abs(ref[key]), (call, key, got[k], ref[key])


def test_budget_noalloc_rejects_grids_beyond_its_scratch(built_lib):
    from lex_gb300 import _lib
    fields = (ctypes.c_void_p * 6)(*([1] * 6))   # never dereferenced: rejected before any launch
    rc = built_lib.lexgb_budget_noalloc(512, 512, 128, 100.0, 100.0, 100.0, 300.0, fields, 1, 1, 1, None)
    assert rc == _lib.LEXGB_ERR_ARG
    assert "exceed the maximum" in _lib.last_error()
