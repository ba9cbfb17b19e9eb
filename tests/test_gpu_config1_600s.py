"""600 s of the benchmarked workload (the 100 m warm bubble on 192 x 192 x 96, dt = 1 s, 600 big steps):
the library in FP32 against the FP64 oracle run on the GPU (its torch form, one big step captured in a
CUDA graph and replayed; the oracle is pinned to the reference's own code at this size by
test_gpu_config1.py).  theta' = theta - 300 K, qv' = qv - qv0, w and pi' on the whole grid.

Bar (FP32 against FP64 after 600 steps of a developing thermal, stated here): relative L2 of theta'
and qv' below 1e-3, of w and pi' below 2e-3.  The measured errors go to config1_600s_report.json.
"""
import json

import numpy as np
import pytest

from conftest import report_path

pytestmark = pytest.mark.gpu
NSTEPS = 600


def test_600s_192x192x96_against_the_fp64_oracle(built_lib):
    import torch
    from oracle.ic import Grid, hydrostatic_columns
    from oracle.dycore import Dycore
    from lex_gb300.solver import Solver
    from lex_gb300.workload import warm_bubble
    phys, prof = warm_bubble(192, 192, 96, 100.0, 100.0, 100.0)
    pi0, rho0 = hydrostatic_columns(prof["theta0"], prof["qv0"], 100.0)
    cols = dict(theta0=prof["theta0"], qv0=prof["qv0"], pi0=pi0, rho0=rho0)
    with Solver(192, 192, 96, 100.0, 100.0, 100.0, 1.0, 32, turb_opt=1) as S:
        S.set_base_columns(cols["theta0"], cols["qv0"], cols["pi0"], cols["rho0"])
        S.upload(phys)
        S.step(NSTEPS)
        out = S.download()
        assert S.count_nonfinite() == 0
    D = Dycore(Grid(192, 192, 96, 100.0, 100.0, 100.0), cols, 1.0, 32, device="cuda")
    x = tuple(t.clone() for t in D.cast(phys))
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        D.step(x)
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        y, _ = D.step(x)
    for a, b in zip(x, D.cast(phys)):
        a.copy_(b)
    for n in range(NSTEPS):
        g.replay()
        if n + 1 < NSTEPS:
            for a, b in zip(x, y):
                a.copy_(b)
    ref = [t.cpu().numpy() for t in y]
    inner = (slice(3, -3), slice(3, -3), slice(1, -1))
    qv0 = prof["qv0"][1:-1][None, None, :]
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    errs = {"theta_p": rel(out[0][inner] - 300.0, ref[0][inner] - 300.0),
            "qv_p": rel(out[5][inner] - qv0, ref[5][inner] - qv0),
            "w": rel(out[3][3:-3, 3:-3, 1:-1], ref[3][3:-3, 3:-3, 1:-1]),
            "pip": rel(out[4][inner], ref[4][inner]),
            "max_w_oracle": float(np.abs(ref[3]).max()), "max_theta_p_oracle": float((ref[0][inner] - 300.0).max())}
    with open(report_path("config1_600s_report.json"), "w") as f:
        json.dump(errs, f, indent=1)
    assert errs["theta_p"] < 1e-3 and errs["qv_p"] < 1e-3, errs
    assert errs["w"] < 2e-3 and errs["pip"] < 2e-3, errs
