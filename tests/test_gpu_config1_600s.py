"""600 s of the benchmarked workload (the 100 m warm bubble on 192 x 192 x 96, dt = 1 s, 600 big steps):
the library in FP32 against
  - the FP64 oracle run on the GPU (its torch form, one big step captured in a CUDA graph and
    replayed), theta' = theta - 300 K, qv' = qv - qv0, w and pi' on the whole grid, and
  - the reference's own FP64 run of the same 600 s (tests/golden/bubble192_600s.npz, made by
    tests/golden/make_golden.py --cases bubble192_600s with the reference source under the torch
    stand-in for jax): every 4th point of the four fields at 600 s, the x-z plane through the bubble
    centre and the fields' norms; the oracle's own distance to that run is checked too.
Bar (FP32 against FP64 after 600 steps of a developing thermal, stated here): relative L2 of theta'
and qv' below 1e-3, of w and pi' below 2e-3; the FP64 oracle against the FP64 reference run below
1e-6.  The measured errors go to config1_600s_report.json.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden, report_path

pytestmark = pytest.mark.gpu
NSTEPS = 600


def test_600s_192x192x96_against_the_fp64_oracle(built_lib):
    import torch
    from oracle.ic import Grid, hydrostatic_columns
    from oracle.dycore import Dycore
    from lex_gb300.solver import Solver
    from lex_gb300.workload import warm_bubble
    gref = load_golden("bubble192_600s.npz") if os.path.exists(os.path.join(GOLDEN, "bubble192_600s.npz")) else None
    seed = int(gref["seed"]) if gref is not None else None
    phys, prof = (warm_bubble(192, 192, 96, 100.0, 100.0, 100.0, seed=seed) if seed is not None
                  else warm_bubble(192, 192, 96, 100.0, 100.0, 100.0))
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
    bars = {"theta_p": 1e-3, "qv_p": 1e-3, "w": 2e-3, "pip": 2e-3}
    if gref is not None:   # the reference's own 600 s run
        lib = {"theta_p": out[0][inner] - 300.0, "qv_p": out[5][inner] - qv0, "w": out[3][3:-3, 3:-3, 1:-1],
               "pip": out[4][inner]}
        ora = {"theta_p": ref[0][inner] - 300.0, "qv_p": ref[5][inner] - qv0, "w": ref[3][3:-3, 3:-3, 1:-1],
               "pip": ref[4][inner]}
        vs = {}
        for k in bars:
            sub = gref["t600_%s_sub4" % k].astype(np.float64)
            xz = gref["t600_%s_xz" % k].astype(np.float64)
            vs[k] = {"library_points": rel(lib[k][::4, ::4, ::4], sub), "library_xz": rel(lib[k][:, 96, :], xz),
                     "library_norm": abs(np.linalg.norm(lib[k]) - float(gref["t600_%s_norm" % k]))
                     / float(gref["t600_%s_norm" % k]),
                     "oracle_points": rel(ora[k][::4, ::4, ::4], sub)}
        errs["vs_reference_run"] = vs
    with open(report_path("config1_600s_report.json"), "w") as f:
        json.dump(errs, f, indent=1)
    for k, bar in bars.items():
        assert errs[k] < bar, errs
    if gref is not None:
        for k, bar in bars.items():
            v = errs["vs_reference_run"][k]
            assert v["library_points"] < bar and v["library_xz"] < bar and v["library_norm"] < bar, (k, v)
            assert v["oracle_points"] < 1e-6, (k, v)
