"""Parity of the CUDA path (through the C ABI) with the oracle / reference golden vectors.

Tolerances are relative L2 norms of FP32 GPU results against FP64 references:
  * single operators on a random state ........................ 2e-6 (WENO operators 5e-6)
  * RK stage tendencies (the reference's tends tuple) ........... 1e-5
  * prognostic states: the error must stay within 1e-5 of the increment (state - initial
    state) plus the FP32 representation floor of the stored field, STATE_FLOOR * ||field||
    (theta is stored as theta - theta_ref, so its floor is taken on theta - theta_ref).
"""
import json
import os

import numpy as np
import pytest

from conftest import rel_l2, report_path

FIELDS = ("theta", "u", "v", "w", "pip", "qv")
REPORT = {}

pytestmark = pytest.mark.gpu


def _solver(g, turb=1, pairs=True):
    from lex_gb300.solver import Solver
    S = Solver(int(g["nx"]), int(g["ny"]), int(g["nz"]), float(g["dx"]), float(g["dy"]), float(g["dz"]),
               float(g["dt"]), int(g["n_sound"]), turb_opt=turb, acoustic_pairs=pairs)
    S.set_base_columns(g["col_theta0"], g["col_qv0"], g["col_pi0"], g["col_rho0"])
    return S


STATE_FLOOR = 1.2e-7   # two FP32 half-ulps, relative


def state_err(a, ref, a0, name, theta_ref=300.0):
    """||a - ref|| / (||ref - a0|| + floor); <= 1e-5 passes."""
    stored = ref - theta_ref if name == "theta" else ref
    denom = np.linalg.norm(ref - a0) + STATE_FLOOR / 1e-5 * np.linalg.norm(stored)
    return float(np.linalg.norm(a - ref) / max(denom, 1e-300))


def inner(a):
    return a[3:-3, 3:-3, 1:-1]


def inner_u(a):
    return a[3:-3, 3:-3, 1:-1]


@pytest.fixture(scope="module", autouse=True)
def report():
    yield
    with open(report_path("parity_report.json"), "w") as f:
        json.dump(REPORT, f, indent=1, sort_keys=True)


OPS = [  # diagnostic, golden key, slicer, tolerance
    ("mass_div", "mass_div", inner, 2e-6),
    ("theta_rho", "theta_rho", inner, 2e-7),
    ("adv_theta", "adv_theta", None, 5e-6),
    ("adv_qv", "adv_qv", None, 5e-6),
    ("adv_u", "adv_u", None, 5e-6),
    ("adv_v", "adv_v", None, 5e-6),
    ("adv_w", "adv_w", None, 5e-6),
    ("buoy_w", "buoy_w", None, 2e-6),
    ("pgf_u", "pgf_u", None, 2e-6),
    ("pgf_v", "pgf_v", None, 2e-6),
    ("pgf_w", "pgf_w", None, 2e-6),
    ("adv_pi", "adv_pi", None, 2e-6),
    ("n2", "n2", inner, 5e-6),
    ("km", "km", inner, 5e-6),
    ("sgs_u", "sgs_u", None, 5e-6),
    ("sgs_v", "sgs_v", None, 5e-6),
    ("sgs_w", "sgs_w", None, 5e-6),
    ("sgs_theta", "sgs_theta", None, 5e-6),
    ("sgs_qv", "sgs_qv", None, 5e-6),
]


@pytest.mark.parametrize("name,key,sl,tol", OPS, ids=[o[0] for o in OPS])
def test_operator_matches_reference(built_lib, ops_golden, name, key, sl, tol):
    g = ops_golden
    with _solver(g) as S:
        S.upload(tuple(g["in_" + f] for f in FIELDS))
        out = S.diagnose(name)
    ref = g[key] if sl is None else sl(g[key])
    assert out.shape == ref.shape
    err = rel_l2(out, ref)
    REPORT["op_" + name] = err
    assert err <= tol, (name, err)


def test_rk3_stages_match_reference(built_lib, ops_golden):
    g = ops_golden
    x0 = tuple(g["in_" + f] for f in FIELDS)
    with _solver(g) as S:
        S.upload(x0)
        S.step_record()
        for s in range(3):
            fields, tends = S.stage(s)
            for f, a, a0 in zip(FIELDS, fields, x0):
                ref = g["stage%d_%s" % (s, f)]
                err = state_err(a, ref, a0, f)
                REPORT["stage%d_%s" % (s, f)] = err
                assert err <= 1e-5, (s, f, err)
            # our tendencies come in field order (theta, u, v, w, pi', qv)
            for n, a in zip(("dtheta", "du", "dv", "dw", "dpip", "dqv"), tends):
                ref = g["stage%d_%s" % (s, n)]
                if ref.shape != a.shape:
                    ref = inner(ref) if n in ("dpip", "dw") else inner_u(ref)
                err = rel_l2(a, ref)
                REPORT["stage%d_%s" % (s, n)] = err
                assert err <= 1e-5, (s, n, err)


@pytest.mark.parametrize("pairs", [True, False], ids=["two_substeps_per_launch", "one_substep_per_launch"])
def test_step_matches_reference_graph_and_eager(built_lib, ops_golden, pairs):
    g = ops_golden
    x0 = tuple(g["in_" + f] for f in FIELDS)
    outs = []
    for graph in (False, True):
        with _solver(g, pairs=pairs) as S:
            S.upload(x0)
            S.step(1, graph=graph)
            outs.append(S.download())
    for f, a, b, a0 in zip(FIELDS, outs[0], outs[1], x0):
        np.testing.assert_array_equal(a, b)   # graph replay is bit-identical to eager launches
        ref = g["step_" + f]
        err = state_err(a, ref, a0, f)
        REPORT["step_%s_%s" % ("pairs" if pairs else "single", f)] = err
        assert err <= 1e-5, (f, err)


def test_warm_bubble_three_steps(built_lib, bubble_golden):
    g = bubble_golden
    x0 = tuple(g["in_" + f] for f in FIELDS)
    with _solver(g) as S:
        S.upload(x0)
        for n in range(1, 4):
            S.step(1)
            st = S.download()
            for f, a, a0 in zip(FIELDS, st, x0):
                ref = g["f64_step%d_%s" % (n, f)]
                err = state_err(a, ref, a0, f)
                f32 = state_err(g["f32_step%d_%s" % (n, f)], ref, a0, f)
                REPORT["bubble_step%d_%s" % (n, f)] = err
                REPORT["bubble_step%d_%s_reference_fp32" % (n, f)] = f32
                assert err <= 1e-5, (n, f, err)


def test_roundtrip_and_ghosts(built_lib, ops_golden):
    g = ops_golden
    x0 = tuple(g["in_" + f] for f in FIELDS)
    with _solver(g) as S:
        S.upload(x0)
        back = S.download()
    for f, a, b in zip(FIELDS, back, x0):
        # FP32 device storage (theta stored minus theta_ref): compare to FP32 rounding
        np.testing.assert_allclose(a, b, rtol=2e-7, atol=1e-9 if f != "theta" else 1e-6, err_msg=f)


def test_budget_and_finite(built_lib, bubble_golden):
    from oracle.ic import RD, CP, P00, REPSM1
    g = bubble_golden
    x0 = tuple(g["in_" + f] for f in FIELDS)
    with _solver(g) as S:
        S.upload(x0)
        b = S.budget()
        assert S.count_nonfinite() == 0
    th, u, v, w, pip, qv = (inner(a) for a in x0)
    pi = g["col_pi0"][1:-1][None, None, :] + pip
    rho = pi ** (CP / RD) * P00 / RD / ((1.0 + REPSM1 * qv) * (pi * th))
    dV = float(g["dx"] * g["dy"] * g["dz"])
    # the budget integrates the FP32-stored state in FP64: compare at the FP32 storage level
    assert abs(b["mass"] - rho.sum() * dV) / (rho.sum() * dV) < 1e-9
    assert abs(b["vapour"] - (rho * qv).sum() * dV) / ((rho * qv).sum() * dV) < 1e-7
    r0 = g["col_rho0"][1:-1][None, None, :]
    assert abs(b["rho_theta"] - (r0 * th).sum() * dV) / ((r0 * th).sum() * dV) < 1e-9
    assert b["kinetic"] == 0.0
    # total energy: internal cv T (T = pi theta) + potential g z at the cell centres + kinetic (0 at rest)
    from oracle.ic import CV, G
    z = (np.arange(th.shape[2]) + 0.5) * float(g["dz"])
    e = (rho * (CV * pi * th + G * z[None, None, :])).sum() * dV
    assert abs(b["total_energy"] - e) / e < 1e-9


def test_budgets_over_a_600_s_run(built_lib):
    """The FP64 budgets along 600 s of the 32^3 warm bubble (600 m x 600 m x 300 m, dt 3 s,
    Smagorinsky): the flux-form step conserves air mass to within 1e-6 and total energy (internal
    + potential + kinetic) to within 1e-5 of their initial values (measured: 1.8e-7 and 6.8e-7)."""
    from lex_gb300.solver import Solver
    from lex_gb300.workload import warm_bubble
    phys, prof = warm_bubble(32, 32, 32, 600.0, 600.0, 300.0, seed=1)
    with Solver(32, 32, 32, 600.0, 600.0, 300.0, 3.0, 32, turb_opt=1) as S:
        S.integrate_base_state(prof["theta0"], prof["qv0"])
        S.upload(phys, dtype=np.float32)
        b0 = S.budget()
        drift = {"mass": 0.0, "total_energy": 0.0}
        for _ in range(4):
            S.step(50)
            b = S.budget()
            for key in drift:
                drift[key] = max(drift[key], abs(b[key] - b0[key]) / abs(b0[key]))
        assert b["kinetic"] > 0.0
    assert drift["mass"] < 1e-6 and drift["total_energy"] < 1e-5, drift


def test_fp64_hydrostatic_base_state_on_gpu(built_lib):
    """lexgb_integrate_base_state (FP64 on the GPU) vs the oracle's hydrostatic integration."""
    from lex_gb300.solver import Solver
    from lex_gb300.workload import warm_bubble
    from oracle.ic import hydrostatic_columns
    nx, ny, nz, dz = 16, 16, 40, 250.0
    _, prof = warm_bubble(nx, ny, nz, 500.0, 500.0, dz)
    with Solver(nx, ny, nz, 500.0, 500.0, dz, 2.0) as S:
        pi0, rho0 = S.integrate_base_state(prof["theta0"], prof["qv0"])
    pr, rr = hydrostatic_columns(prof["theta0"], prof["qv0"], dz)
    REPORT["base_pi0"] = rel_l2(pi0, pr)
    REPORT["base_rho0"] = rel_l2(rho0, rr)
    assert rel_l2(pi0, pr) < 1e-14 and rel_l2(rho0, rr) < 1e-13


def test_warm_bubble_600s_32cube(built_lib):
    """600 s (200 RK3 steps) of the 32^3 warm bubble vs the reference run in FP64
    (tests/golden/bubble32_600s.npz): relative L2 of theta', qv', w and pi'."""
    from conftest import load_golden
    from lex_gb300.solver import Solver
    from lex_gb300.workload import warm_bubble
    g = load_golden("bubble32_600s.npz")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    dx, dy, dz, dt = float(g["dx"]), float(g["dy"]), float(g["dz"]), float(g["dt"])
    phys, prof = warm_bubble(nx, ny, nz, dx, dy, dz, seed=int(g["seed"]))
    with Solver(nx, ny, nz, dx, dy, dz, dt, int(g["n_sound"]), turb_opt=1) as S:
        S.integrate_base_state(prof["theta0"], prof["qv0"])
        S.upload(phys)
        S.step(int(g["nsteps"]))
        th, u, v, w, pip, qv = S.download()
        assert S.count_nonfinite() == 0
    qv0 = prof["qv0"][1:-1][None, None, :]
    errs = {"theta_p": rel_l2(inner(th) - 300.0, g["theta_p"]), "qv_p": rel_l2(inner(qv) - qv0, g["qv_p"]),
            "w": rel_l2(w[3:-3, 3:-3, 1:-1], g["w"]), "pip": rel_l2(inner(pip), g["pip"])}
    for k, e in errs.items():
        REPORT["bubble600s_" + k] = e
    # FP32 after 200 steps of a developing thermal: theta' and qv' within 1e-3, w within 2e-3
    assert errs["theta_p"] < 1e-3 and errs["qv_p"] < 1e-3 and errs["w"] < 2e-3, errs


@pytest.mark.parametrize("cor", [1, 2], ids=["coriolis", "coriolis_lspgrad"])
def test_coriolis_stages_match_reference(built_lib, cor):
    """cor_opt 1 and 2 (calculate_coriolis_force / _with_lspgrad, pressure_gradient_coriolis.py:80-113,
    added to R_u and R_v at one_step_integration.py:127-132): every stage tendency within 1e-5 of the
    reference's (tests/golden/ops_coriolis.npz) and the step within 1e-5 of its increment."""
    from conftest import load_golden
    from lex_gb300.solver import Solver
    g = load_golden("ops_coriolis.npz")
    x0 = tuple(g["in_" + f] for f in FIELDS)
    with Solver(int(g["nx"]), int(g["ny"]), int(g["nz"]), float(g["dx"]), float(g["dy"]), float(g["dz"]),
                float(g["dt"]), int(g["n_sound"]), turb_opt=1, cor_opt=cor, f_cor=float(g["f_cor"])) as S:
        S.set_base_columns(g["col_theta0"], g["col_qv0"], g["col_pi0"], g["col_rho0"])
        S.upload(x0)
        S.step_record()
        for s in range(3):
            _, tends = S.stage(s)
            for n, a in zip(("dtheta", "du", "dv", "dw", "dpip", "dqv"), tends):
                ref = g["cor%d_stage%d_%s" % (cor, s, n)]
                if ref.shape != a.shape:
                    ref = inner(ref)
                err = rel_l2(a, ref)
                REPORT["cor%d_stage%d_%s" % (cor, s, n)] = err
                assert err <= 1e-5, (cor, s, n, err)
        S.upload(x0)
        S.step(1)
        for f, a, a0 in zip(FIELDS, S.download(), x0):
            err = state_err(a, g["cor%d_step_%s" % (cor, f)], a0, f)
            REPORT["cor%d_step_%s" % (cor, f)] = err
            assert err <= 1e-5, (cor, f, err)
