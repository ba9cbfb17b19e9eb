"""Generate golden vectors by running the reference's own source (LEX) under the NumPy jax stand-in.

Run in a container that has the reference checkout (read-only); its path is the required argument:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py REF_DIR [--cases ...] [--long]

Writes tests/golden/*.npz.  The fixtures pin the oracle (oracle/dycore.py, oracle/ic.py)
to the reference, and feed the GPU parity tests; nothing at test time reads the reference.

Cases
  ops_random.npz   random padded state on a 16x12x8 grid (nx != ny): every operator on the
                   path (divergences, WENO advection of scalars/u/v/w, advection_pi, pressure
                   gradient, buoyancy, deformation, N^2, Smagorinsky tendencies), one full RK3
                   step with the three stages' states and tendencies (FP64).
  bubble_steps.npz the warm-bubble workload on a 16x16x12 grid at 600/600/300 m, dt=3 s:
                   interior fields after 1, 2, 3 RK3 steps in FP64, and the same from an FP32
                   run of the reference (to document its own FP32 drift).
  bubble32_600s.npz the 32x32x32 warm-bubble workload (600/600/300 m, dt = 3 s, Smagorinsky) after
                   600 s = 200 RK3 steps of the reference in FP64: theta - 300 K, qv - qv0, w and
                   pi' on the interior, stored as FP32.
  base_option1.npz the reference's own option-1 base state (setup_lex.py:74-146) columns,
                   pinning the hydrostatic integration of oracle/ic.py.
  dl_packing.npz   the learned correction's interface on a 16x12x8 grid: the network input the
                   reference's phys_state_tuple2array (dl_models.py:125-155) makes from a random
                   padded state and keepdims scaling_params, and the correction it applies
                   (correct_array2tuple + the scaling of one_sprint_functions.py:139-143) for a
                   random network output; output ranges vary with height only (w's not at all);
                   and the Laplacian of the training loss (dataset_generation.py:320-347) of a
                   random cell field.
"""
import os
import sys
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import jax_standin as js  # noqa: E402
from oracle.ic import WarmBubble, random_state  # noqa: E402

MODEL_OPT = (2, False, False, 0, False, False, 1)   # solver 2, Smagorinsky on, all else off
FIELDS = ("theta", "u", "v", "w", "pip", "qv")


def set_namelist(nl, nx, ny, nz, dx, dy, dz, dt, n_sound=32):
    nl.nx, nl.ny, nl.nz, nl.dx, nl.dy, nl.dz, nl.dt = nx, ny, nz, dx, dy, dz, dt
    nl.n_sound = n_sound
    nl.solver_opt, nl.turb_opt = 2, 1


def columns(base):
    rho0_theta0, rho0, theta0, pi0, qv0, _ = base
    return dict(col_theta0=theta0[0, 0], col_qv0=qv0[0, 0], col_pi0=pi0[0, 0], col_rho0=rho0[0, 0])


def case_ops(R, out):
    nl = R.nl
    nx, ny, nz, dx, dy, dz, dt = 16, 12, 8, 600.0, 500.0, 300.0, 3.0
    set_namelist(nl, nx, ny, nz, dx, dy, dz, dt)
    phys, base, grids = WarmBubble(nx, ny, nz, dx, dy, dz).build()
    state = random_state(phys, nx, ny, nz, seed=11)
    js.set_dtype(np.float64)
    c = js._cast_tree
    state, base, grids = c(state), c(base), c(grids)
    th, u, v, w, pip, qv = state
    _, rho0, theta0, pi0, qv0, _ = base
    x3d, y3d, z3d, x3d4u, y3d4v, z3d4w, cc1, cc2, _, _ = grids
    z2 = np.zeros((nx, ny))
    d = dict(nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, dt=dt, n_sound=32, **columns(base))
    for k, a in zip(FIELDS, state):
        d["in_" + k] = np.asarray(a)
    div = R.adv.get_divergence(rho0, u, v, w, x3d4u, y3d4v, z3d4w)
    d["mass_div"] = div
    d["vel_div"] = R.adv.get_divergence2(u, v, w, x3d4u, y3d4v, z3d4w)
    d["adv_theta"] = R.adv.advection_scalar(rho0, th, u, v, w, 1e-17, div, z2, x3d4u, y3d4v, z3d4w)
    d["adv_qv"] = R.adv.advection_scalar(rho0, qv, u, v, w, 1e-18, div, z2, x3d4u, y3d4v, z3d4w)
    d["adv_u"], d["adv_v"], d["adv_w"] = R.one.prep_momentum_eqn(rho0, u, v, w, div, z2, z2, x3d, y3d, z3d,
                                                                  x3d4u, y3d4v, z3d4w)
    d["adv_pi"] = R.adv.advection_pi(rho0, pi0, pip, u, v, w, x3d, y3d, z3d, cc1, cc2)
    trho = th * (1.0 + nl.reps * qv) / (1.0 + qv)
    d["theta_rho"] = trho
    d["pgf_u"], d["pgf_v"], d["pgf_w"] = R.pres_grad.pressure_gradient_force(pi0, pip, trho, x3d, y3d, z3d)
    d["buoy"], d["buoy_w"] = R.pres_eqn.calculate_buoyancy(theta0, th, qv0, qv)
    s11, s22, s33, s12, s13, s23, s2 = R.turb.compute_deformation(rho0, u, v, w, x3d, y3d, z3d, x3d4u, y3d4v, z3d4w)
    for k, a in zip(("s11", "s22", "s33", "s12", "s13", "s23", "s2"), (s11, s22, s33, s12, s13, s23, s2)):
        d["def_" + k] = a
    n2 = R.turb.compute_nm(th, pi0, qv, z3d)
    d["n2"] = n2
    km, kh = R.turb.compute_k(s2, n2, x3d4u, y3d4v, z3d4w)
    d["km"], d["kh"] = km, kh
    sg = R.turb.compute_smag(rho0, km, kh, s11, s22, s33, s12, s13, s23, th, qv, x3d, y3d, z3d, x3d4u, y3d4v, z3d4w)
    for k, a in zip(("u", "v", "w", "theta", "qv"), sg):
        d["sgs_" + k] = a
    # the three WS-RK3 stages of one big step (one_sprint_functions.py:17-21)
    xi1, t1, sfc, heat, sgs_t = R.one.rk_sub_step0(state, state, base, grids, MODEL_OPT, nl.dt / 3.0)
    xi2, t2 = R.one.rk_sub_step1(state, xi1, base, grids, heat, sfc, sgs_t, MODEL_OPT, nl.dt / 2.0)
    xi3, t3 = R.one.rk_sub_step2(state, xi2, base, grids, heat, sfc, sgs_t, MODEL_OPT, nl.dt)
    tnames = ("dtheta", "dpip", "du", "dv", "dw", "dqv")
    for s, (xi, tt) in enumerate(((xi1, t1), (xi2, t2), (xi3, t3))):
        for k, a in zip(FIELDS, xi):
            d["stage%d_%s" % (s, k)] = a
        for k, a in zip(tnames, tt):
            d["stage%d_%s" % (s, k)] = a
    step, _ = R.sp.ws_rk3_big_step(state, base, grids, MODEL_OPT)
    for k, a in zip(FIELDS, step):
        d["step_" + k] = a
    d = {k: np.asarray(v) for k, v in d.items()}
    np.savez_compressed(out, **d)


def case_bubble(R, out, nsteps=3):
    nl = R.nl
    nx, ny, nz, dx, dy, dz, dt = 16, 16, 12, 600.0, 600.0, 300.0, 3.0
    set_namelist(nl, nx, ny, nz, dx, dy, dz, dt)
    wb = WarmBubble(nx, ny, nz, dx, dy, dz)
    phys, base, grids = wb.build()
    d = dict(nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, dt=dt, n_sound=32, seed=wb.seed, **columns(base))
    for k, a in zip(FIELDS, phys):
        d["in_" + k] = a
    for tag, dtype in (("f64", np.float64), ("f32", np.float32)):
        js.set_dtype(dtype)
        st = phys
        for n in range(nsteps):
            st, _ = R.sp.ws_rk3_big_step(st, base, grids, MODEL_OPT)
            for k, a in zip(FIELDS, st):
                d["%s_step%d_%s" % (tag, n + 1, k)] = np.asarray(a, dtype=dtype)
    np.savez_compressed(out, **{k: np.asarray(v) for k, v in d.items()})


def case_bubble_600s(R, out, nsteps=200):
    nl = R.nl
    nx, ny, nz, dx, dy, dz, dt = 32, 32, 32, 600.0, 600.0, 300.0, 3.0
    set_namelist(nl, nx, ny, nz, dx, dy, dz, dt)
    wb = WarmBubble(nx, ny, nz, dx, dy, dz)
    phys, base, grids = wb.build()
    js.set_dtype(np.float64)
    st = phys
    for _ in range(nsteps):
        st, _ = R.sp.ws_rk3_big_step(st, base, grids, MODEL_OPT)
    th, u, v, w, pip, qv = (np.asarray(a) for a in st)
    qv0 = base[4]
    inner = (slice(3, -3), slice(3, -3), slice(1, -1))
    np.savez_compressed(out, nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, dt=dt, n_sound=32, seed=wb.seed,
                        nsteps=nsteps, theta_p=(th[inner] - 300.0).astype(np.float32),
                        qv_p=(qv[inner] - qv0[inner]).astype(np.float32),
                        w=w[3:-3, 3:-3, 1:-1].astype(np.float32), pip=pip[inner].astype(np.float32))


def case_base(R, out):
    nl = R.nl
    nx, ny, nz, dz = 4, 4, 40, 100.0
    set_namelist(nl, nx, ny, nz, 100.0, 100.0, dz, 1.0)
    js.set_dtype(np.float64)
    phys, base, grids, _ = R.setl.setup_grid_n_ic(1)
    rho0_theta0, rho0, theta0, pi0, qv0, _ = base
    np.savez_compressed(out, nz=nz, dz=dz, rho0=np.asarray(rho0)[0, 0], theta0=np.asarray(theta0)[0, 0],
                        pi0=np.asarray(pi0)[0, 0], qv0=np.asarray(qv0)[0, 0],
                        rho0_theta0=np.asarray(rho0_theta0)[0, 0])


def case_dl(R, ref_dir, out):
    """dl_models.py run under the stand-in: flax.linen and zarr are only needed for its class
    definitions and imports, so minimal stubs stand in for them."""
    import importlib.util
    import types
    linen = types.ModuleType("flax.linen")
    linen.Module = type("Module", (), {})
    linen.compact = lambda f: f
    flax = types.ModuleType("flax")
    flax.linen = linen
    sys.modules.setdefault("flax", flax)
    sys.modules.setdefault("flax.linen", linen)
    sys.modules.setdefault("zarr", types.ModuleType("zarr"))
    jnp = sys.modules["jax.numpy"]
    jnp.stack = np.stack
    jnp.unstack = np.unstack
    spec = importlib.util.spec_from_file_location("dl_models_reference", os.path.join(ref_dir, "dl_models.py"))
    dlm = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(dlm)
    nl = R.nl
    nx, ny, nz, dx, dy, dz, dt = 16, 12, 8, 600.0, 500.0, 300.0, 3.0
    set_namelist(nl, nx, ny, nz, dx, dy, dz, dt)
    js.set_dtype(np.float64)
    phys, _, grids = WarmBubble(nx, ny, nz, dx, dy, dz).build()
    state = random_state(phys, nx, ny, nz, seed=21)
    rng = np.random.default_rng(22)
    interior = lambda a, e: np.asarray(a)[3:3 + nx + e[0], 3:3 + ny + e[1], 1:1 + nz + e[2]]
    scaling = []
    for f, (a, e) in enumerate(zip((state[0], state[1], state[2], state[3], state[5]),
                                   ((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 0, 0)))):
        x = interior(a, e)
        lo = x - rng.uniform(0.1, 0.5, size=x.shape)
        rng_z = rng.uniform(0.5, 2.0, size=x.shape[2])          # output range: per level only,
        if f == 3:                                              # and for w the same on every level
            rng_z[:] = rng_z[0]
        scaling += [lo[None, None], (lo + rng_z[None, None, :])[None, None]]
    scaling += [np.zeros((1, 1, nx, ny, nz))] * 4               # Laplacian ranges (unused here)
    packed = np.asarray(dlm.phys_state_tuple2array(tuple(np.asarray(a) for a in state), tuple(scaling)))
    # the Laplacian of the training loss (dataset_generation.py:320-347) on a random cell field
    jnp.copy = js._simple(np.copy)
    spec = importlib.util.spec_from_file_location("dataset_generation_reference",
                                                  os.path.join(ref_dir, "dataset_generation.py"))
    dgen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(dgen)
    x3d, y3d, z3d, x3d4u, y3d4v, z3d4w = (np.asarray(a) for a in grids[:6])
    lap_in = rng.normal(size=(1, 1, nx, ny, nz))
    lap_out = np.asarray(dgen.laplace_of_tensor_jnp(x3d, x3d4u, y3d, y3d4v, z3d, z3d4w, js._cast_tree(lap_in)))
    corr = rng.normal(size=(nx, ny, nz, 5))
    th_c, u_c, v_c, w_c, q_c = (np.asarray(a) for a in dlm.correct_array2tuple(corr))
    mm = [(scaling[2 * f + 1] - scaling[2 * f]).squeeze() for f in range(5)]
    np.savez(out, nx=nx, ny=ny, nz=nz, **{"in_" + f: np.asarray(a) for f, a in zip(FIELDS, state)},
             **{"sc_%d" % i: a for i, a in enumerate(scaling[:10])}, packed=packed, corr=corr,
             out_theta=th_c * mm[0], out_u=u_c * mm[1], out_v=v_c * mm[2], out_w=w_c * mm[3], out_qv=q_c * mm[4],
             lap_in=lap_in[0, 0], lap_out=lap_out[0, 0], spacing=np.array([dx, dy, dz]))


def case_coriolis(R, out):
    """One big step of the ops_random state with Coriolis on (cor_opt 1 and 2, f = 1e-4): the three
    stages' tendencies, the step's result, and the Coriolis terms themselves (pressure_gradient_coriolis.py:80-113)."""
    nl = R.nl
    nx, ny, nz, dx, dy, dz, dt = 16, 12, 8, 600.0, 500.0, 300.0, 3.0
    set_namelist(nl, nx, ny, nz, dx, dy, dz, dt)
    nl.fCor = 1.0e-4
    phys, base, grids = WarmBubble(nx, ny, nz, dx, dy, dz).build()
    state = random_state(phys, nx, ny, nz, seed=11)
    js.set_dtype(np.float64)
    c = js._cast_tree
    state, base, grids = c(state), c(base), c(grids)
    d = dict(nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, dt=dt, n_sound=32, f_cor=nl.fCor, **columns(base))
    for k, a in zip(FIELDS, state):
        d["in_" + k] = np.asarray(a)
    tnames = ("dtheta", "dpip", "du", "dv", "dw", "dqv")
    for cor in (1, 2):
        mo = (2, False, False, cor, False, False, 1)
        f = R.pres_grad.calculate_coriolis_force if cor == 1 else R.pres_grad.calculate_coriolis_force_with_lspgrad
        fu, fv = f(state[1], state[2])
        d["cor%d_fu" % cor], d["cor%d_fv" % cor] = fu, fv
        xi1, t1, sfc, heat, sgs_t = R.one.rk_sub_step0(state, state, base, grids, mo, nl.dt / 3.0)
        xi2, t2 = R.one.rk_sub_step1(state, xi1, base, grids, heat, sfc, sgs_t, mo, nl.dt / 2.0)
        xi3, t3 = R.one.rk_sub_step2(state, xi2, base, grids, heat, sfc, sgs_t, mo, nl.dt)
        for s, tt in enumerate((t1, t2, t3)):
            for k, a in zip(tnames, tt):
                d["cor%d_stage%d_%s" % (cor, s, k)] = a
        for k, a in zip(FIELDS, xi3):     # the big step's result (padded)
            d["cor%d_step_%s" % (cor, k)] = a
    nl.fCor = 1.0e-4
    np.savez_compressed(out, **{k: np.asarray(v) for k, v in d.items()})


# ---------------------------------------------------------------------------------------------------------
# the 100 m warm bubble on 192 x 192 x 96 (dt = 1 s): reduced records, since whole fields would be ~14 MB each
# ---------------------------------------------------------------------------------------------------------
BIG = dict(nx=192, ny=192, nz=96, dx=100.0, dy=100.0, dz=100.0, dt=1.0)
NSAMPLE = 4096


def sample_index(shape, seed=7):
    """Seeded flat indices (C order) of NSAMPLE points of an array of ``shape``."""
    n = int(np.prod(shape))
    return np.sort(np.random.default_rng(seed + n % 9973).choice(n, NSAMPLE, replace=False))


def reduce_into(d, key, a):
    """FP64 summary of a whole interior field: L2 norm, sum, max |.|, and the values at seeded points."""
    a = np.asarray(a, dtype=np.float64)
    d[key + "_norm"] = np.linalg.norm(a)
    d[key + "_sum"] = a.sum()
    d[key + "_amax"] = np.abs(a).max()
    d[key + "_idx"] = sample_index(a.shape)
    d[key + "_at"] = a.reshape(-1)[d[key + "_idx"]]


def _np(a):
    return a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)


def case_bubble192_step(R, out):
    """One WS-RK3 big step of the 192 x 192 x 96 warm bubble (FP64, NumPy stand-in): per stage, the six
    tendencies (rk_sub_step0/1/2's tuple) and the six interior stage fields, each reduced."""
    nl = R.nl
    g = BIG
    set_namelist(nl, g["nx"], g["ny"], g["nz"], g["dx"], g["dy"], g["dz"], g["dt"])
    wb = WarmBubble(g["nx"], g["ny"], g["nz"], g["dx"], g["dy"], g["dz"])
    phys, base, grids = wb.build()
    js.set_dtype(np.float64)
    c = js._cast_tree
    state, base, grids = c(phys), c(base), c(grids)
    d = dict(seed=wb.seed, **g)
    xi1, t1, sfc, heat, sgs_t = R.one.rk_sub_step0(state, state, base, grids, MODEL_OPT, nl.dt / 3.0)
    xi2, t2 = R.one.rk_sub_step1(state, xi1, base, grids, heat, sfc, sgs_t, MODEL_OPT, nl.dt / 2.0)
    xi3, t3 = R.one.rk_sub_step2(state, xi2, base, grids, heat, sfc, sgs_t, MODEL_OPT, nl.dt)
    tnames = ("dtheta", "dpip", "du", "dv", "dw", "dqv")
    inner = {"theta": (slice(3, -3), slice(3, -3), slice(1, -1)), "u": (slice(3, -3), slice(3, -3), slice(1, -1)),
             "v": (slice(3, -3), slice(3, -3), slice(1, -1)), "w": (slice(3, -3), slice(3, -3), slice(1, -1)),
             "pip": (slice(3, -3), slice(3, -3), slice(1, -1)), "qv": (slice(3, -3), slice(3, -3), slice(1, -1))}
    for s, (xi, tt) in enumerate(((xi1, t1), (xi2, t2), (xi3, t3))):
        for k, a in zip(tnames, tt):
            a = np.asarray(a)
            if a.shape[1] >= g["ny"] + 6:       # u, v, w and pi' tendencies come padded
                a = a[3:-3, 3:-3, 1:-1]
            reduce_into(d, "stage%d_%s" % (s, k), a)
        for k, a in zip(FIELDS, xi):
            a = np.asarray(a)[inner[k]]
            reduce_into(d, "stage%d_%s" % (s, k), a - 300.0 if k == "theta" else a)
    np.savez_compressed(out, **{k: np.asarray(v) for k, v in d.items()})


def case_bubble192_600s(R, jt, out, checkpoint=None, nsteps=600):
    """600 s (600 RK3 steps) of the 192 x 192 x 96 warm bubble under the torch stand-in (FP64): norms at
    60, 300 and 600 s, and at 600 s the x-z plane through the bubble centre (j = 96) and every 4th point
    of theta - 300 K, qv - qv0, w and pi' (FP32).  Resumable from ``checkpoint`` (a state file)."""
    import time
    import torch
    nl = R.nl
    g = BIG
    set_namelist(nl, g["nx"], g["ny"], g["nz"], g["dx"], g["dy"], g["dz"], g["dt"])
    wb = WarmBubble(g["nx"], g["ny"], g["nz"], g["dx"], g["dy"], g["dz"])
    phys, base, grids = wb.build()
    qv0 = base[4][3:-3, 3:-3, 1:-1]
    st, bt, gt = jt.tree(phys), jt.tree(base), jt.tree(grids)
    d = dict(seed=wb.seed, nsteps=nsteps, **g)
    n0 = 0
    if checkpoint and os.path.exists(checkpoint):
        with np.load(checkpoint) as z:
            n0 = int(z["n"])
            st = tuple(torch.as_tensor(z[k]) for k in FIELDS)
            d.update({k: z[k] for k in z.files if k[0] == "t" and k[1:2].isdigit()})

    def record(n, st):
        th, u, v, w, pip, qv = (_np(a) for a in st)
        inner = (slice(3, -3), slice(3, -3), slice(1, -1))
        f = {"theta_p": th[inner] - 300.0, "qv_p": qv[inner] - qv0, "w": w[3:-3, 3:-3, 1:-1], "pip": pip[inner],
             "u": u[3:-3, 3:-3, 1:-1], "v": v[3:-3, 3:-3, 1:-1]}
        for k, a in f.items():
            d["t%d_%s_norm" % (n, k)] = np.linalg.norm(a)
            d["t%d_%s_amax" % (n, k)] = np.abs(a).max()
        if n == nsteps:
            for k in ("theta_p", "qv_p", "w", "pip"):
                d["t%d_%s_xz" % (n, k)] = f[k][:, g["ny"] // 2, :].astype(np.float32)
                d["t%d_%s_sub4" % (n, k)] = f[k][::4, ::4, ::4].astype(np.float32)

    with torch.no_grad():
        for n in range(n0 + 1, nsteps + 1):
            t0 = time.time()
            st, _ = R.sp.ws_rk3_big_step(st, bt, gt, MODEL_OPT)
            if n in (60, 300, nsteps):
                record(n, st)
            if checkpoint and (n % 20 == 0 or n == nsteps):
                tmp = checkpoint + ".tmp.npz"
                np.savez(tmp, n=n, **{k: _np(a) for k, a in zip(FIELDS, st)},
                         **{k: v for k, v in d.items() if k[0] == "t" and k[1:2].isdigit()})
                os.replace(tmp, checkpoint)
            print("step %d %.1f s" % (n, time.time() - t0), flush=True)
    np.savez_compressed(out, **{k: np.asarray(v) for k, v in d.items()})


def case_adjoint(R, jt, out):
    """torch.autograd through the reference's ws_rk3_big_step (torch stand-in, FP64) as the stand-in for
    jax.vjp: on the ops_random state (16 x 12 x 8, Smagorinsky on), the adjoint of the interior state for
    seeded output seeds, after one big step and after a three-step rollout, with cor_opt 0 and 1.  The
    same reverse mode run in FP32 is compared with it too: ``..._fp32err_<field>`` is the relative L2
    difference of the reference's own FP32 adjoint from its FP64 adjoint (w on faces 1..nz-1).

    Inputs and outputs are in the device layout of the library (interior only, x fastest: [z][y][x],
    u and v without the duplicated periodic face, w on the nz+1 faces): the padding the reference applies
    to its inputs (padding3*_array) is part of the differentiated function, so its adjoint folds the ghost
    cells back onto the interior values they copy."""
    import torch
    from oracle.ic import pad_scalar, pad_u, pad_v
    nl = R.nl
    nx, ny, nz, dx, dy, dz, dt = 16, 12, 8, 600.0, 500.0, 300.0, 3.0
    set_namelist(nl, nx, ny, nz, dx, dy, dz, dt)
    nl.fCor = 1.0e-4
    phys, base, grids = WarmBubble(nx, ny, nz, dx, dy, dz).build()
    state = random_state(phys, nx, ny, nz, seed=11)
    bt, gt = jt.tree(base), jt.tree(grids)
    inner = (slice(3, -3), slice(3, -3), slice(1, -1))

    def to_dev(k, a):   # padded reference array -> device layout [z][y][x]
        a = a[inner]
        if k == "u":
            a = a[:-1]
        elif k == "v":
            a = a[:, :-1]
        return a.permute(2, 1, 0) if hasattr(a, "permute") else np.transpose(a, (2, 1, 0))

    def from_dev(k, a):  # device layout -> padded reference array (differentiable)
        a = a.permute(2, 1, 0)
        if k == "u":
            return pad_u(torch.cat((a, a[:1]), 0))
        if k == "v":
            return pad_v(torch.cat((a, a[:, :1]), 1))
        return pad_scalar(a)

    x0 = [torch.as_tensor(np.ascontiguousarray(to_dev(k, np.asarray(a)))) for k, a in zip(FIELDS, state)]
    rng = np.random.default_rng(31)
    ybar = [torch.as_tensor(rng.standard_normal(tuple(x.shape))) for x in x0]
    ybar[3][0] = 0.0      # w on the bottom and lid faces is zero by construction
    ybar[3][-1] = 0.0
    d = dict(nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, dt=dt, n_sound=32, f_cor=nl.fCor, **columns(base))
    for k, x in zip(FIELDS, x0):
        d["x_" + k] = x.numpy()
    for k, y in zip(FIELDS, ybar):
        d["ybar_" + k] = y.numpy()
    def vjp(cor, nsteps, dtype):
        jt.set_dtype(dtype)
        b, g_ = jt.tree(base), jt.tree(grids)
        xs = [x.to(dtype).clone().requires_grad_(True) for x in x0]
        st = tuple(from_dev(k, x) for k, x in zip(FIELDS, xs))
        for _ in range(nsteps):
            st, _ = R.sp.ws_rk3_big_step(st, b, g_, (2, False, False, cor, False, False, 1))
        y = [to_dev(k, a) for k, a in zip(FIELDS, st)]
        dot = sum((a * yb.to(dtype)).sum() for a, yb in zip(y, ybar))
        return y, torch.autograd.grad(dot, xs)

    for cor in (0, 1):
        for nsteps in (1, 3):
            y, gr = vjp(cor, nsteps, torch.float64)
            _, g32 = vjp(cor, nsteps, torch.float32)
            for k, a, gg, g4 in zip(FIELDS, y, gr, g32):
                d["cor%d_n%d_y_%s" % (cor, nsteps, k)] = a.detach().numpy()
                d["cor%d_n%d_xbar_%s" % (cor, nsteps, k)] = gg.numpy()
                ref, got = gg.numpy(), g4.double().numpy()
                if k == "w":
                    ref, got = ref[1:-1], got[1:-1]
                d["cor%d_n%d_fp32err_%s" % (cor, nsteps, k)] = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    jt.set_dtype(torch.float64)
    np.savez_compressed(out, **{k: np.asarray(v) for k, v in d.items()})


FAST = ("ops", "bubble", "base", "dl", "coriolis")


def main(argv):
    import argparse
    ap = argparse.ArgumentParser(description="golden vectors from the reference's own source")
    ap.add_argument("ref_dir", help="checkout of the reference (read-only)")
    ap.add_argument("--cases", default=",".join(FAST),
                    help="comma-separated: ops, bubble, base, dl, coriolis (fast); bubble32_600s, "
                         "bubble192_step (about 2 min), bubble192_600s (hours; torch stand-in), adjoint")
    ap.add_argument("--long", action="store_true", help="also bubble32_600s (the original long case)")
    ap.add_argument("--checkpoint", default=None, help="bubble192_600s: resumable state file")
    ap.add_argument("--threads", type=int, default=0, help="torch CPU threads for the torch stand-in cases")
    a = ap.parse_args(argv)
    cases = [c for c in a.cases.split(",") if c]
    if a.long:
        cases.append("bubble32_600s")
    torch_cases = [c for c in cases if c in ("bubble192_600s", "adjoint")]
    numpy_cases = [c for c in cases if c not in torch_cases]
    if numpy_cases and torch_cases:
        raise SystemExit("the NumPy and torch stand-ins cannot share a process: run the torch cases separately")
    if numpy_cases:
        R = js.load_reference(a.ref_dir)
        out = lambda n: os.path.join(HERE, n)
        for c in numpy_cases:
            {"ops": lambda: case_ops(R, out("ops_random.npz")),
             "bubble": lambda: case_bubble(R, out("bubble_steps.npz")),
             "base": lambda: case_base(R, out("base_option1.npz")),
             "dl": lambda: case_dl(R, a.ref_dir, out("dl_packing.npz")),
             "coriolis": lambda: case_coriolis(R, out("ops_coriolis.npz")),
             "bubble32_600s": lambda: case_bubble_600s(R, out("bubble32_600s.npz")),
             "bubble192_step": lambda: case_bubble192_step(R, out("bubble192_step.npz"))}[c]()
    if torch_cases:
        import torch
        import jax_standin_torch as jt
        if a.threads:
            torch.set_num_threads(a.threads)
        R = jt.load_reference(a.ref_dir)
        for c in torch_cases:
            if c == "bubble192_600s":
                case_bubble192_600s(R, jt, os.path.join(HERE, "bubble192_600s.npz"), a.checkpoint)
            else:
                case_adjoint(R, jt, os.path.join(HERE, "adjoint_vjp.npz"))


if __name__ == "__main__":
    main(sys.argv[1:])
