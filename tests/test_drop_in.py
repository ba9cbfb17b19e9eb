"""The drop-in sprint API (lex_gb300/one_sprint_functions.py) mirrors one_sprint_functions.py:
argument checking and the surface tuple on the CPU, the integration itself on the GPU."""
import types

import numpy as np
import pytest

from conftest import load_golden
from test_gpu_parity import FIELDS, state_err

OK = (2, 0, 0, 0, 0, 0, 1)


def namelist(g, sprint_n=1):
    return types.SimpleNamespace(nx=int(g["nx"]), ny=int(g["ny"]), nz=int(g["nz"]), dx=float(g["dx"]),
                                 dy=float(g["dy"]), dz=float(g["dz"]), dt=float(g["dt"]),
                                 n_sound=int(g["n_sound"]), sprint_n=sprint_n, fCor=1.0e-4)


def base_state(g):
    nx, ny = int(g["nx"]) + 6, int(g["ny"]) + 6
    col = lambda c: np.broadcast_to(np.asarray(c, dtype=np.float64), (nx, ny, c.size)).copy()
    rho0, th0 = col(g["col_rho0"]), col(g["col_theta0"])
    return (rho0 * th0, rho0, th0, col(g["col_pi0"]), col(g["col_qv0"]), np.zeros((nx - 6, ny - 6)))


@pytest.mark.parametrize("opt,exc", [((1, 0, 0, 0, 0, 0, 1), NotImplementedError),
                                     ((3, 0, 0, 0, 0, 0, 1), NotImplementedError),
                                     ((2, 1, 0, 0, 0, 0, 1), NotImplementedError),
                                     ((2, 0, 1, 0, 0, 0, 1), NotImplementedError),
                                     ((2, 0, 0, 0, 1, 0, 1), NotImplementedError),
                                     ((2, 0, 0, 0, 0, 0, 2), NotImplementedError),
                                     ((2, 0, 0, 3, 0, 0, 1), ValueError),
                                     ((2, 0, 0, 0, 0, 0), ValueError)])
def test_model_opt_outside_the_gpu_path_is_refused(opt, exc):
    from lex_gb300 import one_sprint_functions as sp
    with pytest.raises(exc):
        sp.check_model_opt(opt)


def test_first_step_flux_is_the_zero_surface_tuple():
    from lex_gb300 import one_sprint_functions as sp
    g = load_golden("bubble_steps.npz")
    sp.configure(namelist(g))
    sfc = sp.get_first_step_flux(None, None, None, OK)
    assert len(sfc) == 9 and sfc[0] == -999 and sfc[1] == -999   # one_step_integration.py:181-186
    for a in sfc[2:]:
        assert a.shape == (int(g["nx"]), int(g["ny"])) and not a.any()


@pytest.mark.gpu
def test_big_step_and_sprint_match_reference(built_lib):
    from lex_gb300 import one_sprint_functions as sp
    g = load_golden("bubble_steps.npz")
    x0 = tuple(g["in_" + f].copy() for f in FIELDS)
    keep = tuple(a.copy() for a in x0)
    base = base_state(g)
    sp.configure(namelist(g, sprint_n=2))
    x1, sfc = sp.ws_rk3_big_step(x0, base, None, OK)
    assert len(sfc) == 9
    for f, a, a0, k in zip(FIELDS, x1, x0, keep):
        np.testing.assert_array_equal(a0, k)            # inputs are not modified
        assert state_err(a, g["f64_step1_" + f], a0, f) <= 1e-5, f
    x3, _ = sp.ws_rk3_sprint(x1, base, None, OK)         # resident state: no upload
    for f, a, a0 in zip(FIELDS, x3, x0):
        assert state_err(a, g["f64_step3_" + f], a0, f) <= 1e-5, f
    sp.configure(namelist(g))                            # releases the solver


def _flax_params(seed, scale=0.05):
    """Random simpleCNN parameters in flax's layout: kernel [3, 3, 3, cin, cout] over (x, y, z)."""
    rng = np.random.default_rng(seed)
    p = {}
    for li, (cin, cout) in enumerate([(5, 32), (32, 32), (32, 32), (32, 5)]):
        p["Conv_%d" % li] = {"kernel": rng.normal(0, (2.0 / (27 * cin)) ** 0.5, (3, 3, 3, cin, cout)) *
                             (scale if li == 3 else 1.0), "bias": rng.normal(0, 0.01, cout)}
    return p


def _flax_conv(x, k, b):
    """flax nn.Conv (cross-correlation, zero 'SAME' padding) on x [X][Y][Z][cin], float64."""
    X, Y, Z, _ = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((X, Y, Z, k.shape[4])) + b
    for a in range(3):
        for c in range(3):
            for e in range(3):
                out += np.einsum("xyzi,io->xyzo", xp[a:a + X, c:c + Y, e:e + Z], k[a, c, e])
    return out


def test_flax_kernels_convert_to_the_library_layout():
    torch = pytest.importorskip("torch")
    from lex_gb300 import one_sprint_functions as sp
    k = _flax_params(3)["Conv_1"]["kernel"][:, :, :, :16, :8]
    # the conversion of _sgs_tensors, on the CPU
    w = k.transpose(2, 1, 0, 4, 3).reshape(27, 8, 16)
    x = np.random.default_rng(4).normal(size=(6, 5, 4, 16))        # [x][y][z][c]
    ref = _flax_conv(x, k, np.zeros(8))
    # the library's convolution: device layout [z][y][x][c], weights [27][cout][cin] with the
    # offset (dz+1)*9 + (dy+1)*3 + (dx+1), as torch conv3d over (z, y, x)
    wt = torch.tensor(w).reshape(3, 3, 3, 8, 16).permute(3, 4, 0, 1, 2)
    xt = torch.tensor(x.transpose(2, 1, 0, 3)).permute(3, 0, 1, 2).unsqueeze(0)
    out = torch.nn.functional.conv3d(xt, wt, padding=1)[0].permute(3, 2, 1, 0).numpy()
    assert np.abs(out - ref).max() < 1e-10
    assert callable(sp.ws_rk3_sprint_dl)


@pytest.mark.gpu
def test_sprint_dl_applies_the_correction_inside_the_step(built_lib):
    import torch
    from lex_gb300 import one_sprint_functions as sp
    g = load_golden("bubble_steps.npz")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    assert nx % 16 == 0
    x0 = tuple(g["in_" + f].copy() for f in FIELDS)
    base = base_state(g)
    sp.configure(namelist(g, sprint_n=1))            # one corrected step: pi' stays the plain step's
    plain, _ = sp.ws_rk3_sprint(x0, base, None, OK)
    # scaling_params with keepdims shapes; ranges from the input state's interior
    inner = lambda a, ex=(0, 0, 0): a[3:3 + nx + ex[0], 3:3 + ny + ex[1], 1:1 + nz + ex[2]][None, None]
    sc = []
    for a, ex in zip((x0[0], x0[1], x0[2], x0[3], x0[5]), ((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 0, 0))):
        sc += [inner(a, ex) - 0.5, inner(a, ex) + 0.5]
    zero = _flax_params(5, scale=0.0)
    for li in range(4):
        zero["Conv_%d" % li]["bias"][:] = 0.0
    same, _ = sp.ws_rk3_sprint_dl(x0, base, None, OK, zero, tuple(sc))
    for a, b in zip(same, plain):                  # a zero network changes nothing
        assert np.array_equal(a, b)
    corr, _ = sp.ws_rk3_sprint_dl(x0, base, None, OK, _flax_params(5), tuple(sc))
    d = [float(np.abs(a - b).max()) for a, b in zip(corr, plain)]
    assert all(np.isfinite(a).all() for a in corr)
    assert d[0] > 0 and d[1] > 0 and d[3] > 0 and d[5] > 0 and d[4] == 0.0, d   # pi' is not corrected
    again, _ = sp.ws_rk3_sprint(x0, base, None, OK)    # the plain sprint detaches the network
    for a, b in zip(again, plain):
        assert np.array_equal(a, b)


def test_scaling_params_convert_to_the_library_layout():
    from lex_gb300 import one_sprint_functions as sp
    nx, ny, nz = 4, 3, 5
    r = np.random.default_rng(7)
    shapes = [(nx, ny, nz), (nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1), (nx, ny, nz)]
    sc = []
    for shp in shapes:                                   # keepdims shapes of dataset_generation.py:81-90
        mn = r.normal(size=shp)[None, None]
        sc += [mn, mn + r.uniform(0.5, 2.0, size=shp)[None, None]]
    ws, bs, out = sp.sgs_arrays(_flax_params(1), tuple(sc) + (None,) * 4, nx, ny, nz)
    assert [w.shape for w in ws] == [(27, 32, 16), (27, 32, 32), (27, 32, 32), (27, 8, 32)]
    assert not ws[0][:, :, 5:].any() and not ws[3][:, 5:, :].any() and not bs[3][5:].any()
    assert out["lo"].shape == (5, nz + 1) and out["rout"].shape == (5, nz + 1, ny, nx)
    top = lambda a: np.append(a, a[-1])                  # entry nz repeats the top level but for w
    lvl = lambda a: np.concatenate([a, a[:, :, -1:]], axis=2)
    th_min, th_max = sc[0][0, 0], sc[1][0, 0]
    assert np.allclose(out["lo"][0], top(th_min.min(axis=(0, 1))))
    assert np.allclose(out["rin"][0], top(th_max.max(axis=(0, 1)) - th_min.min(axis=(0, 1)) + 0.01))
    assert np.allclose(out["rout"][0], lvl(th_max - th_min).transpose(2, 1, 0))
    w_min, w_max = sc[6][0, 0], sc[7][0, 0]                # w per face level, faces 0..nz
    assert np.allclose(out["lo"][3], w_min.min(axis=(0, 1)))
    assert np.allclose(out["rout"][3], (w_max - w_min).transpose(2, 1, 0))
    ru = sc[3][0, 0] - sc[2][0, 0]                          # u on x faces 0..nx-1
    assert np.allclose(out["rout"][1], lvl(ru[:nx]).transpose(2, 1, 0))
    q_min, q_max = sc[8][0, 0], sc[9][0, 0]
    assert np.allclose(out["rin"][4], top(q_max.max(axis=(0, 1)) - q_min.min(axis=(0, 1)) + 1e-5))


def test_dl_packing_matches_the_reference():
    """The network input and the applied correction against the reference's own
    phys_state_tuple2array / correct_array2tuple (tests/golden/dl_packing.npz), all five channels and
    every stored face (u and v faces 0..nx-1 / 0..ny-1: the reference's correction also changes the
    duplicated periodic face nx / ny, to the value of face 1, which the device layout does not store)."""
    torch = pytest.importorskip("torch")
    from lex_gb300 import one_sprint_functions as sp, sgs_cnn
    g = load_golden("dl_packing.npz")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    _, _, sc = sp.sgs_arrays(_flax_params(0, scale=0.0), tuple(g["sc_%d" % i] for i in range(10)), nx, ny, nz)
    scale = {k: torch.tensor(v) for k, v in sc.items()}
    ext = {"theta": (0, 0, 0), "u": (0, 0, 0), "v": (0, 0, 0), "w": (0, 0, 1), "pip": (0, 0, 0), "qv": (0, 0, 0)}
    state = tuple(torch.tensor(np.ascontiguousarray(
        g["in_" + f][3:3 + nx + e[0], 3:3 + ny + e[1], 1:1 + nz + e[2]].transpose(2, 1, 0))) for f, e in ext.items())
    x = sgs_cnn.pack(state, scale).numpy().reshape(nz, ny, nx, 5).transpose(2, 1, 0, 3)
    ref = g["packed"][0]
    for c in range(5):
        assert np.allclose(x[..., c], ref[..., c], rtol=1e-12, atol=1e-12), c
    corr = torch.tensor(np.ascontiguousarray(g["corr"].transpose(2, 1, 0, 3).reshape(-1, 5)))
    d = [a.numpy() for a in sgs_cnn.unpack(corr, scale, (nx, ny, nz))]
    t = lambda a: a.transpose(2, 1, 0)
    assert np.allclose(d[0], t(g["out_theta"]), rtol=1e-12, atol=1e-12)
    assert np.allclose(d[5], t(g["out_qv"]), rtol=1e-12, atol=1e-12)
    assert np.allclose(d[1], t(g["out_u"][:nx]), rtol=1e-12, atol=1e-12)
    assert np.allclose(d[2], t(g["out_v"][:, :ny]), rtol=1e-12, atol=1e-12)
    assert np.allclose(d[3], t(g["out_w"]), rtol=1e-12, atol=1e-12)
    assert not d[4].any()


@pytest.mark.gpu
def test_relay_sequence_keeps_the_state_on_the_device(built_lib, tmp_path):
    """lex_relay.py's calls (lex_relay.py:17-61) through the drop-in on the 32^3 warm bubble at
    600 m / dt 3 s for 600 s (the CPU-runnable case): get_first_step_flux, save2nc_base, save2nc, then
    sprints of 20 steps with a save every 5 sprints.  The state stays on the device between sprints:
    one host copy of the six fields per save and none in between.  The final state matches the
    reference's own 600 s run (tests/golden/bubble32_600s.npz) as test_gpu_parity's 600 s case does;
    a state read after later sprints (kept by the caller) still holds its own values; host copies
    are read-only."""
    from lex_gb300 import one_sprint_functions as sp, write_netcdf as write
    from oracle.ic import WarmBubble
    g = load_golden("bubble32_600s.npz")
    nx, ny, nz = int(g["nx"]), int(g["ny"]), int(g["nz"])
    bubble = lambda: WarmBubble(nx, ny, nz, float(g["dx"]), float(g["dy"]), float(g["dz"]), seed=int(g["seed"])).build()
    phys, base, grids = bubble()
    nl = types.SimpleNamespace(nx=nx, ny=ny, nz=nz, dx=float(g["dx"]), dy=float(g["dy"]), dz=float(g["dz"]),
                               dt=float(g["dt"]), n_sound=int(g["n_sound"]), sprint_n=20, fCor=1.0e-4,
                               file_name_format=str(tmp_path / "lex_%04d.nc"), base_file_name=str(tmp_path / "base.nc"),
                               output_format=1, sfc_opt=0, pic_opt=0)
    sp.configure(nl)
    sfc = sp.get_first_step_flux(phys, base, grids, OK)
    write.save2nc_base(base, grids)
    write.save2nc(phys, sfc, grids, 0, 0.0)
    d0 = sp._ResidentState.downloads
    relay_n, save_n = int(g["nsteps"]) // nl.sprint_n, 5
    kept = None
    for i in range(relay_n):
        phys, sfc = sp.ws_rk3_sprint(phys, base, grids, OK)
        if i == 2:
            kept = phys                                   # read only after later sprints
        if (i + 1) % save_n == 0:
            write.save2nc(phys, sfc, grids, (i + 1) // save_n, (i + 1) * nl.sprint_n * nl.dt)
    assert sp._ResidentState.downloads - d0 == relay_n // save_n    # one host copy per save
    th = np.asarray(phys[0])
    assert not th.flags.writeable
    with pytest.raises(ValueError):
        th[0, 0, 0] = 0.0
    saved = np.load(str(tmp_path / ("lex_%04d.npz" % (relay_n // save_n))))
    np.testing.assert_array_equal(saved["theta"][0], th[3:-3, 3:-3, 1:-1].astype(np.float32))
    inner = (slice(3, -3), slice(3, -3), slice(1, -1))
    qv0 = base[4][inner]
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    errs = {"theta_p": rel(th[inner] - 300.0, g["theta_p"]), "qv_p": rel(np.asarray(phys[5])[inner] - qv0, g["qv_p"]),
            "w": rel(np.asarray(phys[3])[3:-3, 3:-3, 1:-1], g["w"])}
    assert errs["theta_p"] < 1e-3 and errs["qv_p"] < 1e-3 and errs["w"] < 2e-3, errs
    # the state of sprint 3, read now: 60 steps from the start, unaffected by the later sprints
    sp.configure(nl)
    again = bubble()[0]
    for _ in range(3):
        again, _ = sp.ws_rk3_sprint(again, base, grids, OK)
    for a, b in zip(kept, again):
        np.testing.assert_array_equal(np.asarray(a), np.asarray(b))
    sp.configure(nl)
