"""Host-side logic of the learned SGS correction on CPU tensors: coarse-graining of a fine state,
per-level scales, and the packing and un-packing (staggering) of the network's fields."""
import pytest

torch = pytest.importorskip("torch")


def _state(nx, ny, nz, seed=0):
    g = torch.Generator().manual_seed(seed)
    r = lambda *s: torch.rand(*s, generator=g, dtype=torch.float64)
    return (300.0 + r(nz, ny, nx), r(nz, ny, nx), r(nz, ny, nx), r(nz + 1, ny, nx), r(nz, ny, nx), 0.01 * r(nz, ny, nx))


def test_coarse_grain_means_over_cells_and_faces():
    from lex_gb300.learned_sgs import coarse_grain
    fine = _state(12, 12, 6)
    th, u, v, w, p, q = coarse_grain(fine, (6, 6, 3))
    assert th.shape == (2, 2, 2) and u.shape == (2, 2, 2) and v.shape == (2, 2, 2) and w.shape == (3, 2, 2)
    # cells: box means
    assert torch.allclose(th[1, 0, 1], fine[0][3:6, 0:6, 6:12].mean())
    assert torch.allclose(q[0, 1, 0], fine[5][0:3, 6:12, 0:6].mean())
    assert torch.allclose(th.mean(), fine[0].mean())
    # u: the fine faces that make up the coarse west face of cell (k, j, i)
    assert torch.allclose(u[1, 1, 1], fine[1][3:6, 6:12, 6].mean())
    assert torch.allclose(v[0, 1, 0], fine[2][0:3, 6, 0:6].mean())
    # w: fine faces 0, 3, 6 averaged over the 6 x 6 fine cells of a coarse face
    assert torch.allclose(w[1, 0, 1], fine[3][3, 0:6, 6:12].mean())
    assert torch.allclose(w[2, 1, 0], fine[3][6, 6:12, 0:6].mean())


def test_scale_is_per_level_with_margins():
    from lex_gb300.sgs_cnn import make_scale
    a, b = _state(4, 3, 5, 1), _state(4, 3, 5, 2)
    sc = make_scale([a, b])
    nz = 5
    assert sc["lo"].shape == (5, nz + 1) and sc["rin"].shape == (5, nz + 1) and sc["rout"].shape == (5, nz + 1, 3, 4)
    for f, i in enumerate((0, 1, 2, 3, 5)):            # each field on its own points; w per face level
        levels = nz + 1 if f == 3 else nz
        for k in range(nz + 1):
            kk = min(k, levels - 1)                     # entry nz repeats the top level but for w
            lo = min(a[i][kk].min(), b[i][kk].min())
            hi = max(a[i][kk].max(), b[i][kk].max())
            assert torch.isclose(sc["lo"][f, k], lo)
            margin = 1e-5 if f == 4 else 0.01
            assert torch.isclose(sc["rin"][f, k], hi - lo + margin)
            assert torch.allclose(sc["rout"][f, k], (hi - lo).expand(3, 4))


def test_pack_normalises_then_averages_the_winds():
    """dl_models.phys_state_tuple2array: every field normalised on its own points (w per face
    level), then u, v, w averaged to the cell centre."""
    from lex_gb300.sgs_cnn import make_scale, pack
    st = _state(4, 3, 5, 3)
    sc = make_scale([st])
    x = pack(st, sc)
    assert x.shape == (60, 5)
    lo, rin = sc["lo"], sc["rin"]
    n = lambda a, f, m: (a - lo[f, :m].view(-1, 1, 1)) / rin[f, :m].view(-1, 1, 1)
    assert torch.equal(x[:, 0], n(st[0], 0, 5).reshape(-1))
    assert torch.equal(x[:, 4], n(st[5], 4, 5).reshape(-1))
    wn = n(st[3], 3, 6)
    assert torch.equal(x[:, 3], (0.5 * (wn[:-1] + wn[1:])).reshape(-1))
    # x fastest: point 1 is (k, j, i) = (0, 0, 1); ui there averages the normalised u faces 1 and 2
    un = lambda i: (st[1][0, 0, i] - lo[1, 0]) / rin[1, 0]
    assert torch.isclose(x[1, 1], 0.5 * (un(1) + un(2)))


def test_unpack_staggers_the_correction_as_the_reference():
    """dl_models.correct_array2tuple / stagger_uvw: a face i >= 1 gets the mean of the cells beside
    it, face 0 the value of face nx-1 (the face next to the far end), w zero on the bottom and the
    lid; each field times its range at its own point."""
    from lex_gb300.sgs_cnn import unpack
    nx, ny, nz = 4, 3, 5
    rout = torch.ones(5, nz + 1, ny, nx, dtype=torch.float64) * torch.arange(1, 6, dtype=torch.float64).view(5, 1, 1, 1)
    corr = torch.zeros(nx * ny * nz, 5, dtype=torch.float64)
    corr[:, 0] = 1.0
    cu = torch.zeros(nz, ny, nx, dtype=torch.float64)
    cu[2, 1, 3] = 1.0                                  # the last cell of a row
    corr[:, 1] = cu.reshape(-1)
    cv = torch.zeros(nz, ny, nx, dtype=torch.float64)
    cv[1, 0, 2] = 1.0                                  # the first cell of a column
    corr[:, 2] = cv.reshape(-1)
    cw = torch.zeros(nz, ny, nx, dtype=torch.float64)
    cw[0, 0, 0] = 1.0                                  # the bottom cell's w correction
    corr[:, 3] = cw.reshape(-1)
    th, u, v, w, p, q = unpack(corr, {"rout": rout}, (nx, ny, nz))
    assert torch.equal(th, torch.ones(nz, ny, nx, dtype=torch.float64))
    # u: face 3 (west of cell 3) gets half, times the range 2; face 0 copies face 3 (face nx-1)
    assert u[2, 1, 3] == 1.0 and u[2, 1, 0] == 1.0 and float(u.abs().sum()) == 2.0
    # v: face 1 (north of cell 0) gets half, times 3; face 0 copies face ny-1 = 2, which is zero
    assert v[1, 1, 2] == 1.5 and float(v.abs().sum()) == 1.5
    # w: interior face 1 gets half of the bottom cell's correction (range 4); face 0 stays zero
    assert w[1, 0, 0] == 2.0 and float(w.abs().sum()) == 2.0 and float(w[0].abs().sum()) == 0.0
    assert float(p.abs().sum()) == 0.0 and float(q.abs().sum()) == 0.0


def test_bubble_generators():
    import numpy as np
    from lex_gb300.workload import random_bubbles, warm_bubble, warm_bubbles
    a, pa = warm_bubble(16, 12, 10, 600.0, 600.0, 300.0, seed=4)
    b, pb = warm_bubbles(16, 12, 10, 600.0, 600.0, 300.0, [(2.0, 2000.0, 4800.0, 3600.0)], seed=4)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    four = random_bubbles(3, 4, 76800.0, 76800.0)
    assert four == random_bubbles(3, 4, 76800.0, 76800.0)          # seeded
    for i, (amp, rh, xc, yc) in enumerate(four):
        assert 1.0 <= amp <= 3.0 and 1500.0 <= rh <= 3000.0
        assert rh <= xc <= 76800.0 - rh and rh <= yc <= 76800.0 - rh
        for amp2, rh2, xc2, yc2 in four[:i]:
            assert (xc - xc2) ** 2 + (yc - yc2) ** 2 > (rh + rh2) ** 2
    one = random_bubbles(5, 1, 19200.0, 19200.0, centred=True)
    assert one[0][2:] == (9600.0, 9600.0)


def test_laplacian_matches_the_reference():
    """Against the reference's own laplace_of_tensor_jnp (tests/golden/dl_packing.npz)."""
    import numpy as np
    from conftest import load_golden
    from lex_gb300.learned_sgs import laplacian
    g = load_golden("dl_packing.npz")
    a = torch.tensor(np.ascontiguousarray(g["lap_in"].transpose(2, 1, 0)))
    got = laplacian(a, tuple(float(v) for v in g["spacing"])).numpy().transpose(2, 1, 0)
    assert np.allclose(got, g["lap_out"], rtol=1e-12, atol=1e-15)


def test_loss_options():
    from lex_gb300.learned_sgs import field_scale, loss_fn
    st = _state(6, 5, 4, 1)
    sc = field_scale([st, _state(6, 5, 4, 2)], spacing=(600.0, 600.0, 300.0))
    assert len(sc["la"]) == 2 and sc["la"][0] > 0 and sc["la"][1] > 0
    sp = (600.0, 600.0, 300.0)
    assert float(loss_fn(st, st, sc, sp, True, True)) == 0.0       # qv >= 0 here
    neg = tuple(a.clone() for a in st)
    neg[5][0, 0, 0] = -1e-3
    base = float(loss_fn(neg, st, sc))
    assert float(loss_fn(neg, st, sc, sp, False, True)) > base
    assert float(loss_fn(neg, st, sc, sp, True, False)) > base
