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
    from lex_gb300.sgs_cnn import cell_fields, make_scale
    a, b = _state(4, 3, 5, 1), _state(4, 3, 5, 2)
    sc = make_scale([a, b])
    assert sc["lo"].shape == (5, 5) and sc["rin"].shape == (5, 5) and sc["rout"].shape == (5, 5, 3, 4)
    for f, (fa, fb) in enumerate(zip(cell_fields(a), cell_fields(b))):
        for k in range(5):
            lo = min(fa[k].min(), fb[k].min())
            hi = max(fa[k].max(), fb[k].max())
            assert torch.isclose(sc["lo"][f, k], lo)
            margin = 1e-5 if f == 4 else 0.01
            assert torch.isclose(sc["rin"][f, k], hi - lo + margin)
            assert torch.allclose(sc["rout"][f, k], (hi - lo).expand(3, 4))


def test_pack_normalises_cell_centred_fields():
    from lex_gb300.sgs_cnn import cell_fields, make_scale, pack
    st = _state(4, 3, 5, 3)
    sc = make_scale([st])
    x = pack(st, sc)
    assert x.shape == (60, 5)
    for f, a in enumerate(cell_fields(st)):
        ref = ((a - sc["lo"][f].view(-1, 1, 1)) / sc["rin"][f].view(-1, 1, 1)).reshape(-1)
        assert torch.equal(x[:, f], ref)
    # x fastest: point 1 is (k, j, i) = (0, 0, 1); ui there averages u faces 1 and 2
    ui = 0.5 * (st[1][0, 0, 1] + st[1][0, 0, 2])
    assert torch.isclose(x[1, 1], (ui - sc["lo"][1, 0]) / sc["rin"][1, 0])


def test_unpack_staggers_the_correction():
    from lex_gb300.sgs_cnn import unpack
    nx, ny, nz = 4, 3, 5
    rout = torch.ones(5, nz, ny, nx, dtype=torch.float64) * torch.arange(1, 6, dtype=torch.float64).view(5, 1, 1, 1)
    corr = torch.zeros(nx * ny * nz, 5, dtype=torch.float64)
    corr[:, 0] = 1.0
    cu = torch.zeros(nz, ny, nx, dtype=torch.float64)
    cu[2, 1, 3] = 1.0                                  # one cell's u correction
    corr[:, 1] = cu.reshape(-1)
    cw = torch.zeros(nz, ny, nx, dtype=torch.float64)
    cw[0, 0, 0] = 1.0                                  # the bottom cell's w correction
    corr[:, 3] = cw.reshape(-1)
    th, u, v, w, p, q = unpack(corr, {"rout": rout}, (nx, ny, nz))
    assert torch.equal(th, torch.ones(nz, ny, nx, dtype=torch.float64))
    # u faces west (i = 3) and east (i = 0, periodic) of the cell get half of it, times the range 2
    assert u[2, 1, 3] == 1.0 and u[2, 1, 0] == 1.0 and float(u.abs().sum()) == 2.0
    # w: interior face 1 gets half of the bottom cell's correction (range 4); face 0 stays zero
    assert w[1, 0, 0] == 2.0 and float(w.abs().sum()) == 2.0 and float(w[0].abs().sum()) == 0.0
    assert float(v.abs().sum()) == 0.0 and float(p.abs().sum()) == 0.0 and float(q.abs().sum()) == 0.0


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
