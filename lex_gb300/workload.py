"""Synthetic warm-bubble workloads in the reference's padded layout.

The benchmark cases are warm bubbles on a neutral hydrostatic base state:
  theta0 = 300 K, qv0(z) = 14 g/kg * exp(-z / 2.5 km), u = v = w = pi' = 0,
  theta = theta0 + 2 K cos^2(pi r / 2) for r <= 1,
  r^2 = ((x-xc)/2 km)^2 + ((y-yc)/2 km)^2 + ((z-1.5 km)/1.5 km)^2, centred mid-domain,
  plus uniform +-0.01 K noise from numpy.random.default_rng(seed) over the interior, C order.
Coordinates follow setup_lex.py:12-24 (cell centres at (i + 1/2) dx).  The hydrostatic
pi0 / rho0 columns are integrated in FP64 on the GPU by Solver.integrate_base_state.
"""
import numpy as np

NGX, NGY, NGZ = 3, 3, 1


def _pad(a, kind):
    """Reference ghost filling (padding3_array / padding3u_array / padding3v_array)."""
    if kind == "u":
        a = np.concatenate((a[-(NGX + 1):-1], a, a[1:NGX + 1]), axis=0)
    else:
        a = np.concatenate((a[-NGX:], a, a[:NGX]), axis=0)
    if kind == "v":
        a = np.concatenate((a[:, -(NGY + 1):-1], a, a[:, 1:NGY + 1]), axis=1)
    else:
        a = np.concatenate((a[:, -NGY:], a, a[:, :NGY]), axis=1)
    return np.concatenate((a[:, :, :1], a, a[:, :, -1:]), axis=2)


def level_heights(nz, dz):
    """Heights of the padded scalar levels (setup_lex.py:14)."""
    return np.linspace(0.0 - (NGZ - 0.5) * dz, (nz + NGZ - 0.5) * dz, nz + 2 * NGZ)


def warm_bubble(nx, ny, nz, dx, dy, dz, amplitude=2.0, radius_h=2000.0, radius_v=1500.0, z_center=1500.0,
                theta_base=300.0, qv_surface=0.014, qv_scale_height=2500.0, noise=0.01, seed=2025, center=None):
    """Return (phys_state, profile): the padded FP64 (theta, u, v, w, pi', qv) tuple and the padded
    base-state columns {'theta0', 'qv0'} from which the hydrostatic pi0/rho0 are integrated."""
    z = level_heights(nz, dz)
    theta0 = np.full(z.shape, float(theta_base))
    qv0 = qv_surface * np.exp(-z / qv_scale_height)
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dy
    zi = z[NGZ:-NGZ]
    xc, yc = (0.5 * nx * dx, 0.5 * ny * dy) if center is None else center
    X, Y, Z = np.meshgrid(x, y, zi, indexing="ij")
    r = np.sqrt(((X - xc) / radius_h) ** 2 + ((Y - yc) / radius_h) ** 2 + ((Z - z_center) / radius_v) ** 2)
    dtheta = np.where(r <= 1.0, amplitude * np.cos(0.5 * np.pi * r) ** 2, 0.0)
    if noise:
        dtheta = dtheta + np.random.default_rng(seed).uniform(-noise, noise, size=dtheta.shape)
    theta = _pad(theta0[NGZ:-NGZ][None, None, :] + dtheta, "s")
    qv = _pad(np.broadcast_to(qv0[NGZ:-NGZ], dtheta.shape).copy(), "s")
    shp = (nx + 2 * NGX, ny + 2 * NGY, nz + 2 * NGZ)
    phys = (theta, np.zeros((shp[0] + 1, shp[1], shp[2])), np.zeros((shp[0], shp[1] + 1, shp[2])),
            np.zeros((shp[0], shp[1], shp[2] + 1)), np.zeros(shp), qv)
    return phys, {"theta0": theta0, "qv0": qv0}


def warm_bubbles(nx, ny, nz, dx, dy, dz, bubbles, radius_v=1500.0, z_center=1500.0, theta_base=300.0,
                 qv_surface=0.014, qv_scale_height=2500.0, noise=0.01, seed=2025):
    """Several warm bubbles on the base state of warm_bubble: ``bubbles`` is a list of
    (amplitude K, horizontal radius m, x centre m, y centre m); perturbations add.  Returns
    (phys_state, profile) like warm_bubble."""
    z = level_heights(nz, dz)
    theta0 = np.full(z.shape, float(theta_base))
    qv0 = qv_surface * np.exp(-z / qv_scale_height)
    X, Y, Z = np.meshgrid((np.arange(nx) + 0.5) * dx, (np.arange(ny) + 0.5) * dy, z[NGZ:-NGZ], indexing="ij")
    dtheta = np.zeros(X.shape)
    for amp, rh, xc, yc in bubbles:
        r = np.sqrt(((X - xc) / rh) ** 2 + ((Y - yc) / rh) ** 2 + ((Z - z_center) / radius_v) ** 2)
        dtheta += np.where(r <= 1.0, amp * np.cos(0.5 * np.pi * r) ** 2, 0.0)
    if noise:
        dtheta = dtheta + np.random.default_rng(seed).uniform(-noise, noise, size=dtheta.shape)
    theta = _pad(theta0[NGZ:-NGZ][None, None, :] + dtheta, "s")
    qv = _pad(np.broadcast_to(qv0[NGZ:-NGZ], dtheta.shape).copy(), "s")
    shp = (nx + 2 * NGX, ny + 2 * NGY, nz + 2 * NGZ)
    phys = (theta, np.zeros((shp[0] + 1, shp[1], shp[2])), np.zeros((shp[0], shp[1] + 1, shp[2])),
            np.zeros((shp[0], shp[1], shp[2] + 1)), np.zeros(shp), qv)
    return phys, {"theta0": theta0, "qv0": qv0}


def random_bubbles(seed, n, lx, ly, amplitude=(1.0, 3.0), radius=(1500.0, 3000.0), centred=False, tries=10000):
    """n bubbles with amplitude and horizontal radius drawn uniformly (seeded); centred: one
    bubble at mid-domain, else positions drawn at random so that no two bubbles overlap and
    none crosses the domain edge."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        amp = float(rng.uniform(*amplitude))
        rh = float(rng.uniform(*radius))
        if centred:
            out.append((amp, rh, 0.5 * lx, 0.5 * ly))
            continue
        for _ in range(tries):
            xc, yc = float(rng.uniform(rh, lx - rh)), float(rng.uniform(rh, ly - rh))
            if all((xc - b[2]) ** 2 + (yc - b[3]) ** 2 > (rh + b[1]) ** 2 for b in out):
                break
        else:
            raise ValueError("no room for %d non-overlapping bubbles" % n)
        out.append((amp, rh, xc, yc))
    return out

