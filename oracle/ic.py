"""Oracle: grids, base state and warm-bubble initial state in the reference's padded layout.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` and ``--impl reference`` legs of ``bench.py`` may import this package; the
product path never does.

Layout follows LEX exactly: C-order ``[x][y][z]`` arrays with ``ngx=ngy=3``
lateral ghost cells and ``ngz=1`` ghost level, scalars ``(nx+6, ny+6, nz+2)``,
u ``(nx+7, ny+6, nz+2)``, v ``(nx+6, ny+7, nz+2)``, w ``(nx+6, ny+6, nz+3)``.

Reference formulas followed:
  * coordinates, cc1/cc2:               setup_lex.py:12-29
  * hydrostatic pi0 by cumulative sum:   setup_lex.py:103-111, :123-132
  * rho0*theta0 = pi0^(Cv/Rd) p00/Rd,
    rho0 = rho0theta0/theta_rho0:        setup_lex.py:128-131
  * rho0_theta0 = rho0*theta0 on output: setup_lex.py:62
  * periodic/ghost padding:             one_step_integration.py:950-985
The warm bubble itself (2 K cos^2, radii 2 km / 1.5 km, mid-domain at 1.5 km,
qv0 = 14 g/kg exp(-z/2.5 km), additive +-0.01 K seeded noise) is the synthetic
workload; the reference's own option-1 bubble (setup_lex.py:74-146) is
reproduced by ``reference_option1_base_state`` to pin the base-state formulas.
"""
from dataclasses import dataclass, field
import numpy as np
from .xp import concat

NGX, NGY, NGZ = 3, 3, 1

# namelist_n_constants.py:64-75
RD = 287.04
RV = 461.5
CP = 1004.64
CV = CP - RD
EPS = RD / RV
REPS = RV / RD
REPSM1 = RV / RD - 1.0
G = 9.80616
P00 = 100000.0


@dataclass
class Grid:
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    x1d: np.ndarray = field(init=False)
    y1d: np.ndarray = field(init=False)
    z1d: np.ndarray = field(init=False)
    x1d4u: np.ndarray = field(init=False)
    y1d4v: np.ndarray = field(init=False)
    z1d4w: np.ndarray = field(init=False)

    def __post_init__(self):
        nx, ny, nz, dx, dy, dz = self.nx, self.ny, self.nz, self.dx, self.dy, self.dz
        # setup_lex.py:12-24
        self.x1d = np.linspace(0.0 - (NGX - 0.5) * dx, (nx + NGX - 0.5) * dx, nx + 2 * NGX)
        self.y1d = np.linspace(0.0 - (NGY - 0.5) * dy, (ny + NGY - 0.5) * dy, ny + 2 * NGY)
        self.z1d = np.linspace(0.0 - (NGZ - 0.5) * dz, (nz + NGZ - 0.5) * dz, nz + 2 * NGZ)
        self.x1d4u = np.linspace(0.0 - NGX * dx, (nx + NGX) * dx, nx + 1 + 2 * NGX)
        self.y1d4v = np.linspace(0.0 - NGY * dy, (ny + NGY) * dy, ny + 1 + 2 * NGY)
        self.z1d4w = np.linspace(0.0 - NGZ * dz, (nz + NGZ) * dz, nz + 1 + 2 * NGZ)

    def grids_tuple(self):
        """The reference's ``grids`` tuple (setup_lex.py:68): 3-D coordinate arrays, cc1, cc2, tau."""
        x3d, y3d, z3d = np.meshgrid(self.x1d, self.y1d, self.z1d, indexing="ij")
        x3d4u, _, _ = np.meshgrid(self.x1d4u, self.y1d, self.z1d, indexing="ij")
        _, y3d4v, _ = np.meshgrid(self.x1d, self.y1d4v, self.z1d, indexing="ij")
        _, _, z3d4w = np.meshgrid(self.x1d, self.y1d, self.z1d4w, indexing="ij")
        s = (slice(NGX, -NGX), slice(NGY, -NGY))
        cc1 = (z3d4w[s + (slice(NGZ + 1, -NGZ),)] - z3d[s + (slice(NGZ, -NGZ),)]) / (
            z3d4w[s + (slice(NGZ + 1, -NGZ),)] - z3d4w[s + (slice(NGZ, -NGZ - 1),)])
        cc2 = 1.0 - cc1
        tauh = np.zeros_like(z3d)
        tauf = np.zeros_like(z3d4w)
        return (x3d, y3d, z3d, x3d4u, y3d4v, z3d4w, cc1, cc2, tauh, tauf)


def pad_scalar(a):
    """padding3_array (one_step_integration.py:950-959): periodic x/y, z ghost = edge copy."""
    a = concat((a[-NGX:], a, a[:NGX]), axis=0)
    a = concat((a[:, -NGY:], a, a[:, :NGY]), axis=1)
    return concat((a[:, :, :1], a, a[:, :, -1:]), axis=2)


def pad_u(a):
    """padding3u_array (one_step_integration.py:962-972): the duplicated periodic face is skipped."""
    a = concat((a[-(NGX + 1):-1], a, a[1:NGX + 1]), axis=0)
    a = concat((a[:, -NGY:], a, a[:, :NGY]), axis=1)
    return concat((a[:, :, :1], a, a[:, :, -1:]), axis=2)


def pad_v(a):
    """padding3v_array (one_step_integration.py:975-985)."""
    a = concat((a[-NGX:], a, a[:NGX]), axis=0)
    a = concat((a[:, -(NGY + 1):-1], a, a[:, 1:NGY + 1]), axis=1)
    return concat((a[:, :, :1], a, a[:, :, -1:]), axis=2)


def random_state(phys, nx, ny, nz, seed):
    """A random padded state around a warm-bubble state ``phys``: theta + N(0, 0.5 K), u and v
    N(0, 2 m/s), w N(0, 1 m/s) with zero end faces, pi' N(0, 1e-4), qv (1 + N(0, 0.05)).
    Halos filled as the reference's padding functions do."""
    rng = np.random.default_rng(seed)
    rnd = lambda shape, s: rng.standard_normal(shape) * s
    th = pad_scalar(phys[0][3:-3, 3:-3, 1:-1] + rnd((nx, ny, nz), 0.5))
    ui = rnd((nx, ny, nz), 2.0)
    u = pad_u(np.concatenate([ui, ui[:1]], 0))
    vi = rnd((nx, ny, nz), 2.0)
    v = pad_v(np.concatenate([vi, vi[:, :1]], 1))
    wi = rnd((nx, ny, nz + 1), 1.0)
    wi[:, :, 0] = 0.0
    wi[:, :, -1] = 0.0
    w = pad_scalar(wi)
    pip = pad_scalar(rnd((nx, ny, nz), 1e-4))
    qv = pad_scalar(phys[5][3:-3, 3:-3, 1:-1] * (1.0 + rnd((nx, ny, nz), 0.05)))
    return (th, u, v, w, pip, qv)


def hydrostatic_columns(theta0_col, qv0_col, dz):
    """FP64 hydrostatic base state on the padded column (setup_lex.py:123-132).

    theta0_col, qv0_col: (nz+2,) values at padded scalar levels.
    Returns pi0, rho0 (nz+2,) with the ghost levels copied from the edge levels for pi0.
    """
    theta_rho0 = theta0_col * (1.0 + REPS * qv0_col) / (1.0 + qv0_col)
    d_pi0_dz = -G / CP / theta_rho0
    pi_faces = np.concatenate(([1.0], np.cumsum(d_pi0_dz[NGZ:-NGZ]) * dz + 1.0))
    pi0 = np.empty_like(theta0_col)
    pi0[NGZ:-NGZ] = 0.5 * (pi_faces[:-1] + pi_faces[1:])
    pi0[0] = pi0[NGZ]
    pi0[-1] = pi0[-(NGZ + 1)]
    rho0_theta0 = pi0 ** (CV / RD) * P00 / RD
    rho0 = rho0_theta0 / theta0_col / ((1.0 + REPS * qv0_col) / (1.0 + qv0_col))
    return pi0, rho0


@dataclass
class WarmBubble:
    """The synthetic warm-bubble workload (neutral 300 K, exponential qv0)."""
    nx: int = 32
    ny: int = 32
    nz: int = 32
    dx: float = 600.0
    dy: float = 600.0
    dz: float = 300.0
    theta_base: float = 300.0
    qv_surface: float = 0.014
    qv_scale_height: float = 2500.0
    amplitude: float = 2.0
    radius_h: float = 2000.0
    radius_v: float = 1500.0
    z_center: float = 1500.0
    noise: float = 0.01
    seed: int = 2025

    def build(self):
        """Return (phys_state, base_state, grids) as padded FP64 NumPy arrays."""
        g = Grid(self.nx, self.ny, self.nz, self.dx, self.dy, self.dz)
        z = g.z1d
        theta0_col = np.full(z.shape, self.theta_base)
        qv0_col = self.qv_surface * np.exp(-z / self.qv_scale_height)
        pi0_col, rho0_col = hydrostatic_columns(theta0_col, qv0_col, self.dz)
        shp = (self.nx + 2 * NGX, self.ny + 2 * NGY, self.nz + 2 * NGZ)
        col = lambda c: np.broadcast_to(c, shp).copy()
        theta0, qv0, pi0, rho0 = col(theta0_col), col(qv0_col), col(pi0_col), col(rho0_col)
        rho0_theta0 = rho0 * theta0          # setup_lex.py:62
        surface_t = np.full((self.nx, self.ny), self.theta_base)

        xc = 0.5 * self.nx * self.dx
        yc = 0.5 * self.ny * self.dy
        xi, yi, zi = np.meshgrid(g.x1d[NGX:-NGX], g.y1d[NGY:-NGY], g.z1d[NGZ:-NGZ], indexing="ij")
        r = np.sqrt(((xi - xc) / self.radius_h) ** 2 + ((yi - yc) / self.radius_h) ** 2
                    + ((zi - self.z_center) / self.radius_v) ** 2)
        dtheta = np.where(r <= 1.0, self.amplitude * np.cos(0.5 * np.pi * r) ** 2, 0.0)
        rng = np.random.default_rng(self.seed)
        dtheta = dtheta + rng.uniform(-self.noise, self.noise, size=dtheta.shape)
        theta = pad_scalar(theta0_col[NGZ:-NGZ][None, None, :] + dtheta)
        qv = pad_scalar(np.broadcast_to(qv0_col[NGZ:-NGZ], dtheta.shape).copy())
        pip = np.zeros(shp)
        u = np.zeros((shp[0] + 1, shp[1], shp[2]))
        v = np.zeros((shp[0], shp[1] + 1, shp[2]))
        w = np.zeros((shp[0], shp[1], shp[2] + 1))
        phys = (theta, u, v, w, pip, qv)
        base = (rho0_theta0, rho0, theta0, pi0, qv0, surface_t)
        return phys, base, g.grids_tuple()


def rslf(p, t):
    """Bolton (1980) saturation mixing ratio (setup_lex.py:159-167)."""
    esl = 611.2 * np.exp(17.67 * (t - 273.15) / (t - 29.65))
    esl = np.where(esl > p * 0.5, p * 0.5, esl)
    return EPS * esl / (p - esl)


def reference_option1_base_state(nx, ny, nz, dz):
    """Column restatement of the reference's option-1 base state (setup_lex.py:101-137).

    theta0 = 300 K with qv0 at 10 % relative humidity, iterated to hydrostatic balance.
    Used only to pin ``hydrostatic_columns`` against the reference's own set-up.
    Returns (rho0, theta0, pi0, qv0) padded columns.
    """
    g = Grid(nx, ny, nz, 100.0, 100.0, dz)
    theta0 = np.full(g.z1d.shape, 300.0)
    qv0 = np.zeros_like(theta0)
    pi0, _ = hydrostatic_columns(theta0, qv0, dz)
    pressure0 = pi0 ** (CP / RD) * P00
    qv0 = rslf(pressure0, theta0 * pi0) * 0.1
    # The reference's balance loop (setup_lex.py:119-136) binds qv0_prev to the same array that
    # it then updates in place, so the loop body runs exactly once: pi0 and rho0 are balanced
    # against the first-guess qv0, and qv0 is refreshed once from that pi0.
    pi0, rho0 = hydrostatic_columns(theta0, qv0, dz)
    pressure0 = pi0 ** (CP / RD) * P00
    qv0 = rslf(pressure0, theta0 * pi0) * 0.1
    return rho0, theta0, pi0, qv0
