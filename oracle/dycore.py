"""Oracle: a NumPy restatement of LEX's fully compressible dynamical-core step (solver_opt=2).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` and ``--impl reference`` legs of ``bench.py`` may import this package; the
product path never does.  The CUDA kernels are tested against it, and it is pinned in turn
against golden vectors produced by the reference's own source (tests/golden/).

Everything works on the reference's padded ``[x][y][z]`` arrays (see oracle/ic.py)
in the dtype of the inputs (FP64 for the oracle proper; FP32 reproduces what an
FP32 run of the reference computes, up to operation order).  The base state is
horizontally uniform, so it is passed as padded columns of shape (nz+2,).

Reference correspondence (file:line):
  WENO5-Z / WENO3 reconstruction ........ advection.py:305-416 (vertical), :419-516 (horizontal)
  advection_scalar ...................... advection.py:9-34
  advection_u / _v / _w ................. advection.py:37-149 (+ fluxes :561-1281)
  advection_pi .......................... advection.py:152-197
  get_divergence / get_divergence2 ...... advection.py:200-236
  pressure_gradient_force ............... pressure_gradient_coriolis.py:7-37
  calculate_coriolis_force (+ _with_lspgrad) pressure_gradient_coriolis.py:80-113
  calculate_buoyancy .................... pressure_equations.py:123-172
  Smagorinsky ........................... turbulence.py:9-111, :298-446, :474-504
  acoustic sub-steps .................... one_step_integration.py:519-556 / :638-675 / :757-794
  set_w_bc .............................. boundary_conditions.py:104-109
  RK stages ............................. one_step_integration.py:16-447
  Wicker-Skamarock RK3 big step ......... one_sprint_functions.py:10-30
"""
import numpy as np
from . import xp
from .ic import NGX, NGY, NGZ, RD, CP, CV, G, REPS, REPSM1, pad_scalar, pad_u, pad_v

WEPS_MOM = 1.0e-16     # one_step_integration.py:896
WEPS_THETA = 1.0e-17   # one_step_integration.py:905
WEPS_QV = 1.0e-18      # one_step_integration.py:913
PRANDTL = 1.0 / 3.0    # turbulence.py:432
CS = 0.18              # turbulence.py:433
DIV_DAMP = 1.1         # one_step_integration.py:546


# ----------------------------------------------------------------------------------------------
# reconstruction primitives
# ----------------------------------------------------------------------------------------------
def weno5(a, b, c, d, e, eps):
    """Upwind WENO5 value at the face right of ``c`` for a stencil ordered upwind->downwind.

    a..e = s[-2], s[-1], s[0], s[+1], s[+2] relative to the upwind cell.  Smoothness
    indicators of Jiang & Shu, Borges et al. (2008) WENO-Z weights with the reference's
    fmin(1e30, .) cap (advection.py:311-324).
    """
    b1 = (13.0 / 12.0) * (a - 2.0 * b + c) ** 2 + 0.25 * (a - 4.0 * b + 3.0 * c) ** 2
    b2 = (13.0 / 12.0) * (b - 2.0 * c + d) ** 2 + 0.25 * (b - d) ** 2
    b3 = (13.0 / 12.0) * (c - 2.0 * d + e) ** 2 + 0.25 * (3.0 * c - 4.0 * d + e) ** 2
    tau = abs(b1 - b3)
    w1 = 0.1 * (1.0 + xp.fmin(1.0e30, tau / (b1 + eps)) ** 2)
    w2 = 0.6 * (1.0 + xp.fmin(1.0e30, tau / (b2 + eps)) ** 2)
    w3 = 0.3 * (1.0 + xp.fmin(1.0e30, tau / (b3 + eps)) ** 2)
    q1 = (2.0 / 6.0) * a + (-7.0 / 6.0) * b + (11.0 / 6.0) * c
    q2 = (-1.0 / 6.0) * b + (5.0 / 6.0) * c + (2.0 / 6.0) * d
    q3 = (2.0 / 6.0) * c + (5.0 / 6.0) * d + (-1.0 / 6.0) * e
    return (w1 * q1 + w2 * q2 + w3 * q3) / (w1 + w2 + w3)


def weno3(a, b, c, eps):
    """Upwind WENO3 value at the face right of ``b``; a, b, c = s[-1], s[0], s[+1] (advection.py:327-337)."""
    b1 = (a - b) ** 2
    b2 = (b - c) ** 2
    tau = abs(b1 - b2)
    w1 = (1.0 / 3.0) * (1.0 + xp.fmin(1.0e30, tau / (b1 + eps)) ** 2)
    w2 = (2.0 / 3.0) * (1.0 + xp.fmin(1.0e30, tau / (b2 + eps)) ** 2)
    return (w1 * ((-1.0 / 2.0) * a + (3.0 / 2.0) * b) + w2 * ((1.0 / 2.0) * b + (1.0 / 2.0) * c)) / (w1 + w2)


def _ax(arr, axis, start, stop):
    idx = [slice(None)] * arr.ndim
    idx[axis] = slice(start, stop)
    return arr[tuple(idx)]


def recon_lateral(s, axis, lo, n, eps):
    """WENO5 values at the n faces between s[p] and s[p+1], p = lo..lo+n-1, along a periodic axis.

    Returns (positive-flow value, negative-flow value) (advection.py:424-503).
    """
    sh = lambda off: _ax(s, axis, lo + off, lo + off + n)
    pos = weno5(sh(-2), sh(-1), sh(0), sh(1), sh(2), eps)
    neg = weno5(sh(3), sh(2), sh(1), sh(0), sh(-1), eps)
    return pos, neg


def recon_vertical(s, eps):
    """Face values between consecutive z levels of ``s`` (N levels -> N-1 faces, axis 2).

    Face 0 and face N-2 carry zero (no flux through the ghost faces); faces next to the
    ends fall back to centred / WENO3 exactly as advection.py:305-416 (and the u, v, w
    versions :561-676, :816-931, :1070-1184) do.  Returns (upward, downward).
    """
    N = s.shape[2]
    nf = N - 1
    lv = lambda k: s[:, :, k:k + 1]
    up = xp.zeros(tuple(s.shape[:2]) + (nf,), like=s)
    dn = xp.zeros_like(up)
    # upward (w >= 0): centred at face 1, WENO3 at face 2 and face nf-2, WENO5 in between
    up[:, :, 1:2] = 0.5 * (lv(1) + lv(2))
    up[:, :, 2:3] = weno3(lv(1), lv(2), lv(3), eps)
    f = xp.arange(3, nf - 2, like=s)
    if xp.size(f):
        up[:, :, 3:nf - 2] = weno5(s[:, :, f - 2], s[:, :, f - 1], s[:, :, f], s[:, :, f + 1], s[:, :, f + 2], eps)
    up[:, :, nf - 2:nf - 1] = weno3(lv(N - 4), lv(N - 3), lv(N - 2), eps)
    # downward (w < 0): WENO3 at face 1 and face nf-3, centred at face nf-2, WENO5 in between
    dn[:, :, 1:2] = weno3(lv(3), lv(2), lv(1), eps)
    f = xp.arange(2, nf - 3, like=s)
    if xp.size(f):
        dn[:, :, 2:nf - 3] = weno5(s[:, :, f + 3], s[:, :, f + 2], s[:, :, f + 1], s[:, :, f], s[:, :, f - 1], eps)
    dn[:, :, nf - 3:nf - 2] = weno3(lv(N - 2), lv(N - 3), lv(N - 4), eps)
    dn[:, :, nf - 2:nf - 1] = 0.5 * (lv(N - 2) + lv(N - 3))
    return up, dn


def upwind_flux(m, pos, neg):
    """jax.lax.select(m >= 0, m*pos, m*neg): ties go to the positive branch."""
    return xp.where(m >= 0.0, m * pos, m * neg)


def col(c):
    return c[None, None, :]


IX = slice(NGX, -NGX)
IY = slice(NGY, -NGY)
IZ = slice(NGZ, -NGZ)


class Dycore:
    """Restated LEX solver_opt=2 dynamical core on padded arrays.

    grid: oracle.ic.Grid (uniform dx, dy, dz); base: dict of padded FP64 columns
    theta0, qv0, pi0, rho0 (each (nz+2,)); dt, n_sound; dtype FP64 or FP32.
    device: None for NumPy arrays; a torch device ("cpu", "cuda") to evaluate the same
    expressions on torch tensors of that dtype (``cast`` converts a NumPy state).
    """

    def __init__(self, grid, base, dt, n_sound=32, dtype=np.float64, turb=True, cs=CS, cor_opt=0, f_cor=1.0e-4,
                 device=None):
        self.device = device
        self.g = grid
        self.cs = cs
        self.cor_opt = int(cor_opt)
        self.f_cor = f_cor
        self.nx, self.ny, self.nz = grid.nx, grid.ny, grid.nz
        self.dt = dt
        self.n_sound = n_sound
        self.turb = turb
        self.dtype = np.dtype(dtype).type
        if device is None:
            t = self.dtype
            arr = lambda a: np.asarray(a, dtype=t)
        else:
            import torch
            tdt = torch.float64 if self.dtype == np.float64 else torch.float32
            t = float if tdt == torch.float64 else (lambda v: float(np.float32(v)))
            arr = lambda a: xp.to_torch(a, device, tdt)
        self._arr = arr
        self._s = t
        self.dx, self.dy, self.dz = t(grid.dx), t(grid.dy), t(grid.dz)
        self.theta0 = col(arr(base["theta0"]))
        self.qv0 = col(arr(base["qv0"]))
        self.pi0 = col(arr(base["pi0"]))
        self.rho0 = col(arr(base["rho0"]))
        # cc1/cc2 of setup_lex.py:25-29 for a uniform grid
        self.cc1 = t(0.5)
        self.cc2 = t(1.0) - self.cc1

    def cast(self, state):
        return tuple(self._arr(a) for a in state)

    # ------------------------------------------------------------------ divergence
    def mass_divergence(self, u, v, w):
        """get_divergence (advection.py:200-226) on the whole padded scalar array."""
        r = self.rho0
        rw = xp.concat((xp.zeros_like(r[:, :, :1]), 0.5 * (r[:, :, :-1] + r[:, :, 1:]),
                        xp.zeros_like(r[:, :, :1])), axis=2)
        dvx = (r * u[1:] - r * u[:-1]) / self.dx
        dvy = (r * v[:, 1:] - r * v[:, :-1]) / self.dy
        dvz = (rw[:, :, 1:] * w[:, :, 1:] - rw[:, :, :-1] * w[:, :, :-1]) / self.dz
        return dvx + dvy + dvz

    def velocity_divergence(self, u, v, w):
        """get_divergence2 (advection.py:229-236)."""
        return (u[1:] - u[:-1]) / self.dx + (v[:, 1:] - v[:, :-1]) / self.dy + (w[:, :, 1:] - w[:, :, :-1]) / self.dz

    # ------------------------------------------------------------------ advection
    def advect_scalar(self, s, u, v, w, div, eps):
        """advection_scalar (advection.py:9-34) with zero surface flux."""
        nx, ny = self.nx, self.ny
        r = self.rho0
        rz = 0.5 * (r[:, :, :-1] + r[:, :, 1:])
        # x faces p=2..nx+2 between s[p], s[p+1] (u points 3..nx+3); interior y, z
        pos, neg = recon_lateral(s[:, IY, IZ], 0, 2, nx + 1, eps)
        fx = upwind_flux(r[:, :, IZ] * u[3:nx + 4, IY, IZ], pos, neg)
        pos, neg = recon_lateral(s[IX, :, IZ], 1, 2, ny + 1, eps)
        fy = upwind_flux(r[:, :, IZ] * v[IX, 3:ny + 4, IZ], pos, neg)
        up, dn = recon_vertical(s[IX, IY, :], eps)
        fz = upwind_flux(rz * w[IX, IY, 1:-1], up, dn)
        fz[:, :, 0] = 0.0
        conv = -((fx[1:] - fx[:-1]) / self.dx + (fy[:, 1:] - fy[:, :-1]) / self.dy
                 + (fz[:, :, 1:] - fz[:, :, :-1]) / self.dz)
        return (conv + s[IX, IY, IZ] * div[IX, IY, IZ]) / r[:, :, IZ]

    def advect_u(self, u, v, w, div, eps=WEPS_MOM):
        """advection_u (advection.py:37-74) with its fluxes horizontal_flux_u / vertical_flux_u2."""
        nx, ny = self.nx, self.ny
        r = self.rho0
        # x flux at scalar points p=2..nx+3 (between u[p] and u[p+1])
        pos, neg = recon_lateral(u[:, IY, IZ], 0, 2, nx + 2, eps)
        fx = upwind_flux(0.5 * (u[2:nx + 4, IY, IZ] + u[3:nx + 5, IY, IZ]) * r[:, :, IZ], pos, neg)
        # y flux at corners (u points q=3..nx+3, v faces 3..ny+3)
        pos, neg = recon_lateral(u[3:nx + 4, :, IZ], 1, 2, ny + 1, eps)
        m = r[:, :, IZ] * v[:, 3:ny + 4, IZ]
        m8u = 0.5 * (m[2:nx + 3] + m[3:nx + 4])
        fy = upwind_flux(m8u, pos, neg)
        # z flux at (u point, w face)
        up, dn = recon_vertical(u[3:nx + 4, IY, :], eps)
        mw = 0.5 * (r[:, :, :-1] + r[:, :, 1:]) * w[:, IY, 1:-1]
        mw8u = 0.5 * (mw[2:nx + 3] + mw[3:nx + 4])
        fz = upwind_flux(mw8u, up, dn)
        fz[:, :, 0] = 0.0
        conv = -((fx[1:] - fx[:-1]) / self.dx + (fy[:, 1:] - fy[:, :-1]) / self.dy
                 + (fz[:, :, 1:] - fz[:, :, :-1]) / self.dz)
        d8u = 0.5 * (div[2:nx + 3, IY, IZ] + div[3:nx + 4, IY, IZ])
        return (conv + u[3:nx + 4, IY, IZ] * d8u) / r[:, :, IZ]

    def advect_v(self, u, v, w, div, eps=WEPS_MOM):
        """advection_v (advection.py:77-114) with horizontal_flux_v / vertical_flux_v2."""
        nx, ny = self.nx, self.ny
        r = self.rho0
        # x flux at corners (u faces 3..nx+3, v points 3..ny+3)
        pos, neg = recon_lateral(v[:, 3:ny + 4, IZ], 0, 2, nx + 1, eps)
        m = r[:, :, IZ] * u[3:nx + 4, :, IZ]
        m8v = 0.5 * (m[:, 2:ny + 3] + m[:, 3:ny + 4])
        fx = upwind_flux(m8v, pos, neg)
        # y flux at scalar points
        pos, neg = recon_lateral(v[IX, :, IZ], 1, 2, ny + 2, eps)
        fy = upwind_flux(0.5 * (v[IX, 2:ny + 4, IZ] + v[IX, 3:ny + 5, IZ]) * r[:, :, IZ], pos, neg)
        up, dn = recon_vertical(v[IX, 3:ny + 4, :], eps)
        mw = 0.5 * (r[:, :, :-1] + r[:, :, 1:]) * w[IX, :, 1:-1]
        mw8v = 0.5 * (mw[:, 2:ny + 3] + mw[:, 3:ny + 4])
        fz = upwind_flux(mw8v, up, dn)
        fz[:, :, 0] = 0.0
        conv = -((fx[1:] - fx[:-1]) / self.dx + (fy[:, 1:] - fy[:, :-1]) / self.dy
                 + (fz[:, :, 1:] - fz[:, :, :-1]) / self.dz)
        d8v = 0.5 * (div[IX, 2:ny + 3, IZ] + div[IX, 3:ny + 4, IZ])
        return (conv + v[IX, 3:ny + 4, IZ] * d8v) / r[:, :, IZ]

    def advect_w(self, u, v, w, div, eps=WEPS_MOM):
        """advection_w (advection.py:117-149) with horizontal_flux_w / vertical_flux_w2."""
        nx, ny, nz = self.nx, self.ny, self.nz
        r = self.rho0
        # x flux at (u faces 3..nx+3, w faces 0..nz)
        pos, neg = recon_lateral(w[:, IY, 1:-1], 0, 2, nx + 1, eps)
        m = r * u[3:nx + 4, IY, :]
        m8w = 0.5 * (m[:, :, :-1] + m[:, :, 1:])
        fx = upwind_flux(m8w, pos, neg)
        pos, neg = recon_lateral(w[IX, :, 1:-1], 1, 2, ny + 1, eps)
        m = r * v[IX, 3:ny + 4, :]
        m8w = 0.5 * (m[:, :, :-1] + m[:, :, 1:])
        fy = upwind_flux(m8w, pos, neg)
        # z flux at scalar levels 0..nz+1 (between w[L] and w[L+1])
        up, dn = recon_vertical(w[IX, IY, :], eps)
        fz = upwind_flux(0.5 * (w[IX, IY, :-1] + w[IX, IY, 1:]) * r, up, dn)
        conv = -((fx[1:] - fx[:-1]) / self.dx + (fy[:, 1:] - fy[:, :-1]) / self.dy
                 + (fz[:, :, 1:] - fz[:, :, :-1]) / self.dz)
        d8w = 0.5 * (div[IX, IY, :-1] + div[IX, IY, 1:])
        r8w = 0.5 * (r[:, :, :-1] + r[:, :, 1:])
        out = (conv + w[IX, IY, 1:-1] * d8w) / r8w
        out[:, :, 0] = 0.0
        out[:, :, -1] = 0.0
        return out

    def advect_pi(self, pis, u, v, w):
        """advection_pi (advection.py:152-197): low-order advection of pi' by the new winds."""
        nx, ny = self.nx, self.ny
        r = self.rho0
        dpx = (pis[3:nx + 4, IY, IZ] - pis[2:nx + 3, IY, IZ]) / self.dx
        dpy = (pis[IX, 3:ny + 4, IZ] - pis[IX, 2:ny + 3, IZ]) / self.dy
        dp0 = (self.pi0[:, :, 1:] - self.pi0[:, :, :-1]) / self.dz
        dpz = dp0 + (pis[IX, IY, 1:] - pis[IX, IY, :-1]) / self.dz
        ux = u[3:nx + 4, IY, IZ] * dpx
        vy = v[IX, 3:ny + 4, IZ] * dpy
        wz = w[IX, IY, 1:-1] * dpz
        wz[:, :, 0] = 0.0
        wz[:, :, -1] = 0.0
        r8w = 0.5 * (r[:, :, :-1] + r[:, :, 1:])
        return -(0.5 * (ux[1:] + ux[:-1]) + 0.5 * (vy[:, 1:] + vy[:, :-1])
                 + (self.cc1 * wz[:, :, :-1] * r8w[:, :, :-1] + self.cc2 * wz[:, :, 1:] * r8w[:, :, 1:])
                 / r[:, :, IZ])

    # ------------------------------------------------------------------ forces
    def pgf(self, pip, trho):
        """pressure_gradient_force (pressure_gradient_coriolis.py:7-37); pi0 horizontally uniform."""
        nx, ny = self.nx, self.ny
        pu = -CP * 0.5 * (trho[3:nx + 4, IY, IZ] + trho[2:nx + 3, IY, IZ]) * (
            (pip[3:nx + 4, IY, IZ] - pip[2:nx + 3, IY, IZ]) / self.dx)
        pv = -CP * 0.5 * (trho[IX, 3:ny + 4, IZ] + trho[IX, 2:ny + 3, IZ]) * (
            (pip[IX, 3:ny + 4, IZ] - pip[IX, 2:ny + 3, IZ]) / self.dy)
        pw = -CP * 0.5 * (trho[IX, IY, 1:] + trho[IX, IY, :-1]) * (
            (pip[IX, IY, 1:] - pip[IX, IY, :-1]) / self.dz)
        pw[:, :, 0] = 0.0
        pw[:, :, -1] = 0.0
        if xp.is_torch(pu):
            return pu, pv, pw
        return pu.astype(self.dtype), pv.astype(self.dtype), pw.astype(self.dtype)

    def coriolis(self, u, v):
        """calculate_coriolis_force / calculate_coriolis_force_with_lspgrad (pressure_gradient_coriolis.py:80-113).

        Returns (fu at v points (nx, ny+1, nz), fv at u points (nx+1, ny, nz)): four-point averages of
        the other wind times f; cor_opt 2 subtracts a 1 m/s geostrophic wind from u's average.
        """
        nx, ny = self.nx, self.ny
        f = self._s(self.f_cor)
        fv = 0.25 * (v[2:nx + 3, 3:ny + 3, IZ] + v[2:nx + 3, 4:ny + 4, IZ]
                     + v[3:nx + 4, 3:ny + 3, IZ] + v[3:nx + 4, 4:ny + 4, IZ])
        fu = 0.25 * (u[3:nx + 3, 2:ny + 3, IZ] + u[3:nx + 3, 3:ny + 4, IZ]
                     + u[4:nx + 4, 2:ny + 3, IZ] + u[4:nx + 4, 3:ny + 4, IZ])
        if self.cor_opt == 2:
            return f * (fu - 1.0), f * (fv - 0.0)
        return f * fu, f * fv

    @staticmethod
    def extrapolate_ends(a):
        """extrapolate_bottom_top (pressure_equations.py:141-159): quadratic to the end levels."""
        bot = 1.875 * a[:, :, 0] - 1.25 * a[:, :, 1] + 0.375 * a[:, :, 2]
        top = 1.875 * a[:, :, -1] - 1.25 * a[:, :, -2] + 0.375 * a[:, :, -3]
        return bot[:, :, None], top[:, :, None]

    def to_w(self, a):
        """interpolate_scalar2w (pressure_equations.py:123-128) on an interior array."""
        bot, top = self.extrapolate_ends(a)
        return xp.concat((bot, 0.5 * (a[:, :, :-1] + a[:, :, 1:]), top), axis=2)

    @staticmethod
    def to_w0(a):
        """interpolate_scalar2w_0 (pressure_equations.py:131-138): zero at the end faces."""
        z = xp.zeros_like(a[:, :, :1])
        return xp.concat((z, 0.5 * (a[:, :, :-1] + a[:, :, 1:]), z), axis=2)

    def buoyancy(self, theta, qv):
        """calculate_buoyancy (pressure_equations.py:162-172) -> (b at scalars, b at w faces)."""
        trho0 = self.theta0 * (1.0 + REPS * self.qv0) / (1.0 + self.qv0)
        trho = theta * (1.0 + REPS * qv) / (1.0 + qv)
        b = (G * (trho - trho0) / trho0)[IX, IY, IZ]
        return b, self.to_w(b)

    # ------------------------------------------------------------------ Smagorinsky
    def deformation(self, u, v, w):
        """compute_deformation (turbulence.py:298-388): rho-weighted S_ij at scalar points, padded."""
        nx, ny = self.nx, self.ny
        r = self.rho0[:, :, IZ]
        dx, dy, dz = self.dx, self.dy, self.dz
        s11 = r * (u[4:nx + 4, IY, IZ] - u[3:nx + 3, IY, IZ]) / dx
        s22 = r * (v[IX, 4:ny + 4, IZ] - v[IX, 3:ny + 3, IZ]) / dy
        s33 = r * (w[IX, IY, 2:-1] - w[IX, IY, 1:-2]) / dz
        dudy = (u[3:nx + 4, 3:ny + 4, IZ] - u[3:nx + 4, 2:ny + 3, IZ]) / dy
        dvdx = (v[3:nx + 4, 3:ny + 4, IZ] - v[2:nx + 3, 3:ny + 4, IZ]) / dx
        e12 = 0.5 * (dudy + dvdx)
        s12 = r * (0.25 * (e12[:-1, :-1] + e12[1:, 1:] + e12[:-1, 1:] + e12[1:, :-1]))
        dudz = (u[3:nx + 4, IY, 2:-1] - u[3:nx + 4, IY, 1:-2]) / dz
        dwdx = (w[3:nx + 4, IY, 2:-2] - w[2:nx + 3, IY, 2:-2]) / dx
        e13 = 0.5 * (dudz + dwdx)
        b0, t0 = self.extrapolate_ends(e13)
        s13 = xp.concat((0.5 * (b0[1:] + b0[:-1]),
                              0.25 * (e13[:-1, :, :-1] + e13[1:, :, 1:] + e13[:-1, :, 1:] + e13[1:, :, :-1]),
                              0.5 * (t0[1:] + t0[:-1])), axis=2)
        s13 = r * s13
        dvdz = (v[IX, 3:ny + 4, 2:-1] - v[IX, 3:ny + 4, 1:-2]) / dz
        dwdy = (w[IX, 3:ny + 4, 2:-2] - w[IX, 2:ny + 3, 2:-2]) / dy
        e23 = 0.5 * (dvdz + dwdy)
        b0, t0 = self.extrapolate_ends(e23)
        s23 = xp.concat((0.5 * (b0[:, 1:] + b0[:, :-1]),
                              0.25 * (e23[:, :-1, :-1] + e23[:, 1:, 1:] + e23[:, :-1, 1:] + e23[:, 1:, :-1]),
                              0.5 * (t0[:, 1:] + t0[:, :-1])), axis=2)
        s23 = r * s23
        s2 = (2.0 * (s11 ** 2 + s22 ** 2 + s33 ** 2) + 4.0 * (s12 ** 2 + s13 ** 2 + s23 ** 2)) / r ** 2
        return tuple(pad_scalar(a) for a in (s11, s22, s33, s12, s13, s23, s2))

    def brunt_vaisala(self, theta, qv):
        """compute_nm (turbulence.py:391-427): N^2 from log(theta*(1+repsm1*qv)), padded."""
        tr = theta * (1.0 + REPSM1 * qv)
        n28w = xp.log(tr[IX, IY, 2:-1] / tr[IX, IY, 1:-2]) / self.dz * G
        bot, top = self.extrapolate_ends(n28w)
        return pad_scalar(xp.concat((bot, 0.5 * (n28w[:, :, :-1] + n28w[:, :, 1:]), top), axis=2))

    def eddy_coefficients(self, s2, n2):
        """compute_k (turbulence.py:430-446)."""
        delta = np.cbrt(self.dx * self.dy * self.dz)
        s2n2 = s2 - n2 / PRANDTL
        s2n2 = xp.where(s2n2 > 0.0, s2n2, xp.zeros_like(s2n2))
        km = (self.cs * delta) ** 2 * xp.sqrt(s2n2)
        return km, km / PRANDTL

    def smagorinsky(self, theta, u, v, w, qv):
        """Smagorinsky SGS tendencies (turbulence.py:9-111) -> (sgs_u, sgs_v, sgs_w, sgs_theta, sgs_qv)."""
        nx, ny = self.nx, self.ny
        dx, dy, dz = self.dx, self.dy, self.dz
        s11, s22, s33, s12, s13, s23, s2 = self.deformation(u, v, w)
        n2 = self.brunt_vaisala(theta, qv)
        km, kh = self.eddy_coefficients(s2, n2)
        r = self.rho0
        t11, t22, t33 = -2.0 * km * s11, -2.0 * km * s22, -2.0 * km * s33
        t12, t13, t23 = -2.0 * km * s12, -2.0 * km * s13, -2.0 * km * s23
        # u
        d11 = (t11[3:nx + 4, IY, IZ] - t11[2:nx + 3, IY, IZ]) / dx
        d12v = (t12[2:nx + 4, 3:ny + 4, IZ] - t12[2:nx + 4, 2:ny + 3, IZ]) / dy
        d12 = 0.25 * (d12v[:-1, :-1] + d12v[1:, 1:] + d12v[:-1, 1:] + d12v[1:, :-1])
        t13w = self.to_w0(t13[:, :, IZ])
        d13s = (t13w[:, :, 1:] - t13w[:, :, :-1]) / dz
        d13 = 0.5 * (d13s[2:nx + 3, IY] + d13s[3:nx + 4, IY])
        sgs_u = -(d11 + d12 + d13) / (0.5 * (r[:, :, IZ] + r[:, :, IZ]))
        # v
        d22 = (t22[IX, 3:ny + 4, IZ] - t22[IX, 2:ny + 3, IZ]) / dy
        d12u = (t12[3:nx + 4, 2:ny + 4, IZ] - t12[2:nx + 3, 2:ny + 4, IZ]) / dx
        d12x = 0.25 * (d12u[:-1, :-1] + d12u[1:, 1:] + d12u[:-1, 1:] + d12u[1:, :-1])
        t23w = self.to_w0(t23[:, :, IZ])
        d23s = (t23w[:, :, 1:] - t23w[:, :, :-1]) / dz
        d23 = 0.5 * (d23s[IX, 2:ny + 3] + d23s[IX, 3:ny + 4])
        sgs_v = -(d12x + d22 + d23) / (0.5 * (r[:, :, IZ] + r[:, :, IZ]))
        # w
        d33 = (t33[IX, IY, 1:] - t33[IX, IY, :-1]) / dz
        d13x = self.to_w0((t13[4:nx + 4, IY, IZ] - t13[2:nx + 2, IY, IZ]) / (2.0 * dx))
        d23y = self.to_w0((t23[IX, 4:ny + 4, IZ] - t23[IX, 2:ny + 2, IZ]) / (2.0 * dy))
        r8w = self.to_w(xp.broadcast_to(r[:, :, IZ], (nx, ny, self.nz)))
        sgs_w = -(d13x + d23y + d33) / r8w
        sgs_w[:, :, 0] = 0.0
        sgs_w[:, :, -1] = 0.0
        # scalars
        kh8u = 0.5 * (kh[3:nx + 4, IY, IZ] + kh[2:nx + 3, IY, IZ])
        kh8v = 0.5 * (kh[IX, 3:ny + 4, IZ] + kh[IX, 2:ny + 3, IZ])
        kh8w = self.to_w(kh[IX, IY, IZ])
        r8 = r[:, :, IZ]

        def scalar_sgs(s):
            gx = (s[3:nx + 4, IY, IZ] - s[2:nx + 3, IY, IZ]) / dx
            gy = (s[IX, 3:ny + 4, IZ] - s[IX, 2:ny + 3, IZ]) / dy
            gz = (s[IX, IY, 1:] - s[IX, IY, :-1]) / dz
            gz[:, :, 0] = 0.0
            gz[:, :, -1] = 0.0
            fx = -r8 * kh8u * gx
            fy = -r8 * kh8v * gy
            fz = -r8w * kh8w * gz
            fz[:, :, 0] = 0.0
            fz[:, :, -1] = 0.0
            return -((fx[1:] - fx[:-1]) / dx + (fy[:, 1:] - fy[:, :-1]) / dy
                     + (fz[:, :, 1:] - fz[:, :, :-1]) / dz) / r8

        return sgs_u, sgs_v, sgs_w, scalar_sgs(theta), scalar_sgs(qv)

    # ------------------------------------------------------------------ acoustic loop
    def acoustic(self, u, v, w, pip, pis, rhs_u, rhs_v, rhs_w, trho, n, dts):
        """sound_rk_step0/1/2 (one_step_integration.py:519-556): n forward-backward sub-steps."""
        piadv = (self.pi0 + pis)[IX, IY, IZ]
        for _ in range(n):
            pu, pv, pw = self.pgf(pip, trho)
            un = u[3:-3, IY, IZ] + (pu + rhs_u) * dts
            vn = v[IX, 3:-3, IZ] + (pv + rhs_v) * dts
            wn = w[IX, IY, 1:-1] + (pw + rhs_w) * dts
            u, v, w = pad_u(un), pad_v(vn), pad_scalar(wn)
            w[:, :, 0:2] = 0.0       # set_w_bc (boundary_conditions.py:104-109)
            w[:, :, -2:] = 0.0
            div = self.velocity_divergence(u, v, w)
            apl = self.advect_pi(pis, u, v, w)
            dpdt = -RD / CV * (piadv * div[IX, IY, IZ]) + apl
            pip = pad_scalar(pip[IX, IY, IZ] + DIV_DAMP * dpdt * dts)
        return u, v, w, pip

    # ------------------------------------------------------------------ RK stage / step
    def stage(self, xi0, xis, dts, sgs, n_sound):
        """One Wicker-Skamarock stage (rk_sub_step0/1/2, one_step_integration.py:16-447).

        Returns (next padded state, tendencies (dtheta, dpip, du, dv, dw, dqv)).
        """
        th0, u0, v0, w0, p0, q0 = xi0
        th, u, v, w, pis, q = xis
        _, b8w = self.buoyancy(th, q)
        div = self.mass_divergence(u, v, w)
        au = self.advect_u(u, v, w, div)
        av = self.advect_v(u, v, w, div)
        aw = self.advect_w(u, v, w, div)
        if self.cor_opt:
            # one_step_integration.py:83-86, :127-132: rhs_u = adv4u + fv (+ sgs), rhs_v = adv4v - fu (+ sgs)
            fu, fv = self.coriolis(u, v)
            au, av = au + fv, av - fu
        if sgs is not None:
            rhs_u, rhs_v, rhs_w = au + sgs[0], av + sgs[1], aw + b8w + sgs[2]
        else:
            rhs_u, rhs_v, rhs_w = au, av, aw + b8w
        trho = th * (1.0 + REPS * q) / (1.0 + q)
        dtau = self._s(self._dtau(dts, n_sound))
        un, vn, wn, pn = self.acoustic(u0, v0, w0, p0, pis, rhs_u, rhs_v, rhs_w, trho, n_sound, dtau)
        dth = self.advect_scalar(th, u, v, w, div, WEPS_THETA)
        dq = self.advect_scalar(q, u, v, w, div, WEPS_QV)
        thn = th0[IX, IY, IZ] + dth * dts
        qn = q0[IX, IY, IZ] + dq * dts
        if sgs is not None:
            thn = thn + sgs[3] * dts
            dth = dth + sgs[3]
            qn = qn + sgs[4] * dts
            dq = dq + sgs[4]
        thn, qn = pad_scalar(thn), pad_scalar(qn)
        tends = (dth, (pn - p0)[IX, IY, IZ] / dts, (un - u0)[3:-3, IY, IZ] / dts,
                 (vn - v0)[IX, 3:-3, IZ] / dts, (wn - w0)[IX, IY, 1:-1] / dts, dq)
        return (thn, un, vn, wn, pn, qn), tends

    def _dtau(self, dts, n_sound):
        # stage 0: one sub-step of the stage length; stages 1/2: dt/n_sound (one_step_integration.py:121-122, :253-254)
        return dts if n_sound == 1 else self.dt / self.n_sound

    def stage_plan(self):
        """(stage length, number of acoustic sub-steps) for the three WS-RK3 stages."""
        dt = self.dt
        n1 = int(round((dt / 2.0) / (dt / self.n_sound)))
        n2 = int(round(dt / (dt / self.n_sound)))
        return [(dt / 3.0, 1), (dt / 2.0, n1), (dt, n2)]

    def step(self, state, return_stages=False):
        """ws_rk3_big_step (one_sprint_functions.py:10-30). Returns (new state, last-stage tendencies)."""
        xi0 = self.cast(state)
        sgs = self.smagorinsky(xi0[0], xi0[1], xi0[2], xi0[3], xi0[5]) if self.turb else None
        xs = xi0
        stages = []
        for dts, n in self.stage_plan():
            xs, tends = self.stage(xi0, xs, self._s(dts), sgs, n)
            stages.append((xs, tends))
        if return_stages:
            return xs, tends, stages, sgs
        return xs, tends
