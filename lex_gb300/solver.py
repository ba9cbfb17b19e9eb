"""Host-side solver object over the C ABI.

``Solver`` owns one device context: the prognostic state stays resident in HBM across
steps and only crosses to the host on ``download``/``diagnose``.  Arrays exchanged with the
host use the reference's padded layout (see include/lexgb.h), so the tuples LEX builds in
setup_lex.py:66-69 can be passed straight through.
"""
import ctypes
import numpy as np

from . import _lib
from ._lib import check, Config

NGX, NGY, NGZ = 3, 3, 1
FIELDS = ("theta", "u", "v", "w", "pip", "qv")


def padded_shape(nx, ny, nz, field):
    """Padded reference shape of one prognostic field (setup_lex.py:39-49)."""
    return (nx + 2 * NGX + (field == "u"), ny + 2 * NGY + (field == "v"), nz + 2 * NGZ + (field == "w"))


def interior_shape(nx, ny, nz, field):
    return (nx + (field == "u"), ny + (field == "v"), nz + (field == "w"))


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Solver:
    """LEX solver_opt=2 dynamical core on one GPU.

    Parameters mirror namelist_n_constants.py: grid (nx, ny, nz, dx, dy, dz), big-step dt,
    n_sound acoustic sub-steps per big step, turb_opt (0/1), cor_opt (0/1/2), f_cor.
    theta_ref is the constant subtracted from theta on the device (0: theta0 at level 1).
    acoustic_pairs: advance two acoustic sub-steps per kernel launch (temporal blocking).
    l2_persist: keep the acoustic sub-steps' per-stage inputs in a persisting L2 window.
    acoustic_kernel: "auto" (the fastest measured form for the grid), "rows" or "tile" (one kernel
    launch per sub-step) or "persistent" (one cooperative launch per stage); a form the grid does not
    allow falls back to "auto" (see ``acoustic_form``).
    cs: the Smagorinsky constant (None: 0.18, turbulence.py:433).
    """

    def __init__(self, nx, ny, nz, dx, dy, dz, dt, n_sound=32, turb_opt=1, cor_opt=0, f_cor=1.0e-4,
                 theta_ref=0.0, acoustic_pairs=False, l2_persist=True, cs=None, acoustic_kernel="auto"):
        self.lib = _lib.load()
        cfg = Config()
        check(self.lib.lexgb_default_config(ctypes.byref(cfg)))
        cfg.nx, cfg.ny, cfg.nz = nx, ny, nz
        cfg.dx, cfg.dy, cfg.dz, cfg.dt = dx, dy, dz, dt
        cfg.n_sound, cfg.turb_opt, cfg.cor_opt = n_sound, turb_opt, cor_opt
        cfg.f_cor, cfg.theta_ref = f_cor, theta_ref
        cfg.acoustic_pairs = 1 if acoustic_pairs else 0
        cfg.l2_persist = 0 if l2_persist else -1
        cfg.cs = float(cs) if cs is not None else 0.0
        if acoustic_kernel not in _lib.ACOUSTIC_KERNELS:
            raise ValueError("acoustic_kernel must be one of %s" % sorted(_lib.ACOUSTIC_KERNELS))
        cfg.acoustic_kernel = _lib.ACOUSTIC_KERNELS[acoustic_kernel]
        self.cs = float(cs) if cs is not None else 0.18
        self.cfg = cfg
        self.nx, self.ny, self.nz = nx, ny, nz
        self.dt = dt
        self.n_sound = n_sound
        h = ctypes.c_void_p()
        check(self.lib.lexgb_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h

    # -------------------------------------------------------------------------------- lifetime
    def close(self):
        if getattr(self, "handle", None):
            self.lib.lexgb_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_handle):
        """Order work on a CUDA stream given as an integer handle (e.g. torch.cuda.Stream().cuda_stream)."""
        check(self.lib.lexgb_set_stream(self.handle, ctypes.c_void_p(stream_handle)))

    # -------------------------------------------------------------------------------- base state
    def _col(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        if a.size != self.nz + 2:
            raise ValueError("base columns need nz+2 = %d padded levels, got %d" % (self.nz + 2, a.size))
        return a

    def set_base_columns(self, theta0, qv0, pi0, rho0):
        cols = [self._col(c) for c in (theta0, qv0, pi0, rho0)]
        check(self.lib.lexgb_set_base_columns(self.handle, *[_dptr(c) for c in cols]))
        self._base = cols

    def set_base_state(self, base_state):
        """From the reference's base_state tuple (rho0_theta0, rho0, theta0, pi0, qv0, surface_t)."""
        _, rho0, theta0, pi0, qv0, _ = base_state
        cols = []
        for name, a in (("theta0", theta0), ("qv0", qv0), ("pi0", pi0), ("rho0", rho0)):
            a = np.asarray(a, dtype=np.float64)
            c = a[0, 0, :]
            if not np.array_equal(a, np.broadcast_to(c, a.shape)):
                raise ValueError("base state %s is not horizontally uniform" % name)
            cols.append(c)
        self.set_base_columns(*cols)

    def integrate_base_state(self, theta0, qv0):
        """FP64 hydrostatic integration on the GPU; returns padded (pi0, rho0) columns."""
        t, q = self._col(theta0), self._col(qv0)
        pi0 = np.empty(self.nz + 2)
        rho0 = np.empty(self.nz + 2)
        check(self.lib.lexgb_integrate_base_state(self.handle, _dptr(t), _dptr(q), _dptr(pi0), _dptr(rho0)))
        self._base = [t, q, pi0.copy(), rho0.copy()]
        return pi0, rho0

    # -------------------------------------------------------------------------------- state transfer
    def upload(self, state, dtype=None):
        """Upload the phys_state tuple (theta, u, v, w, pi', qv) in the padded reference layout."""
        if len(state) != 6:
            raise ValueError("state must have 6 fields (theta, u, v, w, pip, qv)")
        if dtype is None:
            dtype = np.float64 if np.asarray(state[0]).dtype == np.float64 else np.float32
        arrs = []
        for name, a in zip(FIELDS, state):
            a = np.ascontiguousarray(a, dtype=dtype)
            if a.shape != padded_shape(self.nx, self.ny, self.nz, name):
                raise ValueError("%s has shape %s, expected %s" % (name, a.shape,
                                                                    padded_shape(self.nx, self.ny, self.nz, name)))
            arrs.append(a)
        ptrs = (ctypes.c_void_p * 6)(*[a.ctypes.data for a in arrs])
        code = _lib.LEXGB_F64 if dtype == np.float64 else _lib.LEXGB_F32
        check(self.lib.lexgb_upload_state(self.handle, ptrs, code))

    def upload_ptrs(self, ptrs, f64):
        """Upload from raw host pointers (e.g. pinned buffers) already in the padded layout."""
        arr = (ctypes.c_void_p * 6)(*ptrs)
        check(self.lib.lexgb_upload_state(self.handle, arr, _lib.LEXGB_F64 if f64 else _lib.LEXGB_F32))

    def download_ptrs(self, ptrs, f64):
        arr = (ctypes.c_void_p * 6)(*ptrs)
        check(self.lib.lexgb_download_state(self.handle, arr, _lib.LEXGB_F64 if f64 else _lib.LEXGB_F32))

    def download(self, dtype=np.float64):
        outs = [np.empty(padded_shape(self.nx, self.ny, self.nz, n), dtype=dtype) for n in FIELDS]
        ptrs = (ctypes.c_void_p * 6)(*[a.ctypes.data for a in outs])
        code = _lib.LEXGB_F64 if dtype == np.float64 else _lib.LEXGB_F32
        check(self.lib.lexgb_download_state(self.handle, ptrs, code))
        return tuple(outs)

    # -------------------------------------------------------------------------------- stepping
    def step(self, nsteps=1, graph=True):
        """Advance nsteps RK3 big steps (asynchronous on the context's stream)."""
        check(self.lib.lexgb_step(self.handle, int(nsteps), 1 if graph else 0))

    def set_cs(self, cs):
        """Smagorinsky constant for the following steps."""
        check(self.lib.lexgb_set_cs(self.handle, float(cs)))
        self.cs = float(cs)
        self._kept_token = None   # the library discards a kept step when Cs changes

    def cs_grad(self, reset=True):
        """d(seed . output)/dCs accumulated by the reverse-mode calls since the last reset."""
        g = ctypes.c_double()
        check(self.lib.lexgb_get_cs_grad(self.handle, ctypes.byref(g), 1 if reset else 0))
        return g.value

    def step_record(self):
        check(self.lib.lexgb_step_record(self.handle))

    def stage(self, s):
        """After step_record: (padded stage state, interior tendencies) of stage s as FP64 tuples."""
        f = [np.empty(padded_shape(self.nx, self.ny, self.nz, n)) for n in FIELDS]
        t = [np.empty(interior_shape(self.nx, self.ny, self.nz, n)) for n in FIELDS]
        fp = (ctypes.c_void_p * 6)(*[a.ctypes.data for a in f])
        tp = (ctypes.c_void_p * 6)(*[a.ctypes.data for a in t])
        check(self.lib.lexgb_download_stage(self.handle, int(s), fp, tp))
        return tuple(f), tuple(t)

    def synchronize(self):
        """Wait for the solver's stream; raises LexError(LEXGB_ERR_TIMEOUT) when a bounded device-side
        wait gave up since the last check (the state must then be uploaded again)."""
        check(self.lib.lexgb_synchronize(self.handle))

    @property
    def acoustic_form(self):
        """The acoustic form this solver runs: "rows", "tile" or "persistent"."""
        k = ctypes.c_int()
        check(self.lib.lexgb_acoustic_kernel(self.handle, ctypes.byref(k)))
        return {v: n for n, v in _lib.ACOUSTIC_KERNELS.items()}[k.value]

    def set_barrier_limit(self, polls):
        """Polls a grid-barrier wait of the persistent acoustic kernel makes before it gives up (0: default;
        negative: test mode, every wait expects an arrival that never comes and gives up after -polls)."""
        check(self.lib.lexgb_set_barrier_limit(self.handle, int(polls)))

    # -------------------------------------------------------------------------------- reverse mode
    def step_vjp(self, ybar, nstages=3):
        """Vector-Jacobian product of one big step (or its first `nstages` stages) at the resident
        state.  ybar / result: interior arrays in reference order [x][y][z] for (theta, u, v, w,
        pi', qv), w with nz+1 levels; the result is the adjoint of the resident state."""
        shapes = [interior_shape(self.nx, self.ny, self.nz, n) for n in FIELDS]
        shapes[1], shapes[2] = (self.nx, self.ny, self.nz), (self.nx, self.ny, self.nz)   # periodic u, v
        dev = []
        for a, shp in zip(ybar, shapes):
            a = np.asarray(a, dtype=np.float32)
            if a.shape != shp:
                raise ValueError("adjoint seed shape %s, expected %s" % (a.shape, shp))
            dev.append(np.ascontiguousarray(a.transpose(2, 1, 0)))
        out = [np.empty(shp[::-1], dtype=np.float32) for shp in shapes]
        yp = (ctypes.c_void_p * 6)(*[a.ctypes.data for a in dev])
        xp = (ctypes.c_void_p * 6)(*[a.ctypes.data for a in out])
        check(self.lib.lexgb_step_vjp(self.handle, int(nstages), yp, xp, 0))
        return tuple(np.ascontiguousarray(a.transpose(2, 1, 0)) for a in out)

    # -------------------------------------------------------------------------------- diagnostics
    _DIAG_SHAPES = {"adv_u": "u", "adv_v": "v", "adv_w": "w", "buoy_w": "w", "pgf_u": "u", "pgf_v": "v",
                    "pgf_w": "w", "sgs_u": "u", "sgs_v": "v", "sgs_w": "w"}

    def diagnose(self, name):
        """One operator of the path evaluated on the current state (FP64, reference C order)."""
        idx = _lib.DIAGNOSTICS.index(name)
        out = np.empty(interior_shape(self.nx, self.ny, self.nz, self._DIAG_SHAPES.get(name, "theta")))
        check(self.lib.lexgb_diagnose(self.handle, idx, _dptr(out)))
        return out

    def budget(self):
        """FP64 global sums of the current state: air mass, water vapour mass, kinetic energy
        (0.5 rho0 |u|^2), rho0 theta and total energy (rho (cv T + g z + 0.5 |u|^2))."""
        out = np.empty(5)
        check(self.lib.lexgb_budget(self.handle, _dptr(out), 5))
        return dict(mass=out[0], vapour=out[1], kinetic=out[2], rho_theta=out[3], total_energy=out[4])

    def count_nonfinite(self):
        n = ctypes.c_longlong()
        check(self.lib.lexgb_check_finite(self.handle, ctypes.byref(n)))
        return n.value

    def check_finite(self):
        """Raise FloatingPointError if the state holds a NaN or an infinity (one device count)."""
        n = self.count_nonfinite()
        if n:
            raise FloatingPointError("%d non-finite values in the solver state" % n)

    # -------------------------------------------------------------------------------- checkpoints
    _CFG = ("nx", "ny", "nz", "dx", "dy", "dz", "dt", "n_sound", "turb_opt", "cor_opt", "f_cor", "theta_ref",
            "acoustic_pairs", "l2_persist", "acoustic_kernel")

    def save(self, path):
        """Checkpoint to an .npz archive: the configuration, the Smagorinsky constant, the base
        columns and the state (padded reference layout, FP64: the device's FP32 values and the
        theta offset are exact in it, so a restored solver continues bit for bit)."""
        if getattr(self, "_base", None) is None:
            raise RuntimeError("no base state has been set")
        out = {"cfg_" + k: np.asarray(getattr(self.cfg, k)) for k in self._CFG}
        out["cfg_cs"] = np.asarray(self.cs)
        for name, c in zip(("theta0", "qv0", "pi0", "rho0"), self._base):
            out["base_" + name] = c
        for name, a in zip(FIELDS, self.download(np.float64)):
            out["state_" + name] = a
        np.savez(path, **out)

    @classmethod
    def restore(cls, path):
        """A new solver from a checkpoint written by save()."""
        with np.load(path) as z:
            c = {k: z["cfg_" + k].item() for k in cls._CFG if "cfg_" + k in z.files}
            S = cls(int(c["nx"]), int(c["ny"]), int(c["nz"]), c["dx"], c["dy"], c["dz"], c["dt"], int(c["n_sound"]),
                    turb_opt=int(c["turb_opt"]), cor_opt=int(c["cor_opt"]), f_cor=c["f_cor"],
                    theta_ref=c["theta_ref"], acoustic_pairs=bool(c["acoustic_pairs"]),
                    l2_persist=int(c["l2_persist"]) == 0, cs=z["cfg_cs"].item(),
                    acoustic_kernel={v: n for n, v in _lib.ACOUSTIC_KERNELS.items()}[int(c.get("acoustic_kernel", 0))])
            S.set_base_columns(*[z["base_" + n] for n in ("theta0", "qv0", "pi0", "rho0")])
            S.upload(tuple(z["state_" + f] for f in FIELDS))
        return S

    def step_kernel_count(self):
        n = ctypes.c_int()
        check(self.lib.lexgb_step_kernel_count(self.handle, ctypes.byref(n)))
        return n.value

    def time_kernel(self, name, reps=20):
        """Average duration [ms] of one launch of a step kernel, CUDA events on the solver's stream."""
        ms = ctypes.c_float()
        check(self.lib.lexgb_time_kernel(self.handle, _lib.KERNELS.index(name), int(reps), ctypes.byref(ms)))
        return ms.value

    def device_ptrs(self):
        arr = (ctypes.c_void_p * 6)()
        check(self.lib.lexgb_state_device_ptrs(self.handle, arr))
        return [arr[i] for i in range(6)]
