"""Benchmark of the LEX fully compressible dynamical-core step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl lexgb|reference]

Workload: the 100 m warm bubble on a 192 x 192 x 96 grid (19.2 x 19.2 x 9.6 km), dt = 1 s,
Wicker-Skamarock RK3 with 1 + 16 + 32 acoustic sub-steps, WENO5 advection, Smagorinsky
Cs = 0.18, FP32 on the device.  Synthetic seeded initial state (2 K cos^2 bubble + 0.01 K
noise on a neutral 300 K hydrostatic base state with qv0 = 14 g/kg exp(-z/2.5 km)).

One "step" is one RK3 big step over the whole grid.  The timed region is bracketed by a
barrier and a device synchronisation and timed with CUDA events on the solver's stream;
rank 0 prints one JSON line.  Under torchrun (N > 1) each rank advances its own replica on
its own GPU (the solver has no domain decomposition): weak scaling, no collective on the
data path.

--impl reference times the reference algorithm's CPU implementation on the host cores: the
reference itself is Python/JAX and cannot be installed here, so its restatement in
oracle/ (bit-identical to the reference in FP64, pinned by tests/golden/) is timed on a
bounded sub-domain sample.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-pt·RK3-steps/s @192×192×96 vs HBM roofline; adjoint/forward cost; SGS err"
UNIT = "grid-pt·RK3-steps/s"
GRID = dict(nx=192, ny=192, nz=96, dx=100.0, dy=100.0, dz=100.0, dt=1.0, n_sound=32)
# algorithmic bytes per grid point per RK3 step on the reference's field-level dataflow (FP32):
# 3 stages x 17 slow-mode fields + 3 x 3 theta_rho fields + 49 acoustic sub-steps x 13 fields
B_ALG = 4 * (51 + 9 + 49 * 13)
# one acoustic sub-step: read u, v, w, pi', R_u, R_v, R_w, theta_rho, pi'_s; write u, v, w, pi'
B_ACOUSTIC = 4 * 13
FALLBACK_HBM_GBS = 6800.0


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def build_case(nx, ny, nz, dx, dy, dz, **_):
    """Synthetic warm bubble in the reference's padded layout, generated on the host."""
    from lex_gb300.workload import warm_bubble
    return warm_bubble(nx, ny, nz, dx, dy, dz)


SAMPLE = (48, 48, GRID["nz"])


def _oracle_worker(k, warm, barrier, out, dtype="f32"):
    """One core: `warm` RK3 steps of the oracle (NumPy, FP32 or FP64 arithmetic) on the sample
    sub-domain, a barrier with the other cores, then `k` timed steps; puts the CLOCK_MONOTONIC
    start and end of the timed steps."""
    from oracle.ic import WarmBubble, Grid
    from oracle.dycore import Dycore
    nx, ny, nz = SAMPLE
    phys, base, _ = WarmBubble(nx, ny, nz, GRID["dx"], GRID["dy"], GRID["dz"]).build()
    cols = dict(theta0=base[2][0, 0], qv0=base[4][0, 0], pi0=base[3][0, 0], rho0=base[1][0, 0])
    D = Dycore(Grid(nx, ny, nz, GRID["dx"], GRID["dy"], GRID["dz"]), cols, GRID["dt"], GRID["n_sound"],
               dtype=np.float32 if dtype == "f32" else np.float64)
    st = D.cast(phys)
    for _ in range(warm):
        st, _ = D.step(st)
    barrier.wait(timeout=600)
    t0 = time.monotonic()
    for _ in range(k):
        st, _ = D.step(st)
    out.put((t0, time.monotonic()))


def oracle_throughput(k, warm, dtype="f32"):
    """The oracle on every host core at once (spawned processes, one sample sub-domain each, timed
    together after a barrier): (grid-pt-steps/s over the union of the timed windows, cores, s)."""
    import multiprocessing as mp
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    ctx = mp.get_context("spawn")
    barrier, out = ctx.Barrier(cores), ctx.Queue()
    procs = [ctx.Process(target=_oracle_worker, args=(k, warm, barrier, out, dtype)) for _ in range(cores)]
    for p in procs:
        p.start()
    try:
        spans = [out.get(timeout=1200) for _ in procs]
    finally:
        for p in procs:
            p.join(timeout=60)
    t0, t1 = min(a for a, _ in spans), max(b for _, b in spans)
    pts = SAMPLE[0] * SAMPLE[1] * SAMPLE[2] * k * cores
    return pts / (t1 - t0), cores, t1 - t0


def _sample_text(k, cores, seconds, dtype="f32"):
    nx, ny, nz = SAMPLE
    return ("%d RK3 step(s) of a %dx%dx%d sub-domain of the workload (same dz, dt, physics) on each of %d host "
            "cores at once (one process per core), NumPy %s restatement of the reference (oracle/; the reference "
            "is Python/JAX and not installable here), %.1f s" % (k, nx, ny, nz, cores,
                                                                 "FP32" if dtype == "f32" else "FP64", seconds))


def cpu_baseline():
    """The oracle (NumPy) on every host core, a bounded sample of the workload: in FP32, the
    reference's precision, and (second line) in FP64."""
    value, cores, sec = oracle_throughput(2, 1, "f32")
    v64, c64, s64 = oracle_throughput(2, 1, "f64")
    return {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "dtype": "f32",
            "sample": _sample_text(2, cores, sec, "f32"),
            "fp64": {"value": v64, "unit": UNIT, "cores": c64, "sample": _sample_text(2, c64, s64, "f64")}}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    k = min(max(1, args.steps), 3)
    warm = max(0, min(args.warmup, 1))
    value, cores, sec = oracle_throughput(k, warm, "f32")
    sample = _sample_text(k, cores, sec, "f32")
    nx, ny, _ = SAMPLE
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": k,
            "warmup": warm, "ms_per_step": 1e3 * GRID["nx"] * GRID["ny"] * GRID["nz"] / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": "warm bubble 192x192x96 @ 100 m, dt = 1 s (sampled on %dx%dx%d per core)"
                                   % SAMPLE, "grid": [GRID["nx"], GRID["ny"], GRID["nz"]]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def max_over_ranks(x, dist=None):
    """The largest value of x over the ranks of the process group (x itself without one); the
    reduction tensor lives where the backend wants it (CUDA for NCCL, host memory for gloo)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(ms_local, ws, npts, steps, dist=None):
    """Whole-job throughput of ws independent replicas, each timing `steps` steps of `npts`
    points in ms_local: the job takes as long as its slowest replica -> (ms, points*steps/s)."""
    ms = max_over_ranks(ms_local, dist)
    return ms, ws * npts * steps / (ms * 1e-3)


def run_lexgb(args):
    import torch
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from lex_gb300.solver import Solver, padded_shape, FIELDS

    g = GRID
    phys, profile = build_case(**g)
    S = Solver(g["nx"], g["ny"], g["nz"], g["dx"], g["dy"], g["dz"], g["dt"], g["n_sound"], turb_opt=1,
               acoustic_kernel=args.acoustic_kernel)
    stream = torch.cuda.Stream()
    S.set_stream(stream.cuda_stream)
    S.integrate_base_state(profile["theta0"], profile["qv0"])   # FP64 hydrostatic balance on the GPU
    S.upload(phys, dtype=np.float32)
    npts = g["nx"] * g["ny"] * g["nz"]

    def barrier():
        if dist is not None:
            dist.barrier()

    # ---- device-resident throughput (value)
    S.step(max(3, args.warmup), graph=True)
    S.synchronize()
    kernels_per_step = S.step_kernel_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    with torch.cuda.stream(stream):
        e0.record()
        S.step(args.steps, graph=True)
        e1.record()
    e1.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier()
    ms, value = replica_throughput(e0.elapsed_time(e1), ws, npts, args.steps, dist)
    ms_per_step = ms / args.steps
    n_bad = S.count_nonfinite()
    if args.profile:   # warm-up + timed steps only (for profiler captures)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": ms_per_step,
                              "steps": args.steps, "profile_mode": True}), flush=True)
        S.close()
        return

    # ---- end to end through the public API with host buffers (pinned), copies in the timed region
    host_in = [torch.empty(padded_shape(g["nx"], g["ny"], g["nz"], f), dtype=torch.float32).pin_memory()
               for f in FIELDS]
    host_out = [torch.empty_like(h).pin_memory() for h in host_in]
    for h, a in zip(host_in, phys):
        h.numpy()[...] = a
    h2d = sum(h.numel() * 4 for h in host_in)
    d2h = sum(h.numel() * 4 for h in host_out)
    ptr_in = [h.data_ptr() for h in host_in]
    ptr_out = [h.data_ptr() for h in host_out]
    e2e_steps = max(1, min(args.steps, 10))
    for _ in range(2):
        S.upload_ptrs(ptr_in, False)
        S.step(1, graph=True)
        S.download_ptrs(ptr_out, False)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        S.upload_ptrs(ptr_in, False)
        S.step(1, graph=True)
        S.download_ptrs(ptr_out, False)
    torch.cuda.synchronize()
    el = max_over_ranks(time.perf_counter() - t0, dist)
    e2e = ws * npts * e2e_steps / el

    # ---- dominant kernel: one acoustic sub-step, timed alone with CUDA events
    S.upload(phys, dtype=np.float32)
    S.step(2, graph=True)
    kern = {k: S.time_kernel(k, reps=32 if k == "acoustic" else 8) for k in
            ("acoustic", "div_trho", "adv_scalars", "adv_momentum", "smag_a", "smag_b")}
    peak, peak_kind = peaks()
    ac_ms = kern["acoustic"]
    achieved = B_ACOUSTIC * npts / (ac_ms * 1e-3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "acoustic_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            t = json.load(f)
        traffic = t["bytes_per_point"] * npts
    # ---- reverse mode: one big step forward plus its vector-Jacobian product, device pointers
    adjoint = None
    if not args.no_adjoint:
        import ctypes
        from lex_gb300 import _lib
        shp = [(g["nz"], g["ny"], g["nx"])] * 6
        shp[3] = (g["nz"] + 1, g["ny"], g["nx"])
        gen = torch.Generator(device="cuda").manual_seed(1)
        ybar = [torch.randn(sh, device="cuda", generator=gen) for sh in shp]
        xbar = [torch.empty(sh, device="cuda") for sh in shp]
        yp = (ctypes.c_void_p * 6)(*[t.data_ptr() for t in ybar])
        xp = (ctypes.c_void_p * 6)(*[t.data_ptr() for t in xbar])
        S.upload(phys, dtype=np.float32)
        torch.cuda.synchronize()
        _lib.check(S.lib.lexgb_step_vjp(S.handle, 3, yp, xp, 1))   # allocates the workspace
        reps = 3
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a0.record()
            for _ in range(reps):
                _lib.check(S.lib.lexgb_step_vjp(S.handle, 3, yp, xp, 1))
            a1.record()
        a1.synchronize()
        vjp_ms = a0.elapsed_time(a1) / reps
        # non-checkpointed: the forward keeps its intermediates, the reverse reuses them
        S.upload(phys, dtype=np.float32)
        torch.cuda.synchronize()
        k0 = torch.cuda.Event(enable_timing=True)
        k1 = torch.cuda.Event(enable_timing=True)
        k2 = torch.cuda.Event(enable_timing=True)
        keep_ms = kept_ms = 0.0
        for _ in range(reps):
            with torch.cuda.stream(stream):
                k0.record()
                _lib.check(S.lib.lexgb_step_keep(S.handle))
                k1.record()
                _lib.check(S.lib.lexgb_step_vjp_kept(S.handle, yp, xp, 1))
                k2.record()
            k2.synchronize()
            keep_ms += k0.elapsed_time(k1) / reps
            kept_ms += k1.elapsed_time(k2) / reps
        adjoint = {"forward_ms": ms_per_step,
                   "kept_forward_ms": keep_ms, "kept_reverse_ms": kept_ms,
                   "forward_plus_adjoint_over_forward": (keep_ms + kept_ms) / ms_per_step,
                   "checkpointed_reverse_ms": vjp_ms,
                   "checkpointed_forward_plus_adjoint_over_forward": (ms_per_step + vjp_ms) / ms_per_step,
                   "note": "forward_plus_adjoint: lexgb_step_keep + lexgb_step_vjp_kept (intermediates kept by "
                           "the forward); checkpointed: graph forward + lexgb_step_vjp, which recomputes the "
                           "step; xbar finite: %s" % bool(all(torch.isfinite(t).all().item() for t in xbar))}
    # ---- learned SGS correction fused into the coarse step (600 m x 600 m x 300 m, 32^3, dt = 3 s)
    sgs = None
    if not args.no_sgs:
        from lex_gb300 import learned_sgs as lsgs, sgs_cnn, autograd as lag, _lib
        from lex_gb300.workload import warm_bubble
        net = sgs_cnn.SGSNet(seed=0, zero_last=False)
        net.w[3] *= 0.01   # corrections of the size a trained network makes
        net.refresh()

        def corrected_cost(dims, n):
            Sc = lsgs.coarse_solver(dims=dims)
            cphys, _ = warm_bubble(*dims, 600.0, 600.0, 300.0)
            Sc.upload(cphys, dtype=np.float32)
            Sc.step(20)
            xc = lag.get_state(Sc)
            cplain = lsgs.step_cost(Sc, xc, n=n)
            clearn = lsgs.step_cost(Sc, xc, net, sgs_cnn.make_scale([xc]), n=n)
            Sc.close()
            return cplain, clearn

        def train_cost(dims, kernel, reps):
            # one forward + backward of the network (input, weight and bias gradients), as a
            # training step through the solver runs it per corrected step
            lib = _lib.load()
            _lib.check(lib.lexgb_cnn_set_kernel(kernel))
            n = dims[0] * dims[1] * dims[2]
            gen = torch.Generator(device="cpu").manual_seed(5)
            x = torch.rand(n, 5, generator=gen).cuda().requires_grad_(True)
            seed = torch.randn(n, 5, generator=gen).cuda()
            params = [t.detach().clone().requires_grad_(True) for t in net.params()]
            tnet = sgs_cnn.SGSNet(seed=0, zero_last=False)
            tnet.w, tnet.b = params[:4], params[4:]
            tnet.refresh()

            def once():
                out = sgs_cnn.net_apply(tnet, x, dims)
                return torch.autograd.grad((out * seed).sum(), [x] + params)
            once()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                once()
            e1.record()
            torch.cuda.synchronize()
            _lib.check(lib.lexgb_cnn_set_kernel(0))
            return e0.elapsed_time(e1) / reps

        cplain, clearn = corrected_cost((32, 32, 32), 300)
        lplain, llearn = corrected_cost((128, 128, 64), 100)
        t_tc = train_cost((128, 128, 64), 2, 10)
        t_legacy = train_cost((128, 128, 64), 1, 3)
        sgs = {"grid": [32, 32, 32], "dx_m": [600.0, 600.0, 300.0], "dt_s": 3.0,
               "ms_per_step_plain": cplain, "ms_per_step_learned": clearn, "cost_ratio": clearn / cplain,
               "grid_128x128x64": {"ms_per_step_plain": lplain, "ms_per_step_learned": llearn,
                                   "cost_ratio": llearn / lplain},
               "network_fwd_bwd_128x128x64_ms": {"tcgen05": t_tc, "mma_sync_and_cuda_core_dw": t_legacy,
                                                 "note": "net_apply + autograd.grad of the input and all "
                                                         "parameters: four convolutions, four input-gradient "
                                                         "convolutions, four weight gradients"},
               "note": "CNN 5-32-32-32-5 (3x3x3, BF16 tensor cores: tcgen05 where the grid fits its tiles) "
                       "applied after every big step inside the step's CUDA graph (lexgb_set_sgs_net); CUDA "
                       "events over 300 (32^3) and 100 (128x128x64) steps each"}
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "warm bubble 192x192x96 @ 100 m (19.2x19.2x9.6 km), dt = 1 s, WS-RK3 with "
                               "1+16+32 acoustic sub-steps, WENO5, Smagorinsky Cs=0.18",
                   "grid": [g["nx"], g["ny"], g["nz"]], "dx_m": g["dx"], "dt_s": g["dt"], "n_sound": g["n_sound"],
                   "l2": "inputs larger than L2: ~0.7 GB of fields touched per step vs 129 MB L2",
                   "acoustic_form": S.acoustic_form,
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "kernel": "k_acoustic (one acoustic sub-step)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": B_ACOUSTIC * npts, "ms_per_launch": ac_ms,
                     "step_frac_of_roofline": value / ws * B_ALG / (peak * 1e9),
                     "step_bytes_per_point": B_ALG},
        "kernel_ms": kern,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "path": "lexgb_upload_state (pinned FP32 host) + lexgb_step + "
                                            "lexgb_download_state (pinned FP32 host)"},
        "gpu_launches": kernels_per_step * args.steps,
        "nonfinite_after": n_bad,
        "clocks": clk,
    }
    if adjoint is not None:
        line["adjoint"] = adjoint
    if sgs is not None:
        line["learned_sgs"] = sgs
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    print(json.dumps(line), flush=True)
    S.close()
    if dist is not None:
        dist.destroy_process_group()


def profile_sgs(args):
    """Warm-up + timed coarse steps (600 m x 600 m x 300 m; 32^3 or --sgs-dims) with the fused CNN
    correction."""
    import torch
    from lex_gb300 import learned_sgs as lsgs, sgs_cnn, autograd as lag
    from lex_gb300.workload import warm_bubble
    dims = tuple(int(v) for v in args.sgs_dims.split(","))
    S = lsgs.coarse_solver(dims=dims)
    phys, _ = warm_bubble(*dims, 600.0, 600.0, 300.0)
    S.upload(phys, dtype=np.float32)
    S.step(args.warmup)
    x = lag.get_state(S)
    net = sgs_cnn.SGSNet(seed=0, zero_last=False)
    net.w[3] *= 0.01
    net.refresh()
    sgs_cnn.attach(S, net, sgs_cnn.make_scale([x]))
    S.step(args.warmup)
    torch.cuda.synchronize()
    S.step(args.steps)
    torch.cuda.synchronize()
    S.close()
    print(json.dumps({"profile_sgs": True, "steps": args.steps, "warmup": args.warmup}))


def profile_cnn(args):
    """CUDA-event times of the correction's layer shapes at --sgs-dims (default here 128,128,64):
    lexgb_cnn_conv3d without the FP32 pre-activation (as in the step graph) and
    lexgb_cnn_conv3d_dw, each on the tcgen05 kernel and on the legacy one (mma.sync convolution,
    FP32 CUDA-core weight gradient); --steps launches each after --warmup."""
    import ctypes
    import torch
    from lex_gb300 import _lib
    lib = _lib.load()
    dims = tuple(int(v) for v in args.sgs_dims.split(","))
    nx, ny, nz = dims
    n = nx * ny * nz
    gen = torch.Generator(device="cpu").manual_seed(7)
    P = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None

    def timed(call, reps):
        for _ in range(args.warmup):
            _lib.check(call())
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            call()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps * 1e3

    out = {"profile_cnn": True, "grid": list(dims), "unit": "us per launch", "layers": {}}
    for cin, cout, gstride in ((16, 32, 32), (32, 32, 32), (32, 8, 16)):
        x = torch.randn(n, cin, generator=gen).to(torch.bfloat16).cuda()
        w = (0.2 * torch.randn(27, cout, cin, generator=gen)).to(torch.bfloat16).cuda()
        b = torch.randn(cout, generator=gen).cuda()
        g = torch.randn(n, gstride, generator=gen).to(torch.bfloat16).cuda()
        yb = torch.empty(n, cout, dtype=torch.bfloat16, device="cuda")
        yf = torch.empty(n, cout, device="cuda")
        dw = torch.zeros(27, cout, cin, device="cuda")
        last = cout == 8
        flop = 2 * 27 * cin * cout * n
        rec = {}
        for name, code in (("tcgen05", 2), ("legacy", 1)):
            _lib.check(lib.lexgb_cnn_set_kernel(code))
            conv = lambda: lib.lexgb_cnn_conv3d(nx, ny, nz, cin, cout, P(x), P(w), P(b), None,
                                                None if last else P(yb), P(yf) if last else None,
                                                0 if last else 1, 5 if last else cout, None)
            dwc = lambda: lib.lexgb_cnn_conv3d_dw(nx, ny, nz, cin, cout, gstride, P(x), P(g), P(dw), None, None)
            tc = timed(conv, args.steps)
            td = timed(dwc, args.steps if name == "tcgen05" else max(1, args.steps // 10))
            rec[name] = {"conv3d": tc, "conv3d_dw": td, "conv3d_tflops": flop / tc / 1e6,
                         "conv3d_dw_tflops": flop / td / 1e6}
        _lib.check(lib.lexgb_cnn_set_kernel(0))
        out["layers"]["%d->%d" % (cin, cout)] = rec
    t = ctypes.c_uint(0)
    _lib.check(lib.lexgb_cnn_take_timeouts(ctypes.byref(t)))
    out["tcgen05_timeouts"] = t.value
    print(json.dumps(out))


def profile_adjoint(args):
    """Warm-up + timed forward-with-intermediates + reverse passes of the benchmarked step
    (lexgb_step_keep + lexgb_step_vjp_kept), for profiler captures."""
    import ctypes
    import torch
    from lex_gb300.solver import Solver
    from lex_gb300 import _lib
    g = GRID
    phys, profile = build_case(**g)
    S = Solver(g["nx"], g["ny"], g["nz"], g["dx"], g["dy"], g["dz"], g["dt"], g["n_sound"], turb_opt=1)
    S.integrate_base_state(profile["theta0"], profile["qv0"])
    S.upload(phys, dtype=np.float32)
    shp = [(g["nz"], g["ny"], g["nx"])] * 6
    shp[3] = (g["nz"] + 1, g["ny"], g["nx"])
    gen = torch.Generator(device="cuda").manual_seed(1)
    ybar = [torch.randn(sh, device="cuda", generator=gen) for sh in shp]
    xbar = [torch.empty(sh, device="cuda") for sh in shp]
    yp = (ctypes.c_void_p * 6)(*[t.data_ptr() for t in ybar])
    xp = (ctypes.c_void_p * 6)(*[t.data_ptr() for t in xbar])
    for _ in range(args.warmup + args.steps):
        _lib.check(S.lib.lexgb_step_keep(S.handle))
        _lib.check(S.lib.lexgb_step_vjp_kept(S.handle, yp, xp, 1))
    torch.cuda.synchronize()
    S.close()
    print(json.dumps({"profile_adjoint": True, "steps": args.steps, "warmup": args.warmup}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="lexgb", choices=["lexgb", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the forward+adjoint cost measurement")
    ap.add_argument("--no-sgs", action="store_true", help="skip the learned-SGS step cost measurement")
    ap.add_argument("--profile", action="store_true", help="only warm-up + timed steps (profiler captures)")
    ap.add_argument("--profile-sgs", action="store_true",
                    help="only a few coarse 32^3 steps with the fused learned SGS correction (profiler captures)")
    ap.add_argument("--profile-cnn", action="store_true",
                    help="only CUDA-event times of the correction's convolutions and weight gradients, tcgen05 "
                         "against the legacy kernels, at --sgs-dims")
    ap.add_argument("--sgs-dims", default=None, help="nx,ny,nz of --profile-sgs (32,32,32) / --profile-cnn "
                                                      "(128,128,64)")
    ap.add_argument("--acoustic-kernel", default="auto", choices=["auto", "rows", "tile", "persistent"],
                    help="form of the acoustic sub-steps (auto: the fastest measured for the grid)")
    ap.add_argument("--profile-adjoint", action="store_true",
                    help="only forward-with-intermediates + reverse passes of the step (profiler captures)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "lexgb":
        args.warmup = 3
    if args.sgs_dims is None:
        args.sgs_dims = "128,128,64" if args.profile_cnn else "32,32,32"
    if args.profile_sgs:
        profile_sgs(args)
    elif args.profile_cnn:
        profile_cnn(args)
    elif args.profile_adjoint:
        profile_adjoint(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_lexgb(args)


if __name__ == "__main__":
    main()
