"""Precision of the gradient of the differentiable-step case (64^3, 300 x 300 x 150 m, dt 2 s): the
library's FP32 reverse mode against torch.autograd through the oracle in FP64 (the exact derivative
of the discrete step) and in FP32 (the reference's arithmetic in FP32), over 30 and 300 steps; whole
dL/dtheta0 vectors, four seeded directions and dL/dCs.  Test infrastructure (imports the oracle);
the numbers are summarised in profiles/gradcheck_64cube.md.

    python tests/gradcheck_precision.py [out.json]      # on a GPU, about 15 minutes
"""
import sys, os, json, time
here = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(here)); sys.path.insert(0, here)
import numpy as np, torch
from torch.utils.checkpoint import checkpoint
from test_gpu_gradcheck import library_gradient, N, SPACING as SP, DT, CS0, SEED
from oracle.ic import Grid, pad_scalar
from oracle.dycore import Dycore
out = {}
inner = (slice(3, -3), slice(3, -3), slice(1, -1))
for steps in (30, 300):
    t0 = time.time()
    L, g_theta, gcs_lib, cols, phys, phys_t = library_gradient(steps)
    g_lib = g_theta.permute(2, 1, 0).contiguous()     # (x, y, z)
    res = {"loss_lib": L, "t_lib": time.time() - t0, "dLdCs_lib": gcs_lib}
    grads = {}
    for name, dt in (("f64", np.float64), ("f32", np.float32)):
        t1 = time.time()
        D = Dycore(Grid(N, N, N, *SP), cols, DT, 32, dtype=dt, device="cuda")
        with torch.no_grad():
            y = D.cast(phys_t)
            for _ in range(steps):
                y, _ = D.step(y)
            tt = y[0][inner].double() - 300.0
        xs = D.cast(phys)
        th_i = xs[0][inner].clone().requires_grad_(True)
        csv = torch.tensor(CS0, dtype=torch.float64 if dt == np.float64 else torch.float32, device="cuda",
                           requires_grad=True)
        D.cs = csv
        def one(th, *rest):
            n, _ = D.step((pad_scalar(th),) + rest)
            return (n[0][inner],) + tuple(n[1:])
        s = (th_i,) + tuple(xs[1:])
        for _ in range(steps):
            s = checkpoint(one, *s, use_reentrant=False)
        Lo = ((s[0].double() - 300.0 - tt) ** 2).mean()
        Lo.backward()
        grads[name] = th_i.grad.double()
        res["loss_" + name] = float(Lo)
        res["dLdCs_" + name] = float(csv.grad)
        res["t_" + name] = time.time() - t1
        del D, s, Lo
        torch.cuda.empty_cache()
    g64 = grads["f64"]
    rel = lambda a: float((a - g64).norm() / g64.norm())
    res["full_rel_err_lib"] = rel(g_lib)
    res["full_rel_err_oracle_f32"] = rel(grads["f32"])
    gen = torch.Generator(device="cuda").manual_seed(SEED)
    dd = []
    for k in range(4):
        v = torch.randn((N, N, N), device="cuda", generator=gen, dtype=torch.float64).permute(2, 1, 0)
        dd.append({"lib": float((g_lib * v).sum()), "f64": float((g64 * v).sum()), "f32": float((grads["f32"] * v).sum())})
    res["directions"] = dd
    out[steps] = res
    print(steps, json.dumps(res), flush=True)
if len(sys.argv) > 1:
    json.dump(out, open(sys.argv[1], "w"), indent=1)
