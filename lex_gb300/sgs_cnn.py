"""Learned SGS correction: the 3-D CNN of the reference (simpleCNN, dl_models.py:19-30) on the
library's BF16 tensor-core kernels, as a torch.autograd operation.

    x (5 normalised fields at cell centres) -> conv 5->32, GELU -> conv 32->32, GELU
      -> conv 32->32, GELU -> conv 32->5 -> correction (5 fields)

All convolutions are 3x3x3 with zero padding ('SAME'), biases on, tanh-GELU (flax ``nn.gelu``).
The forward runs ``lexgb_cnn_conv3d`` (BF16 operands, FP32 accumulation); the backward runs the
same kernel on the mirrored, transposed weights for the input gradients, ``lexgb_cnn_gelu_bwd``
and ``lexgb_cnn_conv3d_dw`` for the weight and bias gradients.  ``adam_step`` updates the FP32
master weights with ``lexgb_cnn_adam`` (the reference uses optax.lamb, lex_dl_train.py).

Packing, as the reference's (dl_models.py:125-182, one_sprint_functions.py:136-151): theta, u, v, w,
qv are min-max normalised on their own points with per-level constants (w per face level), the
normalised winds averaged to cell centres (unstagger_uvw); the correction's winds go back to the
faces as stagger_uvw puts them (the mean of the two cells beside a face, face 0 of u and v taking the
value of face nx-1 / ny-1, w zero on the bottom and the lid) and every field is scaled by the output
range at its own point.  Packing runs as torch element-wise operations here (differentiable, for
training) and as the kernels of ``lexgb_set_sgs_net`` inside the library's step (inference,
:func:`attach`); both round the same way.

A scale is a dict of CUDA tensors, fields (theta, u, v, w, qv): ``lo`` and ``rin`` [5, nz+1]
(input minimum and range per level; entry nz is used by w's lid face only, the other fields repeat
their top level there) and ``rout`` [5, nz+1, ny, nx] (output range at each field's points: cells
for theta and qv, west / south faces for u / v, faces 0..nz for w).
"""
import ctypes

import torch

from . import _lib

CIN0, C, COUT_REAL = 5, 32, 5
LAYERS = ((16, 32, True), (32, 32, True), (32, 32, True), (32, 8, False))  # (cin padded, cout padded, GELU)


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    h = torch.cuda.current_stream().cuda_stream
    return ctypes.c_void_p(h if h else 1)   # 1: cudaStreamLegacy (torch's default stream)


class SGSNet:
    """Parameters (FP32 masters + BF16 copies) and Adam moments of the four convolutions."""

    def __init__(self, seed=0, init_scale=1.0, zero_last=True):
        """He-normal weights, zero biases; zero_last: the last layer starts at zero, so that
        training starts from the uncorrected model."""
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.w, self.b, self.wbf = [], [], []
        for li, (cin, cout, _) in enumerate(LAYERS):
            rin = CIN0 if li == 0 else C
            rout = COUT_REAL if li == 3 else C
            w = torch.zeros(27, cout, cin)
            std = init_scale * (2.0 / (27 * rin)) ** 0.5
            w[:, :rout, :rin] = torch.randn(27, rout, rin, generator=g) * std
            if li == 3 and zero_last:
                w.zero_()
            self.w.append(w.cuda())
            self.b.append(torch.zeros(cout, device="cuda"))
        self.m = [torch.zeros_like(t) for t in self.w + self.b]
        self.v = [torch.zeros_like(t) for t in self.w + self.b]
        self.step_count = 0
        self.refresh()

    def refresh(self):
        self.wbf = [w.to(torch.bfloat16).contiguous() for w in self.w]

    def params(self):
        return self.w + self.b

    def state_dict(self):
        return {"w": [t.cpu() for t in self.w], "b": [t.cpu() for t in self.b]}

    def load_state_dict(self, d):
        self.w = [t.cuda() for t in d["w"]]
        self.b = [t.cuda() for t in d["b"]]
        self.refresh()


def conv3d(x_bf16, w_bf16, bias, nx, ny, nz, cin, cout, gelu, creal, want_pre=True, out_f32=False):
    """One convolution; x_bf16 [npts, cin] -> (pre FP32 or None, y BF16 or None, y FP32 or None)."""
    n = nx * ny * nz
    pre = torch.empty(n, cout, device="cuda") if want_pre else None
    ybf = None if out_f32 else torch.empty(n, cout, device="cuda", dtype=torch.bfloat16)
    yf = torch.empty(n, cout, device="cuda") if out_f32 else None
    _lib.check(_lib.load().lexgb_cnn_conv3d(nx, ny, nz, cin, cout, _p(x_bf16), _p(w_bf16), _p(bias), _p(pre),
                                            _p(ybf), _p(yf), 1 if gelu else 0, creal, _stream()))
    return pre, ybf, yf


def _mirror(w_bf16):
    """[27][cout][cin] -> [27][cin][cout] with the offsets reversed: the input-gradient weights."""
    return w_bf16.flip(0).transpose(1, 2).contiguous()


def _pad_channels(t, c):
    if t.shape[1] == c:
        return t.contiguous()
    out = torch.zeros(t.shape[0], c, device=t.device, dtype=t.dtype)
    out[:, :t.shape[1]] = t
    return out


class _NetFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, net, dims, *params):
        nx, ny, nz = dims
        a = _pad_channels(x.to(torch.bfloat16), 16)
        acts, pres = [a], []
        for li, (cin, cout, gelu) in enumerate(LAYERS):
            last = li == len(LAYERS) - 1
            pre, ybf, yf = conv3d(acts[-1], net.wbf[li], net.b[li], nx, ny, nz, cin, cout, gelu,
                                  COUT_REAL if last else cout, want_pre=not last, out_f32=last)
            pres.append(pre)
            if not last:
                acts.append(ybf)
            else:
                out = yf[:, :COUT_REAL].contiguous()
        ctx.net, ctx.dims, ctx.acts, ctx.pres = net, dims, acts, pres
        return out

    @staticmethod
    def backward(ctx, gout):
        net, (nx, ny, nz) = ctx.net, ctx.dims
        lib = _lib.load()
        n = nx * ny * nz
        st = _stream()
        # gradient at the last layer's output: no GELU; channels padded to 16 for the input-gradient conv
        dy = _pad_channels(gout.float().contiguous(), 8)
        g = torch.empty(n, 16, device="cuda", dtype=torch.bfloat16)
        _lib.check(lib.lexgb_cnn_gelu_bwd(n, 8, 16, _p(dy), None, _p(g), st))
        gstride = 16
        grads_w = [None] * len(LAYERS)
        grads_b = [None] * len(LAYERS)
        dx = None
        for li in range(len(LAYERS) - 1, -1, -1):
            cin, cout, _ = LAYERS[li]
            dw = torch.zeros(27, cout, cin, device="cuda")
            db = torch.zeros(cout, device="cuda")
            _lib.check(lib.lexgb_cnn_conv3d_dw(nx, ny, nz, cin, cout, gstride, _p(ctx.acts[li]), _p(g), _p(dw),
                                               _p(db), st))
            grads_w[li], grads_b[li] = dw, db
            # input gradient: mirrored weights, padded so that the gradient's channels are the k16 input
            wm = _mirror(net.wbf[li])                       # [27][cin][cout]
            if gstride != cout:
                wm = torch.cat([wm, torch.zeros(27, cin, gstride - cout, device="cuda", dtype=wm.dtype)], 2)
            _, _, da = conv3d(g, wm.contiguous(), None, nx, ny, nz, gstride, cin, False, cin,
                              want_pre=False, out_f32=True)
            if li == 0:
                dx = da[:, :CIN0].contiguous()
                break
            g = torch.empty(n, cin, device="cuda", dtype=torch.bfloat16)
            _lib.check(lib.lexgb_cnn_gelu_bwd(n, cin, cin, _p(da), _p(ctx.pres[li - 1]), _p(g), st))
            gstride = cin
        return (dx, None, None) + tuple(grads_w) + tuple(grads_b)


def net_apply(net, x, dims):
    """Correction for x [npts, 5] (FP32, differentiable in x and the parameters)."""
    return _NetFn.apply(x, net, dims, *net.params())


def adam_step(net, grads, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step of the network's FP32 master parameters on the GPU (lexgb_cnn_adam)."""
    lib = _lib.load()
    net.step_count += 1
    for i, (p, gr) in enumerate(zip(net.params(), grads)):
        if gr is None:
            continue
        gr = gr.contiguous().float()
        _lib.check(lib.lexgb_cnn_adam(p.numel(), _p(p), _p(gr), _p(net.m[i]), _p(net.v[i]), None,
                                      lr, beta1, beta2, eps, net.step_count, _stream()))
    net.refresh()


# ------------------------------------------------------------------------------------------------
# packing of the device-layout state (theta, u, v, w, pi', qv) (dl_models.py:125-182)
# ------------------------------------------------------------------------------------------------
FIELDS5 = ("theta", "u", "v", "w", "qv")


def pack(state, scale):
    """state: six CUDA tensors (nz, ny, nx) / w (nz+1, ny, nx) -> [npts, 5] normalised, x fastest."""
    th, u, v, w, _, q = state
    nz = th.shape[0]
    lo, rin = scale["lo"], scale["rin"]
    n = lambda a, f, m: (a - lo[f, :m].view(-1, 1, 1)) / rin[f, :m].view(-1, 1, 1)
    un, vn, wn = n(u, 1, nz), n(v, 2, nz), n(w, 3, nz + 1)
    cols = (n(th, 0, nz), 0.5 * (un + torch.roll(un, -1, dims=2)), 0.5 * (vn + torch.roll(vn, -1, dims=1)),
            0.5 * (wn[:-1] + wn[1:]), n(q, 4, nz))
    return torch.stack([c.reshape(-1) for c in cols], 1)


def stagger(c, dim):
    """Cell values -> faces as stagger_uvw puts them (dl_models.py:172-182): face i >= 1 the mean of
    cells i-1 and i, face 0 the value of face n-1 (the face next to the far end)."""
    s = 0.5 * (c + torch.roll(c, 1, dims=dim))
    n = c.shape[dim]
    return torch.cat([s.narrow(dim, n - 1, 1), s.narrow(dim, 1, n - 1)], dim)


def unpack(corr, scale, dims):
    """[npts, 5] correction -> additions to (theta, u, v, w, pi', qv) on the staggered grid."""
    nx, ny, nz = dims
    c = [corr[:, i].reshape(nz, ny, nx) for i in range(5)]
    r = scale["rout"]
    z = torch.zeros(1, ny, nx, device=corr.device, dtype=corr.dtype)
    w = torch.cat([z, 0.5 * (c[3][:-1] + c[3][1:]), z], 0) * r[3]
    th = c[0] * r[0, :nz]
    return (th, stagger(c[1], 2) * r[1, :nz], stagger(c[2], 1) * r[2, :nz], w, torch.zeros_like(th),
            c[4] * r[4, :nz])


def correct(net, state, scale, dims):
    """state + CNN correction (one_sprint_functions.py:128-163), differentiable."""
    d = unpack(net_apply(net, pack(state, scale), dims), scale, dims)
    return tuple(a + b for a, b in zip(state, d))


def level_extrema(state):
    """Per-level minima and maxima of (theta, u, v, w, qv) on their own points, [5, nz+1] each
    (w per face level; the other fields repeat their top level in entry nz)."""
    th, u, v, w, _, q = state
    lo, hi = [], []
    for a in (th, u, v, w, q):
        mn, mx = a.amin(dim=(1, 2)), a.amax(dim=(1, 2))
        if mn.shape[0] == th.shape[0]:
            mn, mx = torch.cat([mn, mn[-1:]]), torch.cat([mx, mx[-1:]])
        lo.append(mn)
        hi.append(mx)
    return torch.stack(lo), torch.stack(hi)


def make_scale(states, margins=(0.01, 0.01, 0.01, 0.01, 1.0e-5)):
    """Per-level minimum and maximum over `states` (dataset_generation.py:80-90): input range
    max - min + margin per level (dl_models.py:128-152); output range max - min of the level, at
    every point of it (the reference's scaling_params carry a range per point; a few training
    states do not determine one, so the library's training uses the level's)."""
    lo, hi = None, None
    for st in states:
        mn, mx = level_extrema(st)
        lo = mn if lo is None else torch.minimum(lo, mn)
        hi = mx if hi is None else torch.maximum(hi, mx)
    nz, ny, nx = states[0][0].shape
    m = torch.tensor(margins, device=lo.device, dtype=lo.dtype).view(5, 1)
    rout = (hi - lo).view(5, nz + 1, 1, 1).expand(5, nz + 1, ny, nx).contiguous()
    return {"lo": lo.contiguous(), "rin": (hi - lo + m).contiguous(), "rout": rout}


def attach(solver, net, scale):
    """Apply the network after every big step of ``solver.step`` inside the library's step graph
    (lexgb_set_sgs_net); call again after the weights change.  ``attach(solver, None, None)``
    turns the correction off."""
    from .autograd import _bind_stream
    lib = _lib.load()
    _bind_stream(solver)
    if net is None:
        _lib.check(lib.lexgb_set_sgs_net(solver.handle, None, None, None, None, None, 0))
        return
    P4 = ctypes.c_void_p * 4
    w = P4(*[t.data_ptr() for t in net.wbf])
    b = P4(*[t.data_ptr() for t in net.b])
    _lib.check(lib.lexgb_set_sgs_net(solver.handle, w, b, _p(scale["lo"]), _p(scale["rin"]), _p(scale["rout"]), 1))
