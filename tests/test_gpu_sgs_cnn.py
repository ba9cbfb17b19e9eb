"""The learned-SGS CNN kernels against a plain PyTorch fp32 reference of the same network
(torch conv3d on the same BF16-rounded weights): forward, input and parameter gradients, Adam.
Tolerances are BF16 level (activations are stored in BF16 between layers)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reference(net, x, dims):
    import torch
    import torch.nn.functional as F
    from lex_gb300.sgs_cnn import LAYERS
    nx, ny, nz = dims
    ws, bs = [], []
    a = x.reshape(nz, ny, nx, -1).permute(3, 0, 1, 2).unsqueeze(0)     # [1, C, z, y, x]
    a = a.to(torch.bfloat16).float()
    for li, (cin, cout, gelu) in enumerate(LAYERS):
        w = net.w[li].to(torch.bfloat16).float().detach().clone().requires_grad_(True)
        b = net.b[li].detach().clone().requires_grad_(True)
        ws.append(w)
        bs.append(b)
        wt = w.reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)         # [cout, cin, dz, dy, dx]
        if a.shape[1] < cin:
            a = torch.cat([a, torch.zeros(1, cin - a.shape[1], nz, ny, nx, device="cuda")], 1)
        a = F.conv3d(a, wt, b, padding=1)
        if gelu:
            a = F.gelu(a, approximate="tanh")
            a = a.to(torch.bfloat16).float()       # the kernels store activations in BF16
    out = a[0, :5].permute(1, 2, 3, 0).reshape(-1, 5)
    return out, ws, bs


def _rel(a, b):
    return float((a - b).norm() / b.norm())


@pytest.fixture
def conv_kernel(built_lib):
    """Select the convolution kernel for one test (lexgb_cnn_set_kernel), back to AUTO after it;
    a tcgen05 test also checks that none of its bounded waits gave up."""
    import ctypes
    chosen = {}

    def use(name):
        chosen["name"] = name
        code = {"auto": 0, "mma": 1, "tcgen05": 2}[name]
        assert built_lib.lexgb_cnn_set_kernel(code) == 0
    yield use
    n = ctypes.c_uint(0)
    assert built_lib.lexgb_cnn_take_timeouts(ctypes.byref(n)) == 0
    built_lib.lexgb_cnn_set_kernel(0)
    assert n.value == 0, n.value


KERNEL_CASES = [("mma", (16, 8, 6)), ("tcgen05", (16, 16, 6)), ("tcgen05", (32, 32, 8))]


@pytest.mark.parametrize("kernel,dims", KERNEL_CASES, ids=["%s-%dx%dx%d" % ((k,) + d) for k, d in KERNEL_CASES])
def test_cnn_forward_and_gradients_match_torch(conv_kernel, kernel, dims):
    torch = pytest.importorskip("torch")
    from lex_gb300 import sgs_cnn
    conv_kernel(kernel)
    n = dims[0] * dims[1] * dims[2]
    net = sgs_cnn.SGSNet(seed=1, init_scale=1.0, zero_last=False)
    for t in net.params():
        t.requires_grad_(True)
    g = torch.Generator(device="cpu").manual_seed(2)
    x = torch.rand(n, 5, generator=g).cuda().requires_grad_(True)
    out = sgs_cnn.net_apply(net, x, dims)
    xr = x.detach().clone().requires_grad_(True)
    ref, ws, bs = _reference(net, xr, dims)
    assert _rel(out.detach(), ref.detach()) < 2e-2
    seed = torch.randn(n, 5, generator=g).cuda()
    gx, *gp = torch.autograd.grad((out * seed).sum(), [x] + net.params())
    rx, *rp = torch.autograd.grad((ref * seed).sum(), [xr] + ws + bs)
    assert _rel(gx, rx) < 3e-2, _rel(gx, rx)
    for i, (a, b) in enumerate(zip(gp, rp)):
        if b.norm() > 0:
            assert _rel(a, b) < 3e-2, (i, _rel(a, b))


def test_adam_matches_formula(built_lib):
    torch = pytest.importorskip("torch")
    from lex_gb300 import sgs_cnn
    net = sgs_cnn.SGSNet(seed=3)
    w0 = [t.detach().clone() for t in net.params()]
    m = [torch.zeros_like(t) for t in w0]
    v = [torch.zeros_like(t) for t in w0]
    g = torch.Generator(device="cpu").manual_seed(4)
    lr, b1, b2, eps = 1e-3, 0.9, 0.999, 1e-8
    for step in range(1, 4):
        grads = [torch.randn(t.shape, generator=g).cuda() for t in w0]
        sgs_cnn.adam_step(net, grads, lr, b1, b2, eps)
        for i, gr in enumerate(grads):
            m[i] = b1 * m[i] + (1 - b1) * gr
            v[i] = b2 * v[i] + (1 - b2) * gr * gr
            w0[i] = w0[i] - lr * (m[i] / (1 - b1 ** step)) / ((v[i] / (1 - b2 ** step)).sqrt() + eps)
    for a, b in zip(net.params(), w0):
        assert float((a - b).abs().max()) < 1e-6


@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 32), (32, 8), (16, 8)])
def test_tcgen05_convolution_matches_mma_sync(conv_kernel, cin, cout):
    """One convolution layer (zero padding, bias, FP32 pre-activation) on the tcgen05 kernel against
    the mma.sync kernel on the same BF16 inputs: both accumulate the same BF16 products in FP32, in a
    different order, so they agree to FP32 summation rounding."""
    torch = pytest.importorskip("torch")
    nx, ny, nz = 32, 16, 5
    g = torch.Generator(device="cpu").manual_seed(cin + cout)
    x = torch.randn(nz * ny * nx, cin, generator=g).to(torch.bfloat16).cuda()
    w = (0.2 * torch.randn(27, cout, cin, generator=g)).to(torch.bfloat16).cuda()
    b = torch.randn(cout, generator=g).cuda()
    outs = {}
    for kernel in ("mma", "tcgen05"):
        conv_kernel(kernel)
        pre = torch.empty(nz * ny * nx, cout, device="cuda")
        yb = torch.empty(nz * ny * nx, cout, dtype=torch.bfloat16, device="cuda")
        rc = _conv_call(nx, ny, nz, cin, cout, x, w, b, pre, yb)
        assert rc == 0
        torch.cuda.synchronize()
        outs[kernel] = (pre, yb)
    a, r = outs["tcgen05"][0], outs["mma"][0]
    assert _rel(a, r) < 1e-5, _rel(a, r)
    assert _rel(outs["tcgen05"][1].float()[:, :5], outs["mma"][1].float()[:, :5]) < 1e-2


def _conv_call(nx, ny, nz, cin, cout, x, w, b, pre, yb):
    """lexgb_cnn_conv3d with GELU, 5 real output channels, the default stream."""
    import ctypes
    from lex_gb300 import _lib
    lib = _lib.load()
    return lib.lexgb_cnn_conv3d(nx, ny, nz, cin, cout, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(w.data_ptr()),
                                ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(pre.data_ptr()),
                                ctypes.c_void_p(yb.data_ptr()), None, 1, 5, None)


DW_CASES = [(16, 32, 32, (32, 32, 8)), (32, 32, 32, (32, 32, 8)), (32, 8, 16, (32, 32, 8)), (16, 8, 16, (16, 16, 6)),
            (32, 32, 32, (20, 13, 5)), (16, 32, 32, (9, 17, 3))]


@pytest.mark.parametrize("cin,cout,gstride,dims", DW_CASES,
                         ids=["%d-%d-%d-%dx%dx%d" % ((a, b, c) + d) for a, b, c, d in DW_CASES])
def test_tcgen05_weight_gradient_matches_cuda_cores(conv_kernel, cin, cout, gstride, dims):
    """lexgb_cnn_conv3d_dw on the tensor cores (tcgen05, the AUTO choice) against the FP32 CUDA-core
    reduction (the LEXGB_CNN_MMA choice) on the same BF16 activations and gradients, including grids
    that the 8 x 16 tiles do not divide: both sum the same exact BF16 products in FP32, in a
    different order, so they agree to FP32 summation rounding; the bias gradient is the same kernel
    on both."""
    torch = pytest.importorskip("torch")
    import ctypes
    from lex_gb300 import _lib
    lib = _lib.load()
    nx, ny, nz = dims
    n = nx * ny * nz
    gen = torch.Generator(device="cpu").manual_seed(cin * 7 + cout + gstride + nx)
    x = torch.randn(n, cin, generator=gen).to(torch.bfloat16).cuda()
    g = torch.randn(n, gstride, generator=gen).to(torch.bfloat16).cuda()
    outs = {}
    for kernel in ("mma", "tcgen05"):
        conv_kernel(kernel)
        dw = torch.zeros(27, cout, cin, device="cuda")
        db = torch.zeros(cout, device="cuda")
        rc = lib.lexgb_cnn_conv3d_dw(nx, ny, nz, cin, cout, gstride, ctypes.c_void_p(x.data_ptr()),
                                     ctypes.c_void_p(g.data_ptr()), ctypes.c_void_p(dw.data_ptr()),
                                     ctypes.c_void_p(db.data_ptr()), None)
        assert rc == 0
        torch.cuda.synchronize()
        outs[kernel] = (dw, db)
    a, r = outs["tcgen05"][0], outs["mma"][0]
    assert _rel(a, r) < 1e-5, _rel(a, r)
    # every offset on its own (the edge offsets see fewer points)
    for tap in range(27):
        assert _rel(a[tap], r[tap]) < 1e-5, (tap, _rel(a[tap], r[tap]))
    assert _rel(outs["tcgen05"][1], outs["mma"][1]) < 1e-6
