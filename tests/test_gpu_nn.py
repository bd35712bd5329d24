"""GPU: the warm-start network's tensor-core kernels (tcgen05.mma).

- forward convolution against torch's FP32 conv2d on the same bf16 inputs
  (FP32 accumulation on both sides: tolerance 1e-4 relative);
- data and weight gradients of one layer against torch autograd in FP32
  (the GPU rounds dz to bf16: tolerance 2e-2 relative);
- the whole network's parameter gradients against the CPU oracle
  (oracle/nn_oracle.py) with the same bf16 roundings of activations and dz
  (tolerance 1e-2 relative per layer), and without them (float64 throughout:
  the layer-0 gradient then differs by the accumulated bf16 error, < 2e-1);
- training lowers the loss.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("stride,up,cin,cout", [(1, 0, 16, 48), (2, 0, 48, 48), (1, 1, 48, 16),
                                                (2, 0, 16, 16)])
def test_conv_forward_and_grads_vs_torch(built, stride, up, cin, cout):
    import torch
    import torch.nn.functional as F
    import imexlb as im
    from imexlb.neural import _p
    torch.manual_seed(0)
    n, h, w = 2, 12, 20
    x = torch.randn(n, h, w, cin, device="cuda").to(torch.bfloat16)
    wt = (torch.randn(cout, 9 * cin, device="cuda") * 0.2).to(torch.bfloat16)
    b = torch.randn(cout, device="cuda")
    hg, wg = (2 * h, 2 * w) if up else (h, w)
    d = im.ConvDesc(n, h, w, cin, (hg - 1) // stride + 1, (wg - 1) // stride + 1, cout, 0, stride, up)
    y = torch.empty(n, d.hout, d.wout, cout, device="cuda")
    L = im.lib()
    import ctypes as C
    assert L.imexlb_nn_conv_fwd(C.byref(d), _p(x), _p(wt), _p(b), 0, None, _p(y), None) == 0
    # torch reference in FP32
    xr = x.float().permute(0, 3, 1, 2).requires_grad_(True)
    wr = wt.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2).requires_grad_(True)
    xin = F.interpolate(xr, scale_factor=2, mode="nearest") if up else xr
    yr = F.conv2d(xin, wr, b, stride=stride, padding=1)
    torch.cuda.synchronize()
    assert _rel(y.cpu().numpy(), yr.permute(0, 2, 3, 1).detach().cpu().numpy()) < 1e-4
    # gradients: dz = random, no activation
    dy = torch.randn_like(y)
    dz = torch.empty_like(y, dtype=torch.bfloat16)
    gb = torch.zeros(cout, device="cuda")
    assert L.imexlb_nn_act_grad(_p(dy), None, dy.numel(), cout, 0, _p(dz), _p(gb), None) == 0
    gw = torch.zeros(cout, 9 * cin, device="cuda")
    assert L.imexlb_nn_conv_bwd_weight(C.byref(d), _p(x), _p(dz), _p(gw), None) == 0
    dgrid = torch.empty(n, hg, wg, cin, device="cuda")
    dx = torch.empty(n, h, w, cin, device="cuda") if up else None
    wtt = torch.empty(cin, 9 * cout, dtype=torch.bfloat16, device="cuda")
    assert L.imexlb_nn_conv_bwd_data(C.byref(d), _p(dz), _p(wt), _p(wtt), _p(dgrid), _p(dx), None) == 0
    yr.backward(dz.float().permute(0, 3, 1, 2))
    torch.cuda.synchronize()
    gx = (dx if up else dgrid).cpu().numpy()
    assert _rel(gx, xr.grad.permute(0, 2, 3, 1).cpu().numpy()) < 2e-2
    gw_ref = wr.grad.permute(0, 2, 3, 1).reshape(cout, 9 * cin).cpu().numpy()
    assert _rel(gw.cpu().numpy(), gw_ref) < 2e-2
    # the bias gradient sums the FP32 dy (before rounding dz to bf16)
    assert _rel(gb.cpu().numpy(), dy.sum((0, 1, 2)).cpu().numpy()) < 1e-4
    st = C.c_int(-1)
    assert L.imexlb_nn_status(C.byref(st)) == 0 and st.value == 0


def test_network_gradients_vs_cpu_oracle(built):
    import torch
    from imexlb import neural
    from oracle import nn_oracle
    net = neural.Net(seed=3)
    rng = np.random.default_rng(1)
    n, H, W = 2, 16, 32
    frac = (rng.uniform(size=(n, H, W)) > 0.2).astype(np.float32)
    re = np.array([60.0, 150.0])
    x = neural.make_input(frac, re, torch)
    tgt = rng.standard_normal((n, H, W, 3)).astype(np.float32)
    T = torch.tensor(tgt, device="cuda")
    y = net.forward(x, keep=True)
    loss, dy = net.loss(y, T)
    grads = net.backward(dy)
    torch.cuda.synchronize()
    ws = [w.float().cpu().numpy().astype(np.float64) for w in net.wb]
    bs = [b.cpu().numpy().astype(np.float64) for b in net.b]
    x64 = x.float().cpu().numpy().astype(np.float64)
    nl = len(neural.LAYERS)
    for mimic, tol in ((True, 1e-2), (False, 2e-1)):
        lo, gws, gbs = nn_oracle.net_grads(x64, ws, bs, neural.LAYERS, tgt.astype(np.float64),
                                           mimic_bf16=mimic)
        assert abs(float(loss.item()) - lo) / lo < tol
        for i in range(nl):
            gw = grads[i].cpu().numpy()
            assert _rel(gw, gws[i]) < tol, (mimic, i, _rel(gw, gws[i]))
            gb = grads[nl + i].cpu().numpy()
            if np.linalg.norm(gbs[i]) > 0:
                assert _rel(gb, gbs[i]) < tol, (mimic, i, _rel(gb, gbs[i]))


def test_training_lowers_the_loss(built):
    from imexlb import neural
    rng = np.random.default_rng(0)
    n, H, W = 8, 32, 64
    yy, xx = np.mgrid[0:H, 0:W]
    frac = np.ones((n, H, W), dtype=np.float32)
    fields = np.zeros((n, 3, H, W), dtype=np.float32)
    re = rng.uniform(40, 200, n)
    for k in range(n):
        cx, cy, r = 16, H / 2 + rng.uniform(-2, 2), rng.uniform(3, 7)
        frac[k][(xx - cx) ** 2 + (yy - cy) ** 2 < r * r] = 0.0
        fields[k, 1] = 0.05 * frac[k] * (1 - np.exp(-np.abs(xx - cx) / (r * re[k] / 60)))
        fields[k, 0] = 0.0025 * np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (4 * r * r))
    net = neural.Net(seed=0)
    hist = neural.train(net, frac, re, fields, steps=150, batch=4, lr=3e-3)
    assert hist[-1][1] < 0.5 * hist[0][1]


@pytest.mark.parametrize("stride,up,cin,cout", [(1, 1, 48, 48), (2, 0, 16, 48), (1, 0, 48, 16)])
def test_conv_network_sizes_vs_torch(built, stride, up, cin, cout):
    """The layer shapes of the network at its training batch (16 images,
    128 x 256 input): many 128-row tiles per block, several pixel slices of
    the weight gradient."""
    import ctypes as C
    import torch
    import torch.nn.functional as F
    import imexlb as im
    from imexlb.neural import _p
    torch.manual_seed(1)
    n, h, w = 16, (64 if up else 128), (128 if up else 256)
    x = torch.randn(n, h, w, cin, device="cuda").to(torch.bfloat16)
    wt = (torch.randn(cout, 9 * cin, device="cuda") * 0.1).to(torch.bfloat16)
    b = torch.randn(cout, device="cuda")
    hg, wg = (2 * h, 2 * w) if up else (h, w)
    d = im.ConvDesc(n, h, w, cin, (hg - 1) // stride + 1, (wg - 1) // stride + 1, cout, 0, stride, up)
    L = im.lib()
    y = torch.empty(n, d.hout, d.wout, cout, device="cuda")
    assert L.imexlb_nn_conv_fwd(C.byref(d), _p(x), _p(wt), _p(b), 0, None, _p(y), None) == 0
    xr = x.float().permute(0, 3, 1, 2).requires_grad_(True)
    wr = wt.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2).requires_grad_(True)
    xin = F.interpolate(xr, scale_factor=2, mode="nearest") if up else xr
    yr = F.conv2d(xin, wr, b, stride=stride, padding=1)
    torch.cuda.synchronize()
    assert _rel(y.cpu().numpy(), yr.permute(0, 2, 3, 1).detach().cpu().numpy()) < 1e-4
    dz = (torch.randn_like(y) * 0.1).to(torch.bfloat16)
    gw = torch.zeros(cout, 9 * cin, device="cuda")
    assert L.imexlb_nn_conv_bwd_weight(C.byref(d), _p(x), _p(dz), _p(gw), None) == 0
    dgrid = torch.empty(n, hg, wg, cin, device="cuda")
    dx = torch.empty(n, h, w, cin, device="cuda") if up else None
    wtt = torch.empty(cin, 9 * cout, dtype=torch.bfloat16, device="cuda")
    assert L.imexlb_nn_conv_bwd_data(C.byref(d), _p(dz), _p(wt), _p(wtt), _p(dgrid), _p(dx), None) == 0
    yr.backward(dz.float().permute(0, 3, 1, 2))
    torch.cuda.synchronize()
    gx = (dx if up else dgrid).cpu().numpy()
    assert _rel(gx, xr.grad.permute(0, 2, 3, 1).cpu().numpy()) < 1e-4
    gw_ref = wr.grad.permute(0, 2, 3, 1).reshape(cout, 9 * cin).cpu().numpy()
    assert _rel(gw.cpu().numpy(), gw_ref) < 1e-4
    st = C.c_int(-1)
    assert L.imexlb_nn_status(C.byref(st)) == 0 and st.value == 0
