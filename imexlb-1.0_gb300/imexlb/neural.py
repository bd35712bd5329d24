"""Warm-start neural operator: a 6-layer convolutional encoder-decoder that
maps (obstacle fluid fraction, Reynolds number) on a 256 x 128 grid to the
(p, ux, uy) field of a developed flow, trained and evaluated with the
library's tensor-core kernels (include/imexlb_nn.h).

Layout: NHWC bfloat16 activations, weights w[co][tap*Cin + ci]; FP32
accumulation, FP32 master weights with Adam. torch only holds device memory
and streams; every arithmetic step is a library kernel.

Layers (H x W = 128 x 256 input, 48 channels):
  1 conv s2  16->48 ReLU  (64 x 128)      4 up2+conv 48->48 ReLU (64 x 128)
  2 conv s2  48->48 ReLU  (32 x 64)       5 up2+conv 48->48 ReLU (128 x 256)
  3 conv     48->48 ReLU  (32 x 64)       6 conv     48->16 (3 used), linear
"""
import ctypes as C

import numpy as np

from . import ConvDesc, lib

CH = 48
CIN = 16       # input channels incl. zero padding: 0 fluid fraction, 1 Re/200
COUT = 16      # GEMM width of the last layer; 3 channels used
USED = 3
LAYERS = [  # (cin, cout, stride, upsample, relu)
    (CIN, CH, 2, 0, 1), (CH, CH, 2, 0, 1), (CH, CH, 1, 0, 1),
    (CH, CH, 1, 1, 1), (CH, CH, 1, 1, 1), (CH, COUT, 1, 0, 0)]

# target normalisation: p / U^2, u / U with the inlet speed U
U_REF = 0.05


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _ck(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed (%d)" % (what, rc))


class Net:
    """Parameters, optimiser state and the forward/backward passes."""

    def __init__(self, seed=0, device="cuda"):
        import torch
        self.torch = torch
        self.dev = device
        g = np.random.default_rng(seed)
        self.w, self.b, self.wb = [], [], []
        for cin, cout, _, _, _ in LAYERS:
            fan_in = 9 * cin
            w = g.standard_normal((cout, 9 * cin)) * np.sqrt(2.0 / fan_in)
            if cout == COUT:
                w[USED:] = 0.0
                w *= 0.1
            self.w.append(torch.tensor(w, dtype=torch.float32, device=device))
            self.b.append(torch.zeros(cout, dtype=torch.float32, device=device))
        self.wb = [w.to(torch.bfloat16) for w in self.w]
        self.params = self.w + self.b
        self.m = [torch.zeros_like(p) for p in self.params]
        self.v = [torch.zeros_like(p) for p in self.params]
        self.t = 0

    # ---- shapes -------------------------------------------------------------
    @staticmethod
    def descs(n, h, w):
        out = []
        for cin, cout, stride, up, _ in LAYERS:
            hg, wg = (2 * h, 2 * w) if up else (h, w)
            ho, wo = (hg - 1) // stride + 1, (wg - 1) // stride + 1
            out.append(ConvDesc(n, h, w, cin, ho, wo, cout, 0, stride, up))
            h, w = ho, wo
        return out

    # ---- forward ------------------------------------------------------------
    def forward(self, x, keep=False):
        """x: (n, h, w, 16) bfloat16 device tensor -> (n, h, w, 16) float32."""
        torch = self.torch
        n, h, w, _ = x.shape
        ds = self.descs(n, h, w)
        acts = [x]
        L = lib()
        for i, (d, (cin, cout, _, _, relu)) in enumerate(zip(ds, LAYERS)):
            last = i == len(LAYERS) - 1
            shape = (n, d.hout, d.wout, cout)
            y = torch.empty(shape, dtype=torch.float32 if last else torch.bfloat16, device=self.dev)
            _ck(L.imexlb_nn_conv_fwd(C.byref(d), _p(acts[-1]), _p(self.wb[i]), _p(self.b[i]), relu,
                                     None if last else _p(y), _p(y) if last else None, None),
                "conv_fwd")
            acts.append(y)
        if keep:
            self._acts, self._descs = acts, ds
        return acts[-1]

    # ---- backward -----------------------------------------------------------
    def backward(self, dy):
        """dy: gradient of the loss wrapt the last output (n, h, w, 16) f32.
        Returns the list of parameter gradients (weights, then biases)."""
        torch = self.torch
        L = lib()
        acts, ds = self._acts, self._descs
        gw = [torch.zeros_like(w) for w in self.w]
        gb = [torch.zeros_like(b) for b in self.b]
        for i in range(len(LAYERS) - 1, -1, -1):
            cin, cout, _, up, relu = LAYERS[i]
            d = ds[i]
            y = acts[i + 1]
            dz = torch.empty(y.shape, dtype=torch.bfloat16, device=self.dev)
            _ck(L.imexlb_nn_act_grad(_p(dy), _p(y) if relu else None, dy.numel(), cout, relu,
                                     _p(dz), _p(gb[i]), None), "act_grad")
            _ck(L.imexlb_nn_conv_bwd_weight(C.byref(d), _p(acts[i]), _p(dz), _p(gw[i]), None),
                "bwd_weight")
            if i > 0:
                hg, wg = (2 * d.hin, 2 * d.win) if up else (d.hin, d.win)
                dgrid = torch.empty((d.n, hg, wg, cin), dtype=torch.float32, device=self.dev)
                dx = torch.empty((d.n, d.hin, d.win, cin), dtype=torch.float32, device=self.dev) if up else None
                wt = torch.empty((cin, 9 * cout), dtype=torch.bfloat16, device=self.dev)
                _ck(L.imexlb_nn_conv_bwd_data(C.byref(d), _p(dz), _p(self.wb[i]), _p(wt), _p(dgrid),
                                              _p(dx), None), "bwd_data")
                dy = dx if up else dgrid
        return gw + gb

    def adam(self, grads, lr=2e-3, wd=0.0):
        L = lib()
        self.t += 1
        nw = len(self.w)
        for k, (p, g, m, v) in enumerate(zip(self.params, grads, self.m, self.v)):
            pb = self.wb[k] if k < nw else None
            _ck(L.imexlb_nn_adam(_p(p), _p(g), _p(m), _p(v), _p(pb), p.numel(), lr, 0.9, 0.999, 1e-8,
                                 self.t, wd, None), "adam")

    def loss(self, y, target, weight=None):
        """MSE over the first 3 channels; returns (loss tensor, dy)."""
        torch = self.torch
        dy = torch.empty_like(y)
        out = torch.zeros(1, dtype=torch.float32, device=self.dev)
        npix = y.shape[0] * y.shape[1] * y.shape[2]
        _ck(lib().imexlb_nn_mse(_p(y), _p(target), _p(weight), npix, COUT, USED, _p(dy), _p(out),
                                None), "mse")
        return out, dy

    def state(self):
        return {"w": [w.cpu().numpy() for w in self.w], "b": [b.cpu().numpy() for b in self.b]}


def make_input(frac, re, torch, device="cuda"):
    """frac: (n, H, W) fluid fraction; re: (n,) Reynolds numbers -> NHWC bf16."""
    n, H, W = frac.shape
    x = np.zeros((n, H, W, CIN), dtype=np.float32)
    x[..., 0] = frac
    x[..., 1] = (np.asarray(re, dtype=np.float32) / 200.0)[:, None, None]
    return torch.tensor(x, device=device).to(torch.bfloat16)


def make_target(p, ux, uy, torch, device="cuda"):
    t = np.stack([p / U_REF ** 2, ux / U_REF, uy / U_REF], axis=-1).astype(np.float32)
    return torch.tensor(t, device=device)


def train(net, frac, re, fields, steps=2000, batch=16, lr=2e-3, seed=0, log=None):
    """frac (n,H,W), re (n,), fields (n,3,H,W) = p, ux, uy. Returns the loss history."""
    torch = net.torch
    rng = np.random.default_rng(seed)
    n = frac.shape[0]
    X = make_input(frac, re, torch, net.dev)
    T = make_target(fields[:, 0], fields[:, 1], fields[:, 2], torch, net.dev)
    hist = []
    for it in range(steps):
        idx = torch.tensor(rng.choice(n, size=min(batch, n), replace=False), device=net.dev)
        xb, tb = X.index_select(0, idx).contiguous(), T.index_select(0, idx).contiguous()
        y = net.forward(xb, keep=True)
        loss, dy = net.loss(y, tb)
        grads = net.backward(dy)
        net.adam(grads, lr=lr * (0.5 * (1 + np.cos(np.pi * it / steps))))
        if it % 50 == 0 or it == steps - 1:
            hist.append((it, float(loss.item())))
            if log:
                log("train %5d loss %.5f" % (it, hist[-1][1]))
    return hist


def predict(net, frac, re):
    """(n,H,W) fluid fraction, (n,) Re -> (n,3,H,W) physical p, ux, uy."""
    torch = net.torch
    y = net.forward(make_input(frac, re, torch, net.dev)).cpu().numpy()
    return np.stack([y[..., 0] * U_REF ** 2, y[..., 1] * U_REF, y[..., 2] * U_REF], axis=1)


def time_layer(layer=4, batch=16, reps=10, warmup=3, seed=0):
    """CUDA-event time of one layer's forward convolution and weight gradient
    on `batch` random images of the network's 128 x 256 input (layer 4 is
    the second up2+conv, 64 x 128 x 48 channels in, 128 x 256 x 48 out):
    `warmup` untimed launches of each, then `reps` timed. Returns a dict with
    ms per launch and TFLOP/s (2 x GEMM M x N x K per launch)."""
    import torch
    net = Net(seed=seed)
    d = net.descs(batch, 128, 256)[layer]
    cin, cout, _, _, relu = LAYERS[layer]
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randn((batch, d.hin, d.win, cin), generator=g, device="cuda").to(torch.bfloat16)
    y = torch.empty((batch, d.hout, d.wout, cout), dtype=torch.bfloat16, device="cuda")
    dz = torch.randn(y.shape, generator=g, device="cuda").to(torch.bfloat16)
    dw = torch.zeros_like(net.w[layer])
    L = lib()
    fwd = lambda: _ck(L.imexlb_nn_conv_fwd(C.byref(d), _p(x), _p(net.wb[layer]), _p(net.b[layer]),
                                           relu, _p(y), None, None), "conv_fwd")
    wgrad = lambda: _ck(L.imexlb_nn_conv_bwd_weight(C.byref(d), _p(x), _p(dz), _p(dw), None),
                        "bwd_weight")
    flops = 2.0 * batch * d.hout * d.wout * cout * 9 * cin
    out = {"layer": layer, "batch": batch, "gflop": round(flops / 1e9, 2)}
    for name, fn in (("fwd", fwd), ("wgrad", wgrad)):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[name] = {"ms": round(ms, 4), "tflops": round(flops / (ms / 1e3) / 1e12, 1)}
    return out


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="time one layer of the warm-start network")
    ap.add_argument("--layer", type=int, default=4)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--reps", type=int, default=10)
    a = ap.parse_args()
    print(json.dumps(time_layer(a.layer, a.batch, a.reps)))
