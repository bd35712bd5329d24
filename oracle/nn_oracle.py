"""CPU float64 restatement of the warm-start network (test infrastructure
only): the same 3x3 convolutions (stride, nearest x2 upsampling, ReLU), loss
and gradients as the library's tensor-core kernels, written with numpy so the
GPU gradients can be checked against it. Layout NHWC, weights
w[co][tap*Cin + ci], tap = ky*3 + kx, zero padding of 1. The network has no
reference counterpart; these gradients are themselves checked against
central finite differences (tests/test_nn_oracle_fd.py)."""
import numpy as np


def bf16(a):
    """Round to bfloat16 (nearest even) and return float64."""
    f = np.asarray(a, dtype=np.float32)
    bits = f.view(np.uint32).astype(np.uint64)
    bits = (bits + 0x7FFF + ((bits >> 16) & 1)) & 0xFFFF0000
    return bits.astype(np.uint32).view(np.float32).astype(np.float64)


def conv_fwd(x, w, b, stride, up, relu):
    """Returns (y, cache) for x (n, h, w, cin), w (cout, 9*cin), b (cout,)."""
    xg = x.repeat(2, axis=1).repeat(2, axis=2) if up else x
    n, H, W, cin = xg.shape
    Ho, Wo = (H - 1) // stride + 1, (W - 1) // stride + 1
    xp = np.pad(xg, ((0, 0), (1, 1), (1, 1), (0, 0)))
    cols = np.empty((n, Ho, Wo, 9 * cin))
    for ky in range(3):
        for kx in range(3):
            t = ky * 3 + kx
            cols[..., t * cin:(t + 1) * cin] = xp[:, ky:ky + stride * Ho:stride, kx:kx + stride * Wo:stride, :]
    z = cols @ w.T + b
    y = np.maximum(z, 0.0) if relu else z
    return y, (cols, z, xg.shape, x.shape, stride, up, relu)


def conv_bwd(dy, w, cache, round_dz=False):
    """Returns (dx, dw, db); round_dz rounds dz to bfloat16 for the products
    as the GPU kernels do (the bias gradient uses the unrounded values)."""
    cols, z, gshape, xshape, stride, up, relu = cache
    dz = dy * (z > 0) if relu else dy
    db = dz.reshape(-1, w.shape[0]).sum(0)
    if round_dz:
        dz = bf16(dz)
    cout = w.shape[0]
    dw = dz.reshape(-1, cout).T @ cols.reshape(-1, cols.shape[-1])
    dcols = dz @ w
    n, H, W, cin = gshape
    Ho, Wo = dz.shape[1], dz.shape[2]
    dxp = np.zeros((n, H + 2, W + 2, cin))
    for ky in range(3):
        for kx in range(3):
            t = ky * 3 + kx
            dxp[:, ky:ky + stride * Ho:stride, kx:kx + stride * Wo:stride, :] += dcols[..., t * cin:(t + 1) * cin]
    dx = dxp[:, 1:-1, 1:-1, :]
    if up:
        dx = dx.reshape(n, H // 2, 2, W // 2, 2, cin).sum(axis=(2, 4))
    return dx, dw, db


def net_grads(x, ws, bs, layers, target, used=3, mimic_bf16=False):
    """Loss = mean over pixels and the first `used` channels of (y - t)^2.
    Returns (loss, [dw...], [db...]). mimic_bf16 rounds what the GPU stores
    in bfloat16 (hidden activations, dz); accumulation stays float64."""
    caches, h = [], x
    for i, (w, b, (cin, cout, stride, up, relu)) in enumerate(zip(ws, bs, layers)):
        h, c = conv_fwd(h, w, b, stride, up, relu)
        if mimic_bf16 and i < len(ws) - 1:
            h = bf16(h)
        caches.append(c)
    y = h
    cnt = y.shape[0] * y.shape[1] * y.shape[2] * used
    d = y[..., :used] - target
    loss = (d * d).sum() / cnt
    dy = np.zeros_like(y)
    dy[..., :used] = 2.0 * d / cnt
    gws, gbs = [None] * len(ws), [None] * len(ws)
    for i in range(len(ws) - 1, -1, -1):
        dy, gws[i], gbs[i] = conv_bwd(dy, ws[i], caches[i], round_dz=mimic_bf16)
        if mimic_bf16:
            dy = dy.astype(np.float32).astype(np.float64)  # GPU keeps dx in f32
    return loss, gws, gbs
