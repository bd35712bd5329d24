"""The network oracle's analytic gradients against central finite differences.

The GPU forward / backward kernels of the warm-start network are checked
against oracle/nn_oracle.py; this pins the oracle itself: on a small network
with every layer kind of the real one (stride-2 and stride-1 convolutions
with ReLU, a nearest x2 upsampling convolution, a linear output), float64
throughout, each sampled weight and bias gradient must match
(L(w + h) - L(w - h)) / 2h.
"""
import numpy as np

from oracle import nn_oracle as nn

# (cin, cout, stride, up, relu)
LAYERS = [(4, 6, 2, False, True), (6, 6, 1, False, True), (6, 5, 1, True, True),
          (5, 3, 1, False, False)]


def _net(seed):
    rng = np.random.default_rng(seed)
    ws = [rng.normal(0.0, np.sqrt(2.0 / (9 * ci)), size=(co, 9 * ci)) for ci, co, *_ in LAYERS]
    bs = [rng.normal(0.0, 0.1, size=co) for _, co, *_ in LAYERS]
    x = rng.normal(size=(2, 8, 8, 4))
    target = rng.normal(size=(2, 8, 8, 3))
    return x, ws, bs, target, rng


def _loss(x, ws, bs, target):
    return nn.net_grads(x, ws, bs, LAYERS, target)[0]


def test_weight_and_bias_gradients_match_finite_differences():
    x, ws, bs, target, rng = _net(7)
    loss, gws, gbs = nn.net_grads(x, ws, bs, LAYERS, target)
    assert np.isfinite(loss) and loss > 0
    h = 1e-6
    checked = 0
    for li in range(len(LAYERS)):
        # a sample of weights and every bias of the layer
        flat = [(ws, li, np.unravel_index(k, ws[li].shape))
                for k in rng.choice(ws[li].size, size=12, replace=False)]
        flat += [(bs, li, (k,)) for k in range(bs[li].size)]
        for params, i, idx in flat:
            keep = params[i][idx]
            params[i][idx] = keep + h
            up = _loss(x, ws, bs, target)
            params[i][idx] = keep - h
            dn = _loss(x, ws, bs, target)
            params[i][idx] = keep
            fd = (up - dn) / (2 * h)
            an = (gws if params is ws else gbs)[i][idx]
            assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)) + 1e-8, (li, params is ws, idx, fd, an)
            checked += 1
    assert checked == sum(12 + co for _, co, *_ in LAYERS)


def test_loss_covers_only_the_used_channels():
    """With used=2 the third output channel carries no loss: its output
    weights and bias get no gradient, and the loss does not change when that
    channel's weights do."""
    x, ws, bs, target, _ = _net(11)
    base, gws, gbs = nn.net_grads(x, ws, bs, LAYERS, target[..., :2], used=2)
    assert np.all(gws[-1][2] == 0.0) and gbs[-1][2] == 0.0
    assert np.any(gws[-1][:2] != 0.0)
    ws[-1][2] += 1.0
    assert nn.net_grads(x, ws, bs, LAYERS, target[..., :2], used=2)[0] == base
