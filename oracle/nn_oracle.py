"""CPU oracle of the warm-start U-Net (test infrastructure: only tests and smoke() use it).

A NumPy restatement of the network that ``pfm.nn`` runs on the tensor cores: 3x3x3
cross-correlation with zero padding, weights ``W [cout][cin][27]`` with tap = 9 a + 3 b + c for the
offsets (a-1, b-1, c-1), 2x2x2 average pooling, nearest upsampling, ReLU, the scaled input
``div / rms(div)`` and the loss ``mean(e^2) - mean(e)^2`` of ``e = pred - p / rms(div)``.

Fields are planar ``[C][n0][n1][n2]``.  With ``rounding=True`` every tensor the GPU stores in BF16
(weights, activations, gradients of activations) is rounded to BF16 here at the same place, and
every sum is taken in float64 (the GPU sums in FP32), so the two agree to the accumulation
order; with ``rounding=False`` the whole network is float64, which the finite-difference test
uses to pin the backward pass.

The reference solver has no network: this oracle is pinned by finite differences of its own
float64 loss (tests/test_nn_oracle.py), not by reference outputs.
"""
import numpy as np

LAYERS = [  # name, c1, c2, cout, relu, level (as pfm.nn.LAYERS)
    ("enc0a", 16, 0, 16, True, 0),
    ("enc0b", 16, 0, 16, True, 0),
    ("enc1a", 16, 0, 32, True, 1),
    ("enc1b", 32, 0, 32, True, 1),
    ("bot_a", 32, 0, 64, True, 2),
    ("bot_b", 64, 0, 64, True, 2),
    ("dec1a", 32, 64, 32, True, 1),
    ("dec1b", 32, 0, 32, True, 1),
    ("dec0a", 16, 32, 16, True, 0),
    ("dec0b", 16, 0, 16, True, 0),
    ("out", 16, 0, 1, False, 0),
]

TAPS = [(t // 9, (t // 3) % 3, t % 3) for t in range(27)]


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r.astype(np.uint32)).view(np.float32).reshape(a.shape)


def _id(x):
    return x


def conv3(x, W, b=None):
    """y[co] = sum over taps and ci of W[co][ci][t] x[ci][v + off(t)] (+ b[co]), float64."""
    cin, n0, n1, n2 = x.shape
    xp = np.pad(np.asarray(x, np.float64), ((0, 0), (1, 1), (1, 1), (1, 1)))
    W = np.asarray(W, np.float64)
    y = np.zeros((W.shape[0], n0, n1, n2))
    for t, (a, bb, c) in enumerate(TAPS):
        y += np.tensordot(W[:, :, t], xp[:, a:a + n0, bb:bb + n1, c:c + n2], axes=(1, 0))
    if b is not None:
        y += np.asarray(b, np.float64)[:, None, None, None]
    return y


def conv3_dgrad(dy, W):
    """dx[ci] = sum over taps and co of W[co][ci][t] dy[co][v - off(t)] (the flipped convolution)."""
    Wf = np.transpose(np.asarray(W, np.float64)[:, :, ::-1], (1, 0, 2))
    return conv3(dy, Wf)


def conv3_wgrad(x, dy):
    """dW[co][ci][t] = sum over voxels of dy[co][v] x[ci][v + off(t)], float64."""
    cin, n0, n1, n2 = x.shape
    xp = np.pad(np.asarray(x, np.float64), ((0, 0), (1, 1), (1, 1), (1, 1)))
    dy = np.asarray(dy, np.float64)
    dW = np.zeros((dy.shape[0], cin, 27))
    for t, (a, bb, c) in enumerate(TAPS):
        dW[:, :, t] = np.tensordot(dy, xp[:, a:a + n0, bb:bb + n1, c:c + n2], axes=([1, 2, 3], [1, 2, 3]))
    return dW


def pool(x):
    C, n0, n1, n2 = x.shape
    return np.asarray(x, np.float64).reshape(C, n0 // 2, 2, n1 // 2, 2, n2 // 2, 2).sum(axis=(2, 4, 6)) * 0.125


def pool_bwd(dy):
    return up(dy) * 0.125


def up(x):
    return np.repeat(np.repeat(np.repeat(np.asarray(x, np.float64), 2, axis=1), 2, axis=2), 2, axis=3)


def up_bwd(dy):
    C, n0, n1, n2 = dy.shape
    return np.asarray(dy, np.float64).reshape(C, n0 // 2, 2, n1 // 2, 2, n2 // 2, 2).sum(axis=(2, 4, 6))


def unflatten(params):
    """Flat parameter vector (the layout of pfm.nn.UNet3D.params) -> {name: (W, b)}."""
    out, off = {}, 0
    params = np.asarray(params)
    for (name, c1, c2, cout, _, _) in LAYERS:
        nw = cout * (c1 + c2) * 27
        W = params[off:off + nw].reshape(cout, c1 + c2, 27)
        off += nw
        out[name] = (W, params[off:off + cout])
        off += cout
    return out


def flatten(grads):
    return np.concatenate([np.concatenate([grads[n][0].ravel(), grads[n][1].ravel()]) for (n, *_r) in LAYERS])


def input_scale(div):
    """1 / rms(div) as the GPU forms it (float64 sum, rounded to f32)."""
    return np.float32(1.0 / np.sqrt(np.mean(np.asarray(div, np.float64) ** 2)))


def forward(params, div, rounding=True):
    """Network output on the scaled input (pred = net(div / rms)), plus the cache for backward."""
    R = bf16 if rounding else _id
    P = unflatten(params)
    Wr = {n: (R(W.astype(np.float32)) if rounding else W, b) for n, (W, b) in P.items()}
    div = np.asarray(div, np.float32 if rounding else np.float64)
    s = input_scale(div) if rounding else 1.0 / np.sqrt(np.mean(div.astype(np.float64) ** 2))
    x = np.zeros((16,) + div.shape, np.float64)
    x[0] = R((div * s).astype(np.float32)) if rounding else div * s
    c = {"x": x, "s": s}

    def layer(name, inp):
        W, b = Wr[name]
        y = conv3(inp, W, b)
        return y

    def act(name, inp):
        y = np.maximum(layer(name, inp), 0.0)
        return R(y.astype(np.float32)).astype(np.float64) if rounding else y

    def rr(y):
        return R(y.astype(np.float32)).astype(np.float64) if rounding else y

    c["e0a"] = act("enc0a", x)
    c["e0"] = act("enc0b", c["e0a"])
    c["p0"] = rr(pool(c["e0"]))
    c["e1a"] = act("enc1a", c["p0"])
    c["e1"] = act("enc1b", c["e1a"])
    c["p1"] = rr(pool(c["e1"]))
    c["ba"] = act("bot_a", c["p1"])
    c["b"] = act("bot_b", c["ba"])
    c["u1"] = up(c["b"])
    c["d1a"] = act("dec1a", np.concatenate([c["e1"], c["u1"]]))
    c["d1"] = act("dec1b", c["d1a"])
    c["u0"] = up(c["d1"])
    c["d0a"] = act("dec0a", np.concatenate([c["e0"], c["u0"]]))
    c["d0"] = act("dec0b", c["d0a"])
    pred = layer("out", c["d0"])[0]
    if rounding:
        pred = pred.astype(np.float32).astype(np.float64)
    c["pred"] = pred
    c["W"] = Wr
    c["rounding"] = rounding
    return pred, c


def loss(pred, p, s):
    e = np.asarray(pred, np.float64) - np.asarray(p, np.float64) * s
    me = e.mean()
    return float((e * e).mean() - me * me), e - me


def backward(c, p):
    """Gradients of the loss against the solver pressure p; returns (loss, flat gradient)."""
    rounding = c["rounding"]
    R = bf16 if rounding else _id

    def rr(y):
        return R(y.astype(np.float32)).astype(np.float64) if rounding else y

    Wr = c["W"]
    s = c["s"]
    L, ec = loss(c["pred"], p, s)
    V = ec.size
    g = np.zeros((16,) + ec.shape)
    g[0] = rr(2.0 * ec / V)
    G = {}

    def lay(name, x, dy, cout):
        W, _ = Wr[name]
        G[name] = (conv3_wgrad(x, dy[:cout]), dy[:cout].sum(axis=(1, 2, 3)))
        return rr(conv3_dgrad(dy[:cout], W))

    gx = lay("out", c["d0"], g, 1)
    gx = gx * (c["d0"] > 0)
    gx = lay("dec0b", c["d0a"], gx, 16) * (c["d0a"] > 0)
    gcat = lay("dec0a", np.concatenate([c["e0"], c["u0"]]), gx, 16)
    gS0, gU0 = gcat[:16], gcat[16:]
    gx = rr(up_bwd(gU0)) * (c["d1"] > 0)
    gx = lay("dec1b", c["d1a"], gx, 32) * (c["d1a"] > 0)
    gcat = lay("dec1a", np.concatenate([c["e1"], c["u1"]]), gx, 32)
    gS1, gU1 = gcat[:32], gcat[32:]
    gx = rr(up_bwd(gU1)) * (c["b"] > 0)
    gx = lay("bot_b", c["ba"], gx, 64) * (c["ba"] > 0)
    gx = lay("bot_a", c["p1"], gx, 64)
    gx = rr(rr(pool_bwd(gx)) + gS1) * (c["e1"] > 0)
    gx = lay("enc1b", c["e1a"], gx, 32) * (c["e1a"] > 0)
    gx = lay("enc1a", c["p0"], gx, 32)
    gx = rr(rr(pool_bwd(gx)) + gS0) * (c["e0"] > 0)
    gx = lay("enc0b", c["e0a"], gx, 16) * (c["e0a"] > 0)
    W, _ = Wr["enc0a"]
    G["enc0a"] = (conv3_wgrad(c["x"], gx), gx.sum(axis=(1, 2, 3)))
    return L, flatten(G)
