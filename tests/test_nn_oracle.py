"""CPU checks of the warm-start U-Net oracle (oracle/nn_oracle.py): the convolution against a
direct loop, its data and weight gradients as adjoints of the forward, and the whole network's
backward pass against central finite differences of its float64 loss."""
import numpy as np
import pytest

import nn_oracle as O


def _direct_conv(x, W, b):
    cin, n0, n1, n2 = x.shape
    y = np.zeros((W.shape[0], n0, n1, n2))
    for co in range(W.shape[0]):
        for i in range(n0):
            for j in range(n1):
                for k in range(n2):
                    s = b[co]
                    for t, (a, bb, c) in enumerate(O.TAPS):
                        ii, jj, kk = i + a - 1, j + bb - 1, k + c - 1
                        if 0 <= ii < n0 and 0 <= jj < n1 and 0 <= kk < n2:
                            s += W[co, :, t] @ x[:, ii, jj, kk]
                    y[co, i, j, k] = s
    return y


def test_conv_matches_direct_loop():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((3, 4, 5, 3))
    W = rng.standard_normal((2, 3, 27))
    b = rng.standard_normal(2)
    np.testing.assert_allclose(O.conv3(x, W, b), _direct_conv(x, W, b), rtol=1e-12, atol=1e-12)


def test_conv_gradients_are_adjoints():
    """<conv(x), dy> = <x, dgrad(dy)> = <W, wgrad(x, dy)> (the convolution is bilinear)."""
    rng = np.random.default_rng(1)
    x = rng.standard_normal((4, 5, 6, 7))
    W = rng.standard_normal((3, 4, 27))
    dy = rng.standard_normal((3, 5, 6, 7))
    lhs = np.sum(O.conv3(x, W) * dy)
    assert abs(lhs - np.sum(x * O.conv3_dgrad(dy, W))) < 1e-9 * abs(lhs)
    assert abs(lhs - np.sum(W * O.conv3_wgrad(x, dy))) < 1e-9 * abs(lhs)


def test_resample_adjoints():
    rng = np.random.default_rng(2)
    f = rng.standard_normal((2, 4, 6, 8))
    c = rng.standard_normal((2, 2, 3, 4))
    assert abs(np.sum(O.pool(f) * c) - np.sum(f * O.pool_bwd(c))) < 1e-12
    assert abs(np.sum(O.up(c) * f) - np.sum(c * O.up_bwd(f))) < 1e-12


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e-3], np.float32)
    r = O.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == np.float32(1.0 + 2 ** -7)
    assert r[3] == -2.5
    assert abs(r[4] - 3.0e-3) <= 3.0e-3 * 2 ** -8


def _params(seed):
    rng = np.random.default_rng(seed)
    chunks = []
    for (_, c1, c2, cout, relu, _) in O.LAYERS:
        cin = c1 + c2
        chunks.append(rng.standard_normal(cout * cin * 27) * np.sqrt((2.0 if relu else 1.0) / (cin * 27)))
        chunks.append(rng.standard_normal(cout) * 0.1)
    return np.concatenate(chunks)


@pytest.mark.parametrize("seed", [0, 1])
def test_unet_backward_matches_finite_differences(seed):
    rng = np.random.default_rng(10 + seed)
    dims = (8, 8, 8)
    div = rng.standard_normal(dims)
    p = rng.standard_normal(dims)
    th = _params(seed)

    def L(t):
        pred, c = O.forward(t, div, rounding=False)
        return O.loss(pred, p, c["s"])[0]

    pred, c = O.forward(th, div, rounding=False)
    L0, g = O.backward(c, p)
    assert abs(L0 - L(th)) < 1e-12 * max(1.0, abs(L0))
    for k in range(3):
        d = rng.standard_normal(th.size)
        d /= np.linalg.norm(d)  # a step of 1e-6 in parameter norm: no ReLU kink in between
        eps = 1e-6
        fd = (L(th + eps * d) - L(th - eps * d)) / (2 * eps)
        an = float(g @ d)
        assert abs(fd - an) <= 1e-5 * max(abs(fd), 1e-3), (k, fd, an)


def test_product_layer_table_matches_oracle():
    """pfm.nn runs the same network the oracle restates, and every layer fits the tensor-core
    kernels: inputs in multiples of 16 channels, outputs in multiples of 8 (the 1-channel output
    layer is written in f32), skip concatenations joining tensors of the same resolution."""
    import pfm.nn as N
    assert [tuple(l) for l in N.LAYERS] == [tuple(l) for l in O.LAYERS]
    level_of = {}
    for (name, c1, c2, cout, relu, level) in N.LAYERS:
        assert c1 % 16 == 0 and c2 % 16 == 0 and c1 + c2 <= 128
        assert cout == 1 or cout % 8 == 0
        level_of[name] = level
    assert level_of["dec1a"] == level_of["enc1b"] and level_of["dec0a"] == level_of["enc0b"]
    n_params = sum(cout * (c1 + c2) * 27 + cout for (_, c1, c2, cout, _, _) in N.LAYERS)
    assert n_params == 360177
