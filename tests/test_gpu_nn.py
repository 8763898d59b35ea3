"""GPU parity of the warm-start U-Net (pfm_nn_* through the C ABI) against the CPU oracle
(oracle/nn_oracle.py): the tensor-core convolution forward, data gradient and weight gradient on
single layers (tight tolerances: the inputs are BF16, the sums FP32 against float64), the
element-wise layers, and the whole network's prediction and gradient (loose tolerances: BF16
rounding of every stored activation flips differently once sums differ in the last bit)."""
import ctypes

import numpy as np
import pytest
import torch

import nn_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import pfm
    from pfm import _lib
    torch.cuda.set_device(0)
    return _lib.load()


def blocked(x):
    """planar float [C][n0][n1][n2] -> BF16 channel-blocked [C/8][n0][n1][n2][8] (device, flat)"""
    x = torch.as_tensor(np.ascontiguousarray(x, np.float32))
    C = x.shape[0]
    t = x.reshape(C // 8, 8, *x.shape[1:]).permute(0, 2, 3, 4, 1).contiguous()
    return t.to(torch.bfloat16).reshape(-1).cuda()


def planar(t, C, dims):
    t = t.reshape(C // 8, *dims, 8).permute(0, 4, 1, 2, 3).reshape(C, *dims)
    return t.float().cpu().numpy()


def P(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def r16(c):
    return (c + 15) // 16 * 16


def pack(lib, W, flip, kin, npad):
    Wt = torch.as_tensor(W, dtype=torch.float32).cuda().contiguous()
    out = torch.empty(27 * kin * npad, dtype=torch.bfloat16, device="cuda")
    assert lib.pfm_nn_pack_weights(P(Wt), W.shape[0], W.shape[1], flip, kin, npad, P(out), None) == 0
    return out


def conv(lib, dims, x1, c1, x2, c2, wp, bias, cout, relu, y1=None, cy1=None, y2=None, yf=None):
    from pfm import _lib
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    a = _lib.Conv3Args(dims[0], dims[1], dims[2], P(x1), c1, P(x2), c2, P(wp), P(bias), cout, relu, P(y1),
                       cy1 or cout, P(y2), P(yf), None, P(err))
    st = lib.pfm_nn_conv3(ctypes.byref(a), None)
    assert st == 0, st
    torch.cuda.synchronize()
    assert int(err.item()) == 0


CONV_CASES = [  # c1, c2, cout, dims
    (16, 0, 16, (2, 16, 8)),
    (16, 0, 32, (3, 20, 11)),   # partial tiles along d1 and d2
    (32, 64, 32, (2, 16, 16)),  # concatenated inputs
    (16, 32, 16, (3, 18, 9)),
    (64, 0, 64, (4, 8, 8)),
    (16, 0, 1, (4, 12, 12)),    # the output layer (N padded to 16)
    (96, 0, 48, (2, 7, 5)),     # small grid, several taps out of range everywhere
]


@pytest.mark.parametrize("c1,c2,cout,dims", CONV_CASES)
def test_conv_forward(lib, c1, c2, cout, dims):
    rng = np.random.default_rng(c1 + 7 * c2 + cout)
    cin = c1 + c2
    x = O.bf16(rng.standard_normal((cin,) + dims).astype(np.float32))
    W = rng.standard_normal((cout, cin, 27)).astype(np.float32) * 0.1
    b = rng.standard_normal(cout).astype(np.float32)
    wp = pack(lib, W, 0, cin, r16(cout))
    bias = torch.as_tensor(b).cuda()
    yf = torch.empty((cout,) + dims, device="cuda")
    x1 = blocked(x[:c1])
    x2 = blocked(x[c1:]) if c2 else None
    conv(lib, dims, x1, c1, x2, c2, wp, bias, cout, 0, yf=yf)
    Wb = O.bf16(W)
    ref = O.conv3(x, Wb, b)
    bound = O.conv3(np.abs(x), np.abs(Wb), np.abs(b))
    got = yf.cpu().numpy()
    assert np.all(np.abs(got - ref) <= 1e-4 * bound + 1e-6), np.max(np.abs(got - ref) / (bound + 1e-6))
    if cout % 8 == 0:  # BF16 output with ReLU, split into two tensors when cout allows
        cy1 = cout // 2 if cout % 16 == 0 else cout
        y1 = torch.zeros(cy1 * int(np.prod(dims)), dtype=torch.bfloat16, device="cuda")
        y2 = torch.zeros((cout - cy1) * int(np.prod(dims)), dtype=torch.bfloat16, device="cuda") if cy1 < cout else None
        conv(lib, dims, x1, c1, x2, c2, wp, bias, cout, 1, y1=y1, cy1=cy1, y2=y2)
        got = planar(y1, cy1, dims)
        if y2 is not None:
            got = np.concatenate([got, planar(y2, cout - cy1, dims)])
        refr = np.maximum(ref, 0)
        assert np.all(np.abs(got - refr) <= 2 ** -8 * np.abs(refr) + 1e-4 * bound + 1e-6)


@pytest.mark.parametrize("c1,c2,cout,dims", CONV_CASES)
def test_conv_data_gradient(lib, c1, c2, cout, dims):
    rng = np.random.default_rng(100 + c1 + 7 * c2 + cout)
    cin = c1 + c2
    kin = r16(cout)
    W = rng.standard_normal((cout, cin, 27)).astype(np.float32) * 0.1
    dy = np.zeros((kin,) + dims, np.float32)
    dy[:cout] = O.bf16(rng.standard_normal((cout,) + dims).astype(np.float32))
    wq = pack(lib, W, 1, kin, r16(cin))
    yf = torch.empty((cin,) + dims, device="cuda")
    conv(lib, dims, blocked(dy), kin, None, 0, wq, None, cin, 0, yf=yf)
    Wb = O.bf16(W)
    ref = O.conv3_dgrad(dy[:cout], Wb)
    bound = O.conv3_dgrad(np.abs(dy[:cout]), np.abs(Wb))
    got = yf.cpu().numpy()
    assert np.all(np.abs(got - ref) <= 1e-4 * bound + 1e-6)


@pytest.mark.parametrize("c1,c2,cout,dims", CONV_CASES)
def test_conv_weight_gradient(lib, c1, c2, cout, dims):
    from pfm import _lib
    rng = np.random.default_rng(200 + c1 + 7 * c2 + cout)
    cin = c1 + c2
    cdy = r16(cout) if cout < 16 else cout  # the gradient tensor's channels (a multiple of 8)
    x = O.bf16(rng.standard_normal((cin,) + dims).astype(np.float32))
    dy = np.zeros((cdy,) + dims, np.float32)
    dy[:cout] = O.bf16(rng.standard_normal((cout,) + dims).astype(np.float32))
    x1 = blocked(x[:c1])
    x2 = blocked(x[c1:]) if c2 else None
    dyt = blocked(dy)
    dw = torch.full((cout, cin, 27), np.nan, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    a = _lib.Conv3WgradArgs(dims[0], dims[1], dims[2], P(x1), c1, P(x2), c2, P(dyt), cdy, cout, P(dw), None, 0, P(err))
    nb = ctypes.c_size_t()
    assert lib.pfm_nn_wgrad_workspace(ctypes.byref(a), ctypes.byref(nb)) == 0
    part = torch.empty(nb.value // 4 + 1, device="cuda")
    a.partial, a.partial_bytes = P(part), part.numel() * 4
    assert lib.pfm_nn_conv3_wgrad(ctypes.byref(a), None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = O.conv3_wgrad(x, dy[:cout])
    bound = O.conv3_wgrad(np.abs(x), np.abs(dy[:cout]))
    got = dw.cpu().numpy()
    assert np.all(np.abs(got - ref) <= 1e-4 * bound + 1e-6), np.nanmax(np.abs(got - ref) / (bound + 1e-6))


def test_resample_elementwise_bias_loss_adam(lib):
    rng = np.random.default_rng(5)
    dims = (4, 6, 8)
    f = O.bf16(rng.standard_normal((16,) + dims).astype(np.float32))
    c = O.bf16(rng.standard_normal((16, 2, 3, 4)).astype(np.float32))
    ft, ct = blocked(f), blocked(c)
    out_c = torch.empty_like(ct)
    out_f = torch.empty_like(ft)
    for mode, src, dst, ref in [(0, ft, out_c, O.pool(f)), (3, ft, out_c, O.up_bwd(f)), (2, ct, out_f, O.up(c)),
                                (1, ct, out_f, O.pool_bwd(c))]:
        assert lib.pfm_nn_resample(P(src), P(dst), 16, *dims, mode, None) == 0
        torch.cuda.synchronize()
        got = planar(dst, 16, ref.shape[1:])
        np.testing.assert_allclose(got, O.bf16(ref.astype(np.float32)), rtol=2 ** -8, atol=1e-6)
    g = O.bf16(rng.standard_normal((16,) + dims).astype(np.float32))
    gt = blocked(g)
    assert lib.pfm_nn_elementwise(P(gt), P(ft), gt.numel(), 0, None) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(planar(gt, 16, dims), g * (f > 0))
    scratch = torch.zeros(int(lib.pfm_nn_scratch_floats(64)), device="cuda")
    db = torch.empty(16, device="cuda")
    assert lib.pfm_nn_bias_grad(P(ft), 16, *dims, 16, P(db), P(scratch), None) == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(db.cpu().numpy(), f.sum(axis=(1, 2, 3)), rtol=1e-5, atol=1e-4)
    pred = rng.standard_normal(dims).astype(np.float32)
    tgt = rng.standard_normal(dims).astype(np.float32)
    out4 = torch.empty(4, device="cuda")
    inv = torch.tensor([0.5], device="cuda")
    gr = torch.empty(16 * int(np.prod(dims)), dtype=torch.bfloat16, device="cuda")
    assert lib.pfm_nn_loss(P(torch.as_tensor(pred).cuda()), P(torch.as_tensor(tgt).cuda()), P(inv), *dims, P(out4),
                           P(gr), P(scratch), None) == 0
    torch.cuda.synchronize()
    L, ec = O.loss(pred, tgt, np.float32(0.5))
    assert abs(out4[0].item() - L) < 1e-5 * L
    gg = planar(gr, 16, dims)
    np.testing.assert_allclose(gg[0], O.bf16((2 * ec / ec.size).astype(np.float32)), rtol=2 ** -7, atol=1e-9)
    assert np.all(gg[1:] == 0)
    n = 1000
    p0 = rng.standard_normal(n).astype(np.float32)
    gv = rng.standard_normal(n).astype(np.float32)
    pt, gt2 = torch.as_tensor(p0).cuda(), torch.as_tensor(gv).cuda()
    m, v = torch.zeros(n, device="cuda"), torch.zeros(n, device="cuda")
    for step in (1, 2):
        assert lib.pfm_nn_adam(P(pt), P(gt2), P(m), P(v), n, 1e-3, 0.9, 0.999, 1e-8, step, 1.0, None) == 0
    torch.cuda.synchronize()
    mm, vv, pp = np.zeros(n), np.zeros(n), p0.astype(np.float64)
    for step in (1, 2):
        mm = 0.9 * mm + 0.1 * gv
        vv = 0.999 * vv + 0.001 * gv.astype(np.float64) ** 2
        pp -= 1e-3 * (mm / (1 - 0.9 ** step)) / (np.sqrt(vv / (1 - 0.999 ** step)) + 1e-8)
    np.testing.assert_allclose(pt.cpu().numpy(), pp, rtol=1e-5, atol=1e-6)


def _fields(seed, dims):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*[np.linspace(0, 1, n) for n in dims], indexing="ij")
    div = np.zeros(dims)
    for _ in range(4):
        c = rng.uniform(0.2, 0.8, 3)
        s = rng.uniform(0.05, 0.15)
        div += rng.uniform(-1, 1) * np.exp(-((z - c[0]) ** 2 + (y - c[1]) ** 2 + (x - c[2]) ** 2) / (2 * s * s))
    div -= div.mean()
    p = rng.standard_normal(dims) * 0.1 + div * 0.3
    return div.astype(np.float32), p.astype(np.float32)


def test_unet_forward_and_gradient_match_oracle(lib):
    from pfm.nn import UNet3D
    dims = (16, 16, 16)
    net = UNet3D(seed=3)
    div, p = _fields(1, dims)
    dt, pt = torch.as_tensor(div).cuda(), torch.as_tensor(p).cuda()
    out = net.predict(dt)
    torch.cuda.synchronize()
    net.check()
    params = net.params.cpu().numpy().astype(np.float64)
    pred, cache = O.forward(params, div, rounding=True)
    s = 1.0 / cache["s"]
    got = out.cpu().numpy()
    rel = np.linalg.norm(got - pred * s) / np.linalg.norm(pred * s)
    assert rel < 1e-2, rel
    stats = net.loss_and_grad(dt, pt)
    torch.cuda.synchronize()
    net.check()
    L, g = O.backward(cache, p)
    assert abs(stats[0].item() - L) < 2e-2 * L
    gg = net.grads.cpu().numpy().astype(np.float64)
    rel_g = np.linalg.norm(gg - g) / np.linalg.norm(g)
    cos = float(gg @ g / (np.linalg.norm(gg) * np.linalg.norm(g)))
    assert rel_g < 5e-2 and cos > 0.998, (rel_g, cos)
    # per layer: every layer's gradient agrees, not only the total
    off = 0
    for (name, c1, c2, cout, _, _) in O.LAYERS:
        n = cout * (c1 + c2) * 27 + cout
        a, b = gg[off:off + n], g[off:off + n]
        assert np.linalg.norm(a - b) <= 0.1 * np.linalg.norm(b) + 1e-12, name
        off += n


def _poisson_pairs(seeds, dims):
    """(divergence, MGPCG pressure) pairs: the pressure the solver returns for each field."""
    import pfm
    sc = pfm.Scene(3, dims, 1.0 / dims[1], 0)
    out = []
    for s in seeds:
        div, _ = _fields(s, dims)
        d = torch.as_tensor(div).cuda()
        p = torch.zeros_like(d)
        sc.mgpcg_solve(d, p, k=-1.0, tol=1e-6, tol_mode=1)
        out.append((d, p))
    return out


def test_unet_training_reduces_loss(lib):
    from pfm.nn import UNet3D
    dims = (16, 16, 16)
    net = UNet3D(seed=0, lr=2e-3)
    pairs = _poisson_pairs(range(4), dims)
    first = [net.loss_and_grad(d, p)[0].item() for d, p in pairs]
    for it in range(200):
        d, p = pairs[it % 4]
        net.train_step(d, p)
    torch.cuda.synchronize()
    net.check()
    last = [net.loss_and_grad(d, p)[0].item() for d, p in pairs]
    assert np.mean(last) < 0.5 * np.mean(first), (first, last)


def test_unet_state_roundtrip_and_partial_tiles(lib):
    """A saved and reloaded network predicts bitwise the same; grids that are not a multiple of the
    16 x 8 tile (24 x 20 x 12: levels 24x20x12, 12x10x6, 6x5x3) match the oracle too."""
    from pfm.nn import UNet3D
    dims = (24, 20, 12)
    div, p = _fields(7, dims)
    dt = torch.as_tensor(div).cuda()
    a = UNet3D(seed=5)
    for _ in range(3):
        a.train_step(dt, torch.as_tensor(p).cuda())
    sd = a.state_dict()
    b = UNet3D(seed=99)
    b.load_state_dict(sd)
    ya, yb = a.predict(dt), b.predict(dt)
    torch.cuda.synchronize()
    a.check()
    b.check()
    assert torch.equal(ya, yb)
    pred, cache = O.forward(a.params.cpu().numpy().astype(np.float64), div, rounding=True)
    ref = pred / cache["s"]
    got = ya.cpu().numpy()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-2


def test_conv_argument_checks(lib):
    """The host side rejects what the kernels cannot take: channel counts that are not multiples of
    16 (inputs) or 8 (bf16 outputs), more than 128 channels, unaligned pointers, null pointers; no
    kernel runs for a rejected call."""
    from pfm import _lib
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    dims = (4, 16, 8)
    V = int(np.prod(dims))
    x = torch.zeros(32 * V + 8, dtype=torch.bfloat16, device="cuda")
    w = torch.zeros(27 * 32 * 32, dtype=torch.bfloat16, device="cuda")
    y = torch.zeros(32 * V + 8, dtype=torch.bfloat16, device="cuda")

    def call(c1=16, c2=0, cout=16, cy1=None, xp=None, wp=None, yp=None, errp=None):
        a = _lib.Conv3Args(dims[0], dims[1], dims[2], xp if xp is not None else P(x), c1, P(x) if c2 else None, c2,
                           wp if wp is not None else P(w), None, cout, 0, yp if yp is not None else P(y),
                           cy1 or cout, None, None, None, errp if errp is not None else P(err))
        return lib.pfm_nn_conv3(ctypes.byref(a), None)

    assert call() == 0
    torch.cuda.synchronize()
    assert call(c1=8) == 2 and call(c1=16, c2=8) == 2 and call(c1=144) == 2
    assert call(cout=12) == 2 and call(cout=16, cy1=12) == 2 and call(cout=136) == 2
    assert call(xp=ctypes.c_void_p(x.data_ptr() + 2)) == 7
    assert call(yp=ctypes.c_void_p(y.data_ptr() + 8)) == 7
    assert call(xp=ctypes.c_void_p(0)) == 1 and call(errp=ctypes.c_void_p(0)) == 1
    torch.cuda.synchronize()
    assert int(err.item()) == 0
