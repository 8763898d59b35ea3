"""Learned warm start for the pressure solve: a 3-level 3D convolutional U-Net that maps a
divergence field to an initial pressure, trained and run on the tensor cores through libpfm.so
(``pfm_nn_*`` in include/pfm.h).

The network (widths 16/32/64 by default, 3x3x3 kernels, BF16 weights and activations, FP32
accumulation) is::

    x (div / rms(div), 16 channels, channel 0 used)
    enc0a, enc0b          conv+ReLU at full resolution       -> e0
    pool 2x2x2 (average)  enc1a, enc1b  at 1/2               -> e1
    pool                  bot_a, bot_b  at 1/4               -> b
    upsample (nearest)    dec1a([e1, up(b)]), dec1b   at 1/2 -> d1
    upsample              dec0a([e0, up(d1)]), dec0b  at 1   -> d0
    out                   conv, linear, 1 channel, times rms(div)

The Poisson problem is linear, so dividing the input by its RMS and multiplying the output by it
makes the network independent of the field's scale.  The loss is the mean squared error of the
prediction against the solver's pressure up to a constant (the all-Neumann pressure is defined up
to one), on the scaled fields.  Training is plain Adam on FP32 master weights; after every update
the weights are re-packed to BF16 for the forward and (flipped, transposed) for the data gradient.

Every grid size needs d0, d1, d2 divisible by 4.  The network never replaces the solver: MGPCG
runs from its guess to the same residual (``warm_start=True``).
"""
import ctypes
import math

import torch

from . import _lib
from ._lib import PfmError

__all__ = ["UNet3D", "LAYERS"]

# name, input channels (first, concatenated second), output channels, ReLU, level
LAYERS = [
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


def _r16(c):
    return (c + 15) // 16 * 16


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class _Layer:
    def __init__(self, spec, w, b, gw, gb):
        self.name, self.c1, self.c2, self.cout, self.relu, self.level = spec
        self.cin = self.c1 + self.c2
        self.w, self.b, self.gw, self.gb = w, b, gw, gb  # views into the flat parameter / gradient buffers
        self.npad = _r16(self.cout)
        self.kin_t = _r16(self.cout)  # channels of the gradient fed to the data-gradient convolution
        self.wp = None  # forward packing [27][cin/8][npad][8]
        self.wq = None  # data-gradient packing [27][kin_t/8][r16(cin)][8]


class UNet3D:
    """The warm-start network: parameters, Adam state and per-grid activation buffers."""

    def __init__(self, device="cuda", seed=0, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        self.lib = _lib.load()
        self.device = torch.device(device)
        sizes = []
        for (_, c1, c2, cout, _, _) in LAYERS:
            sizes += [cout * (c1 + c2) * 27, cout]
        self.n_params = sum(sizes)
        self.params = torch.zeros(self.n_params, device=self.device)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.lr, self.betas, self.eps = lr, betas, eps
        self.step_count = 0
        self.layers = []
        off = 0
        g = torch.Generator().manual_seed(seed)
        init = torch.zeros(self.n_params)
        for spec in LAYERS:
            _, c1, c2, cout, relu, _ = spec
            cin = c1 + c2
            nw = cout * cin * 27
            std = math.sqrt((2.0 if relu else 1.0) / (cin * 27))  # He et al. 2015 for ReLU layers
            init[off:off + nw] = torch.randn(nw, generator=g) * std
            w = self.params[off:off + nw].view(cout, cin, 27)
            gw = self.grads[off:off + nw].view(cout, cin, 27)
            off += nw
            b = self.params[off:off + cout]
            gb = self.grads[off:off + cout]
            off += cout
            self.layers.append(_Layer(spec, w, b, gw, gb))
        self.params.copy_(init.to(self.device))
        self.L = {l.name: l for l in self.layers}
        for l in self.layers:
            l.wp = torch.empty(27 * l.cin * l.npad, dtype=torch.bfloat16, device=self.device)
            l.wq = torch.empty(27 * l.kin_t * _r16(l.cin), dtype=torch.bfloat16, device=self.device)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.scratch = torch.zeros(int(self.lib.pfm_nn_scratch_floats(64)), device=self.device)
        self.stats = torch.zeros(4, device=self.device)   # loss of the last training step
        self.in_stats = torch.zeros(4, device=self.device)  # {., ., 1/rms, rms} of the last input
        self._bufs = {}
        self.pack()

    # -- plumbing -------------------------------------------------------------------------------
    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _check(self, status, what):
        if status != 0:
            raise PfmError(status, what)

    def check(self):
        """Synchronizes and raises if a kernel's bounded wait gave up."""
        e = int(self.err.item())
        if e != 0:
            raise PfmError(6, f"U-Net kernel wait expired (code {e})")

    def pack(self):
        """Re-packs every layer's BF16 weights from the FP32 masters."""
        st = self._stream()
        for l in self.layers:
            self._check(self.lib.pfm_nn_pack_weights(_p(l.w), l.cout, l.cin, 0, l.cin, l.npad, _p(l.wp), st),
                        "pack forward weights")
            self._check(self.lib.pfm_nn_pack_weights(_p(l.w), l.cout, l.cin, 1, l.kin_t, _r16(l.cin), _p(l.wq), st),
                        "pack data-gradient weights")

    def state_dict(self):
        return {"params": self.params.detach().cpu(), "m": self.m.cpu(), "v": self.v.cpu(), "step": self.step_count}

    def load_state_dict(self, sd):
        self.params.copy_(sd["params"].to(self.device))
        if "m" in sd:
            self.m.copy_(sd["m"].to(self.device))
            self.v.copy_(sd["v"].to(self.device))
        self.step_count = int(sd.get("step", 0))
        self.pack()

    def _blk(self, c, dims):
        return torch.empty(c * dims[0] * dims[1] * dims[2], dtype=torch.bfloat16, device=self.device)

    def buffers(self, dims, train):
        key = (tuple(dims), bool(train))
        if key in self._bufs:
            return self._bufs[key]
        d0, d1, d2 = dims
        if d0 % 4 or d1 % 4 or d2 % 4:
            raise PfmError(2, f"U-Net grid {dims} must be divisible by 4")
        F, H, Q = tuple(dims), (d0 // 2, d1 // 2, d2 // 2), (d0 // 4, d1 // 4, d2 // 4)
        B = {"F": F, "H": H, "Q": Q}
        for name, c, g in [("x", 16, F), ("e0a", 16, F), ("e0", 16, F), ("p0", 16, H), ("e1a", 32, H), ("e1", 32, H),
                           ("p1", 32, Q), ("ba", 64, Q), ("b", 64, Q), ("u1", 64, H), ("d1a", 32, H), ("d1", 32, H),
                           ("u0", 32, F), ("d0a", 16, F), ("d0", 16, F)]:
            B[name] = self._blk(c, g)
        B["pred"] = torch.empty(F, device=self.device)
        if train:
            for name, c, g in [("gout", 16, F), ("gA", 16, F), ("gB", 16, F), ("gS0", 16, F), ("gU0", 32, F),
                               ("gH32a", 32, H), ("gH32b", 32, H), ("gS1", 32, H), ("gU1", 64, H), ("gP0", 16, H),
                               ("gQa", 64, Q), ("gQb", 64, Q), ("gP1", 32, Q)]:
                B[name] = self._blk(c, g)
            need = 0
            for l in self.layers:
                g = {0: F, 1: H, 2: Q}[l.level]
                a = _lib.Conv3WgradArgs(g[0], g[1], g[2], None, l.c1, None, l.c2, None, l.kin_t, l.cout)
                nb = ctypes.c_size_t()
                self._check(self.lib.pfm_nn_wgrad_workspace(ctypes.byref(a), ctypes.byref(nb)), "wgrad workspace")
                need = max(need, nb.value)
            B["partial"] = torch.empty(need // 4 + 1, device=self.device)
        self._bufs[key] = B
        return B

    # -- layers ---------------------------------------------------------------------------------
    def _conv(self, l, g, x1, x2, y1=None, y2=None, cy1=None, yf=None, yf_scale=None):
        a = _lib.Conv3Args(g[0], g[1], g[2], _p(x1), l.c1, _p(x2), l.c2, _p(l.wp), _p(l.b), l.cout, int(l.relu),
                           _p(y1), cy1 or l.cout, _p(y2), _p(yf), _p(yf_scale), _p(self.err))
        self._check(self.lib.pfm_nn_conv3(ctypes.byref(a), self._stream()), f"conv {l.name}")

    def _dgrad(self, l, g, dy, gx1, gx2=None):
        a = _lib.Conv3Args(g[0], g[1], g[2], _p(dy), l.kin_t, None, 0, _p(l.wq), None, l.cin, 0, _p(gx1), l.c1,
                           _p(gx2), None, None, _p(self.err))
        self._check(self.lib.pfm_nn_conv3(ctypes.byref(a), self._stream()), f"dgrad {l.name}")

    def _wgrad(self, l, g, x1, x2, dy, B):
        a = _lib.Conv3WgradArgs(g[0], g[1], g[2], _p(x1), l.c1, _p(x2), l.c2, _p(dy), l.kin_t, l.cout, _p(l.gw),
                                _p(B["partial"]), B["partial"].numel() * 4, _p(self.err))
        st = self._stream()
        self._check(self.lib.pfm_nn_conv3_wgrad(ctypes.byref(a), st), f"wgrad {l.name}")
        self._check(self.lib.pfm_nn_bias_grad(_p(dy), l.kin_t, g[0], g[1], g[2], l.cout, _p(l.gb), _p(self.scratch), st),
                    f"bias grad {l.name}")

    def _resample(self, x, y, c, fine, mode):
        self._check(self.lib.pfm_nn_resample(_p(x), _p(y), c, fine[0], fine[1], fine[2], mode, self._stream()),
                    "resample")

    def _ew(self, g, y, mode):
        self._check(self.lib.pfm_nn_elementwise(_p(g), _p(y), g.numel(), mode, self._stream()), "elementwise")

    # -- network --------------------------------------------------------------------------------
    def _input(self, div, B):
        d0, d1, d2 = B["F"]
        st = self._stream()
        self._check(self.lib.pfm_nn_loss(None, _p(div), None, d0, d1, d2, _p(self.in_stats), None, _p(self.scratch), st),
                    "input scale")
        self._check(self.lib.pfm_nn_pack_scalar(_p(div), d0, d1, d2, _p(self.in_stats[2:3]), _p(B["x"]), st),
                    "pack input")

    def _forward(self, B, out, out_scale):
        L, F, H, Q = self.L, B["F"], B["H"], B["Q"]
        self._conv(L["enc0a"], F, B["x"], None, B["e0a"])
        self._conv(L["enc0b"], F, B["e0a"], None, B["e0"])
        self._resample(B["e0"], B["p0"], 16, F, 0)
        self._conv(L["enc1a"], H, B["p0"], None, B["e1a"])
        self._conv(L["enc1b"], H, B["e1a"], None, B["e1"])
        self._resample(B["e1"], B["p1"], 32, H, 0)
        self._conv(L["bot_a"], Q, B["p1"], None, B["ba"])
        self._conv(L["bot_b"], Q, B["ba"], None, B["b"])
        self._resample(B["b"], B["u1"], 64, H, 2)
        self._conv(L["dec1a"], H, B["e1"], B["u1"], B["d1a"])
        self._conv(L["dec1b"], H, B["d1a"], None, B["d1"])
        self._resample(B["d1"], B["u0"], 32, F, 2)
        self._conv(L["dec0a"], F, B["e0"], B["u0"], B["d0a"])
        self._conv(L["dec0b"], F, B["d0a"], None, B["d0"])
        self._conv(L["out"], F, B["d0"], None, yf=out, yf_scale=out_scale)

    def predict(self, div, out=None):
        """Initial pressure for the divergence ``div`` [d0][d1][d2] (f32, device): ``out`` (f32, same
        shape) = rms(div) * net(div / rms(div)).  Asynchronous; no host synchronization."""
        dims = tuple(div.shape)
        B = self.buffers(dims, False)
        if out is None:
            out = torch.empty(dims, device=self.device)
        self._input(div.contiguous(), B)
        self._forward(B, out, self.in_stats[3:4])
        return out

    def loss_and_grad(self, div, p):
        """Forward and backward on one (divergence, pressure) pair; fills self.grads.  Returns the
        device tensor {loss, mean error, ., .} (loss on the scaled fields, up to a constant)."""
        dims = tuple(div.shape)
        B = self.buffers(dims, True)
        L, F, H, Q = self.L, B["F"], B["H"], B["Q"]
        self._input(div.contiguous(), B)
        self._forward(B, B["pred"], None)
        st = self._stream()
        self._check(self.lib.pfm_nn_loss(_p(B["pred"]), _p(p.contiguous()), _p(self.in_stats[2:3]), F[0], F[1], F[2],
                                         _p(self.stats), _p(B["gout"]), _p(self.scratch), st), "loss")
        # out
        self._wgrad(L["out"], F, B["d0"], None, B["gout"], B)
        self._dgrad(L["out"], F, B["gout"], B["gA"])
        self._ew(B["gA"], B["d0"], 0)
        # dec0b, dec0a
        self._wgrad(L["dec0b"], F, B["d0a"], None, B["gA"], B)
        self._dgrad(L["dec0b"], F, B["gA"], B["gB"])
        self._ew(B["gB"], B["d0a"], 0)
        self._wgrad(L["dec0a"], F, B["e0"], B["u0"], B["gB"], B)
        self._dgrad(L["dec0a"], F, B["gB"], B["gS0"], B["gU0"])
        self._resample(B["gU0"], B["gH32a"], 32, F, 3)
        self._ew(B["gH32a"], B["d1"], 0)
        # dec1b, dec1a
        self._wgrad(L["dec1b"], H, B["d1a"], None, B["gH32a"], B)
        self._dgrad(L["dec1b"], H, B["gH32a"], B["gH32b"])
        self._ew(B["gH32b"], B["d1a"], 0)
        self._wgrad(L["dec1a"], H, B["e1"], B["u1"], B["gH32b"], B)
        self._dgrad(L["dec1a"], H, B["gH32b"], B["gS1"], B["gU1"])
        self._resample(B["gU1"], B["gQa"], 64, H, 3)
        self._ew(B["gQa"], B["b"], 0)
        # bottleneck
        self._wgrad(L["bot_b"], Q, B["ba"], None, B["gQa"], B)
        self._dgrad(L["bot_b"], Q, B["gQa"], B["gQb"])
        self._ew(B["gQb"], B["ba"], 0)
        self._wgrad(L["bot_a"], Q, B["p1"], None, B["gQb"], B)
        self._dgrad(L["bot_a"], Q, B["gQb"], B["gP1"])
        self._resample(B["gP1"], B["gH32a"], 32, H, 1)
        self._ew(B["gH32a"], B["gS1"], 1)
        self._ew(B["gH32a"], B["e1"], 0)
        # enc1b, enc1a
        self._wgrad(L["enc1b"], H, B["e1a"], None, B["gH32a"], B)
        self._dgrad(L["enc1b"], H, B["gH32a"], B["gH32b"])
        self._ew(B["gH32b"], B["e1a"], 0)
        self._wgrad(L["enc1a"], H, B["p0"], None, B["gH32b"], B)
        self._dgrad(L["enc1a"], H, B["gH32b"], B["gP0"])
        self._resample(B["gP0"], B["gA"], 16, F, 1)
        self._ew(B["gA"], B["gS0"], 1)
        self._ew(B["gA"], B["e0"], 0)
        # enc0b, enc0a
        self._wgrad(L["enc0b"], F, B["e0a"], None, B["gA"], B)
        self._dgrad(L["enc0b"], F, B["gA"], B["gB"])
        self._ew(B["gB"], B["e0a"], 0)
        self._wgrad(L["enc0a"], F, B["x"], None, B["gB"], B)
        return self.stats

    def adam_step(self, lr=None):
        self.step_count += 1
        b1, b2 = self.betas
        self._check(self.lib.pfm_nn_adam(_p(self.params), _p(self.grads), _p(self.m), _p(self.v), self.n_params,
                                         float(self.lr if lr is None else lr), b1, b2, self.eps, self.step_count, 1.0,
                                         self._stream()), "adam")
        self.pack()

    def train_step(self, div, p, lr=None):
        """One Adam step on one pair; returns the device loss tensor (read it when needed)."""
        s = self.loss_and_grad(div, p)
        self.adam_step(lr)
        return s
