"""Failure detection of the MGPCG solve and the workspace binding, with every failure made on the
host: an iteration limit too small to converge, a NaN placed in the host velocity before it is
uploaded, and a workspace one byte shorter than pfm_workspace_size.  No kernel is made to fault.

The reference prints and returns when MGPCG hits its iteration limit (3D/mgpcg.py:279-280) and has
no checks for non-finite values or undersized buffers (Taichi owns its fields); here each case
returns a status code through the C ABI (include/pfm.h: PFM_ERR_NOT_CONVERGED, PFM_ERR_NONFINITE,
PFM_ERR_WORKSPACE), the Python layer raises PfmError unless told otherwise, and the handle stays
usable afterwards."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import pfm  # noqa: E402
from pfm import _lib  # noqa: E402
from pfm._lib import PfmError  # noqa: E402

RES = (32, 32, 32)
DX = 1.0 / 32


def _ring():
    import __graft_entry__ as G
    return G._ring_velocity(RES, DX)


def _scene():
    return pfm.Scene(3, RES, DX, 0)


def _div_max(u):
    ux, uy, uz = (t.double() for t in u)
    div = (ux[1:] - ux[:-1]) + (uy[:, 1:] - uy[:, :-1]) + (uz[:, :, 1:] - uz[:, :, :-1])
    return div.abs().max().item()


def test_not_converged_returns_status_with_results_written():
    """max_iters = 1 at tol 1e-12: PFM_ERR_NOT_CONVERGED, SolveInfo.converged false, one iteration,
    and the projection still applied (the divergence drops and the pressure is written)."""
    sc = _scene()
    u = [torch.from_numpy(a).cuda() for a in _ring()]
    before = _div_max(u)
    p = torch.zeros(RES, device="cuda")
    info = sc.poisson(u, p, max_iters=1, tol=1e-12, tol_mode=0)
    torch.cuda.synchronize()
    assert info.status == _lib.PFM_ERR_NOT_CONVERGED
    assert not info.converged
    assert info.iterations == 1
    assert np.isfinite(info.rTr) and info.rTr > 1e-12
    assert p.abs().max().item() > 0.0
    after = _div_max(u)
    assert after < 0.5 * before, (before, after)
    # the same limit raises when the caller asks for it
    u2 = [torch.from_numpy(a).cuda() for a in _ring()]
    with pytest.raises(PfmError) as e:
        sc.poisson(u2, p, max_iters=1, tol=1e-12, tol_mode=0, raise_on_limit=True)
    assert e.value.status == _lib.PFM_ERR_NOT_CONVERGED
    # and the handle stays usable: a solve with room converges
    u3 = [torch.from_numpy(a).cuda() for a in _ring()]
    ok = sc.poisson(u3, p, max_iters=400, tol=1e-6, tol_mode=1)
    assert ok.converged and ok.status == 0


def test_not_converged_through_mgpcg_solve():
    """MGPCG.solve on a right-hand side (3D/mgpcg.py:202-280) with max_iters = 2."""
    sc = _scene()
    rng = np.random.default_rng(3)
    r = rng.standard_normal(RES).astype(np.float32)
    r -= r.mean()
    x = torch.zeros(RES, device="cuda")
    info = sc.mgpcg_solve(torch.from_numpy(r).cuda(), x, max_iters=2, tol=1e-12)
    assert info.status == _lib.PFM_ERR_NOT_CONVERGED and not info.converged and info.iterations == 2
    assert torch.isfinite(x).all() and x.abs().max().item() > 0.0


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_nonfinite_velocity_is_reported(precision):
    """A NaN written into the host velocity before the upload: the solve stops with
    PFM_ERR_NONFINITE instead of running to the iteration limit, and the next solve on the same
    handle (finite input) converges."""
    sc = _scene()
    host = _ring()
    host[1][7, 9, 11] = np.nan
    u = [torch.from_numpy(a).cuda() for a in host]
    p = torch.zeros(RES, device="cuda")
    with pytest.raises(PfmError) as e:
        sc.poisson(u, p, max_iters=400, tol=1e-6, tol_mode=1, precision=precision)
    assert e.value.status == 5  # PFM_ERR_NONFINITE
    assert "non-finite" in str(e.value)
    u_ok = [torch.from_numpy(a).cuda() for a in _ring()]
    p.zero_()
    info = sc.poisson(u_ok, p, max_iters=400, tol=1e-6, tol_mode=1, precision=precision)
    assert info.converged


def test_workspace_one_byte_short_is_rejected():
    """pfm_set_workspace with pfm_workspace_size - 1 bytes returns PFM_ERR_WORKSPACE and binds
    nothing, so a phase called next reports the missing workspace instead of writing past it; the
    full size then binds and the phase runs."""
    L = _lib.load()
    cfg = _lib.Config()
    cfg.dim = 3
    for a in range(3):
        cfg.res[a] = RES[a]
    cfg.dx = DX
    cfg.particles = 1000
    cfg.base_level = 3
    cfg.mg_levels = 0
    cfg.pre_post_smoothing = 2
    cfg.bottom_smoothing = 50
    for a in range(3):
        cfg.boundary[a][0] = cfg.boundary[a][1] = 2
    cfg.use_apic = 1
    h = ctypes.c_void_p()
    assert L.pfm_create(ctypes.byref(cfg), ctypes.byref(h)) == 0
    try:
        need = ctypes.c_size_t()
        assert L.pfm_workspace_size(h, ctypes.byref(need)) == 0
        ws = torch.empty(int(need.value), dtype=torch.uint8, device="cuda")
        st = L.pfm_set_workspace(h, ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(int(need.value) - 1))
        assert st == 3  # PFM_ERR_WORKSPACE
        assert b"smaller" in L.pfm_last_error(h)
        pos = torch.rand(3, 1000, device="cuda")
        count = torch.empty(RES, dtype=torch.int32, device="cuda")
        order = torch.empty(1000, dtype=torch.int32, device="cuda")
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        st = L.pfm3_sort_particles(h, ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(count.data_ptr()),
                                   ctypes.c_void_p(order.data_ptr()), stream)
        assert st == 3  # no workspace bound
        st = L.pfm_set_workspace(h, ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(int(need.value)))
        assert st == 0
        st = L.pfm3_sort_particles(h, ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(count.data_ptr()),
                                   ctypes.c_void_p(order.data_ptr()), stream)
        assert st == 0
        torch.cuda.synchronize()
        assert int(count.sum().item()) == 1000
    finally:
        L.pfm_destroy(h)
