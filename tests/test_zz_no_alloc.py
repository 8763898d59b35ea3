"""pfm_sort_particles_noalloc: particle binning whose scratch is a fixed array in the library's
device image (no handle, no workspace, no allocation).  Its counts and permutation must equal the
workspace entry points (pfm3_sort_particles / pfm2_sort_particles) bit for bit, on consecutive
calls that reuse the shared scratch.  The file is named to be collected last, so the GPU test also
runs after every other test in the same process."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import pfm  # noqa: E402
from pfm import _lib  # noqa: E402


def _stable(pos, res, dx):
    """numpy restatement of the binning: key = int(pos/dx) clamped, stable argsort."""
    d = len(res)
    c = [np.clip(np.trunc(pos[a] / np.float32(dx)).astype(np.int64), 0, res[a] - 1) for a in range(d)]
    key = c[0] * res[1] + c[1] if d == 2 else (c[0] * res[1] + c[1]) * res[2] + c[2]
    return np.bincount(key, minlength=int(np.prod(res))), np.argsort(key, kind="stable")


def _cases():
    rng = np.random.default_rng(11)
    res3 = (20, 16, 12)
    dx3 = 1.0 / 16
    p3 = pfm.jittered(res3, dx3, 8, seed=3).astype(np.float32)
    p3 = p3[rng.permutation(p3.shape[0])]
    p3[:7] += np.float32(0.4)  # some outside the grid on the high side
    p3[7:13] -= np.float32(0.3)  # and the low side
    res2 = (40, 24)
    dx2 = 1.0 / 24
    p2 = (rng.random((3001, 2)) * np.array([40 / 24, 1.0])).astype(np.float32)
    return [(res3, dx3, np.ascontiguousarray(p3.T)), (res2, dx2, np.ascontiguousarray(p2.T))]


@pytest.mark.gpu
def test_noalloc_sort_matches_workspace_entry_on_consecutive_calls():
    dev = torch.device("cuda:0")
    for rep in range(2):
        for res, dx, pos in _cases():
            P = pos.shape[1]
            pos_d = torch.from_numpy(pos).to(dev)
            sc = pfm.Scene(len(res), res, dx, P)
            want_count, want_order = sc.sort_particles(pos_d)
            count = torch.full((int(np.prod(res)),), -7, dtype=torch.int32, device=dev)
            order = torch.full((P,), -7, dtype=torch.int32, device=dev)
            pfm.sort_particles_noalloc(pos_d, res, dx, count, order)
            torch.cuda.synchronize()
            assert torch.equal(count, want_count.reshape(-1)), (rep, res)
            assert torch.equal(order, want_order), (rep, res)
            ref_count, ref_order = _stable(pos, res, dx)
            assert np.array_equal(count.cpu().numpy(), ref_count)
            assert np.array_equal(order.cpu().numpy(), ref_order)


@pytest.mark.gpu
def test_noalloc_sort_zero_particles():
    dev = torch.device("cuda:0")
    count = torch.full((6 * 5,), 3, dtype=torch.int32, device=dev)
    pos = torch.empty((2, 0), dtype=torch.float32, device=dev)
    order = torch.empty((0,), dtype=torch.int32, device=dev)
    pfm.sort_particles_noalloc(pos, (6, 5), 0.2, count, order)
    torch.cuda.synchronize()
    assert int(count.abs().sum()) == 0


@pytest.mark.gpu
def test_noalloc_sort_all_particles_in_one_cell():
    """The largest input the scratch holds, every particle in one bin (half of them inside the
    cell, half clamped into it from outside the grid), on two consecutive calls: the permutation is
    the stable one, and each call ends within a time bound (the per-bin ordering does O(n log^2 n)
    work spread over a thread block, not O(n^2) dependent steps in one thread)."""
    import time
    dev = torch.device("cuda:0")
    res, dx = (8, 8, 8), 0.125
    P = _lib.NOALLOC_MAX_PARTICLES
    rng = np.random.default_rng(5)
    pos = np.empty((3, P), np.float32)
    half = P // 2
    pos[:, :half] = ((np.array([[7], [7], [7]]) + rng.random((3, half))) * dx).astype(np.float32)
    pos[:, half:] = (1.0 + rng.random((3, P - half))).astype(np.float32)  # beyond the grid: clamped
    pos = np.ascontiguousarray(pos[:, rng.permutation(P)])
    pos_d = torch.from_numpy(pos).to(dev)
    ref_count, ref_order = _stable(pos, res, dx)
    assert ref_count.max() == P
    for _ in range(2):
        count = torch.full((512,), -7, dtype=torch.int32, device=dev)
        order = torch.full((P,), -7, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pfm.sort_particles_noalloc(pos_d, res, dx, count, order)
        torch.cuda.synchronize()
        elapsed = time.perf_counter() - t0
        assert elapsed < 2.0, elapsed
        assert np.array_equal(count.cpu().numpy(), ref_count)
        assert np.array_equal(order.cpu().numpy(), ref_order)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    """Validation happens before any CUDA call, so this runs without a GPU."""
    lib = pfm.load()
    res = (ctypes.c_int * 3)(1 << 10, 1 << 9, 1)  # 2^19 cells > 2^18
    assert lib.pfm_sort_particles_noalloc(2, res, 1.0, 0, None, ctypes.c_void_p(16), None, None) == 2
    res = (ctypes.c_int * 3)(8, 8, 8)
    too_many = _lib.NOALLOC_MAX_PARTICLES + 1
    assert lib.pfm_sort_particles_noalloc(3, res, 1.0, too_many, ctypes.c_void_p(16), ctypes.c_void_p(16),
                                          ctypes.c_void_p(16), None) == 2
    assert lib.pfm_sort_particles_noalloc(4, res, 1.0, 0, None, ctypes.c_void_p(16), None, None) == 7
    assert lib.pfm_sort_particles_noalloc(3, res, 0.0, 0, None, ctypes.c_void_p(16), None, None) == 7
    assert lib.pfm_sort_particles_noalloc(3, res, 1.0, 5, None, ctypes.c_void_p(16), None, None) == 1
    with pytest.raises(pfm.PfmError, match="at most"):
        pfm.sort_particles_noalloc(torch.zeros(2, _lib.NOALLOC_MAX_PARTICLES + 1), (4, 4), 0.25,
                                   torch.zeros(16, dtype=torch.int32), torch.zeros(1, dtype=torch.int32))
