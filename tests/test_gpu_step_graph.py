"""The whole step as one CUDA graph (pfm3_step / pfm2_step): the same kernels as the eager phase
calls of pfm.Sim3D / pfm.Sim2D, with dt, the reinitialisation schedule and the MGPCG loops on the
device, so the graph steps are compared with the eager steps bit for bit over runs that cross the
reinitialisations, the gradient schedule and a frame boundary."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import pfm  # noqa: E402
from __graft_entry__ import _ring_velocity  # noqa: E402

MIXED = dict(tol=1e-6, tol_mode=2, max_iters=400, precision="fp16", warm_start=True, true_residual_every=5)
PLAIN = dict(tol=1e-12, tol_mode=0, max_iters=400)


def _pair3(res, opts, **kw):
    dx = 1.0 / res[1]
    u0 = _ring_velocity(res, dx)
    seeds = pfm.jittered(res, dx, 8, seed=2)
    a = pfm.Sim3D(u0, seeds, res, dx, poisson_opts=opts, **kw)
    b = pfm.Sim3D(u0, seeds, res, dx, poisson_opts=opts, graph=True, **kw)
    return a, b


@pytest.mark.parametrize("opts", [MIXED, PLAIN], ids=["mixed", "plain"])
def test_step3_graph_equals_eager(opts):
    a, b = _pair3((32, 16, 16), opts, reinit_every=3, reinit_every_grad_m=2, visualize_dt=0.02)
    iters = []
    for _ in range(7):
        a.step()
        b.step()
        iters.append([inf.iterations for inf in a.infos[-2:]])
    torch.cuda.synchronize()
    for f in range(3):
        assert torch.equal(a.u[f], b.u[f]), f
    for name in ("pos", "init_imp", "T_init", "T_gm", "init_C", "p", "p_mid"):
        assert torch.equal(getattr(a, name), getattr(b, name)), name
    info = b.step_info()
    assert info.step == 6 and info.step == a.i
    assert info.dt == a.last_dt and info.frame_idx == a.clock.frame_idx and info.sub_t == a.clock.sub_t
    assert [[info.history[s][0], info.history[s][1]] for s in range(7)] == iters
    assert [info.converged[0], info.converged[1]] == [int(inf.converged) for inf in a.infos[-2:]], iters


def test_step3_graph_restart_and_rebuild():
    """pfm_step_reset restarts the device clock; new field pointers rebuild the graph."""
    a, b = _pair3((16, 16, 16), MIXED, reinit_every=4, reinit_every_grad_m=1)
    for _ in range(2):
        a.step()
        b.step()
    # continue the graph run from copies of its state (new pointers) and a reset clock
    c = pfm.Sim3D([t.clone() for t in b.u], b.seeds.clone(), (16, 16, 16), 1.0 / 16, poisson_opts=MIXED,
                  reinit_every=4, reinit_every_grad_m=1, graph=True)
    for name in ("pos", "init_imp", "T_init", "T_gm", "init_C", "p", "p_mid"):
        getattr(c, name).copy_(getattr(b, name))
    c.i, c.ik = a.i, a.ik
    c.clock.sub_t, c.clock.frame_idx = a.clock.sub_t, a.clock.frame_idx
    for _ in range(3):
        a.step()
        c.step()
    torch.cuda.synchronize()
    for f in range(3):
        assert torch.equal(a.u[f], c.u[f])
    assert torch.equal(a.pos, c.pos)
    launches0 = c.scene.launches
    info = c.step_info()
    assert info.step == a.i and c.scene.launches > launches0


def test_step2_graph_equals_eager():
    res = (64, 32)
    dx = 1.0 / 32
    rng = np.random.default_rng(4)
    idx = np.meshgrid(np.arange(65) / 32, (np.arange(32) + 0.5) / 32, indexing="ij")
    ux = (0.3 * np.sin(3 * idx[0]) * np.cos(2 * idx[1])).astype(np.float32)
    idy = np.meshgrid((np.arange(64) + 0.5) / 32, np.arange(33) / 32, indexing="ij")
    uy = (0.2 * np.cos(2 * idy[0]) * np.sin(3 * idy[1])).astype(np.float32)
    seeds = pfm.jittered(res, dx, 4, seed=int(rng.integers(100)))
    kw = dict(reinit_every=4, reinit_every_grad_m=3, visualize_dt=0.05, poisson_opts=PLAIN)
    a = pfm.Sim2D([ux, uy], seeds, res, dx, **kw)
    b = pfm.Sim2D([ux, uy], seeds, res, dx, graph=True, **kw)
    for _ in range(9):
        a.step()
        b.step()
    torch.cuda.synchronize()
    for f in range(2):
        assert torch.equal(a.u[f], b.u[f]), f
        assert torch.equal(a.psi_grid[f], b.psi_grid[f]), f
    for name in ("pos", "imp", "init_imp", "psi", "T", "T_init", "T_gm", "init_C", "C", "p"):
        assert torch.equal(getattr(a, name), getattr(b, name)), name
    info = b.step_info()
    assert info.step == 8 and info.dt == a.last_dt


def test_step_rejects_unbounded_solve():
    a, b = _pair3((16, 16, 16), dict(tol=1e-6, tol_mode=1, max_iters=-1))
    with pytest.raises(pfm.PfmError):
        b.step()


def test_batch_equals_scenes_alone():
    """Scenes of uneven sizes (2D and 3D) advanced together by one batch graph launch per step are
    bitwise the same scenes stepped alone."""
    specs = [(32, 32), (64, 32), (48, 48), (16, 16, 16)]
    opts = dict(tol=1e-6, tol_mode=1, max_iters=400)

    def make(spec, graph):
        if len(spec) == 2:
            dx = 1.0 / spec[1]
            u = pfm.vortex_blobs2(spec, dx, seed=sum(spec))
            return pfm.Sim2D(u, pfm.jittered(spec, dx, 4, seed=1), spec, dx, reinit_every=5, reinit_every_grad_m=2,
                             poisson_opts=opts, graph=graph)
        dx = 1.0 / spec[1]
        return pfm.Sim3D(_ring_velocity(spec, dx), pfm.jittered(spec, dx, 8, seed=1), spec, dx, reinit_every=4,
                         poisson_opts=opts, graph=graph)

    alone = [make(s, False) for s in specs]
    together = [make(s, True) for s in specs]
    batch = pfm.Batch(together)
    for _ in range(6):
        for sim in alone:
            sim.step()
        batch.step()
    torch.cuda.synchronize()
    for a, b in zip(alone, together):
        for f in range(len(a.u)):
            assert torch.equal(a.u[f], b.u[f])
        assert torch.equal(a.pos, b.pos) and torch.equal(a.p, b.p)
        info = b.step_info()
        assert info.step == a.i == 5 and info.dt == a.last_dt


@pytest.mark.parametrize("dim", [2, 3])
def test_batch_worklist_equals_scenes_alone(dim):
    """The work-list form (the scenes' MGPCG iterations as batched persistent kernels over a
    (scene, block) work list, joined at each solve) is bitwise the scenes stepped alone: scenes of
    uneven sizes whose solves converge at different iterations and whose hierarchies have different
    depths, with and without a one-block V-cycle tail, in plain FP32 and in the mixed form."""
    from pfm import _lib

    def make(spec, graph, opts):
        dx = 1.0 / spec[1]
        if len(spec) == 2:
            return pfm.Sim2D(pfm.vortex_blobs2(spec, dx, seed=sum(spec)), pfm.jittered(spec, dx, 4, seed=1), spec, dx,
                             reinit_every=5, reinit_every_grad_m=2, poisson_opts=opts, graph=graph)
        return pfm.Sim3D(_ring_velocity(spec, dx), pfm.jittered(spec, dx, 8, seed=1), spec, dx, reinit_every=4,
                         poisson_opts=opts, graph=graph)

    specs = [(32, 32), (64, 32), (128, 128), (48, 48), (256, 64)] if dim == 2 else [(16, 16, 16), (32, 16, 24),
                                                                                    (24, 24, 24)]
    for opts in (dict(tol=1e-6, tol_mode=1, max_iters=400),
                 dict(tol=1e-6, tol_mode=2, max_iters=400, precision="fp16", warm_start=dim == 3,
                      true_residual_every=5)):  # the 2D midpoint solve keeps no pressure to start from
        alone = [make(s, False, opts) for s in specs]
        together = [make(s, True, opts) for s in specs]
        together[0].scene.set_tuning(_lib.TUNE_MG_TAIL_CELLS, 0)  # one scene without a tail
        alone[0].scene.set_tuning(_lib.TUNE_MG_TAIL_CELLS, 0)
        batch = pfm.Batch(together, worklist=True)
        for _ in range(6):
            for sim in alone:
                sim.step()
            batch.step()
        torch.cuda.synchronize()
        for a, b in zip(alone, together):
            for f in range(len(a.u)):
                assert torch.equal(a.u[f], b.u[f])
            assert torch.equal(a.pos, b.pos) and torch.equal(a.p, b.p)
            info = b.step_info()
            assert info.step == a.i == 5 and info.dt == a.last_dt
            assert [info.iterations[0], info.iterations[1]] == [a.infos[-2].iterations, a.infos[-1].iterations]
        # the batch can go back to the branch form and carries on identically
        batch.set_worklist(False)
        for sim in alone:
            sim.step()
        batch.step()
        torch.cuda.synchronize()
        for a, b in zip(alone, together):
            assert all(torch.equal(x, y) for x, y in zip(a.u, b.u))


def test_batch_worklist_rejects_mixed_scenes():
    opts = dict(tol=1e-6, tol_mode=1, max_iters=400)
    s2 = pfm.Sim2D(pfm.vortex_blobs2((32, 32), 1 / 32, seed=1), pfm.jittered((32, 32), 1 / 32, 4, seed=1), (32, 32),
                   1 / 32, poisson_opts=opts, graph=True)
    s3 = pfm.Sim3D(_ring_velocity((16, 16, 16), 1 / 16), pfm.jittered((16, 16, 16), 1 / 16, 8, seed=1), (16, 16, 16),
                   1 / 16, poisson_opts=opts, graph=True)
    batch = pfm.Batch([s2, s3], worklist=True)
    with pytest.raises(pfm.PfmError, match="share the dimension"):
        batch.step()


def test_tunables_do_not_change_results():
    """The autotuner's knobs (2D P2G column length, MGPCG tail threshold) change launch shapes only:
    steps with different values are bitwise equal."""
    from pfm import tune
    res = (64, 48)
    dx = 1.0 / 48
    u = pfm.vortex_blobs2(res, dx, seed=9)
    seeds = pfm.jittered(res, dx, 4, seed=3)
    kw = dict(reinit_every=4, reinit_every_grad_m=2, poisson_opts=dict(tol=1e-6, tol_mode=1, max_iters=400))
    a = pfm.Sim2D(u, seeds, res, dx, graph=True, **kw)
    b = pfm.Sim2D(u, seeds, res, dx, graph=True, **kw)
    b.scene.set_tuning(1, 3)
    b.scene.set_tuning(2, 0)
    for _ in range(5):
        a.step()
        b.step()
    torch.cuda.synchronize()
    for f in range(2):
        assert torch.equal(a.u[f], b.u[f])
    assert torch.equal(a.p, b.p) and torch.equal(a.pos, b.pos)
    chosen = tune.autotune(a, reps=1)
    assert set(chosen) == {"mg_tail_cells", "p2g2_column"}
    assert a.scene.get_tuning(2) == chosen["mg_tail_cells"][0]
    with pytest.raises(pfm.PfmError):
        a.scene.set_tuning(1, 0)
