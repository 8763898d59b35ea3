"""The mixed-precision and warm-started MGPCG (pfm_solve_opts precision / warm_start /
true_residual_every / tol_mode 2) against the FP64 oracle solve of the same divergence field.

Bar (the precision study's): velocity and pressure within 1e-4 relative L2 of the FP64
projection.  The true residual of any f32 pressure has a floor (the FP64 solution rounded to f32
leaves about 1.6e-5 relative at 64^3), so the projected velocity's divergence, checked
independently in f64, is held to 1e-4 relative; the 1e-6 rule applies to the solver's residual, as
in the reference."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import oracle as O  # noqa: E402
import pfm  # noqa: E402


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def div3(u):
    ux, uy, uz = (np.asarray(a, np.float64) for a in u)
    return (ux[1:] - ux[:-1]) + (uy[:, 1:] - uy[:, :-1]) + (uz[:, :, 1:] - uz[:, :, :-1])


@pytest.fixture(scope="module")
def ring64():
    import __graft_entry__ as G
    res = (64, 64, 64)
    u = G._ring_velocity(res, 1.0 / 64)
    ux, uy, uz, p64, it64, _ = O.poisson3(*u, fp64=True, tol=1e-13, tol_mode=1)
    return res, u, (ux, uy, uz), p64


OPTS = dict(tol=1e-6, tol_mode=2, true_residual_every=5)


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
def test_mixed_solve_against_fp64_oracle(ring64, precision):
    res, u, u64, p64 = ring64
    sc = pfm.Scene(3, res, 1 / 64, 0)
    ud = [torch.from_numpy(a).cuda() for a in u]
    p = torch.zeros(res, device="cuda")
    info = sc.poisson(ud, p, precision=precision, **OPTS)
    assert info.converged
    got = [t.cpu().numpy() for t in ud]
    err_u = rel(np.concatenate([g.ravel() for g in got]), np.concatenate([a.ravel() for a in u64]))
    assert err_u < 1e-4, (precision, err_u)
    pg = p.cpu().numpy().astype(np.float64)
    err_p = rel(pg - pg.mean(), p64 - p64.mean())
    assert err_p < 1e-4, (precision, err_p)
    # independent true-residual check: div(u after) = -(b - A p), b = -div(u before) after apply_bc
    ub = [a.copy() for a in u]
    for f, a in enumerate(ub):
        idx = [slice(None)] * 3
        idx[f] = 0
        a[tuple(idx)] = 0
        idx[f] = -1
        a[tuple(idx)] = 0
    b = div3(ub)
    b -= b.mean()
    r = div3(got)
    true_rel = np.linalg.norm(r) / np.linalg.norm(b)
    assert true_rel <= 1e-4, (precision, true_rel)
    # the solver's own true-residual check (before subtract_grad_p) agrees with it
    assert info.rTr_true >= 0
    assert np.sqrt(info.rTr_true / info.bTb) == pytest.approx(true_rel, rel=0.25)
    print(f"{precision}: iterations {info.iterations}, velocity err {err_u:.2e}, pressure err {err_p:.2e}, "
          f"true residual {np.linalg.norm(r) / np.linalg.norm(b):.2e}")


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_warm_start_saves_iterations(ring64, precision):
    res, u, _, _ = ring64
    sc = pfm.Scene(3, res, 1 / 64, 0)
    rng = np.random.default_rng(1)
    pert = [(a * (1 + 1e-3 * rng.standard_normal(a.shape))).astype(np.float32) for a in u]
    p = torch.zeros(res, device="cuda")
    sc.poisson([torch.from_numpy(a).cuda() for a in u], p, precision=precision, **OPTS)
    cold_p = torch.zeros(res, device="cuda")
    cold = sc.poisson([torch.from_numpy(a).cuda() for a in pert], cold_p, precision=precision, **OPTS)
    warm = sc.poisson([torch.from_numpy(a).cuda() for a in pert], p, precision=precision, warm_start=True, **OPTS)
    assert cold.converged and warm.converged
    assert warm.iterations < cold.iterations, (warm.iterations, cold.iterations)
    assert abs(warm.bTb - cold.bTb) <= 1e-6 * cold.bTb
    assert warm.rTr < 1e-12 * warm.bTb * 1.0001


def test_zero_warm_start_and_mode2_equal_the_reference_solve(ring64):
    res, u, _, _ = ring64
    sc = pfm.Scene(3, res, 1 / 64, 0)
    a = [torch.from_numpy(x).cuda() for x in u]
    b = [torch.from_numpy(x).cuda() for x in u]
    pa = torch.zeros(res, device="cuda")
    pb = torch.zeros(res, device="cuda")
    ia = sc.poisson(a, pa, tol=1e-6, tol_mode=1)
    ib = sc.poisson(b, pb, tol=1e-6, tol_mode=2, warm_start=True)
    torch.cuda.synchronize()
    assert ia.iterations == ib.iterations
    assert torch.equal(pa, pb)
    for x, y in zip(a, b):
        assert torch.equal(x, y)


def test_bad_precision_is_rejected():
    sc = pfm.Scene(3, (16, 16, 16), 1 / 16, 0)
    with pytest.raises(pfm.PfmError, match="precision"):
        sc.poisson(sc.alloc_faces(), torch.zeros(16, 16, 16, device="cuda"), precision=5)


@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("res", [(64, 64, 64), (40, 24, 48)])
def test_tma_smoother_is_bitwise_the_global_one(prec, res):
    """The 16-bit levels smoothed from TMA-staged tiles (PFM_TUNE_SMOOTH_TMA = 1) and from global
    memory (0) give bitwise the same solve: pressure, iterations and residual."""
    from pfm import _lib
    rng = np.random.default_rng(21)
    dx = 1.0 / res[1]
    sc = pfm.Scene(3, res, dx, 0)
    r = torch.as_tensor(rng.standard_normal(res).astype(np.float32)).cuda()
    out = []
    for tma in (0, 1):
        sc.set_tuning(_lib.TUNE_SMOOTH_TMA, tma)
        x = torch.zeros_like(r)
        info = sc.mgpcg_solve(r, x, k=-1.0, tol=1e-6, tol_mode=1, max_iters=200, precision=prec)
        torch.cuda.synchronize()
        out.append((x, info.iterations, info.rTr))
    assert torch.equal(out[0][0], out[1][0]) and out[0][1:] == out[1][1:]


def test_vcycle_tail_is_bitwise_the_grid_kernels():
    """The one-block V-cycle tail gives bitwise the solve of the grid-wide kernels, whether its
    levels take the register path (at most four cells per thread: 12x8x8 and 6x4x4) or the generic
    loop (the 24x16x16 level, 6,144 cells): pressure, iterations and residual for tail thresholds
    0 (no tail), 4,096 and 8,192 cells, FP32 levels.  (With 16-bit levels the tail keeps its
    levels in FP32 shared memory while the grid-wide kernels round every store to the level
    storage, so the two differ there by design.)"""
    prec = 0
    from pfm import _lib
    rng = np.random.default_rng(8)
    res = (48, 32, 32)
    sc = pfm.Scene(3, res, 1.0 / 32, 0, base_level=2)
    r = torch.as_tensor(rng.standard_normal(res).astype(np.float32)).cuda()
    out = []
    for cells in (0, 4096, 8192):
        sc.set_tuning(_lib.TUNE_MG_TAIL_CELLS, cells)
        x = torch.zeros_like(r)
        info = sc.mgpcg_solve(r, x, k=-1.0, tol=1e-6, tol_mode=1, max_iters=200, precision=prec)
        torch.cuda.synchronize()
        out.append((x, info.iterations, info.rTr))
    for x, it, rtr in out[1:]:
        assert torch.equal(out[0][0], x) and (it, rtr) == out[0][1:]


def test_extrapolated_warm_start_in_the_step():
    """warm_start 2: each solve starts from 2 p - p_before, the linear extrapolation of its buffer's
    last two solutions (the library keeps p_before per pressure buffer).  On the two-ring scene the
    final solve needs fewer iterations than from the previous pressure alone, the whole-step graph
    is bitwise the eager phase calls, and the results stay within the solver tolerance of the
    warm_start 1 run."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    base = dict(tol=1e-6, tol_mode=2, max_iters=400, precision="fp16", true_residual_every=5)
    runs = {}
    for name, ws, graph in (("prev", True, True), ("extrap", 2, True), ("extrap_eager", 2, False)):
        sim = bench.make_sim(64, 2, dict(base, warm_start=ws), graph=graph)
        its = []
        for _ in range(8):
            sim.step()
            if not graph:
                its.append((sim.infos[-2].iterations, sim.infos[-1].iterations))
        torch.cuda.synchronize()
        if graph:
            info = sim.step_info()
            its = [tuple(info.history[s % 64]) for s in range(info.step - 7, info.step + 1)]
        runs[name] = (its, [t.clone() for t in sim.u], sim.p.clone())
        del sim
    for a, b in zip(runs["extrap"][1] + [runs["extrap"][2]], runs["extrap_eager"][1] + [runs["extrap_eager"][2]]):
        assert torch.equal(a, b)
    assert runs["extrap"][0] == runs["extrap_eager"][0]
    final_prev = sum(i[1] for i in runs["prev"][0][2:])
    final_extrap = sum(i[1] for i in runs["extrap"][0][2:])
    assert final_extrap < final_prev, (runs["prev"][0], runs["extrap"][0])
    for a, b in zip(runs["extrap"][1], runs["prev"][1]):
        assert (a - b).norm().item() <= 1e-5 * b.norm().item()


def test_extrapolated_warm_start_history_per_buffer():
    """The history is kept per pressure buffer (two per handle); a third buffer is refused, and
    pfm_reset_warm_history makes the next solve start from the buffer alone again (bitwise the
    warm_start 1 solve)."""
    res = (32, 32, 32)
    sc = pfm.Scene(3, res, 1 / 32, 0)
    import __graft_entry__ as G
    u = G._ring_velocity(res, 1 / 32)
    kw = dict(tol=1e-6, tol_mode=2, max_iters=400)
    ps = [torch.zeros(res, device="cuda") for _ in range(3)]
    for p in ps[:2]:
        sc.poisson([torch.from_numpy(a).cuda() for a in u], p, warm_start=2, **kw)
    with pytest.raises(pfm.PfmError, match="two pressure buffers"):
        sc.poisson([torch.from_numpy(a).cuda() for a in u], ps[2], warm_start=2, **kw)
    sc.reset_warm_history()
    a, b = ps[0].clone(), ps[0].clone()
    ia = sc.poisson([torch.from_numpy(x).cuda() for x in u], a, warm_start=True, **kw)
    ib = sc.poisson([torch.from_numpy(x).cuda() for x in u], ps[0], warm_start=2, **kw)
    torch.cuda.synchronize()
    assert ia.iterations == ib.iterations and torch.equal(a, ps[0])


def test_quadratic_warm_start_is_the_extrapolation():
    """warm_start 3: the library keeps what the buffer held at the start of its two previous solves
    (in a step loop, the two solutions before the current one) and starts from 3 (p - h1) + h2, the
    quadratic through the three; with one kept value, from the linear 2 p - h1; with none (a fresh
    history), from p.  Each solve is bitwise the warm_start 1 solve from that guess formed with
    torch in the same rounding order."""
    res = (32, 32, 32)
    sc = pfm.Scene(3, res, 1 / 32, 0)
    import __graft_entry__ as G
    base = G._ring_velocity(res, 1 / 32)
    kw = dict(tol=1e-6, tol_mode=2, max_iters=400, precision="fp16")
    p = torch.zeros(res, device="cuda")
    held = []  # the buffer's contents at the start of each solve
    for k in range(4):  # slightly different fields, as successive steps give
        fields = [a * (1.0 + 0.05 * k) for a in base]
        if k == 0:
            guess = p.clone()
        elif k == 1:
            guess = 2 * p - held[-1]
        else:
            guess = 3 * (p - held[-1]) + held[-2]
        held.append(p.clone())
        ia = sc.poisson([torch.from_numpy(f).cuda() for f in fields], p, warm_start=3, **kw)
        ref = guess.clone()
        ib = pfm.Scene(3, res, 1 / 32, 0).poisson([torch.from_numpy(f).cuda() for f in fields], ref,
                                                  warm_start=True, **kw)
        torch.cuda.synchronize()
        assert ia.iterations == ib.iterations and torch.equal(p, ref), k


def test_quadratic_warm_start_in_the_step():
    """warm_start 3 in the whole-step graph: bitwise the eager phase calls; on the two-ring scene
    its solves take no more iterations in total than with the linear extrapolation, and the results
    stay within the solver tolerance of the warm_start 1 run."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    base = dict(tol=1e-6, tol_mode=2, max_iters=400, precision="fp16", true_residual_every=5)
    runs = {}
    for name, ws, graph in (("prev", True, True), ("lin", 2, True), ("quad", 3, True), ("quad_eager", 3, False)):
        sim = bench.make_sim(64, 2, dict(base, warm_start=ws), graph=graph)
        its = []
        for _ in range(10):
            sim.step()
            if not graph:
                its.append((sim.infos[-2].iterations, sim.infos[-1].iterations))
        torch.cuda.synchronize()
        if graph:
            info = sim.step_info()
            its = [tuple(info.history[s % 64]) for s in range(info.step - 9, info.step + 1)]
        runs[name] = (its, [t.clone() for t in sim.u], sim.p.clone())
        del sim
    for a, b in zip(runs["quad"][1] + [runs["quad"][2]], runs["quad_eager"][1] + [runs["quad_eager"][2]]):
        assert torch.equal(a, b)
    assert runs["quad"][0] == runs["quad_eager"][0]
    total = {k: sum(i[0] + i[1] for i in runs[k][0][3:]) for k in ("lin", "quad")}
    assert total["quad"] <= total["lin"], (runs["lin"][0], runs["quad"][0])
    for a, b in zip(runs["quad"][1], runs["prev"][1]):
        assert (a - b).norm().item() <= 1e-5 * b.norm().item()


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_true_residual_replacement_against_fp64_oracle(ring64, precision):
    """true_residual_replace: x accumulates in FP64 and every 5 iterations, and before convergence
    is accepted, b - A x formed in FP64 replaces the recursive residual and decides.  The solve then
    stops on its true residual (|b - A x| < tol |b| with the FP64 x), the delivered velocity and
    pressure stay within 1e-4 of the FP64 oracle, and it takes no fewer iterations than the
    monitor-only solve of the same field."""
    res, u, u64, p64 = ring64
    sc = pfm.Scene(3, res, 1 / 64, 0)
    ud = [torch.from_numpy(a).cuda() for a in u]
    p = torch.zeros(res, device="cuda")
    info = sc.poisson(ud, p, precision=precision, true_residual_replace=True, **OPTS)
    assert info.converged
    assert info.rTr < (1e-6) ** 2 * info.bTb  # the deciding residual is the true one
    got = [t.cpu().numpy() for t in ud]
    err_u = rel(np.concatenate([g.ravel() for g in got]), np.concatenate([a.ravel() for a in u64]))
    pg = p.cpu().numpy().astype(np.float64)
    err_p = rel(pg - pg.mean(), p64 - p64.mean())
    assert err_u < 1e-4 and err_p < 1e-4, (err_u, err_p)
    mon = sc.poisson([torch.from_numpy(a).cuda() for a in u], torch.zeros(res, device="cuda"), precision=precision,
                     **OPTS)
    assert info.iterations >= mon.iterations
    print(f"{precision} replacement: iterations {info.iterations} (monitor {mon.iterations}), velocity err "
          f"{err_u:.2e}, pressure err {err_p:.2e}, true residual {np.sqrt(info.rTr / info.bTb):.2e}")


def test_true_residual_replacement_in_the_step_graph_equals_eager():
    """The replacement solve inside the whole-step graph is bitwise the eager phase calls."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    opts = dict(tol=1e-6, tol_mode=2, max_iters=400, precision="fp16", warm_start=2, true_residual_every=5,
                true_residual_replace=True)
    out = []
    for graph in (True, False):
        sim = bench.make_sim(48, 2, opts, graph=graph)
        for _ in range(5):
            sim.step()
        torch.cuda.synchronize()
        out.append([t.clone() for t in sim.u] + [sim.p.clone(), sim.pos.clone()])
        del sim
    for a, b in zip(*out):
        assert torch.equal(a, b)
