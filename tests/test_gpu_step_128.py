"""Element-wise parity at the 3D workload size: 128^3 unit cube, two coaxial vortex rings on the x
axis through (y, z) = (0.5, 0.5) (radius 0.15, core 0.025 with the 1-exp(-(r/d)^3) mollifier of
3D/init_conditions.py:10-22, circulation 1, centres x = 0.25 and 0.35), 8 jittered particles per
cell from seed 0 (16,777,216 particles), CFL 0.5, reinit every 20 steps, gradient reinit every step,
a 5-level MGPCG to |r| < 1e-6 |b| -- stepped on the GPU (one whole-step CUDA graph launch per step)
and by the oracle's restatement of run_3D.main()'s loop body (3D/run_3D.py:716-822) from the same
initial velocity and seeds.

Bar after steps 1 and 10: grid velocity, particle impulse, T_gm and T_init within 1e-5 relative
L2, positions within 1e-6, mean-free pressure within 2e-5.  The plain FP32 arm solves from zero;
the mixed arm (FP16 multigrid levels, compensated FP64-combined dot products, true residual every
5 iterations, warm-started from the previous step's pressure) stops at the same residual rule and
is held to the same bar against the same FP32 oracle run."""
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import oracle as O  # noqa: E402
import pfm  # noqa: E402

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

N = 128
CHECK = (1, 10)
TOL, PTOL, XTOL = 1e-5, 2e-5, 1e-6
PLAIN = dict(tol=1e-6, tol_mode=1, max_iters=400)
MIXED = dict(tol=1e-6, tol_mode=2, max_iters=400, precision="fp16", warm_start=True, true_residual_every=5)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


def prel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return rel(a - a.mean(), b - b.mean())


def _snapshot_gpu(sim):
    torch.cuda.synchronize()
    return dict(u=[t.cpu().numpy() for t in sim.u], p=sim.p.cpu().numpy(), pos=pfm.aos(sim.pos),
                init_imp=pfm.aos(sim.init_imp), T_gm=pfm.aos_T(sim.T_gm), T_init=pfm.aos_T(sim.T_init))


@pytest.fixture(scope="module")
def start():
    """The shared initial state: the GPU scene's projected two-ring velocity and its seeds."""
    sim = bench.make_sim(N, 2, PLAIN, graph=True)
    u0 = [t.cpu().numpy() for t in sim.u]
    seeds = pfm.aos(sim.seeds)
    del sim
    torch.cuda.empty_cache()
    return u0, seeds


@pytest.fixture(scope="module")
def oracle_states(start):
    u0, seeds = start
    ref = O.Sim3D(u0, seeds, (N, N, N), 1.0 / N, CFL=0.5, visualize_dt=0.1, reinit_every=20, reinit_every_grad_m=1,
                  p2g_threads=O.num_threads(), poisson_opts=dict(tol=1e-6, tol_mode=1, max_iters=400))
    out = {}
    for s in range(1, max(CHECK) + 1):
        ref.step()
        if s in CHECK:
            out[s] = dict(u=[a.copy() for a in ref.u], p=ref.p.copy(), pos=ref.pos.copy(),
                          init_imp=ref.init_imp.copy(), T_gm=ref.T_gm.copy(), T_init=ref.T_init.copy())
    out["iters"] = list(ref.iters)
    return out


def _run_gpu(start, opts):
    u0, seeds = start
    dev = [torch.from_numpy(a).cuda() for a in u0]
    sim = pfm.Sim3D(dev, pfm.soa(seeds), (N, N, N), 1.0 / N, CFL=0.5, visualize_dt=0.1, reinit_every=20,
                    reinit_every_grad_m=1, poisson_opts=opts, graph=True)
    out = {}
    for s in range(1, max(CHECK) + 1):
        sim.step()
        if s in CHECK:
            out[s] = _snapshot_gpu(sim)
    info = sim.step_info()
    out["converged"] = (info.converged[0], info.converged[1])
    del sim
    torch.cuda.empty_cache()
    return out


def _compare(gpu, ref, s):
    errs = {f"u{f}": rel(gpu["u"][f], ref["u"][f]) for f in range(3)}
    errs["p"] = prel(gpu["p"], ref["p"])
    errs["pos"] = rel(gpu["pos"], ref["pos"])
    for k in ("init_imp", "T_gm", "T_init"):
        errs[k] = rel(gpu[k], ref[k])
    print(f"step {s}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    for f in range(3):
        assert errs[f"u{f}"] < TOL, (s, errs)
    assert errs["p"] < PTOL, (s, errs)
    assert errs["pos"] < XTOL, (s, errs)
    for k in ("init_imp", "T_gm", "T_init"):
        assert errs[k] < TOL, (s, k, errs)


def test_step3d_128_plain_vs_oracle(start, oracle_states):
    gpu = _run_gpu(start, PLAIN)
    assert all(gpu["converged"])
    for s in CHECK:
        _compare(gpu[s], oracle_states[s], s)


def test_step3d_128_mixed_vs_oracle(start, oracle_states):
    gpu = _run_gpu(start, MIXED)
    assert all(gpu["converged"])
    for s in CHECK:
        _compare(gpu[s], oracle_states[s], s)
