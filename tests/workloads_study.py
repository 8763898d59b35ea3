"""Throughput of the smaller workloads and of the pressure solve alone.

    python tests/workloads_study.py [--steps2d 200] [--res3d 256]

* 2D leapfrog at 256 x 256 (four Gaussian-core vortices, 262,144 jittered particles, reinit 12/8,
  a 4-level MGPCG to 1e-6 relative): whole-step graph launches, steps/s by CUDA events.
* MGPCG alone at res3d^3 on the two-ring field: the time of one PCG iteration as the slope between
  solves run for 4 and for 12 iterations (the tolerance set below reach), FP32 and FP16 multigrid
  levels, and the kernels one iteration launches (the handle's launch count).
One JSON line each.  Not a pytest module."""
import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "particle-flow-maps_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def timed(fn, reps):
    import torch
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps2d", type=int, default=200)
    ap.add_argument("--res3d", type=int, default=256)
    args = ap.parse_args()
    import torch
    import pfm
    import bench
    from test_gpu_step import four_blobs2
    torch.cuda.set_device(0)
    # 2D leapfrog, whole-step graphs
    res = (256, 256)
    dx = 1.0 / 256
    opts = dict(tol=1e-6, tol_mode=1, max_iters=400)
    u0 = four_blobs2(res, dx)
    sim = pfm.Sim2D(u0, pfm.jittered(res, dx, 4, seed=0), res, dx, mg_levels=4, reinit_every=12,
                    reinit_every_grad_m=8, poisson_opts=opts)
    sim.scene.poisson(sim.u, sim.p, **opts)
    sim.set_graph(True)
    for _ in range(10):
        sim.step()
    l0 = sim.scene.launches
    ms = timed(sim.step, args.steps2d)
    sim.step_info()
    print(json.dumps({"workload": "2D 256^2 leapfrog, 262,144 particles, 4-level MGPCG", "steps_per_s": 1e3 / ms,
                      "ms_per_step": ms, "kernels_per_step": (sim.scene.launches - l0) / args.steps2d}), flush=True)
    del sim
    # MGPCG alone at res3d^3
    n = args.res3d
    base = bench.make_sim(n, 2, dict(tol=1e-6, tol_mode=1, max_iters=400), graph=False)
    u = [t.clone() for t in base.u]
    sc = base.scene
    for prec in ("fp32", "fp16"):
        t = {}
        k = {}
        for it in (4, 12):
            kw = dict(max_iters=it, tol=1e-30, tol_mode=1, precision=prec)
            p = torch.zeros(sc.cell_shape, device="cuda")
            sc.poisson([a.clone() for a in u], p, **kw)  # graphs captured outside the timing
            l0 = sc.launches
            t[it] = timed(lambda: sc.poisson([a for a in u], p, **kw), 3)
            k[it] = (sc.launches - l0) / 3
        print(json.dumps({"workload": f"MGPCG at {n}^3, {prec} multigrid levels", "levels": sc.mg_levels,
                          "ms_per_iteration": (t[12] - t[4]) / 8, "ms_4_iterations": t[4],
                          "kernels_per_iteration": (k[12] - k[4]) / 8}), flush=True)


if __name__ == "__main__":
    main()
