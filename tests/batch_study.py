"""Batched scenes: 64 independent 2D scenes of uneven sizes advanced together, against the same
scenes launched one by one.

    python tests/batch_study.py [--steps 100] [--warmup 3] [--eager-steps 10]

Workload: 32 scenes at 128^2, 16 at 256^2, 12 at 512^2 and 4 at 1024^2 (8,912,896 cells), each
seeded by its index with 2-8 Gaussian vortex blobs (pfm.vortex_blobs2), 4 jittered particles per
cell (35,651,584 particles), reinit every 12 steps, gradient reinit every 8 (the 2D defaults),
CFL 0.5, MGPCG to a 1e-6 relative residual.  Three ways to advance every scene one step:
  batched   one CUDA graph launch for all 64 scenes (pfm_batch_step: one branch per scene, run
            concurrently),
  batched_worklist  the same graph with the branches joined at each MGPCG solve and every
            scene's solver iterations run by batched persistent kernels over a (scene, block) work
            list (pfm_batch_set_worklist),
  graphs    one whole-step graph launch per scene (pfm2_step), the 64 launches in sequence,
  eager     the phase calls of each scene (Sim2D.step), with its host synchronizations.
Each mode is timed with CUDA events around its steps (after warm-up steps) and prints one JSON
line: batch steps/s, scene steps/s and particle updates/s.  The same scenes carry on from mode to
mode.  Not a pytest module."""
import argparse
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "particle-flow-maps_gb300"))
sys.path.insert(0, ROOT)

SIZES = [128] * 32 + [256] * 16 + [512] * 12 + [1024] * 4


def make_scenes(scale=1):
    import pfm
    sims = []
    opts = dict(tol=1e-6, tol_mode=1, max_iters=400)
    for k, n in enumerate(SIZES):
        n = max(16, n // scale)
        res = (n, n)
        dx = 1.0 / n
        sim = pfm.Sim2D(pfm.vortex_blobs2(res, dx, seed=k), pfm.jittered(res, dx, 4, seed=k), res, dx, CFL=0.5,
                        reinit_every=12, reinit_every_grad_m=8, poisson_opts=opts)
        sim.scene.poisson(sim.u, sim.p, **opts)  # the initial projection (2D/run_2D.py:720-722)
        sims.append(sim)
    return sims


def timed(fn, steps):
    import torch
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3, time.perf_counter() - t0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--eager-steps", type=int, default=10)
    ap.add_argument("--scale", type=int, default=1, help="divide every scene's resolution (quick runs)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes")
    args = ap.parse_args()
    import torch
    import pfm
    from pfm import tune
    torch.cuda.set_device(0)
    sims = make_scenes(args.scale)
    if not args.no_tune:  # one autotune per scene size, applied to every scene of that size
        chosen = {}
        for s in sims:
            if s.res not in chosen:
                chosen[s.res] = tune.autotune(s)
            else:
                tune.apply(s, chosen[s.res])
        print(json.dumps({"autotune": {"%dx%d" % r: {k: {"chosen": v[0], "ms": v[1]} for k, v in c.items()}
                                       for r, c in chosen.items()}}), flush=True)
    P = sum(s.P for s in sims)
    cells = sum(s.res[0] * s.res[1] for s in sims)
    n = len(sims)

    def report(mode, seconds, steps, wall):
        rate = steps / seconds
        print(json.dumps({"mode": mode, "scenes": n, "cells": cells, "particles": P, "steps": steps,
                          "batch_steps_per_s": rate, "scene_steps_per_s": rate * n,
                          "particle_updates_per_s": rate * P, "ms_per_batch_step": seconds / steps * 1e3,
                          "wall_s": wall}), flush=True)
        return rate

    # batched: one graph launch for every scene (branch form)
    batch = pfm.Batch(sims)
    for _ in range(args.warmup):
        batch.step()
    t, w = timed(batch.step, args.steps)
    r_batch = report("batched", t, args.steps, w)
    info = [s.step_info() for s in sims]

    # work-list form: the scenes' MGPCG iterations as batched persistent kernels
    batch.set_worklist(True)
    for _ in range(args.warmup):
        batch.step()
    t, w = timed(batch.step, args.steps)
    r_work = report("batched_worklist", t, args.steps, w)
    batch.set_worklist(False)

    # one whole-step graph launch per scene, in sequence
    def one_by_one():
        for s in sims:
            s.scene.step_graph(*s._graph_args())
            s.i += 1
    for _ in range(args.warmup):
        one_by_one()
    t, w = timed(one_by_one, args.steps)
    r_graphs = report("graphs", t, args.steps, w)

    # eager phase calls per scene
    for s in sims:
        s.set_graph(False)

    def eager():
        for s in sims:
            s.step()
    eager()
    t, w = timed(eager, args.eager_steps)
    r_eager = report("eager", t, args.eager_steps, w)
    print(json.dumps({"speedup_batched_vs_graphs": r_batch / r_graphs, "speedup_batched_vs_eager": r_batch / r_eager,
                      "speedup_worklist_vs_graphs": r_work / r_graphs, "worklist_vs_branches": r_work / r_batch,
                      "mgpcg_iters_last_step_first_scenes": [[i.iterations[0], i.iterations[1]] for i in info[:4]]}),
          flush=True)


if __name__ == "__main__":
    main()
