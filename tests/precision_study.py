"""Precision study of the projection: the plain FP32 MGPCG and the mixed-precision, warm-started
MGPCG of the step against an FP64 oracle solve of the identical divergence field.

    python tests/precision_study.py --res 128 --at 1 10 50

For each arm the two-ring scene (bench.py's initial condition) is advanced on the GPU; at the
listed steps the velocity entering the step's final Poisson solve is copied, the GPU solve runs as
part of the step, and the oracle solves the same field in FP64 on the host cores.  One JSON line
per (arm, step): relative L2 error of the projected velocity and of the (mean-free) pressure
against the FP64 solve, MGPCG iterations, and the relative divergence left in the GPU velocity.
Not a pytest module (minutes of host time per FP64 solve at 128^3)."""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "particle-flow-maps_gb300"))
sys.path.insert(0, ROOT)


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def div3(u):
    ux, uy, uz = (np.asarray(a, np.float64) for a in u)
    return (ux[1:] - ux[:-1]) + (uy[:, 1:] - uy[:, :-1]) + (uz[:, :, 1:] - uz[:, :, :-1])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--res", type=int, default=128)
    ap.add_argument("--at", type=int, nargs="+", default=[1, 10, 50])
    ap.add_argument("--oracle-tol", type=float, default=1e-8, help="relative residual of the FP64 oracle solve")
    ap.add_argument("--arms", nargs="+", default=["plain", "mixed"])
    ap.add_argument("--warm-start", type=int, default=3, choices=[1, 2, 3],
                    help="the mixed arm's initial guess (as bench.py): previous pressure, linear or quadratic "
                         "extrapolation")
    args = ap.parse_args()
    import torch
    import bench
    import oracle as O
    arms = {"plain": dict(tol=1e-6, tol_mode=1, max_iters=400),
            "mixed": dict(tol=1e-6, tol_mode=2, max_iters=400, precision="fp16", warm_start=args.warm_start,
                          true_residual_every=5)}
    for arm in args.arms:
        sim = bench.make_sim(args.res, 2, arms[arm], graph=False)  # eager steps: the solves are host calls
        sc = sim.scene
        captured = {}
        calls = {"n": 0}
        real_poisson = sc.poisson

        def poisson(u, p_out=None, **kw):
            calls["n"] += 1
            step = (calls["n"] + 1) // 2  # two solves per step: midpoint, then final
            if calls["n"] % 2 == 0 and step in args.at:
                captured[step] = [t.detach().cpu().numpy().copy() for t in u]
            info = real_poisson(u, p_out, **kw)
            if calls["n"] % 2 == 0 and step in args.at:
                captured[step] = (captured[step], [t.detach().cpu().numpy().copy() for t in u],
                                  p_out.detach().cpu().numpy().copy(), info)
            return info

        sc.poisson = poisson
        for step in range(1, max(args.at) + 1):
            sim.step()
            if step in captured:
                u_in, u_gpu, p_gpu, info = captured.pop(step)
                t0 = time.time()
                ux, uy, uz, p64, it64, _ = O.poisson3(*u_in, fp64=True, tol=args.oracle_tol, tol_mode=1)
                t_or = time.time() - t0
                pg = p_gpu.astype(np.float64)
                b = div3([np.where(_wall(a, f), 0, a) for f, a in enumerate(u_in)])
                print(json.dumps({
                    "arm": arm, "step": step, "res": args.res, "mgpcg_iters": info.iterations,
                    "velocity_rel_l2_vs_fp64": rel(np.concatenate([a.ravel() for a in u_gpu]),
                                                   np.concatenate([a.ravel() for a in (ux, uy, uz)])),
                    "pressure_rel_l2_vs_fp64": rel(pg - pg.mean(), p64 - p64.mean()),
                    "divergence_left_rel": float(np.linalg.norm(div3(u_gpu)) / np.linalg.norm(b - b.mean())),
                    "oracle_iters": it64, "oracle_seconds": round(t_or, 1)}), flush=True)
        del sim
        torch.cuda.empty_cache()


def _wall(a, f):
    """Mask of the wall faces of family f (zeroed by apply_bc before the divergence)."""
    m = np.zeros(a.shape, bool)
    idx = [slice(None)] * 3
    idx[f] = 0
    m[tuple(idx)] = True
    idx[f] = -1
    m[tuple(idx)] = True
    return m


if __name__ == "__main__":
    main()
