"""Learned warm start of the pressure solve on the 3D Boussinesq plume: data, training, evaluation.

    python tests/warmstart_study.py [--small 96] [--large 192] [--sources 8] [--steps 125]
                                    [--train-steps 3000] [--train-seconds 300] [--eval-steps 200]

1. Data: plume runs (pfm.plume.Plume3D: source sphere r 0.05 at (sx, 0.1, sz), density 1,
   buoyancy +1 along y, 8 particles per cell from seed 0, MGPCG to |r| < 1e-6 |b| warm-started
   from the previous pressure) at the small and the large resolution for each of --sources source
   positions drawn uniformly in [0.3, 0.7] x {0.1} x [0.3, 0.7] (numpy default_rng(seed)); after
   --skip steps from rest each step's (divergence, pressure) of the final projection is kept:
   sources x steps pairs per resolution (2 x 8 x 125 = 2,000 by default).
2. Training: pfm.nn.UNet3D (3 levels, 16/32/64 channels, BF16 tensor-core convolutions), Adam,
   one pair per step drawn at random, cosine learning-rate decay, stopped at --train-steps or
   --train-seconds.
3. Evaluation on a held-out source (drawn after the training ones) at the large resolution for
   --eval-steps steps: at every step the same divergence is solved from three initial guesses --
   zero, the previous step's pressure (the method without the network) and the network's
   prediction -- each to the same residual; the run itself continues with the previous-pressure
   solve.  Reported: MGPCG iterations, the solve's wall time (CUDA events; the network's inference
   counted in its solve) and the guess's error against the converged pressure (relative L2 up to a
   constant).

Prints JSON lines.  Not a pytest module.
"""
import argparse
import json
import math
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "particle-flow-maps_gb300"))


def emit(**kw):
    print(json.dumps(kw), flush=True)


def sources(n, seed):
    import numpy as np
    rng = np.random.default_rng(seed)
    return [(float(rng.uniform(0.3, 0.7)), 0.1, float(rng.uniform(0.3, 0.7))) for _ in range(n + 1)]


def gen(res, src, steps, skip):
    import torch
    from pfm.plume import Plume3D
    sim = Plume3D(res=(res, res, res), source=src)
    sim.record = []
    t0 = time.perf_counter()
    for _ in range(skip + steps):
        sim.step()
    torch.cuda.synchronize()
    pairs = sim.record[skip:]
    its = [i.iterations for i in sim.infos[1::2]]
    del sim
    torch.cuda.empty_cache()
    return pairs, time.perf_counter() - t0, its


def rel_err(guess, p):
    g = guess - guess.mean()
    q = p - p.mean()
    return (g - q).norm().item() / max(q.norm().item(), 1e-30)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--small", type=int, default=96)
    ap.add_argument("--large", type=int, default=192)
    ap.add_argument("--sources", type=int, default=8)
    ap.add_argument("--steps", type=int, default=125)
    ap.add_argument("--skip", type=int, default=5)
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--train-seconds", type=float, default=300.0)
    ap.add_argument("--eval-steps", type=int, default=200)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--time-only", action="store_true", help="time the network's forward and training step only")
    args = ap.parse_args()
    import numpy as np
    import torch
    import pfm
    from pfm.nn import UNet3D
    torch.cuda.set_device(0)
    net = UNet3D(seed=args.seed, lr=args.lr)
    emit(network={"parameters": net.n_params, "layers": len(net.layers)})

    def timeit(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    for n in sorted({args.small, args.large}):
        d = torch.randn(n, n, n, device="cuda")
        p = torch.randn(n, n, n, device="cuda")
        out = torch.empty_like(d)
        f_ms = timeit(lambda: net.predict(d, out))
        t_ms = timeit(lambda: net.loss_and_grad(d, p))
        V = n ** 3
        flop_f = sum(2 * 27 * (l.c1 + l.c2) * max(l.cout, 1) * V / 8 ** l.level for l in net.layers)
        emit(timing={"res": n, "forward_ms": f_ms, "forward_backward_ms": t_ms,
                     "forward_tflops": flop_f / (f_ms * 1e-3) / 1e12,
                     "forward_backward_tflops": 3 * flop_f / (t_ms * 1e-3) / 1e12})
        net.check()
    if args.time_only:
        return
    net = UNet3D(seed=args.seed, lr=args.lr)

    # 1. data
    srcs = sources(args.sources, args.seed)
    train_src, held = srcs[:-1], srcs[-1]
    data = []
    for res in (args.small, args.large):
        for s in train_src:
            pairs, sec, its = gen(res, s, args.steps, args.skip)
            data += pairs
            emit(data={"res": res, "source": s, "pairs": len(pairs), "seconds": sec,
                       "mgpcg_iters_mean": float(np.mean(its))})

    # 2. training
    rng = np.random.default_rng(args.seed + 1)
    t0 = time.perf_counter()
    hist = []
    it = 0
    while it < args.train_steps and time.perf_counter() - t0 < args.train_seconds:
        lr = args.lr * 0.5 * (1 + math.cos(math.pi * it / args.train_steps))
        d, p = data[int(rng.integers(len(data)))]
        s = net.train_step(d, p, lr=lr)
        it += 1
        if it % 100 == 0:
            hist.append((it, s[0].item()))
    torch.cuda.synchronize()
    net.check()
    emit(training={"steps": it, "seconds": time.perf_counter() - t0, "pairs": len(data),
                   "loss_every_100": hist[-10:] if len(hist) > 10 else hist})
    del data
    torch.cuda.empty_cache()

    # 3. evaluation
    from pfm.plume import Plume3D
    n = args.large
    sim = Plume3D(res=(n, n, n), source=held)
    for _ in range(args.skip):
        sim.step()
    sc = sim.scene
    opts = dict(sim.poisson_opts)
    rows = []
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def solve(guess_fn):
        u = [a.clone() for a in sim.u]
        p = torch.zeros_like(sim.p)
        torch.cuda.synchronize()
        ev[0].record()
        warm = guess_fn(p)
        info = sc.poisson(u, p, warm_start=warm, **opts)
        ev[1].record()
        torch.cuda.synchronize()
        return info, ev[0].elapsed_time(ev[1]), p

    def compare():
        sim.divergence()
        div = sim.div.clone()
        prev = sim.p.clone()
        i0, t0_, p0 = solve(lambda p: False)
        i1, t1_, _ = solve(lambda p: (p.copy_(prev), True)[1])
        i2, t2_, _ = solve(lambda p: (net.predict(div, p), True)[1])
        guess_nn = torch.empty_like(div)
        net.predict(div, guess_nn)
        rows.append({"zero": [i0.iterations, t0_], "previous": [i1.iterations, t1_], "network": [i2.iterations, t2_],
                     "err_previous": rel_err(prev, p0), "err_network": rel_err(guess_nn, p0)})
        return {"warm_start": sim.i > 0}

    sim.before_poisson = compare
    t0 = time.perf_counter()
    for _ in range(args.eval_steps):
        sim.step()
    torch.cuda.synchronize()
    net.check()
    agg = {k: [float(np.mean([r[k][0] for r in rows])), float(np.mean([r[k][1] for r in rows]))]
           for k in ("zero", "previous", "network")}
    emit(evaluation={"res": n, "source": held, "steps": len(rows), "seconds": time.perf_counter() - t0,
                     "mgpcg_iters_mean": {k: v[0] for k, v in agg.items()},
                     "solve_ms_mean": {k: v[1] for k, v in agg.items()},
                     "guess_rel_err_mean": {"previous": float(np.mean([r["err_previous"] for r in rows])),
                                            "network": float(np.mean([r["err_network"] for r in rows]))},
                     "iters_saved_vs_previous": agg["previous"][0] - agg["network"][0],
                     "iters_saved_vs_zero": agg["zero"][0] - agg["network"][0]})


if __name__ == "__main__":
    main()
