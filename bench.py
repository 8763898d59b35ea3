#!/usr/bin/env python3
"""Throughput of the particle-flow-map time step on GB300.

Workload: 3D two-ring leapfrog scene (rings on the x axis through (y, z) = (0.5, 0.5), radius
0.15, core 0.025 with the reference's 1-exp(-(r/d)^3) mollifier, circulation 1.0, centres x = 0.25
and 0.35), unit cube at res^3 (default 256^3), 8 jittered particles per cell (seed 0), reinit
every 20 steps, gradient reinit every step, RK4, CFL 0.5, MGPCG (the reference's V-cycle) to a
1e-6 relative residual.  One bench step = one full time step (run_3D.py:716-822 loop body).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  N > 1 (under torchrun) runs N independent replicas, one per GPU; value is
the whole-job steps/s (N*K / max-over-ranks time).  --impl reference times the CPU oracle (the
reference's kernels restated in C++/OpenMP) on the host cores.
"""
import argparse
import contextlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(REPO, "particle-flow-maps_gb300"), os.path.join(REPO, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "3D 256³ steps/s: mixed-prec+warm-start vs plain FP32 at equal residual; %HBM peak"
UNIT = "steps/s"
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 20 steps: one particle reinitialisation cycle (reinit every 20 steps), so the timed window
    # always holds one reseeding step and the solves that follow it
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--res", type=int, default=256)
    ap.add_argument("--ppc-axis", type=int, default=2)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--tol-mode", type=int, default=1, help="0: r.r < tol (reference); 1: relative norm")
    ap.add_argument("--cpu-res", type=int, default=64, help="grid of the bounded CPU sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--arms", default="both", choices=["both", "plain", "mixed"],
                    help="plain FP32 MGPCG and/or the mixed-precision warm-started MGPCG (the headline)")
    ap.add_argument("--precision", default="fp16", choices=["fp16", "bf16"],
                    help="multigrid level storage of the mixed arm")
    ap.add_argument("--replace", type=int, default=0, choices=[0, 1],
                    help="mixed arm: the FP64 true residual replaces the recursive one every 5 iterations and "
                         "before convergence is accepted (1) or is only reported (0)")
    ap.add_argument("--warm-start", type=int, default=3, choices=[1, 2, 3],
                    help="mixed arm's initial guess: the previous pressure (1), its linear (2) or quadratic (3) "
                         "extrapolation through the last pressures")
    ap.add_argument("--fp64-res", type=int, default=-1,
                    help="grid of the FP64-oracle check of each arm's projection (-1: the bench grid, 0: off)")
    ap.add_argument("--eager", action="store_true",
                    help="time the eager phase calls instead of the whole-step graph (kernels inside graph "
                         "conditional nodes are invisible to ncu launch lists)")
    return ap.parse_args()


def ring_params():
    """The two coaxial rings of the 3D workload (add_vortex_ring arguments)."""
    common = dict(w=1.0, rad=0.15, delta=0.025, unit_x=(0.0, 0.0, -1.0), unit_y=(0.0, 1.0, 0.0), num_samples=2000)
    return [dict(common, c=(0.25, 0.5, 0.5)), dict(common, c=(0.35, 0.5, 0.5))]


# ------------------------------------------------------------------------------------------------
# GPU scene set-up
# ------------------------------------------------------------------------------------------------
def make_sim(res, ppc_axis, poisson_opts, device="cuda", graph=True):
    import torch
    import pfm
    n = res
    dx = 1.0 / n
    P = n ** 3 * ppc_axis ** 3
    seeds = torch.empty(3, P, device=device)
    zeros = [torch.zeros(s, device=device) for s in ((n + 1, n, n), (n, n + 1, n), (n, n, n + 1))]
    sim = pfm.Sim3D(zeros, seeds, (n, n, n), dx, CFL=0.5, visualize_dt=0.1, reinit_every=20, reinit_every_grad_m=1,
                    poisson_opts=poisson_opts, device=device)  # set-up phases run eagerly
    sc = sim.scene
    sc.seed_jittered(sim.seeds, 0, ppc_axis)
    vc = torch.zeros((n, n, n, 3), device=device)
    for r in ring_params():
        sc.add_vortex_ring(vc, **r)
    sc.split_central_vector(vc, sim.u)
    del vc
    sc.poisson(sim.u, sim.p, **poisson_opts)  # split_central_vector + Poisson (run_3D.py:667-670); p starts at 0
    # the set-up projection's pressure answers a different problem: warm starts begin at the first step
    sim.p.zero_()
    sc.reset_warm_history()
    torch.cuda.synchronize()
    sim.set_graph(graph)  # the timed steps: one CUDA graph launch per step
    return sim


class PhaseTimer:
    """CUDA-event pairs around the step phases (on the launching stream)."""

    def __init__(self):
        self.records = {}

    @contextlib.contextmanager
    def __call__(self, name):
        import torch
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        yield
        b.record()
        self.records.setdefault(name, []).append((a, b))

    def summary(self):
        return {k: [a.elapsed_time(b) for a, b in v] for k, v in self.records.items()}


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def host_round_trip_steps(sim, host_u, steps, down, up):
    """``steps`` steps whose grid velocity makes a round trip through pinned host memory: each step's
    input is uploaded from ``host_u`` and its result read back into ``host_u``, so every step starts
    from the previous step's result as read back.  The read-back of a step and the upload of the
    next are issued per velocity component on two streams (device->host on ``down``, host->device on
    ``up``): the upload of a component waits only for that component's read-back, so the two copy
    directions run at once (one 67 MB face grid each way at 256^3: 0.41 ms together against 0.32 +
    0.35 ms one after the other).  The step itself runs on the current stream, after the last upload."""
    import torch
    cur = torch.cuda.current_stream()
    for d, h in zip(sim.u, host_u):
        d.copy_(h, non_blocking=True)
    for k in range(steps):
        sim.step()
        done = torch.cuda.Event()
        done.record(cur)
        down.wait_event(done)
        last = k + 1 == steps
        for d, h in zip(sim.u, host_u):
            with torch.cuda.stream(down):
                h.copy_(d, non_blocking=True)
            if not last:
                e = torch.cuda.Event()
                e.record(down)
                up.wait_event(e)
                with torch.cuda.stream(up):
                    d.copy_(h, non_blocking=True)
        if not last:
            e = torch.cuda.Event()
            e.record(up)
            cur.wait_event(e)
    e = torch.cuda.Event()
    e.record(down)
    cur.wait_event(e)


def measured_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return FALLBACK_HBM_GBS, "fallback"


def _div3(u):
    import numpy as np
    ux, uy, uz = (np.asarray(a, np.float64) for a in u)
    return (ux[1:] - ux[:-1]) + (uy[:, 1:] - uy[:, :-1]) + (uz[:, :, 1:] - uz[:, :, :-1])


def _rel(a, b):
    import numpy as np
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def fp64_check(sim, oracle_tol=1e-7):
    """Accuracy of one step's final projection against an FP64 oracle solve of the identical field
    (outside every timed region).  One more eager step of ``sim`` runs with the final Poisson
    solve's input velocity and output velocity/pressure copied to the host; the CPU oracle
    (MGPCG_3.Poisson restated in C++, FP64 instance) then solves the copied input to a 1e-7
    relative residual (below that the reference's eps = 1e-12 in alpha stalls the FP64 iteration:
    at 64^3 it reaches 1e-7 in 5 iterations and 1e-8 only after 50).  Returns the relative L2 errors of the GPU velocity and mean-free pressure
    against it, and the divergence the GPU velocity keeps relative to the input's."""
    import numpy as np
    import torch
    import oracle as O
    was_graph = sim.graph
    sim.set_graph(False)
    sc = sim.scene
    real = sc.poisson
    calls = []

    def poisson(u, p_out=None, **kw):
        calls.append(None)
        if len(calls) == 2:  # the step's second solve: the final projection
            u_in = [t.detach().cpu().numpy().copy() for t in u]
            info = real(u, p_out, **kw)
            calls[-1] = (u_in, [t.detach().cpu().numpy().copy() for t in u], p_out.detach().cpu().numpy().copy(),
                         info)
            return info
        return real(u, p_out, **kw)

    sc.poisson = poisson
    try:
        sim.step()
        torch.cuda.synchronize()
    finally:
        del sc.poisson
    sim.set_graph(was_graph)
    u_in, u_gpu, p_gpu, info = calls[1]
    t0 = time.perf_counter()
    ux, uy, uz, p64, it64, _ = O.poisson3(*u_in, fp64=True, tol=oracle_tol, tol_mode=1)
    t_or = time.perf_counter() - t0
    b = []
    for f, a in enumerate(u_in):  # apply_bc zeroes the wall faces before the divergence
        a = a.copy()
        idx = [slice(None)] * 3
        idx[f] = 0
        a[tuple(idx)] = 0
        idx[f] = -1
        a[tuple(idx)] = 0
        b.append(a)
    bdiv = _div3(b)
    pg = p_gpu.astype(np.float64)
    return {"res": int(u_in[1].shape[0]), "step": int(sim.i), "mgpcg_iters": info.iterations,
            "velocity_rel_l2": _rel(np.concatenate([a.ravel() for a in u_gpu]),
                                    np.concatenate([a.ravel() for a in (ux, uy, uz)])),
            "pressure_rel_l2": _rel(pg - pg.mean(), p64 - p64.mean()),
            "divergence_left_rel": float(np.linalg.norm(_div3(u_gpu)) / np.linalg.norm(bdiv - bdiv.mean())),
            "oracle": f"FP64 MGPCG_3.Poisson on the host cores to |r| < {oracle_tol:g} |r0| ({it64} iterations, "
                      f"{t_or:.1f} s)"}


# ------------------------------------------------------------------------------------------------
# CPU oracle sample (cpu_baseline and the reference arm)
# ------------------------------------------------------------------------------------------------
def cpu_ic(n):
    """The same two-ring velocity at n^3, built on the host (numpy Biot-Savart of add_vortex_ring)."""
    import numpy as np
    dx = 1.0 / n
    vc = np.zeros((n, n, n, 3), np.float64)
    g = (np.arange(n) + 0.5) * dx
    X = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1)
    for r in ring_params():
        c, ux, uy = map(np.array, (r["c"], r["unit_x"], r["unit_y"]))
        ns, rad, dl, w = r["num_samples"], r["rad"], r["delta"], r["w"]
        cl = 2 * np.pi * rad / ns
        for l in range(0, ns, 8):  # every 8th sample with 8x the weight keeps the host set-up short
            th = l / ns * 2 * np.pi
            ps = rad * (np.cos(th) * ux + np.sin(th) * uy) + c
            wv = w * (-np.sin(th) * ux + np.cos(th) * uy)
            d = X - ps
            rr = np.linalg.norm(d, axis=-1)
            f = 8 * cl * (-1 / (4 * np.pi * rr ** 3) * (1 - np.exp(-(rr / dl) ** 3)))
            vc += f[..., None] * np.cross(d, wv)
    out = []
    for fam in range(3):
        a = vc[..., fam]
        pad = [(0, 0)] * 3
        pad[fam] = (1, 1)
        e = np.pad(a, pad, mode="edge")
        sl_hi = [slice(None)] * 3
        sl_lo = [slice(None)] * 3
        sl_hi[fam] = slice(1, None)
        sl_lo[fam] = slice(0, -1)
        out.append((0.5 * (e[tuple(sl_hi)] + e[tuple(sl_lo)])).astype(np.float32))
    return out


def cpu_sample(n, ppc_axis, steps=1, tol=1e-6, tol_mode=1):
    """Seconds per oracle step at n^3 (all host threads)."""
    import numpy as np
    import oracle as O
    from pfm.sim import jittered
    dx = 1.0 / n
    u = cpu_ic(n)
    popts = dict(tol=tol, tol_mode=tol_mode)
    u = list(O.poisson3(*u, **popts)[:3])
    seeds = jittered((n, n, n), dx, ppc_axis ** 3, seed=0)
    sim = O.Sim3D(u, seeds, (n, n, n), dx, CFL=0.5, visualize_dt=0.1, reinit_every=20, reinit_every_grad_m=1,
                  p2g_threads=O.num_threads(), poisson_opts=popts)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        sim.step()
        times.append(time.perf_counter() - t0)
    return times, O.num_threads(), int(np.int64(seeds.shape[0]))


def cpu_baseline_entry(args, n_target):
    times, cores, P = cpu_sample(args.cpu_res, args.ppc_axis, tol=args.tol, tol_mode=args.tol_mode)
    scale = (n_target / args.cpu_res) ** 3
    t = statistics.median(times) * scale
    return {"value": 1.0 / t, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"one full oracle step at {args.cpu_res}^3 ({P} particles, same workload scaled), "
                      f"{statistics.median(times):.2f} s, x{scale:.0f} work scale to {n_target}^3"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n_target = args.res
    scale = (n_target / args.cpu_res) ** 3
    times, cores, P = cpu_sample(args.cpu_res, args.ppc_axis, steps=args.warmup + args.steps, tol=args.tol,
                                 tol_mode=args.tol_mode)
    timed = times[args.warmup:] if len(times) > args.warmup else times
    per = statistics.mean(timed) * scale
    value = 1.0 / per
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"3D {n_target}^3 two-ring leapfrog, {args.ppc_axis ** 3} ppc, plain FP32, "
                                   f"MGPCG rel tol {args.tol:g}", "res": n_target},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"each step: one full CPU-oracle step at {args.cpu_res}^3 ({P} particles), "
                                       f"x{scale:.0f} work scale to {n_target}^3"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def job_rate(local_seconds, steps, world, dist=None, device=None):
    """Whole-job steps/s of N independent replicas: every rank ran `steps` steps of its own scene,
    the job took the slowest rank's time (an all-reduce MAX; no data moves between replicas)."""
    elapsed = float(local_seconds)
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([elapsed], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    return world * steps / elapsed, elapsed


# ------------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------------
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def timed_arm(popts):
        """W warm-up steps, then K steps timed with CUDA events (max over ranks), launch counts and
        the SM clocks sampled during the timed region.  Every step is one whole-step CUDA graph
        launch (pfm3_step): no host synchronization between steps.  The phase breakdown comes from
        a few more steps of the same scene through the eager phase calls, bracketed by CUDA events."""
        sim = make_sim(args.res, args.ppc_axis, popts, graph=not args.eager)
        for _ in range(args.warmup):
            sim.step()
        sim.step_info()  # settles the launch count of the warm-up steps
        torch.cuda.synchronize()
        launches0 = sim.scene.launches
        clocks = ClockSampler(local)
        barrier()
        clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record()
        torch.cuda.nvtx.range_push("pfm_timed_steps")  # lets ncu --nvtx-include select the timed steps
        for _ in range(args.steps):
            sim.step()
        torch.cuda.nvtx.range_pop()
        e1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        clk = clocks.stop()
        barrier()
        value, elapsed = job_rate(e0.elapsed_time(e1) / 1e3, args.steps, world, dist, "cuda")
        if args.eager:
            mg_iters = [i.iterations for i in sim.infos[-2 * args.steps:]]
            launches = sim.scene.launches - launches0
        else:
            info = sim.step_info()
            launches = sim.scene.launches - launches0
            last = info.step
            mg_iters = []
            for st in range(max(last - args.steps + 1, last - 63), last + 1):
                mg_iters += [int(info.history[st % 64][0]), int(info.history[st % 64][1])]
        # phase breakdown: eager phase calls with CUDA events on the launching stream
        sim.set_graph(False)
        timer = PhaseTimer()
        sim.timer = timer
        for _ in range(min(3, args.steps)):
            sim.step()
        torch.cuda.synchronize()
        sim.timer = None
        eager_ms = sum(statistics.mean(v) for v in timer.summary().values())
        sim.set_graph(not args.eager)
        check = None
        if rank == 0 and args.fp64_res != 0:
            if args.fp64_res in (-1, args.res):
                check = fp64_check(sim)
            else:  # a smaller scene of the same workload, a few steps in
                small = make_sim(args.fp64_res, args.ppc_axis, popts, graph=True)
                for _ in range(3):
                    small.step()
                check = fp64_check(small)
                del small
                torch.cuda.empty_cache()
        return dict(sim=sim, value=value, elapsed=elapsed, wall=wall, clocks=clk, launches=launches,
                    phases=timer.summary(), mg_iters=mg_iters, eager_ms=eager_ms, fp64_check=check)

    # the two arms of the metric, at the same residual: MGPCG stops at |r| < tol |b| in both
    plain_opts = dict(tol=args.tol, tol_mode=args.tol_mode, max_iters=400, check_every=4)
    mixed_opts = dict(tol=args.tol, tol_mode=2, max_iters=400, check_every=4, precision=args.precision,
                      warm_start=args.warm_start, true_residual_every=5, true_residual_replace=bool(args.replace))
    plain = None
    if args.arms in ("both", "plain"):
        plain = timed_arm(plain_opts)
        if args.arms == "both":
            del plain["sim"]
            torch.cuda.empty_cache()
    head = timed_arm(mixed_opts) if args.arms in ("both", "mixed") else plain
    sim = head["sim"]
    value, elapsed, wall, clk, launches = head["value"], head["elapsed"], head["wall"], head["clocks"], head["launches"]
    phases, mg_iters = head["phases"], head["mg_iters"]

    # roofline of the dominant single-kernel phase: RK4_T_forward (one launch per step)
    P = sim.P
    n = args.res
    F3 = 3 * (n + 1) * n * n
    peak, peak_kind = measured_peak()
    rk4_ms = statistics.mean(phases["rk4"])
    # k_rk4_T_forward3 with the gradient reinitialisation and the P2G records, per particle: pos read
    # and written (24 B), T_gm read and written (72 B), T_init read and written (72 B), init_C
    # written (36 B), init_imp read (12 B), record (64 B) + key + slot (8 B) written = 288 B; the
    # pre-midpoint and midpoint velocity grids once each
    rk4_bytes = P * 288 + 2 * F3 * 4
    achieved = rk4_bytes / (rk4_ms / 1e3) / 1e9
    # DRAM bytes of one launch: dram__bytes_read.sum + dram__bytes_write.sum of an ncu capture of
    # k_rk4_T_forward3<true, true> at 128^3 (1,671,280,384 + 3,168,529,152 B for 16,777,216
    # particles), scaled by the particle count (the grid scales with it at a fixed particle density)
    traffic = (1671280384 + 3168529152) / 16777216 * P
    roofline = {"bound": "hbm", "kernel": "k_rk4_T_forward3", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                "traffic_source": "ncu capture at 128^3 scaled by the particle count",
                "bytes_per_launch": rk4_bytes, "ms_per_launch": rk4_ms}
    # The same launch against the FP32 roofline: executed FP32 flops of an ncu count of
    # k_rk4_T_forward3<true, true> at 128^3 for 16,777,216 particles -- FADD 2,511,667,223, FMUL
    # 5,469,372,416, FFMA 11,005,853,696 (2 flops), packed FMUL2 1,509,949,440 (2 flops) and FFMA2
    # 6,241,124,352 (4 flops): 3,455.7 per particle -- scaled by the particle count, over the
    # FMA-throughput probe of this GPU (the better of scalar and packed FMAs; outside every timed region)
    import pfm
    rk4_flops = (2511667223 + 5469372416 + 2 * 11005853696 + 2 * 1509949440 + 4 * 6241124352) / 16777216 * P
    fp32_peak = pfm.measure_fp32_peak()
    fp32_achieved = rk4_flops / (rk4_ms / 1e3) / 1e12
    roofline_fp32 = {"bound": "fp32", "kernel": "k_rk4_T_forward3", "achieved": fp32_achieved, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": fp32_achieved / fp32_peak,
                     "peak_kind": "measured (pfm_measure_fp32_peak: 8-chain FMA loop, best of scalar and packed f32x2)",
                     "flops_per_launch": rk4_flops,
                     "flops_source": "executed FP32 flops of an ncu count at 128^3 scaled by the particle count"}

    e2e = None
    if not args.no_e2e:
        # through the same C-ABI calls, with the step's grid velocity uploaded from pinned host memory
        # and the projected result read back into the same host buffers every step: the velocity makes
        # a round trip through the host, so each step starts from the previous step's result (events
        # order each component's read-back before its next upload) and the solves do the same work as
        # in the device-timed steps
        host_u = [t.cpu().pin_memory() for t in sim.u]
        down, up = torch.cuda.Stream(), torch.cuda.Stream()
        barrier()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        host_round_trip_steps(sim, host_u, args.steps, down, up)
        b.record()
        torch.cuda.synchronize()
        e_rate, _ = job_rate(a.elapsed_time(b) / 1e3, args.steps, world, dist, "cuda")
        gbytes = sum(h.numel() * 4 for h in host_u)
        if args.eager:
            e_iters = [i.iterations for i in sim.infos[-2 * args.steps:]]
        else:
            hist = sim.step_info()
            last = hist.step
            e_iters = []
            for st in range(max(last - args.steps + 1, last - 63), last + 1):
                e_iters += [int(hist.history[st % 64][0]), int(hist.history[st % 64][1])]
        e2e = {"value": e_rate, "unit": UNIT, "h2d_bytes_per_step": gbytes,
               "d2h_bytes_per_step": gbytes, "mgpcg_iters": e_iters}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline_entry(args, n)

    if rank == 0:
        mixed = args.arms != "plain"
        arm = (f"mixed-precision MGPCG ({args.precision} multigrid levels, FP64 inner products, FP64 true residual "
               f"every 5 iterations {'replacing the recursive one' if args.replace else 'reported'}) warm-started "
               + {1: "from the previous step's pressure", 2: "from the linear extrapolation of the last two steps' pressures",
                  3: "from the quadratic extrapolation of the last three steps' pressures"}[args.warm_start] if mixed else
               "plain FP32 MGPCG from a zero initial guess")
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "step_form": ("eager phase calls (pfm3_* entry points)" if args.eager else
                              "one whole-step CUDA graph launch per step (pfm3_step)"),
                "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "wall_s": wall,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded two-ring initial condition and jittered particles)",
                "config": {"workload": f"3D {n}^3 two-ring leapfrog, {args.ppc_axis ** 3} ppc ({P} particles), "
                                       f"FP32 particle/grid step; {arm}; MGPCG to |r| < {args.tol:g} |b|",
                           "res": n, "particles": P, "parallelism": f"replicas x{world}",
                           "l2": "inputs larger than L2 (particle state %.1f GB)" % (P * 132 / 1e9)},
                "particle_updates_per_s": value * P,
                "mgpcg_iters": mg_iters,
                "phase_ms": {k: statistics.mean(v) for k, v in phases.items()},
                "phase_note": "phase_ms: CUDA events around the eager phase calls of 3 further steps "
                              "(sum %.2f ms/step)" % head["eager_ms"],
                "roofline": roofline, "roofline_fp32": roofline_fp32, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
                "gpu_launches": launches, "fp64_check": head["fp64_check"]}
        if plain is not None and mixed:
            line["plain_fp32"] = {"value": plain["value"], "ms_per_step": plain["elapsed"] / args.steps * 1e3,
                                  "mgpcg_iters": plain["mg_iters"],
                                  "phase_ms": {k: statistics.mean(v) for k, v in plain["phases"].items()},
                                  "clocks": plain["clocks"], "fp64_check": plain["fp64_check"]}
            line["speedup_vs_plain_fp32"] = value / plain["value"]
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
