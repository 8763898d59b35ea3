"""Throughput of the kernels beside the live step (smoke transport, vorticity diagnostics, the
"evolve m" dataflow) at the bench's scale, against the HBM roofline.

    python tests/fields_study.py [--res 256] [--reps 5]

Each kernel runs on a 256^3 scene (8 particles per cell, 134,217,728 particles; the two-ring
velocity of bench.py) through the C ABI, timed with CUDA events on the launching stream (median of
--reps after a warm-up call).  One JSON line per kernel: ms, the algorithmic bytes per launch (the
compulsory reads and writes of the reference's dataflow, formula beside each call), achieved GB/s and
the fraction of the measured HBM copy bandwidth (MEASURED_PEAKS.json).  Not a pytest module."""
import argparse
import json
import os
import statistics
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "particle-flow-maps_gb300"))
sys.path.insert(0, ROOT)


def peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--res", type=int, default=256)
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()
    import torch
    import pfm
    import bench
    torch.cuda.set_device(0)
    n = args.res
    dx = 1.0 / n
    C = n ** 3
    F = 3 * (n + 1) * n * n
    P = C * 8
    sc = pfm.Scene(3, (n, n, n), dx, P)
    dev = sc.device
    u = sc.alloc_faces()
    vc = torch.zeros((n, n, n, 3), device=dev)
    for r in bench.ring_params():
        sc.add_vortex_ring(vc, **r)
    sc.split_central_vector(vc, u)
    pos = torch.empty(3, P, device=dev)
    sc.seed_jittered(pos, 0, 2)
    smoke = torch.zeros((n, n, n, 4), device=dev)
    for k, r in enumerate(bench.ring_params()):
        sc.add_vortex_ring_and_smoke(vc, smoke if k == 0 else torch.zeros_like(smoke), color=(1.0, 0.5, 0.25), **r)
    eye = torch.eye(3, device=dev)[:, :, None].expand(3, 3, P).contiguous()
    s_p = torch.empty(4, P, device=dev)
    G = torch.empty(3, 4, P, device=dev)
    psi = [torch.empty(s + (3,), device=dev) for s in sc.face_shapes]
    sc.midpoint(u, sc.alloc_faces(), 0.2 * dx, psi_out=psi)
    pk, kind = peak()
    gb = 1e9

    def run(name, fn, nbytes, note):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        ms = statistics.median(ts)
        ach = nbytes / (ms / 1e3) / gb
        print(json.dumps({"kernel": name, "res": n, "particles": P, "ms": ms, "algorithmic_bytes": nbytes,
                          "achieved_gbs": ach, "peak_gbs": pk, "frac": ach / pk, "peak_kind": kind, "bytes": note}),
              flush=True)

    s2 = torch.zeros_like(smoke)
    run("init_particles_smoke (k_g2p_smoke3)", lambda: sc.init_particles_smoke(pos, smoke, s_p, G),
        P * (12 + 16 + 48) + C * 16, "pos r 12 + smoke w 16 + grad w 48 per particle, smoke grid once")
    w = torch.zeros((n, n, n), device=dev)
    run("P2G_smoke (record pass, sort, k_tile_smoke3, normalise)",
        lambda: sc.p2g_smoke(s_p, G, pos, eye, eye, s2, w),
        P * (16 + 48 + 12 + 36 + 36 + 80 + 8 + 80) + C * (16 + 4) * 2,
        "record pass: smoke 16 + grad 48 + pos 12 + T_gm 36 + T_init 36 read, 5 float4 records + key/slot "
        "written; tiles read the 80 B records; smoke + weight grids written and normalised")
    run("advect_smoke (k_smoke_semilag3)", lambda: sc.advect_smoke(smoke, s2, psi),
        F * 12 + C * (16 + 16), "psi faces 12 B each, smoke0 read and smoke1 written per cell")
    run("clamp_smoke (k_smoke_semilag3)", lambda: sc.clamp_smoke(smoke, s2, psi),
        F * 12 + C * (16 + 32), "psi faces, smoke0 read, smoke1 read and written per cell")
    v = torch.empty((n, n, n, 3), device=dev)
    run("get_central_vector (k_central3)", lambda: sc.get_central_vector(u, v), F * 4 + C * 12,
        "faces read, cell vectors written")
    wv = torch.empty_like(v)
    run("curl (k_curl3)", lambda: sc.curl(v, wv), C * 24, "cell vectors read and written")
    T2 = eye.clone()
    T3 = eye.clone()
    pos2 = pos.clone()
    run("RK4_T_and_T_grad_m_forward (k_rk4_T2_forward3)", lambda: sc.rk4_T_and_T_grad_m_forward(pos2, T2, T3, u,
                                                                                              0.2 * dx),
        P * (24 + 72 + 72) + F * 4, "pos, T, T_grad_m read and written, the grid once")
    imp = torch.empty(3, P, device=dev)
    run("update_particles_imp (k_update_imp3)", lambda: sc.update_imp3(imp, pos, eye), P * (12 + 36 + 12),
        "init_imp and T read, imp written")
    Cg = torch.empty(3, 3, P, device=dev)
    del G, s_p, T2, T3, pos2
    torch.cuda.empty_cache()
    gT = torch.zeros(3, 3, 3, P, device=dev)
    run("update_particles_grad_m (k_update_grad_m3)", lambda: sc.update_grad_m3(Cg, eye, eye, gT, pos),
        P * (36 + 36 + 108 + 12 + 36), "init_C, T, grad_T_init, init_imp read, C written")
    run("compute_dT_dx, cap 12 (sort + k_compute_dT_dx3)", lambda: sc.compute_dT_dx(pos, pos, eye, 12, gT),
        P * (12 + 12 + 36 + 108 + 12), "pos (sort), init_pos, T read, grad_T_init written, keys/order; the "
                                       "neighbour reads are cache hits")


if __name__ == "__main__":
    main()
