"""Autotuner of a scene's launch shapes (pfm_set_tuning): times the candidates on the scene's own
data with CUDA events and keeps the fastest.  Every candidate gives bitwise the same results (the
tunables only change how the sums map to threads and launches), so tuning never changes a
simulation; it is done once per scene size, before the step or batch graphs are built.

  * ``mg_tail_cells``: the MGPCG levels with at most this many cells run the rest of the V-cycle
    in one thread block (fewer launches, one SM) instead of grid-wide kernels; timed on a solve of
    the scene's current divergence (into a scratch pressure);
  * ``p2g2_column`` (2D): faces per thread of the P2G column gather; timed on the scene's P2G into
    its scratch grids;
  * ``smooth_tma`` (3D, 16-bit MGPCG levels): smoothing from tiles the TMA stages in shared memory
    (1) or from global memory (0); timed on the same solve.
"""
import statistics

import torch

from . import _lib

__all__ = ["autotune", "apply"]

TAILS = (0, 256, 1024, 4096, 16384)
COLUMNS = (2, 4, 8, 16, 32)


def _time(fn, reps):
    fn()  # warm-up (and graph capture where the call builds one)
    times = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    return statistics.median(times)


def autotune(sim, reps=3, tails=TAILS, columns=COLUMNS):
    """Tunes ``sim.scene`` (a Sim2D / Sim3D) in place; returns {key: (chosen value, {value: ms})}."""
    sc = sim.scene
    out = {}
    r = torch.empty(sc.cell_shape, device=sc.device)
    sc.divergence(sim.u, r)
    x = torch.zeros_like(r)
    opts = {k: v for k, v in sim.poisson_opts.items() if k not in ("warm_start", "raise_on_limit")}
    times = {}
    for t in tails:
        try:
            sc.set_tuning(_lib.TUNE_MG_TAIL_CELLS, t)
        except _lib.PfmError:  # the tail levels would not fit in shared memory
            continue
        times[t] = _time(lambda: sc.mgpcg_solve(r, x, **opts), reps)
    best = min(times, key=times.get)
    sc.set_tuning(_lib.TUNE_MG_TAIL_CELLS, best)
    out["mg_tail_cells"] = (best, times)
    if sc.dim == 3 and opts.get("precision", 0) in (1, 2):
        times = {}
        for v in (0, 1):
            sc.set_tuning(_lib.TUNE_SMOOTH_TMA, v)
            times[v] = _time(lambda: sc.mgpcg_solve(r, x, **opts), reps)
        best = min(times, key=times.get)
        sc.set_tuning(_lib.TUNE_SMOOTH_TMA, best)
        out["smooth_tma"] = (best, times)
    if sc.dim == 2:
        times = {}
        for k in columns:
            sc.set_tuning(_lib.TUNE_P2G2_COLUMN, k)
            times[k] = _time(lambda: sc.p2g2(sim.imp, sim.pos, sim.C, sim.psi, sim.u_mid, sim.w,
                                              psi_out=sim.psi_grid), reps)
        best = min(times, key=times.get)
        sc.set_tuning(_lib.TUNE_P2G2_COLUMN, best)
        out["p2g2_column"] = (best, times)
    return out


def apply(sim, tuned):
    """Sets the values an autotune() of a scene of the same size chose."""
    keys = {"mg_tail_cells": _lib.TUNE_MG_TAIL_CELLS, "p2g2_column": _lib.TUNE_P2G2_COLUMN,
            "smooth_tma": _lib.TUNE_SMOOTH_TMA}
    for name, (value, _) in tuned.items():
        sim.scene.set_tuning(keys[name], value)
