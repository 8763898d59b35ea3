"""Adapters behind the drop-in modules (``3D/`` and ``2D/`` beside this package) that keep the
reference's function names and argument lists (zjw49246/particle-flow-maps, 3D/run_3D.py,
2D/run_2D.py, */init_conditions.py, */mgpcg.py).

Field conventions of the drop-in: every Taichi field becomes a CUDA tensor in libpfm's layout.
A particle vector field (``ti.Vector.field(d, float, shape=P)``) is an SoA tensor ``[d, P]``; the
reference's per-row triples (``T_x, T_y, T_z``, ``init_C_x, ...``) are the rows ``T[0], T[1],
T[2]`` of one ``[d, d, P]`` tensor (``vector_rows``).  Grids keep the reference's shapes.  Rows
that are not views of one buffer still work: they are stacked into a scratch buffer and, for
outputs, copied back.
"""
import numpy as np
import torch

from ._lib import PfmError
from .core import Scene

_scenes = {}


def scene(dim, res, dx, particles, boundary=None, use_apic=True, base_level=3):
    """One cached libpfm Scene per (shape, particle count, boundary) the drop-in touches."""
    bkey = None if boundary is None else tuple(map(tuple, np.asarray(boundary).tolist()))
    key = (dim, tuple(int(r) for r in res), float(dx), int(particles), bkey, bool(use_apic), int(base_level))
    sc = _scenes.get(key)
    if sc is None:
        sc = Scene(dim, tuple(int(r) for r in res), dx, int(particles), base_level=base_level,
                   boundary=None if boundary is None else np.asarray(boundary), use_apic=use_apic)
        _scenes[key] = sc
    return sc


def vector_rows(d, P, device="cuda"):
    """A [d, d, P] buffer and its rows: the drop-in form of d per-particle vector fields."""
    buf = torch.zeros(d, d, P, device=device)
    return buf, tuple(buf[v] for v in range(d))


class Rows:
    """Context manager giving a contiguous [d, d, P] tensor for row views ``rows``; when the rows
    are not one buffer, a stacked copy is used and written back on exit if ``out`` is set."""

    def __init__(self, rows, out=False):
        self.rows, self.out = rows, out
        d = len(rows)
        r0 = rows[0]
        base = r0._base if r0._base is not None else None
        self.buf = None
        if (base is not None and base.dim() == 3 and tuple(base.shape[:2]) == (d, d) and base.is_contiguous()
                and all(r.data_ptr() == base[v].data_ptr() and r.shape == base[v].shape for v, r in enumerate(rows))):
            self.buf = base
        self.copy = self.buf is None

    def __enter__(self):
        if self.copy:
            for r in self.rows:
                if not isinstance(r, torch.Tensor) or not r.is_cuda:
                    raise PfmError(2, "particle fields must be CUDA tensors")
            self.buf = torch.stack([r.contiguous() for r in self.rows]).contiguous()
        return self.buf

    def __exit__(self, *exc):
        if self.copy and self.out and exc[0] is None:
            for v, r in enumerate(self.rows):
                r.copy_(self.buf[v])
        return False


def check_soa(t, d, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float32 or t.dim() != 2 or t.shape[0] != d:
        raise PfmError(2, f"{name} must be a float32 CUDA tensor [{d}, P] (libpfm's SoA layout)")
    if not t.is_contiguous():
        raise PfmError(2, f"{name} must be contiguous")


class Scalar:
    """Stand-in for a 0-d Taichi field read as ``field[None]``."""

    def __init__(self, value=0.0):
        self.value = value

    def __getitem__(self, idx):
        return self.value

    def __setitem__(self, idx, v):
        self.value = v


def lattice_device(res, dx, particles_per_cell_axis, device="cuda"):
    """init_particles_pos_uniform's lattice (x fastest, (index + 0.5) * dx / axis) as an SoA
    device tensor, built once per shape on the host and kept on the device; later calls copy it
    device to device."""
    from .sim import lattice2, lattice3, soa
    key = ("lattice", tuple(int(r) for r in res), float(dx), int(particles_per_cell_axis), str(device))
    t = _scenes.get(key)
    if t is None:
        a = int(particles_per_cell_axis)
        pts = lattice3(tuple(res), dx, a) if len(res) == 3 else lattice2(tuple(res), dx, a * a)
        t = soa(pts, device)
        _scenes[key] = t
    return t
