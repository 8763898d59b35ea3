"""Drop-in for the field kernels of the reference's 3D/taichi_utils.py (3D/taichi_utils.py:8-100):
the same names and arguments on CUDA tensors, with the grid stencils running libpfm's sm_103a
kernels.  Vector grids keep the reference's shapes ([nx, ny, nz, n]); the @ti.func interpolation
helpers have no Python-level counterpart here (they live inside the kernels)."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import pfm as _pfm  # noqa: E402
from pfm import dropin as _d  # noqa: E402


def _cells(t):
    res = tuple(int(n) for n in t.shape[:3])
    return _d.scene(3, res, 1.0 / res[1], 0)


def copy_to(source, dest):
    dest.copy_(source)


def add_fields(f1, f2, dest, multiplier):
    """dest = f1 + multiplier * f2 (3D/taichi_utils.py:18-21), by libpfm's elementwise kernel."""
    _pfm.add_fields(f1, f2, dest, multiplier)


def scale_field(a, alpha, result):
    """result = alpha * a (3D/taichi_utils.py:13-16), by libpfm's elementwise kernel."""
    _pfm.scale_field(a, alpha, result)


def get_central_vector(vx, vy, vz, vc):
    """vc = face averages per cell (3D/taichi_utils.py:80-85)."""
    _cells(vc).get_central_vector([vx, vy, vz], vc)


def split_central_vector(vc, vx, vy, vz):
    """faces = averages of the adjacent cell values (3D/taichi_utils.py:87-100)."""
    _cells(vc).split_central_vector(vc, [vx, vy, vz])


def curl(vf, cf, dx):
    """cf = curl of the cell-centred vf by central differences (3D/taichi_utils.py:56-78)."""
    _cells(vf).curl(vf, cf, dx=float(dx))
