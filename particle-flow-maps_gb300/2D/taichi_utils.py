"""Drop-in for the field kernels of the reference's 2D/taichi_utils.py (2D/taichi_utils.py:8-104):
the same names and arguments on CUDA tensors, with the grid stencils running libpfm's sm_103a
kernels.  Vector grids keep the reference's shapes ([nx, ny, n])."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import pfm as _pfm  # noqa: E402
from pfm import dropin as _d  # noqa: E402


def _cells(t):
    res = tuple(int(n) for n in t.shape[:2])
    return _d.scene(2, res, 1.0 / res[1], 0)


def copy_to(source, dest):
    dest.copy_(source)


def add_fields(f1, f2, dest, multiplier):
    """dest = f1 + multiplier * f2 (2D/taichi_utils.py:13-16), by libpfm's elementwise kernel."""
    _pfm.add_fields(f1, f2, dest, multiplier)


def scale_field(a, alpha, result):
    """result = alpha * a (2D/taichi_utils.py:8-11), by libpfm's elementwise kernel."""
    _pfm.scale_field(a, alpha, result)


def get_central_vector(horizontal, vertical, central):
    """central = face averages per cell (2D/taichi_utils.py:50-55)."""
    _cells(central).get_central_vector([horizontal, vertical], central)


def split_central_vector(central, horizontal, vertical):
    """faces = averages of the adjacent cell values (2D/taichi_utils.py:56-67)."""
    _cells(central).split_central_vector(central, [horizontal, vertical])


def curl(vf, cf, dx):
    """cf = (vr.y - vl.y - vt.x + vb.x) / (2 dx) (2D/taichi_utils.py:96-104)."""
    _cells(vf).curl(vf, cf, dx=float(dx))
