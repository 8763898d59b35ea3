"""Drop-in for the reference's 3D/mgpcg.py: MGPCG and MGPCG_3 with the same constructor, methods
and keywords (3D/mgpcg.py:8-280, 350-430), backed by libpfm's sm_103a MGPCG (device-side PCG
loop, deterministic reductions).  Fields are CUDA tensors: cell fields [nx, ny, nz], face grids
[nx+1, ny, nz] / [nx, ny+1, nz] / [nx, ny, nz+1]."""
import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from pfm import dropin as _d  # noqa: E402


class MGPCG:
    """Matrix-free multigrid-preconditioned CG for lap(x) = k r on an N grid (3D/mgpcg.py:8-280).
    ``boundary_types``: [dim][2], 1 = Dirichlet, 2 = Neumann."""

    def __init__(self, boundary_types, N, dim=2, base_level=3, real=float):
        self.boundary_types = np.asarray(boundary_types, dtype=np.int32).reshape(dim, 2)
        self.N = tuple(int(n) for n in N)
        self.dim = dim
        self.base_level = base_level
        self.n_mg_levels = int(np.log2(min(self.N))) - base_level + 1
        self.pre_and_post_smoothing = 2
        self.bottom_smoothing = 50
        self.real = real
        self.scene = _d.scene(dim, self.N, 1.0 / self.N[1], 0, boundary=self.boundary_types, base_level=base_level)
        self.x = torch.zeros(self.N, device=self.scene.device)
        self._rhs = None
        self.last_info = None

    def init(self, r, k):
        """Set up the solve for lap(x) = k r (3D/mgpcg.py:71-79)."""
        self._rhs = (r, float(k))

    def solve(self, max_iters=-1, eps=1e-12, tol=1e-12, verbose=False):
        """PCG with the V-cycle preconditioner until r.r < tol (3D/mgpcg.py:202-280)."""
        if self._rhs is None:
            raise RuntimeError("MGPCG.solve before MGPCG.init")
        r, k = self._rhs
        info = self.scene.mgpcg_solve(r, self.x, k=k, max_iters=max_iters, tol=tol, tol_mode=0)
        self.last_info = info
        if verbose:
            print(f"iter {info.iterations}, |residual|_2={np.sqrt(max(info.rTr, 0.0))}")
        if not info.converged:
            print("[MGPCG] Return without converging at iter: ", info.iterations)
        return info

    def get_result(self, x):
        """Copy the solution into x (3D/mgpcg.py:82-90)."""
        x.copy_(self.x)


class MGPCG_3(MGPCG):
    """3D MAC-grid pressure projection (3D/mgpcg.py:350-430).  ``self.p`` holds the pressure of the
    last Poisson solve (the reference's solver.p)."""

    def __init__(self, boundary_types, N, base_level=3, real=float):
        super().__init__(boundary_types, N, dim=3, base_level=base_level, real=real)
        dev = self.scene.device
        self.u_div = torch.zeros(self.N, device=dev)
        self.p = torch.zeros(self.N, device=dev)

    def apply_bc(self, u_x, u_y, u_z):
        self.scene.apply_bc([u_x, u_y, u_z])

    def divergence(self, u_x, u_y, u_z):
        self.scene.divergence([u_x, u_y, u_z], self.u_div)

    def subtract_grad_p(self, u_x, u_y, u_z):
        self.scene.subtract_grad_p([u_x, u_y, u_z], self.p)

    def solve_pressure_MGPCG(self, verbose):
        self.init(self.u_div, -1)
        self.solve(max_iters=400, verbose=verbose, tol=1.e-12)
        self.get_result(self.p)

    def Poisson(self, u_x, u_y, u_z, verbose=False):
        """apply_bc, divergence, solve, subtract_grad_p, apply_bc (3D/mgpcg.py:425-430) as one
        library call (the same result as the five pieces)."""
        info = self.scene.poisson([u_x, u_y, u_z], self.p, max_iters=400, tol=1.e-12, tol_mode=0)
        self.last_info = info
        if verbose:
            print(f"iter {info.iterations}, |residual|_2={np.sqrt(max(info.rTr, 0.0))}")
        return info
