"""3D Boussinesq smoke plume on the particle-flow-map step, the workload of the learned warm start.

A sphere of radius 0.05 at (0.5, 0.1, 0.5) of the unit cube sets the smoke density to 1 every
step; the density is carried semi-Lagrangian by the step's midpoint velocity; the buoyancy
force ``buoyancy * density`` along y (axis 1) enters through the particles' impulse at the start
of each step (``pfm3_add_buoyancy_impulse``: the impulse handed to P2G grows by f dt, and the
flow map transports it afterwards).  The rest of the step is the reference's 3D step unchanged
(``pfm.Sim3D``: CFL 0.5, reinitialisation every 20 steps, gradient reinitialisation every step),
starting from rest with 8 jittered particles per cell (seed 0).

``pressure_guess`` chooses the initial guess of the final projection each step: ``"previous"``
(the previous step's pressure, the method without the network), ``"zero"``, or a callable
``guess(div, p_out)`` that writes an initial pressure for the divergence ``div`` (the network).
The final solve always runs to the same residual (``|r| < tol |b|``); the midpoint solve keeps the
reference's absolute rule.
"""
import ctypes

import torch

from ._lib import PfmError
from .sim import Sim3D


class Plume3D(Sim3D):
    def __init__(self, res=(192, 192, 192), source=(0.5, 0.1, 0.5), radius=0.05, density=1.0, buoyancy=1.0, ppc=8,
                 seed=0, CFL=0.5, reinit_every=20, tol=1e-6, precision=0, pressure_guess="previous", device="cuda",
                 **kw):
        res = tuple(int(r) for r in res)
        dx = 1.0 / res[1]
        axis = round(ppc ** (1.0 / 3.0))
        if axis ** 3 != ppc:
            raise PfmError(7, "particles per cell must be a cube")
        P = res[0] * res[1] * res[2] * ppc
        seeds = torch.empty(3, P, device=device)  # filled by the device seeding kernel below
        u = [torch.zeros(s, device=device) for s in ((res[0] + 1, res[1], res[2]), (res[0], res[1] + 1, res[2]),
                                                      (res[0], res[1], res[2] + 1))]
        opts = dict(tol=tol, tol_mode=2, max_iters=400, precision=precision)
        super().__init__(u, seeds, res, dx, CFL=CFL, reinit_every=reinit_every, poisson_opts=opts, device=device,
                         graph=False, **kw)
        self.scene.seed_jittered(self.seeds, seed, axis)
        # the midpoint solve keeps the reference's absolute rule r.r < 1e-12 (mgpcg.py:420-423): its
        # right-hand side (the divergence advection leaves in an already projected field) is so small
        # that 1e-6 relative sits below the FP32 floor of the recursive residual
        self.poisson_mid_opts = dict(tol=1e-12, tol_mode=0, max_iters=400, precision=precision)
        self.source, self.radius, self.density, self.buoyancy = tuple(source), float(radius), float(density), float(buoyancy)
        self.rho = torch.zeros(res, device=device)
        self.rho_tmp = torch.zeros_like(self.rho)
        self.div = torch.zeros(res, device=device)
        self.pressure_guess = pressure_guess
        self.record = None  # a list: each step appends (div, p) copies of the final projection
        self.before_rk4 = self._force
        self.before_poisson = self._guess
        self.after_step = self._transport
        lib = self.scene.lib
        self._lib = lib
        self._inject()

    def _st(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.scene.device).cuda_stream)

    def _inject(self):
        cx, cy, cz = self.source
        self.scene._check(self._lib.pfm3_plume_source(self.scene.h, ctypes.c_void_p(self.rho.data_ptr()), cx, cy, cz,
                                                      self.radius, self.density, self._st()))

    def _force(self, dt):
        sc = self.scene
        sc._check(self._lib.pfm3_add_buoyancy_impulse(
            sc.h, ctypes.c_void_p(self.pos.data_ptr()), ctypes.c_void_p(self.T_gm.data_ptr()),
            ctypes.c_void_p(self.T_init.data_ptr()), ctypes.c_void_p(self.init_imp.data_ptr()),
            ctypes.c_void_p(self.rho.data_ptr()), float(dt) * self.buoyancy, 1, self._st()))

    def divergence(self, out=None):
        """The divergence the final projection solves for (walls applied first, as Poisson does)."""
        out = self.div if out is None else out
        self.scene.apply_bc(self.u)
        self.scene.divergence(self.u, out)
        return out

    def _guess(self):
        g = self.pressure_guess
        if self.record is not None or callable(g):
            self.divergence()
        if g == "previous":
            return {"warm_start": self.i > 0}
        if g == "zero":
            return {"warm_start": False}
        g(self.div, self.p)
        return {"warm_start": True}

    def _transport(self, dt):
        if self.record is not None:
            self.record.append((self.div.clone(), self.p.clone()))
        sc = self.scene
        sc._check(self._lib.pfm3_advect_density(
            sc.h, ctypes.c_void_p(self.rho.data_ptr()), ctypes.c_void_p(self.rho_tmp.data_ptr()),
            ctypes.c_void_p(self.u_mid[0].data_ptr()), ctypes.c_void_p(self.u_mid[1].data_ptr()),
            ctypes.c_void_p(self.u_mid[2].data_ptr()), float(dt), self._st()))
        self.rho, self.rho_tmp = self.rho_tmp, self.rho
        self._inject()
