"""Host side of the GB300 particle-flow-map step: one :class:`Scene` per simulated domain.

A Scene owns a libpfm handle and its device workspace (a torch uint8 buffer); torch tensors are
used only as device buffers.  Each method launches the sm_103a kernels of one reference phase on
the current torch CUDA stream.  Particle fields are SoA tensors ``[n, P]`` (``[d, d, P]`` for the
per-particle vector triples T_x/T_y/T_z and init_C_x/..); grids have the reference's shapes.
"""
import ctypes

import torch

from . import _lib
from ._lib import PfmError, SolveOpts, SolveStats

__all__ = ["Scene", "PfmError", "SolveInfo", "sort_particles_noalloc", "add_fields", "scale_field"]


class SolveInfo:
    """Result of one MGPCG solve (what the reference prints: iteration and final residual)."""

    def __init__(self, stats, status):
        self.iterations = int(stats.iterations)
        self.converged = bool(stats.converged)
        self.rTr = float(stats.rTr)
        self.rTr0 = float(stats.rTr0)
        self.bTb = float(stats.bTb)
        self.rTr_true = float(stats.rTr_true)
        self.status = status

    def __repr__(self):
        return (f"SolveInfo(iterations={self.iterations}, converged={self.converged}, "
                f"rTr={self.rTr:.3e})")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class Scene:
    """One scene: grid resolution, cell size, particle count and MGPCG configuration.

    Mirrors the module-level state the reference's kernels read (``dx``, ``res_x/y/z`` from
    hyperparameters.py, ``MGPCG_3(boundary_types, N, base_level)`` in 3D/run_3D.py:28-29).
    """

    def __init__(self, dim, res, dx, particles, base_level=3, mg_levels=0, boundary=None,
                 use_apic=True, pre_post_smoothing=2, bottom_smoothing=50, device=None):
        if not torch.cuda.is_available():
            raise PfmError(6, "CUDA is not available: the particle-flow-map step runs only on the GPU")
        self.lib = _lib.load()
        self.dim = int(dim)
        res = tuple(int(r) for r in res)
        self.res = res[:self.dim]
        self.dx = float(dx)
        self.P = int(particles)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        cfg = _lib.Config()
        cfg.dim = self.dim
        for a in range(3):
            cfg.res[a] = res[a] if a < len(res) else 1
        cfg.dx = self.dx
        cfg.particles = self.P
        cfg.base_level = int(base_level)
        cfg.mg_levels = int(mg_levels)
        cfg.pre_post_smoothing = int(pre_post_smoothing)
        cfg.bottom_smoothing = int(bottom_smoothing)
        bt = boundary if boundary is not None else [[2, 2]] * 3
        for a in range(3):
            row = bt[a] if a < len(bt) else (2, 2)
            cfg.boundary[a][0], cfg.boundary[a][1] = int(row[0]), int(row[1])
        cfg.use_apic = int(bool(use_apic))
        self.cfg = cfg
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            st = self.lib.pfm_create(ctypes.byref(cfg), ctypes.byref(h))
            if st != 0:
                raise PfmError(st, "pfm_create failed (check res, dx, particle count, MG levels)")
            self.h = h
            size = ctypes.c_size_t()
            self._check(self.lib.pfm_workspace_size(h, ctypes.byref(size)))
            self.workspace = torch.empty(max(int(size.value), 256), dtype=torch.uint8, device=self.device)
            self._check(self.lib.pfm_set_workspace(h, _ptr(self.workspace), ctypes.c_size_t(self.workspace.numel())))
            self.max_dev = torch.zeros(1, dtype=torch.float32, device=self.device)
        lv = ctypes.c_int()
        self._check(self.lib.pfm_mg_levels(h, ctypes.byref(lv)))
        self.mg_levels = lv.value

    # ------------------------------------------------------------------------------------------
    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and getattr(self, "lib", None) is not None:
            self.lib.pfm_destroy(h)
            self.h = None

    def _check(self, status, allow=()):
        if status != 0 and status not in allow:
            msg = self.lib.pfm_last_error(self.h) if getattr(self, "h", None) else b""
            raise PfmError(status, (msg or b"").decode())
        return status

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    @property
    def face_shapes(self):
        if self.dim == 3:
            nx, ny, nz = self.res
            return [(nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1)]
        nx, ny = self.res
        return [(nx + 1, ny), (nx, ny + 1)]

    @property
    def cell_shape(self):
        return tuple(self.res)

    def _grid(self, t, fam, name):
        self._dev(t, name)
        if tuple(t.shape) != self.face_shapes[fam]:
            raise PfmError(2, f"{name}: shape {tuple(t.shape)} != {self.face_shapes[fam]}")
        return t

    def _dev(self, t, name, dtype=torch.float32):
        if not isinstance(t, torch.Tensor):
            raise PfmError(1, f"{name} must be a torch tensor")
        if t.device.type != "cuda":
            raise PfmError(7, f"{name} must be a CUDA tensor")
        if t.dtype != dtype:
            raise PfmError(7, f"{name} must be {dtype}")
        if not t.is_contiguous():
            raise PfmError(7, f"{name} must be contiguous")
        return t

    def _part(self, t, n, name, vec=None):
        self._dev(t, name)
        want = (n, self.P) if vec is None else (vec, n, self.P)
        if tuple(t.shape) != want:
            raise PfmError(2, f"{name}: shape {tuple(t.shape)} != {want}")
        return t

    def _grids(self, u, name="u"):
        if len(u) != self.dim:
            raise PfmError(2, f"{name} needs {self.dim} face grids")
        return [self._grid(t, f, f"{name}[{f}]") for f, t in enumerate(u)]

    def alloc_faces(self, fill=0.0):
        return [torch.full(s, fill, dtype=torch.float32, device=self.device) for s in self.face_shapes]

    # ------------------------------------------------------------------------------------------
    # phases
    # ------------------------------------------------------------------------------------------
    def calc_max_speed_async(self, u):
        """calc_max_speed: result stays on the device in ``self.max_dev``."""
        u = self._grids(u)
        if self.dim == 3:
            self._check(self.lib.pfm3_calc_max_speed(self.h, *map(_ptr, u), _ptr(self.max_dev), self._stream()))
        else:
            self._check(self.lib.pfm2_calc_max_speed(self.h, *map(_ptr, u), _ptr(self.max_dev), self._stream()))
        return self.max_dev

    def calc_max_speed(self, u):
        """calc_max_speed + the ``max_speed[None]`` read (a host sync, as in the reference)."""
        return float(self.calc_max_speed_async(u).item())

    def g2p(self, pos, u, imp_out=None, C_out=None):
        """init_particles_imp (imp_out) / init_particles_imp_grad_m (C_out) G2P."""
        d = self.dim
        self._part(pos, d, "pos")
        u = self._grids(u)
        if imp_out is not None:
            self._part(imp_out, d, "imp_out")
        if C_out is not None:
            self._part(C_out, d, "C_out", vec=d)
        fn = self.lib.pfm3_g2p if d == 3 else self.lib.pfm2_g2p
        self._check(fn(self.h, _ptr(pos), *map(_ptr, u), _ptr(imp_out), _ptr(C_out), self._stream()))

    def update_T(self, T_init, T_gm, reset_gm=True):
        """3D update_T + reset_T_to_identity(T_gm)."""
        self._part(T_init, 3, "T_init", vec=3)
        self._part(T_gm, 3, "T_gm", vec=3)
        self._check(self.lib.pfm3_update_T(self.h, _ptr(T_init), _ptr(T_gm), int(bool(reset_gm)), self._stream()))

    def reset_T(self, T):
        d = self.dim
        self._part(T, d, "T", vec=d)
        fn = self.lib.pfm3_reset_T if d == 3 else self.lib.pfm2_reset_T
        self._check(fn(self.h, _ptr(T), self._stream()))

    def rk4_T_forward(self, pos, T, u, dt, advect_psi=True):
        d = self.dim
        self._part(pos, d, "pos")
        self._part(T, d, "T", vec=d)
        u = self._grids(u)
        if d == 3:
            self._check(self.lib.pfm3_rk4_T_forward(self.h, _ptr(pos), _ptr(T), *map(_ptr, u), ctypes.c_float(dt),
                                                    self._stream()))
        else:
            self._check(self.lib.pfm2_rk4_T_forward(self.h, _ptr(pos), _ptr(T), *map(_ptr, u), ctypes.c_float(dt),
                                                    int(bool(advect_psi)), self._stream()))

    def midpoint(self, u0, u1, dt_half, psi_out=None, T_out=None):
        d = self.dim
        u0 = self._grids(u0, "u0")
        u1 = self._grids(u1, "u1")
        arr = ctypes.c_void_p * d
        ps = arr(*[t.data_ptr() for t in psi_out]) if psi_out is not None else None
        ts = arr(*[t.data_ptr() for t in T_out]) if T_out is not None else None
        if d == 3:
            self._check(self.lib.pfm3_midpoint(self.h, *map(_ptr, u0), *map(_ptr, u1), ctypes.c_float(dt_half),
                                               ps, ts, self._stream()))
        else:
            self._check(self.lib.pfm2_midpoint(self.h, *map(_ptr, u0), *map(_ptr, u1), ctypes.c_float(dt_half),
                                               ps, ts, self._stream()))

    def sort_particles(self, pos):
        """get_particles_id_in_every_cell as a deterministic counting sort.

        Returns (cell_count [cells] int32, order [P] int32 stable permutation)."""
        d = self.dim
        self._part(pos, d, "pos")
        count = torch.empty(self.cell_shape, dtype=torch.int32, device=self.device)
        order = torch.empty(max(self.P, 1), dtype=torch.int32, device=self.device)
        fn = self.lib.pfm3_sort_particles if d == 3 else self.lib.pfm2_sort_particles
        self._check(fn(self.h, _ptr(pos), _ptr(count), _ptr(order), self._stream()))
        return count, order[:self.P]

    def p2g3(self, init_imp, pos, T_gm, T_init, init_C, u_out, w_out):
        """3D P2G (3D/run_3D.py:441-552)."""
        self._part(init_imp, 3, "init_imp")
        self._part(pos, 3, "pos")
        self._part(T_gm, 3, "T_gm", vec=3)
        self._part(T_init, 3, "T_init", vec=3)
        self._part(init_C, 3, "init_C", vec=3)
        u_out = self._grids(u_out, "u_out")
        w_out = self._grids(w_out, "w_out")
        self._check(self.lib.pfm3_p2g(self.h, _ptr(init_imp), _ptr(pos), _ptr(T_gm), _ptr(T_init), _ptr(init_C),
                                      *map(_ptr, u_out), *map(_ptr, w_out), self._stream()))

    def rk4_p2g3(self, pos, T_gm, u_adv, dt, init_imp, T_init, init_C, u_out, w_out):
        """RK4_T_forward then P2G in one call (3D/run_3D.py:795-812): bitwise the same as
        rk4_T_forward(pos, T_gm, u_adv, dt) followed by p2g3(...), with the particle state read once."""
        self._part(pos, 3, "pos")
        self._part(T_gm, 3, "T_gm", vec=3)
        self._part(init_imp, 3, "init_imp")
        self._part(T_init, 3, "T_init", vec=3)
        self._part(init_C, 3, "init_C", vec=3)
        u_adv = self._grids(u_adv, "u_adv")
        u_out = self._grids(u_out, "u_out")
        w_out = self._grids(w_out, "w_out")
        self._check(self.lib.pfm3_rk4_p2g(self.h, _ptr(pos), _ptr(T_gm), *map(_ptr, u_adv), ctypes.c_float(dt),
                                          _ptr(init_imp), _ptr(T_init), _ptr(init_C), *map(_ptr, u_out),
                                          *map(_ptr, w_out), self._stream()))

    def rk4_p2g_records3(self, pos, T_gm, u_adv, dt, init_imp, T_init, init_C):
        """RK4_T_forward that also leaves the P2G records and cell keys of the advected particles in
        the workspace (first half of rk4_p2g3)."""
        self._part(pos, 3, "pos")
        self._part(T_gm, 3, "T_gm", vec=3)
        self._part(init_imp, 3, "init_imp")
        self._part(T_init, 3, "T_init", vec=3)
        self._part(init_C, 3, "init_C", vec=3)
        u_adv = self._grids(u_adv, "u_adv")
        self._check(self.lib.pfm3_rk4_p2g_records(self.h, _ptr(pos), _ptr(T_gm), *map(_ptr, u_adv), ctypes.c_float(dt),
                                                  _ptr(init_imp), _ptr(T_init), _ptr(init_C), self._stream()))

    def gradm_rk4_records3(self, pos, T_gm, T_init, init_C, init_imp, u, u_adv, dt):
        """Gradient reinitialisation (init_C = grad u(pos), update_T, T_gm = I) + RK4 in u_adv + P2G
        records in one kernel (bitwise g2p + update_T + rk4_p2g_records3)."""
        self._part(pos, 3, "pos")
        for t, n in ((T_gm, "T_gm"), (T_init, "T_init"), (init_C, "init_C")):
            self._part(t, 3, n, vec=3)
        self._part(init_imp, 3, "init_imp")
        u = self._grids(u, "u")
        u_adv = self._grids(u_adv, "u_adv")
        self._check(self.lib.pfm3_gradm_rk4_p2g_records(self.h, _ptr(pos), _ptr(T_gm), _ptr(T_init), _ptr(init_C),
                                                        _ptr(init_imp), *map(_ptr, u), *map(_ptr, u_adv),
                                                        ctypes.c_float(dt), self._stream()))

    def p2g_from_records3(self, u_out, w_out):
        """The rest of P2G (bin sort, cell tiles, normalisation) from the records of
        rk4_p2g_records3 (second half of rk4_p2g3)."""
        u_out = self._grids(u_out, "u_out")
        w_out = self._grids(w_out, "w_out")
        self._check(self.lib.pfm3_p2g_from_records(self.h, *map(_ptr, u_out), *map(_ptr, w_out), self._stream()))

    def p2g2(self, imp, pos, C, psi, u_out, w_out, psi_out=None):
        """2D P2G (2D/run_2D.py:548-611); psi_out = (psi_x_grid [F,2], psi_y_grid [F,2]) or None."""
        self._part(imp, 2, "imp")
        self._part(pos, 2, "pos")
        self._part(C, 2, "C", vec=2)
        if psi is not None:
            self._part(psi, 2, "psi")
        u_out = self._grids(u_out, "u_out")
        w_out = self._grids(w_out, "w_out")
        px = py = None
        if psi_out is not None:
            px, py = psi_out
            for f, t in enumerate((px, py)):
                self._dev(t, "psi_out")
                if tuple(t.shape) != self.face_shapes[f] + (2,):
                    raise PfmError(2, "psi_out shape")
        self._check(self.lib.pfm2_p2g(self.h, _ptr(imp), _ptr(pos), _ptr(C), _ptr(psi), *map(_ptr, u_out),
                                      _ptr(px), _ptr(py), *map(_ptr, w_out), self._stream()))

    def update_grad_m2(self, C, init_C, T_gm):
        for t, n in ((C, "C"), (init_C, "init_C"), (T_gm, "T_gm")):
            self._part(t, 2, n, vec=2)
        self._check(self.lib.pfm2_update_grad_m(self.h, _ptr(C), _ptr(init_C), _ptr(T_gm), self._stream()))

    def update_T2(self, T, T_init, T_gm):
        for t, n in ((T, "T"), (T_init, "T_init"), (T_gm, "T_gm")):
            self._part(t, 2, n, vec=2)
        self._check(self.lib.pfm2_update_T(self.h, _ptr(T), _ptr(T_init), _ptr(T_gm), self._stream()))

    def update_imp2(self, imp, init_imp, T):
        self._part(imp, 2, "imp")
        self._part(init_imp, 2, "init_imp")
        self._part(T, 2, "T", vec=2)
        self._check(self.lib.pfm2_update_imp(self.h, _ptr(imp), _ptr(init_imp), _ptr(T), self._stream()))

    @staticmethod
    def _opts(max_iters, tol, tol_mode, check_every, eps=1e-12, precision=0, warm_start=False, true_residual_every=0,
              true_residual_replace=False):
        o = SolveOpts()
        o.max_iters, o.eps, o.tol, o.tol_mode, o.check_every = int(max_iters), float(eps), float(tol), int(tol_mode), int(check_every)
        o.precision = {"fp32": 0, "fp16": 1, "bf16": 2}.get(precision, precision)
        o.precision = int(o.precision)
        # False/True -> 0/1 (start from zero / from the caller's pressure); 2 / 3: extrapolate
        # linearly / quadratically from the caller's pressure and the solutions before it (the
        # library keeps those per buffer)
        if isinstance(warm_start, bool) or warm_start in (None, 0, 1):
            o.warm_start = int(bool(warm_start))
        elif warm_start in (2, 3):
            o.warm_start = int(warm_start)
        else:
            raise PfmError(1, f"warm_start must be False/True, 0, 1, 2 or 3, not {warm_start!r}")
        o.true_residual_every = int(true_residual_every)
        o.true_residual_replace = int(bool(true_residual_replace))
        return o

    def poisson(self, u, p_out=None, max_iters=400, tol=1e-12, tol_mode=0, check_every=4, raise_on_limit=False,
                precision=0, warm_start=False, true_residual_every=0, true_residual_replace=False):
        """MGPCG_{2,3}.Poisson in place on u (a sync point).  Returns SolveInfo.

        ``precision`` "fp32" (0, the reference), "fp16" (1) or "bf16" (2) multigrid level storage;
        ``warm_start`` starts from p_out's current pressure (``warm_start=2``: from the linear
        extrapolation 2 p - p_before of it and the solution before it; ``warm_start=3``: from the
        quadratic 3 (p - p_before) + p_before2 through the last three; the library keeps the
        earlier solutions per p_out buffer, two buffers per scene); ``true_residual_every`` K > 0
        recomputes |b - A x| every K iterations and reports it; with ``true_residual_replace`` (FP16/BF16
        levels) x is kept in FP64 and that residual, formed in FP64, replaces the recursive one every K
        iterations and before convergence is accepted."""
        u = self._grids(u)
        if p_out is not None:
            self._dev(p_out, "p_out")
            if tuple(p_out.shape) != self.cell_shape:
                raise PfmError(2, "p_out shape")
        elif warm_start:
            raise PfmError(1, "warm_start needs p_out (the previous pressure)")
        o = self._opts(max_iters, tol, tol_mode, check_every, precision=precision, warm_start=warm_start,
                       true_residual_every=true_residual_every, true_residual_replace=true_residual_replace)
        s = SolveStats()
        fn = self.lib.pfm3_poisson if self.dim == 3 else self.lib.pfm2_poisson
        allow = () if raise_on_limit else (_lib.PFM_ERR_NOT_CONVERGED,)
        st = self._check(fn(self.h, *map(_ptr, u), _ptr(p_out), ctypes.byref(o), ctypes.byref(s), self._stream()),
                         allow=allow)
        return SolveInfo(s, st)

    # ------------------------------------------------------------------------------------------
    # set-up helpers (initial conditions, seeding) and bookkeeping
    # ------------------------------------------------------------------------------------------
    def add_vortex_ring(self, vc, w, rad, delta, c, unit_x, unit_y, num_samples):
        """add_vortex_ring (3D/init_conditions.py:10-22) into the cell-centred field vc [*res, 3]."""
        self._dev(vc, "vc")
        if tuple(vc.shape) != self.cell_shape + (3,):
            raise PfmError(2, "vc must be [nx, ny, nz, 3]")
        f3 = ctypes.c_float * 3
        self._check(self.lib.pfm3_add_vortex_ring(self.h, ctypes.c_float(w), ctypes.c_float(rad), ctypes.c_float(delta),
                                                  f3(*c), f3(*unit_x), f3(*unit_y), int(num_samples), _ptr(vc),
                                                  self._stream()))

    def split_central_vector(self, vc, u):
        """split_central_vector (3D/taichi_utils.py:87-100): cell-centred vc -> face grids u."""
        self._dev(vc, "vc")
        u = self._grids(u)
        uz = u[2] if self.dim == 3 else None
        self._check(self.lib.pfm_split_central_vector(self.h, _ptr(vc), _ptr(u[0]), _ptr(u[1]), _ptr(uz),
                                                      self._stream()))

    def seed_jittered(self, pos, seed, ppc_axis):
        """Device twin of pfm.sim.jittered (bit-identical)."""
        self._part(pos, self.dim, "pos")
        self._check(self.lib.pfm_seed_jittered(self.h, ctypes.c_uint64(seed), int(ppc_axis), _ptr(pos), self._stream()))

    def set_tuning(self, key, value):
        """pfm_set_tuning: a launch-shape tunable (results are the same for every value)."""
        self._check(self.lib.pfm_set_tuning(self.h, int(key), int(value)))

    def get_tuning(self, key):
        v = ctypes.c_int()
        self._check(self.lib.pfm_get_tuning(self.h, int(key), ctypes.byref(v)))
        return v.value

    @property
    def launches(self):
        n = ctypes.c_uint64()
        self._check(self.lib.pfm_launch_count(self.h, ctypes.byref(n)))
        return int(n.value)

    def mgpcg_solve(self, r, x_out, k=-1.0, max_iters=400, tol=1e-12, tol_mode=0, check_every=4, precision=0,
                    warm_start=False, true_residual_every=0, true_residual_replace=False):
        """MGPCG init(r, k) + solve + get_result: lap(x) = k r (k = -1 for the divergence);
        with warm_start the solve starts from x_out's current values."""
        self._cells(r, "r")
        self._cells(x_out, "x_out")
        o = self._opts(max_iters, tol, tol_mode, check_every, precision=precision, warm_start=warm_start,
                       true_residual_every=true_residual_every, true_residual_replace=true_residual_replace)
        s = SolveStats()
        st = self._check(self.lib.pfm_mgpcg_solve(self.h, _ptr(r), ctypes.c_float(k), _ptr(x_out), ctypes.byref(o),
                                                  ctypes.byref(s), self._stream()),
                         allow=(_lib.PFM_ERR_NOT_CONVERGED,))
        return SolveInfo(s, st)

    def _cells(self, t, name):
        self._dev(t, name)
        if tuple(t.shape) != self.cell_shape:
            raise PfmError(2, f"{name} must have the cell shape {self.cell_shape}, got {tuple(t.shape)}")

    def _uz(self, u):
        return _ptr(u[2]) if self.dim == 3 else None

    def apply_bc(self, u):
        """MGPCG apply_bc (3D/mgpcg.py:359-378): zero normal velocity on Neumann walls, in place."""
        u = self._grids(u, "u")
        self._check(self.lib.pfm_apply_bc(self.h, _ptr(u[0]), _ptr(u[1]), self._uz(u), self._stream()))

    def divergence(self, u, div_out):
        """MGPCG divergence (3D/mgpcg.py:380-390) into div_out (cell shape)."""
        u = self._grids(u, "u")
        self._cells(div_out, "div_out")
        self._check(self.lib.pfm_divergence(self.h, _ptr(u[0]), _ptr(u[1]), self._uz(u), _ptr(div_out),
                                            self._stream()))

    # ------------------------------------------------------------------------------------------
    # the whole step as one CUDA graph
    # ------------------------------------------------------------------------------------------
    @staticmethod
    def step_params(CFL=0.5, visualize_dt=0.1, save_frame_each_step=False, reinit_every=20, reinit_every_grad_m=1,
                    use_midpoint_vel=True, reinit_particle_pos=True, max_iters=400, tol=1e-12, tol_mode=0, eps=1e-12,
                    precision=0, warm_start=False, true_residual_every=0, check_every=4, true_residual_replace=False):
        """pfm_step_params: the step loop's hyperparameters and the options of both projections."""
        sp = _lib.StepParams()
        sp.CFL, sp.visualize_dt = float(CFL), float(visualize_dt)
        sp.save_frame_each_step = int(bool(save_frame_each_step))
        sp.reinit_every, sp.reinit_every_grad_m = int(reinit_every), int(reinit_every_grad_m)
        sp.use_midpoint_vel, sp.reinit_particle_pos = int(bool(use_midpoint_vel)), int(bool(reinit_particle_pos))
        sp.poisson = Scene._opts(max_iters, tol, tol_mode, check_every, eps=eps, precision=precision,
                                 warm_start=warm_start, true_residual_every=true_residual_every,
                                 true_residual_replace=true_residual_replace)
        return sp

    def step_graph(self, fields, params):
        """One whole step (pfm3_step / pfm2_step) as a single graph launch on the current stream;
        ``fields`` is a Step3Fields / Step2Fields of device pointers (the caller keeps the tensors
        alive).  No host synchronization."""
        fn = self.lib.pfm3_step if self.dim == 3 else self.lib.pfm2_step
        self._check(fn(self.h, ctypes.byref(fields), ctypes.byref(params), self._stream()))

    def reset_warm_history(self):
        """Forgets the pressures kept for ``warm_start=2`` and ``3`` (the next solve of each buffer
        starts from the buffer's pressure alone)."""
        self._check(self.lib.pfm_reset_warm_history(self.h, self._stream()))

    def step_reset(self, i=-1, ik=0, sub_t=0.0, frame_idx=0):
        """Sets the device step clock (pfm_step_reset); the next graph step is i + 1."""
        self._check(self.lib.pfm_step_reset(self.h, int(i), int(ik), ctypes.c_double(sub_t), int(frame_idx),
                                            self._stream()))

    def step_info(self):
        """The device step state after the last graph step (a host sync): a pfm_step_info_t."""
        info = _lib.StepInfo()
        self._check(self.lib.pfm_step_info(self.h, ctypes.byref(info), self._stream()))
        return info

    # ------------------------------------------------------------------------------------------
    # scalar (smoke) transport and diagnostics
    # ------------------------------------------------------------------------------------------
    def _cellvec(self, t, n, name):
        self._dev(t, name)
        if tuple(t.shape) != self.cell_shape + (n,):
            raise PfmError(2, f"{name} must have shape {self.cell_shape + (n,)}, got {tuple(t.shape)}")
        if t.data_ptr() % 16:
            raise PfmError(7, f"{name} must be 16-byte aligned")
        return t

    def _psi(self, psi, name="psi"):
        if len(psi) != self.dim:
            raise PfmError(2, f"{name} needs {self.dim} face grids")
        for f, t in enumerate(psi):
            self._dev(t, f"{name}[{f}]")
            if tuple(t.shape) != self.face_shapes[f] + (self.dim,):
                raise PfmError(2, f"{name}[{f}]: shape {tuple(t.shape)} != {self.face_shapes[f] + (self.dim,)}")
        return psi

    def get_central_vector(self, u, vc=None):
        """get_central_vector (3D/taichi_utils.py:80-85, 2D/taichi_utils.py:50-55): cell-centred
        face averages [*res, dim]."""
        u = self._grids(u)
        vc = torch.empty(self.cell_shape + (self.dim,), device=self.device) if vc is None else vc
        self._cellvec(vc, self.dim, "vc")
        if self.dim == 3:
            self._check(self.lib.pfm3_get_central_vector(self.h, *map(_ptr, u), _ptr(vc), self._stream()))
        else:
            self._check(self.lib.pfm2_get_central_vector(self.h, *map(_ptr, u), _ptr(vc), self._stream()))
        return vc

    def curl(self, vc, w=None, dx=None):
        """curl (3D/taichi_utils.py:56-78: w [*res, 3]; 2D/taichi_utils.py:96-104: w [*res])."""
        self._cellvec(vc, self.dim, "vc")
        shape = self.cell_shape + ((3,) if self.dim == 3 else ())
        w = torch.empty(shape, device=self.device) if w is None else w
        self._dev(w, "w")
        if tuple(w.shape) != shape:
            raise PfmError(2, f"w must have shape {shape}")
        dxf = ctypes.c_float(self.dx if dx is None else dx)
        fn = self.lib.pfm3_curl if self.dim == 3 else self.lib.pfm2_curl
        self._check(fn(self.h, _ptr(vc), _ptr(w), dxf, self._stream()))
        return w

    def init_particles_smoke(self, pos, smoke, smoke_p=None, grad_smoke=None):
        """init_particles_smoke (3D/init_conditions.py:275-279): particle smoke [4, P] and its
        gradient [3, 4, P] from the smoke grid [*res, 4]."""
        self._need3("init_particles_smoke")
        self._part(pos, 3, "pos")
        self._cellvec(smoke, 4, "smoke")
        if smoke_p is not None:
            self._part(smoke_p, 4, "smoke_p")
        if grad_smoke is not None:
            self._dev(grad_smoke, "grad_smoke")
            if tuple(grad_smoke.shape) != (3, 4, self.P):
                raise PfmError(2, f"grad_smoke must be [3, 4, {self.P}]")
        self._check(self.lib.pfm3_init_particles_smoke(self.h, _ptr(pos), _ptr(smoke), _ptr(smoke_p), _ptr(grad_smoke),
                                                       self._stream()))

    def p2g_smoke(self, smoke_p, grad_smoke, pos, T_gm, T_init, smoke_out, w_out, use_apic_smoke=True):
        """P2G_smoke (3D/run_3D.py:554-593) into smoke_out [*res, 4] and the weights w_out [*res]."""
        self._need3("p2g_smoke")
        self._part(smoke_p, 4, "smoke_p")
        self._dev(grad_smoke, "grad_smoke")
        if tuple(grad_smoke.shape) != (3, 4, self.P):
            raise PfmError(2, f"grad_smoke must be [3, 4, {self.P}]")
        self._part(pos, 3, "pos")
        self._part(T_gm, 3, "T_gm", vec=3)
        self._part(T_init, 3, "T_init", vec=3)
        self._cellvec(smoke_out, 4, "smoke_out")
        self._cells(w_out, "w_out")
        self._check(self.lib.pfm3_p2g_smoke(self.h, _ptr(smoke_p), _ptr(grad_smoke), _ptr(pos), _ptr(T_gm),
                                            _ptr(T_init), int(bool(use_apic_smoke)), _ptr(smoke_out), _ptr(w_out),
                                            self._stream()))

    def advect_smoke(self, smoke0, smoke1, psi, dx=None):
        """advect_smoke (3D/run_3D.py:315-323; 2D/run_2D.py:444-450): smoke1 = smoke0 at the
        cell-centre backward map averaged from the face maps psi (pfm3/pfm2_midpoint's psi_out)."""
        nch = 4 if self.dim == 3 else 3
        self._cellvec(smoke0, nch, "smoke0")
        self._cellvec(smoke1, nch, "smoke1")
        psi = self._psi(psi)
        dxf = ctypes.c_float(self.dx if dx is None else dx)
        if self.dim == 3:
            self._check(self.lib.pfm3_advect_smoke(self.h, _ptr(smoke0), _ptr(smoke1), *map(_ptr, psi), dxf,
                                                   self._stream()))
        else:
            self._check(self.lib.pfm2_advect_smoke(self.h, _ptr(smoke0), _ptr(smoke1), *map(_ptr, psi), dxf,
                                                   self._stream()))

    def clamp_smoke(self, smoke0, smoke1, psi, dx=None):
        """clamp_smoke (3D/run_3D.py:326-334): clamps smoke1 to the range of smoke0's trilinear
        corners at the backward map, in place."""
        self._need3("clamp_smoke")
        self._cellvec(smoke0, 4, "smoke0")
        self._cellvec(smoke1, 4, "smoke1")
        psi = self._psi(psi)
        dxf = ctypes.c_float(self.dx if dx is None else dx)
        self._check(self.lib.pfm3_clamp_smoke(self.h, _ptr(smoke0), _ptr(smoke1), *map(_ptr, psi), dxf,
                                              self._stream()))

    def add_vortex_ring_and_smoke(self, vc, smoke, w, rad, delta, c, unit_x, unit_y, color, num_samples):
        """add_vortex_ring_and_smoke (3D/init_conditions.py:29-56): ring velocity into vc [*res, 3],
        marker into smoke [*res, 4], then smoke = (color, 1) where the marker exceeds 0.002, else 0."""
        self._need3("add_vortex_ring_and_smoke")
        self._dev(vc, "vc")
        if tuple(vc.shape) != self.cell_shape + (3,):
            raise PfmError(2, "vc must be [nx, ny, nz, 3]")
        self._cellvec(smoke, 4, "smoke")
        f3 = ctypes.c_float * 3
        self._check(self.lib.pfm3_add_vortex_ring_and_smoke(
            self.h, ctypes.c_float(w), ctypes.c_float(rad), ctypes.c_float(delta), f3(*c), f3(*unit_x), f3(*unit_y),
            f3(*color), int(num_samples), _ptr(vc), _ptr(smoke), self._stream()))

    # ------------------------------------------------------------------------------------------
    # the reference's alternative ("evolve m") dataflow (3D/run_3D.py:221-292, 353-428)
    # ------------------------------------------------------------------------------------------
    def rk4_T_and_T_grad_m_forward(self, pos, T, T_grad_m, u, dt):
        """RK4_T_and_T_grad_m_forward: positions and both Jacobian sets advanced in place."""
        self._need3("rk4_T_and_T_grad_m_forward")
        self._part(pos, 3, "pos")
        self._part(T, 3, "T", vec=3)
        self._part(T_grad_m, 3, "T_grad_m", vec=3)
        u = self._grids(u)
        self._check(self.lib.pfm3_rk4_T_and_T_grad_m_forward(self.h, _ptr(pos), _ptr(T), _ptr(T_grad_m), *map(_ptr, u),
                                                             ctypes.c_float(dt), self._stream()))

    def update_imp3(self, imp, init_imp, T):
        """update_particles_imp (3D): imp = cols(T) @ init_imp."""
        self._need3("update_imp3")
        self._part(imp, 3, "imp")
        self._part(init_imp, 3, "init_imp")
        self._part(T, 3, "T", vec=3)
        self._check(self.lib.pfm3_update_imp(self.h, _ptr(imp), _ptr(init_imp), _ptr(T), self._stream()))

    def update_grad_m3(self, C, init_C, T, grad_T_init=None, init_imp=None):
        """update_particles_grad_m (3D): C_r = grad_T_init_r @ init_imp + (T^T init_C T)_r;
        grad_T_init [3, 3, 3, P] or None (zero)."""
        self._need3("update_grad_m3")
        for t, n in ((C, "C"), (init_C, "init_C"), (T, "T")):
            self._part(t, 3, n, vec=3)
        if grad_T_init is not None:
            self._dev(grad_T_init, "grad_T_init")
            if tuple(grad_T_init.shape) != (3, 3, 3, self.P):
                raise PfmError(2, f"grad_T_init must be [3, 3, 3, {self.P}]")
            self._part(init_imp, 3, "init_imp")
        self._check(self.lib.pfm3_update_grad_m(self.h, _ptr(C), _ptr(init_C), _ptr(T), _ptr(grad_T_init),
                                                _ptr(init_imp), self._stream()))

    def compute_dT_dx(self, pos, init_pos, T, cap, grad_T_init=None):
        """compute_dT_dx: grad_T_init [3, 3, 3, P] from the neighbours in the cell lists of pos (at
        most cap per cell); cap = 0 gives the reference kernel's own (empty-loop) result."""
        self._need3("compute_dT_dx")
        self._part(pos, 3, "pos")
        self._part(init_pos, 3, "init_pos")
        self._part(T, 3, "T", vec=3)
        out = torch.empty(3, 3, 3, self.P, device=self.device) if grad_T_init is None else grad_T_init
        self._dev(out, "grad_T_init")
        if tuple(out.shape) != (3, 3, 3, self.P):
            raise PfmError(2, f"grad_T_init must be [3, 3, 3, {self.P}]")
        self._check(self.lib.pfm3_compute_dT_dx(self.h, _ptr(pos), _ptr(init_pos), _ptr(T), int(cap), _ptr(out),
                                                self._stream()))
        return out

    def _need3(self, what):
        if self.dim != 3:
            raise PfmError(2, f"{what} is a 3D phase")

    def subtract_grad_p(self, u, p):
        """MGPCG subtract_grad_p (3D/mgpcg.py:392-418): u -= grad p, in place."""
        u = self._grids(u, "u")
        self._cells(p, "p")
        self._check(self.lib.pfm_subtract_grad_p(self.h, _ptr(u[0]), _ptr(u[1]), self._uz(u), _ptr(p),
                                                 self._stream()))


def sort_particles_noalloc(pos, res, dx, cell_count, order):
    """Particle binning through ``pfm_sort_particles_noalloc``: the library allocates nothing
    (no handle, no workspace) and writes into the caller's ``cell_count`` (int32, ``prod(res)``
    entries) and ``order`` (int32, ``P`` entries).  Same result as :meth:`Scene.sort_particles`.

    Bounded by the library's fixed scratch: ``P <= NOALLOC_MAX_PARTICLES`` and
    ``prod(res) <= NOALLOC_MAX_CELLS``.  Calls share that scratch: do not run two at once."""
    dim = len(res)
    P = int(pos.shape[1]) if pos.dim() == 2 else -1
    if dim not in (2, 3) or pos.dim() != 2 or pos.shape[0] != dim:
        raise PfmError(7, f"pos must be [{dim}, P] for a {dim}D grid, got {tuple(pos.shape)}")
    cells = 1
    for r in res:
        cells *= int(r)
    if P > _lib.NOALLOC_MAX_PARTICLES or cells > _lib.NOALLOC_MAX_CELLS:
        raise PfmError(2, f"no-alloc binning holds at most {_lib.NOALLOC_MAX_PARTICLES} particles and "
                          f"{_lib.NOALLOC_MAX_CELLS} cells, got {P} particles and {cells} cells")
    for name, t, n, dt in (("pos", pos, None, torch.float32), ("cell_count", cell_count, cells, torch.int32),
                           ("order", order, P, torch.int32)):
        if t.dtype != dt or not t.is_cuda or not t.is_contiguous() or (n is not None and t.numel() < n):
            raise PfmError(2, f"{name} must be a contiguous CUDA {dt} tensor"
                              + (f" with at least {n} entries" if n is not None else ""))
        if t.device != pos.device:
            raise PfmError(7, f"{name} is on {t.device}, pos on {pos.device}: all three must share a device")
    r = (ctypes.c_int * 3)(*(list(int(x) for x in res) + [1] * (3 - dim)))
    # the entry point takes its scratch on the current device: make it pos's device for the call
    with torch.cuda.device(pos.device):
        st = _lib.load().pfm_sort_particles_noalloc(dim, r, float(dx), P, _ptr(pos), _ptr(cell_count), _ptr(order),
                                                     ctypes.c_void_p(torch.cuda.current_stream(pos.device).cuda_stream))
    if st != 0:
        raise PfmError(st, "pfm_sort_particles_noalloc failed")


def _field_check(name, t, like=None):
    if not isinstance(t, torch.Tensor) or t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous():
        raise PfmError(7, f"{name} must be a contiguous CUDA float32 tensor")
    if like is not None and (t.shape != like.shape or t.device != like.device):
        raise PfmError(2, f"{name} must match the shape and device of the destination")


def add_fields(f1, f2, dest, multiplier):
    """add_fields (3D/taichi_utils.py:18-21): dest = f1 + multiplier * f2 through pfm_add_fields."""
    _field_check("dest", dest)
    _field_check("f1", f1, dest)
    _field_check("f2", f2, dest)
    with torch.cuda.device(dest.device):
        st = _lib.load().pfm_add_fields(_ptr(f1), _ptr(f2), float(multiplier), _ptr(dest), dest.numel(),
                                        ctypes.c_void_p(torch.cuda.current_stream(dest.device).cuda_stream))
    if st != 0:
        raise PfmError(st, "pfm_add_fields failed")


def scale_field(a, alpha, result):
    """scale_field (3D/taichi_utils.py:13-16): result = alpha * a through pfm_scale_field."""
    _field_check("result", result)
    _field_check("a", a, result)
    with torch.cuda.device(result.device):
        st = _lib.load().pfm_scale_field(_ptr(a), float(alpha), _ptr(result), result.numel(),
                                         ctypes.c_void_p(torch.cuda.current_stream(result.device).cuda_stream))
    if st != 0:
        raise PfmError(st, "pfm_scale_field failed")


def measure_fp32_peak(blocks_per_sm=4, iters=65536, reps=3, packed=None, device=None):
    """FP32 FMA throughput of the current GPU in TFLOP/s (``pfm_measure_fp32_peak``): the best of
    ``reps`` timed launches of an 8-chain FMA loop, 2 flops per FMA, with scalar FMAs
    (``packed=False``), packed f32x2 FMAs (``packed=True``) or the better of the two (``None``).
    The denominator of the FP32 roofline beside HBM bandwidth.  Synchronous."""
    device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    sink = torch.zeros(1, dtype=torch.float32, device=device)
    best = 0.0
    for mode in ((0, 1) if packed is None else (1 if packed else 0,)):
        out = ctypes.c_double(0.0)
        st = _lib.load().pfm_measure_fp32_peak(_ptr(sink), int(blocks_per_sm), int(iters), int(reps), mode,
                                               ctypes.byref(out),
                                               ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream))
        if st != 0:
            raise PfmError(st, "pfm_measure_fp32_peak failed")
        best = max(best, out.value)
    return best
