"""Python face of the CPU oracle (test infrastructure: tests, smoke() and the CPU-baseline leg).

``libpfm_oracle.so`` (``oracle/pfm_oracle.cpp``) restates the reference's Taichi kernels; this
module binds it with ctypes and restates the two ``main()`` step loops
(``3D/run_3D.py:716-822`` and ``2D/run_2D.py:772-909``) on top of it.  Arrays use the reference's
Taichi layouts (particle vectors AoS ``[P, n]``, ``T``/``C`` as ``[P, n_vectors, n]``).
The oracle is pinned by ``tests/golden/*.npz``, which ``tests/golden/make_golden.py`` produced by
running the reference's own kernels.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libpfm_oracle.so")
SRC = os.path.join(HERE, "pfm_oracle.cpp")


def build(force=False):
    """Compile the oracle with g++ (no FMA contraction, OpenMP)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC):
        return LIB_PATH
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB_PATH + ".tmp", SRC]
    subprocess.check_call(cmd)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int)
_ci, _cd, _cf = ctypes.c_int, ctypes.c_double, ctypes.c_float


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle3_calc_max_speed.restype = _cf
        L.oracle2_calc_max_speed.restype = _cf
        for name in ("oracle3_poisson_f32", "oracle3_poisson_f64", "oracle2_poisson_f32",
                     "oracle2_poisson_f64"):
            getattr(L, name).restype = _ci
        L.oracle_num_threads.restype = _ci
        _lib = L
    return _lib


def _p(a, dtype=np.float32):
    if a is None:
        return None
    assert a.dtype == dtype and a.flags.c_contiguous, (a.dtype, a.flags)
    ptr = {np.float32: _f32p, np.float64: _f64p, np.int32: _i32p}[dtype]
    return a.ctypes.data_as(ptr)


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def set_threads(n):
    lib().oracle_set_threads(int(n))


def num_threads():
    return int(lib().oracle_num_threads())


# ------------------------------------------------------------------------------------------------
# 3D kernels
# ------------------------------------------------------------------------------------------------
def calc_max_speed3(ux, uy, uz):
    nx, ny, nz = uy.shape[0], ux.shape[1], ux.shape[2]
    return float(lib().oracle3_calc_max_speed(_p(f32(ux)), _p(f32(uy)), _p(f32(uz)), nx, ny, nz))


def g2p3(pos, ux, uy, uz, dx, want_imp=True, want_C=True):
    pos = f32(pos)
    P = pos.shape[0]
    nx, ny, nz = uy.shape[0], ux.shape[1], ux.shape[2]
    imp = np.zeros((P, 3), np.float32) if want_imp else None
    C = np.zeros((P, 3, 3), np.float32) if want_C else None
    lib().oracle3_g2p(_p(pos), P, _p(f32(ux)), _p(f32(uy)), _p(f32(uz)), nx, ny, nz, _cd(dx),
                      _p(imp), _p(C))
    return imp, C


def rk4_T_forward3(pos, T, ux, uy, uz, dx, dt):
    pos = f32(pos).copy()
    T = f32(T).copy()
    nx, ny, nz = uy.shape[0], ux.shape[1], ux.shape[2]
    lib().oracle3_rk4_T_forward(_p(pos), _p(T), pos.shape[0], _p(f32(ux)), _p(f32(uy)), _p(f32(uz)),
                                nx, ny, nz, _cd(dx), _cf(np.float32(dt)))
    return pos, T


def update_T3(T_init, T_gm):
    T_init = f32(T_init).copy()
    lib().oracle3_update_T(_p(T_init), _p(f32(T_gm)), T_init.shape[0])
    return T_init


def p2g3(init_imp, pos, T_gm, T_init, init_C, res, dx, use_apic=True, nthreads=1):
    nx, ny, nz = (int(r) for r in res)
    ux = np.zeros((nx + 1, ny, nz), np.float32); uy = np.zeros((nx, ny + 1, nz), np.float32)
    uz = np.zeros((nx, ny, nz + 1), np.float32)
    wx, wy, wz = np.zeros_like(ux), np.zeros_like(uy), np.zeros_like(uz)
    lib().oracle3_p2g(_p(f32(init_imp)), _p(f32(pos)), _p(f32(T_gm)), _p(f32(T_init)), _p(f32(init_C)),
                      f32(pos).shape[0], _p(ux), _p(uy), _p(uz), _p(wx), _p(wy), _p(wz), nx, ny, nz,
                      _cd(dx), int(use_apic), int(nthreads))
    return (ux, uy, uz), (wx, wy, wz)


def bin_count3(pos, res, dx):
    res = tuple(int(r) for r in res)
    count = np.zeros(res, np.int32)
    lib().oracle3_bin_count(_p(f32(pos)), f32(pos).shape[0], res[0], res[1], res[2], _cd(dx),
                            _p(count, np.int32))
    return count


def midpoint_family3(fam, ux, uy, uz, dx, dt_half):
    nx, ny, nz = uy.shape[0], ux.shape[1], ux.shape[2]
    shape = (nx + (fam == 0), ny + (fam == 1), nz + (fam == 2))
    psi = np.zeros(shape + (3,), np.float32)
    T = np.zeros(shape + (3,), np.float32)
    u = np.zeros(shape, np.float32)
    lib().oracle3_midpoint_family(fam, _p(f32(ux)), _p(f32(uy)), _p(f32(uz)), nx, ny, nz, _cd(dx),
                                  _cf(np.float32(dt_half)), _p(psi), _p(T), _p(u))
    return psi, T, u


def midpoint3(ux, uy, uz, dx, dt_half):
    return tuple(midpoint_family3(f, ux, uy, uz, dx, dt_half)[2] for f in range(3))


def poisson3(ux, uy, uz, base_level=3, boundary=(2, 2, 2, 2, 2, 2), levels=0, max_iters=400,
             tol=1e-12, fp64=False, tol_mode=0):
    """MGPCG_3.Poisson on copies of (ux, uy, uz). Returns (ux, uy, uz, p, iters, final_rTr)."""
    dt = np.float64 if fp64 else np.float32
    ux, uy, uz = (np.ascontiguousarray(a, dtype=dt).copy() for a in (ux, uy, uz))
    N = np.array([uy.shape[0], ux.shape[1], ux.shape[2]], np.int32)
    p = np.zeros(tuple(N), dt)
    bt = np.array(boundary, np.int32)
    rtr = ctypes.c_double(0)
    fn = lib().oracle3_poisson_f64 if fp64 else lib().oracle3_poisson_f32
    it = fn(_p(ux, dt), _p(uy, dt), _p(uz, dt), _p(p, dt), _p(N, np.int32), int(base_level),
            _p(bt, np.int32), int(levels), int(max_iters), _cd(tol), ctypes.byref(rtr), int(tol_mode))
    return ux, uy, uz, p, int(it), rtr.value


# ------------------------------------------------------------------------------------------------
# scalar (smoke) transport and diagnostics (Taichi layouts: smoke [nx, ny, nz, 4], particle smoke
# [P, 4], smoke gradient [P, 3, 4], psi grids [F, 3])
# ------------------------------------------------------------------------------------------------
def central_vector3(ux, uy, uz):
    nx, ny, nz = uy.shape[0], ux.shape[1], ux.shape[2]
    vc = np.zeros((nx, ny, nz, 3), np.float32)
    lib().oracle3_central_vector(_p(f32(ux)), _p(f32(uy)), _p(f32(uz)), nx, ny, nz, _p(vc))
    return vc


def curl3(vc, dx):
    vc = f32(vc)
    w = np.zeros_like(vc)
    lib().oracle3_curl(_p(vc), vc.shape[0], vc.shape[1], vc.shape[2], _cf(np.float32(dx)), _p(w))
    return w


def central_vector2(ux, uy):
    nx, ny = uy.shape[0], ux.shape[1]
    vc = np.zeros((nx, ny, 2), np.float32)
    lib().oracle2_central_vector(_p(f32(ux)), _p(f32(uy)), nx, ny, _p(vc))
    return vc


def curl2(vc, dx):
    vc = f32(vc)
    w = np.zeros(vc.shape[:2], np.float32)
    lib().oracle2_curl(_p(vc), vc.shape[0], vc.shape[1], _cf(np.float32(dx)), _p(w))
    return w


def init_particles_smoke3(pos, smoke, dx):
    pos, smoke = f32(pos), f32(smoke)
    P = pos.shape[0]
    s = np.zeros((P, 4), np.float32)
    G = np.zeros((P, 3, 4), np.float32)
    lib().oracle3_init_particles_smoke(_p(pos), P, _p(smoke), smoke.shape[0], smoke.shape[1], smoke.shape[2],
                                       _cf(np.float32(dx)), _p(s), _p(G))
    return s, G


def p2g_smoke3(s, G, pos, T_gm, T_init, res, dx, use_apic=True):
    nx, ny, nz = (int(r) for r in res)
    smoke = np.zeros((nx, ny, nz, 4), np.float32)
    w = np.zeros((nx, ny, nz), np.float32)
    pos = f32(pos)
    lib().oracle3_p2g_smoke(_p(f32(s)), _p(f32(G)), _p(pos), _p(f32(T_gm)), _p(f32(T_init)), pos.shape[0],
                            _p(smoke), _p(w), nx, ny, nz, _cd(dx), int(use_apic))
    return smoke, w


def advect_smoke3(smoke0, smoke1, psi_x, psi_y, psi_z, dx, clamp=False):
    """advect_smoke (clamp False) / clamp_smoke (clamp True) on a copy of smoke1."""
    s0 = f32(smoke0)
    s1 = f32(smoke1).copy()
    nx, ny, nz = s0.shape[:3]
    lib().oracle3_advect_smoke(_p(s0), _p(s1), _p(f32(psi_x)), _p(f32(psi_y)), _p(f32(psi_z)), nx, ny, nz,
                               _cf(np.float32(dx)), int(bool(clamp)))
    return s1


def advect_smoke2(smoke0, psi_x, psi_y, dx):
    s0 = f32(smoke0)
    s1 = np.zeros_like(s0)
    lib().oracle2_advect_smoke(_p(s0), _p(s1), _p(f32(psi_x)), _p(f32(psi_y)), s0.shape[0], s0.shape[1],
                               _cf(np.float32(dx)))
    return s1


# ------------------------------------------------------------------------------------------------
# the alternative ("evolve m") dataflow
# ------------------------------------------------------------------------------------------------
def rk4_T_and_T_grad_m_forward3(pos, T, T2, ux, uy, uz, dx, dt):
    pos, T, T2 = f32(pos).copy(), f32(T).copy(), f32(T2).copy()
    nx, ny, nz = uy.shape[0], ux.shape[1], ux.shape[2]
    lib().oracle3_rk4_T_and_T_grad_m_forward(_p(pos), _p(T), _p(T2), pos.shape[0], _p(f32(ux)), _p(f32(uy)),
                                             _p(f32(uz)), nx, ny, nz, _cd(dx), _cf(np.float32(dt)))
    return pos, T, T2


def update_imp3(imp0, T):
    imp0 = f32(imp0)
    out = np.zeros_like(imp0)
    lib().oracle3_update_imp(_p(out), _p(imp0), _p(f32(T)), imp0.shape[0])
    return out


def update_grad_m3(C0, T, gT, imp0):
    C0 = f32(C0)
    out = np.zeros_like(C0)
    lib().oracle3_update_grad_m(_p(out), _p(C0), _p(f32(T)), _p(None if gT is None else f32(gT)), _p(f32(imp0)),
                                C0.shape[0])
    return out


def compute_dT_dx3(pos, pos0, T, res, dx, cap):
    pos = f32(pos)
    P = pos.shape[0]
    gT = np.zeros((P, 3, 3, 3), np.float32)
    lib().oracle3_compute_dT_dx(_p(pos), _p(f32(pos0)), _p(f32(T)), P, int(res[0]), int(res[1]), int(res[2]),
                                _cd(dx), int(cap), _p(gT))
    return gT


# ------------------------------------------------------------------------------------------------
# 2D kernels
# ------------------------------------------------------------------------------------------------
def calc_max_speed2(ux, uy):
    nx, ny = uy.shape[0], ux.shape[1]
    return float(lib().oracle2_calc_max_speed(_p(f32(ux)), _p(f32(uy)), nx, ny))


def g2p2(pos, ux, uy, dx, want_imp=True, want_C=True):
    pos = f32(pos)
    P = pos.shape[0]
    nx, ny = uy.shape[0], ux.shape[1]
    imp = np.zeros((P, 2), np.float32) if want_imp else None
    C = np.zeros((P, 2, 2), np.float32) if want_C else None
    lib().oracle2_g2p(_p(pos), P, _p(f32(ux)), _p(f32(uy)), nx, ny, _cd(dx), _p(imp), _p(C))
    return imp, C


def rk4_T_forward2(pos, T, ux, uy, dx, dt, advect_psi=1):
    pos = f32(pos).copy()
    T = f32(T).copy()
    nx, ny = uy.shape[0], ux.shape[1]
    lib().oracle2_rk4_T_forward(_p(pos), _p(T), pos.shape[0], _p(f32(ux)), _p(f32(uy)), nx, ny,
                                _cd(dx), _cf(np.float32(dt)), int(advect_psi))
    return pos, T


def update_grad_m2(C0, T):
    C = np.zeros_like(f32(C0))
    lib().oracle2_update_grad_m(_p(C), _p(f32(C0)), _p(f32(T)), C.shape[0])
    return C


def update_T2(T_init, T_gm):
    T = np.zeros_like(f32(T_init))
    lib().oracle2_update_T(_p(T), _p(f32(T_init)), _p(f32(T_gm)), T.shape[0])
    return T


def update_imp2(imp0, T):
    imp = np.zeros_like(f32(imp0))
    lib().oracle2_update_imp(_p(imp), _p(f32(imp0)), _p(f32(T)), imp.shape[0])
    return imp


def p2g2(imp, pos, C, psi, res, dx, use_apic=True, want_psi=True):
    nx, ny = (int(r) for r in res)
    ux = np.zeros((nx + 1, ny), np.float32); uy = np.zeros((nx, ny + 1), np.float32)
    wx, wy = np.zeros_like(ux), np.zeros_like(uy)
    gx = np.zeros((nx + 1, ny, 2), np.float32) if want_psi else None
    gy = np.zeros((nx, ny + 1, 2), np.float32) if want_psi else None
    lib().oracle2_p2g(_p(f32(imp)), _p(f32(pos)), _p(f32(C)), _p(f32(psi)), f32(pos).shape[0],
                      _p(ux), _p(uy), _p(gx), _p(gy), _p(wx), _p(wy), nx, ny, _cd(dx), int(use_apic))
    return (ux, uy), (wx, wy), (gx, gy)


def midpoint_family2(fam, ux, uy, dx, dt_half):
    nx, ny = uy.shape[0], ux.shape[1]
    shape = (nx + (fam == 0), ny + (fam == 1))
    psi = np.zeros(shape + (2,), np.float32)
    T = np.zeros(shape + (2,), np.float32)
    u = np.zeros(shape, np.float32)
    lib().oracle2_midpoint_family(fam, _p(f32(ux)), _p(f32(uy)), nx, ny, _cd(dx),
                                  _cf(np.float32(dt_half)), _p(psi), _p(T), _p(u))
    return psi, T, u


def poisson2(ux, uy, base_level=3, boundary=(2, 2, 2, 2), levels=0, max_iters=400, tol=1e-12,
             fp64=False, tol_mode=0):
    dt = np.float64 if fp64 else np.float32
    ux, uy = (np.ascontiguousarray(a, dtype=dt).copy() for a in (ux, uy))
    N = np.array([uy.shape[0], ux.shape[1]], np.int32)
    p = np.zeros(tuple(N), dt)
    bt = np.array(boundary, np.int32)
    rtr = ctypes.c_double(0)
    fn = lib().oracle2_poisson_f64 if fp64 else lib().oracle2_poisson_f32
    it = fn(_p(ux, dt), _p(uy, dt), _p(p, dt), _p(N, np.int32), int(base_level), _p(bt, np.int32),
            int(levels), int(max_iters), _cd(tol), ctypes.byref(rtr), int(tol_mode))
    return ux, uy, p, int(it), rtr.value


# ------------------------------------------------------------------------------------------------
# seeding (the reference's lattice) and the step loops
# ------------------------------------------------------------------------------------------------
def lattice3(res, dx, ppc_axis=2):
    """init_particles_pos_uniform (3D/init_conditions.py:238-252): x-fastest lattice order."""
    nx, ny, nz = res
    P = nx * ny * nz * ppc_axis ** 3
    i = np.arange(P, dtype=np.int64)
    px, py = ppc_axis * nx, ppc_axis * ny
    idx = np.stack([i % px, (i // px) % py, (i // px) // py], axis=1)
    dist = np.float32(dx / ppc_axis)
    return ((idx.astype(np.float32) + np.float32(0.5)) * dist).astype(np.float32)


def lattice2(res, dx, ppc):
    """init_particles_pos_uniform (2D/init_conditions.py:139-166)."""
    nx, ny = res
    axis = int(np.sqrt(ppc))
    P = nx * ny * ppc
    i = np.arange(P, dtype=np.int64)
    px = axis * nx
    idx = np.stack([i % px, i // px], axis=1)
    dist = np.float32(dx / axis)
    return ((idx.astype(np.float32) + np.float32(0.5)) * dist).astype(np.float32)


class DtClock:
    """The CFL step and frame clamp of run_3D.py:725-743 / run_2D.py:782-799 (Python doubles)."""

    def __init__(self, CFL, dx, visualize_dt, save_frame_each_step=False):
        self.CFL, self.dx, self.visualize_dt = CFL, dx, visualize_dt
        self.save_frame_each_step = save_frame_each_step
        self.sub_t = 0.0
        self.frame_idx = 0

    def next(self, max_speed):
        curr_dt = self.CFL * self.dx / max_speed
        if self.save_frame_each_step:
            self.frame_idx += 1
            return curr_dt, True
        if self.sub_t + curr_dt >= self.visualize_dt:
            curr_dt = self.visualize_dt - self.sub_t
            self.sub_t = 0.0
            self.frame_idx += 1
            return curr_dt, True
        self.sub_t += curr_dt
        return curr_dt, False


class Sim3D:
    """run_3D.main()'s loop body (3D/run_3D.py:716-822) over the oracle kernels."""

    def __init__(self, u, seeds, res, dx, CFL=0.5, visualize_dt=0.1, reinit_every=20,
                 reinit_every_grad_m=1, use_midpoint_vel=True, reinit_particle_pos=True,
                 use_apic=True, base_level=3, p2g_threads=1, poisson_opts=None):
        self.poisson_opts = dict(poisson_opts or {})
        self.u = [f32(a).copy() for a in u]
        self.seeds = f32(seeds)
        self.res, self.dx = tuple(int(r) for r in res), float(dx)
        self.clock = DtClock(CFL, dx, visualize_dt)
        self.reinit_every, self.grad_m = reinit_every, reinit_every_grad_m
        self.use_midpoint_vel, self.reinit_particle_pos = use_midpoint_vel, reinit_particle_pos
        self.use_apic, self.base_level, self.p2g_threads = use_apic, base_level, p2g_threads
        P = self.seeds.shape[0]
        self.pos = np.zeros((P, 3), np.float32)
        self.init_imp = np.zeros((P, 3), np.float32)
        eye = np.broadcast_to(np.eye(3, dtype=np.float32), (P, 3, 3))
        self.T_init = eye.copy()
        self.T_gm = eye.copy()
        self.init_C = np.zeros((P, 3, 3), np.float32)
        self.i, self.ik = -1, 0
        self.iters = []
        self.p = None

    def step(self):
        self.i += 1
        i = self.i
        j = i % self.reinit_every
        max_speed = calc_max_speed3(*self.u)
        curr_dt, _ = self.clock.next(max_speed)
        self.last_dt = curr_dt
        P = self.pos.shape[0]
        eye = np.broadcast_to(np.eye(3, dtype=np.float32), (P, 3, 3))
        if j == 0:
            if self.reinit_particle_pos or i == 0:
                self.pos = self.seeds.copy()
                self.ik = i
            self.init_imp, _ = g2p3(self.pos, *self.u, self.dx, want_C=False)
            self.T_init = eye.copy()
            self.T_gm = eye.copy()
        k = (i - self.ik) % self.grad_m
        if k == 0:
            _, self.init_C = g2p3(self.pos, *self.u, self.dx, want_imp=False)
            self.T_init = update_T3(self.T_init, self.T_gm)
            self.T_gm = eye.copy()
        u_adv = self.u
        if self.use_midpoint_vel:
            mid = midpoint3(*self.u, self.dx, np.float32(0.5 * curr_dt))
            ux, uy, uz, _, it, _ = poisson3(*mid, base_level=self.base_level, **self.poisson_opts)
            self.iters.append(it)
            u_adv = [ux, uy, uz]
        self.pos, self.T_gm = rk4_T_forward3(self.pos, self.T_gm, *u_adv, self.dx, np.float32(curr_dt))
        (ux, uy, uz), _ = p2g3(self.init_imp, self.pos, self.T_gm, self.T_init, self.init_C, self.res,
                               self.dx, self.use_apic, self.p2g_threads)
        ux, uy, uz, p, it, _ = poisson3(ux, uy, uz, base_level=self.base_level, **self.poisson_opts)
        self.iters.append(it)
        self.u = [ux, uy, uz]
        self.p = p
        return curr_dt


class Sim2D:
    """run_2D.main()'s loop body (2D/run_2D.py:772-909) over the oracle kernels."""

    def __init__(self, u, seeds, res, dx, CFL=0.5, visualize_dt=0.1, reinit_every=12,
                 reinit_every_grad_m=8, use_midpoint_vel=True, reinit_particle_pos=True,
                 use_apic=True, base_level=3, poisson_opts=None):
        self.poisson_opts = dict(poisson_opts or {})
        self.u = [f32(a).copy() for a in u]
        self.seeds = f32(seeds)
        self.res, self.dx = tuple(int(r) for r in res), float(dx)
        self.clock = DtClock(CFL, dx, visualize_dt)
        self.reinit_every, self.grad_m = reinit_every, reinit_every_grad_m
        self.use_midpoint_vel, self.reinit_particle_pos = use_midpoint_vel, reinit_particle_pos
        self.use_apic, self.base_level = use_apic, base_level
        P = self.seeds.shape[0]
        eye = np.broadcast_to(np.eye(2, dtype=np.float32), (P, 2, 2))
        self.pos = self.seeds.copy()
        self.imp = np.zeros((P, 2), np.float32)
        self.init_imp = np.zeros((P, 2), np.float32)
        self.T, self.T_init, self.T_gm = eye.copy(), eye.copy(), eye.copy()
        self.init_C = np.zeros((P, 2, 2), np.float32)
        self.C = np.zeros((P, 2, 2), np.float32)
        self.psi = self.seeds.copy()
        self.i, self.ik = -1, 0
        self.iters = []
        self.p = None
        self.psi_grid = None

    def step(self):
        self.i += 1
        i = self.i
        j = i % self.reinit_every
        max_speed = calc_max_speed2(*self.u)
        curr_dt, _ = self.clock.next(max_speed)
        self.last_dt = curr_dt
        P = self.pos.shape[0]
        eye = np.broadcast_to(np.eye(2, dtype=np.float32), (P, 2, 2))
        if j == 0:
            if self.reinit_particle_pos or i == 0:
                self.pos = self.seeds.copy()
            self.ik = i
            imp, _ = g2p2(self.pos, *self.u, self.dx, want_C=False)
            self.imp, self.init_imp = imp.copy(), imp.copy()
            self.psi = self.pos.copy()
            self.T = eye.copy()
            self.T_init = eye.copy()
        k = (i - self.ik) % self.grad_m
        if k == 0:
            _, self.init_C = g2p2(self.pos, *self.u, self.dx, want_imp=False)
            self.T_gm = eye.copy()
            self.T_init = self.T.copy()
        u_adv = self.u
        if self.use_midpoint_vel:
            mids = [midpoint_family2(f, *self.u, self.dx, np.float32(0.5 * curr_dt))[2] for f in range(2)]
            ux, uy, _, it, _ = poisson2(*mids, base_level=self.base_level, **self.poisson_opts)
            self.iters.append(it)
            u_adv = [ux, uy]
        self.pos, self.T_gm = rk4_T_forward2(self.pos, self.T_gm, *u_adv, self.dx, np.float32(curr_dt), 1)
        self.C = update_grad_m2(self.init_C, self.T_gm)
        self.T = update_T2(self.T_init, self.T_gm)
        self.imp = update_imp2(self.init_imp, self.T)
        (ux, uy), _, self.psi_grid = p2g2(self.imp, self.pos, self.C, self.psi, self.res, self.dx,
                                          self.use_apic)
        ux, uy, p, it, _ = poisson2(ux, uy, base_level=self.base_level, **self.poisson_opts)
        self.iters.append(it)
        self.u = [ux, uy]
        self.p = p
        return curr_dt
