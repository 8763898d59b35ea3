"""Drop-in for the reference's 3D/run_3D.py: the same module-level fields, the same step-phase
functions with the same arguments, and main(from_frame, testing) with the same schedule
(3D/run_3D.py:20-95, 96-552, 618-871), running libpfm's sm_103a kernels.

Fields are CUDA tensors (allocated at import, as the reference allocates its Taichi fields, when
a GPU is present): particle vector fields are SoA [3, P]; T_x_init/T_y_init/T_z_init,
T_x_grad_m/..., init_C_x/... are the rows of one [3, 3, P] tensor each; grids keep the
reference's shapes.  main() writes the reference's checkpoints (ckpts/vel_{x,y,z}_numpy_<frame>.npy
and frame_time/frame_times.npy under logs/<exp_name>); the PNG/VTK writers are not built.
"""
import os
import sys
import time

import numpy as np
import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, _HERE)
sys.path.insert(0, os.path.dirname(_HERE))
from pfm import dropin as _d  # noqa: E402
from hyperparameters import *  # noqa: E402,F401,F403
from init_conditions import (init_particles_imp, init_particles_imp_grad_m,  # noqa: E402,F401
                             init_particles_pos_uniform, init_particles_smoke, init_vorts_leapfrog)
from mgpcg import MGPCG_3  # noqa: E402
from taichi_utils import curl, get_central_vector  # noqa: E402,F401

dx = 1. / res_y  # noqa: F405
particles_per_cell_axis = 2
dist_between_neighbor = dx / particles_per_cell_axis
one_sixth = 1. / 6
boundary_types = np.array([[2, 2], [2, 2], [2, 2]], np.int32)  # 1 Dirichlet, 2 Neumann
initial_particle_num = res_x * res_y * res_z * particles_per_cell  # noqa: F405
particle_num = initial_particle_num * total_particles_num_ratio  # noqa: F405
cell_max_particle_num = int(cell_max_particle_num_ratio * particles_per_cell)  # noqa: F405
max_speed = _d.Scalar(0.0)
_res = (res_x, res_y, res_z)  # noqa: F405
_face_shapes = [(res_x + 1, res_y, res_z), (res_x, res_y + 1, res_z), (res_x, res_y, res_z + 1)]  # noqa: F405


def _scene():
    return _d.scene(3, _res, dx, particle_num, boundary=boundary_types, use_apic=use_APIC)  # noqa: F405


def _allocate():
    g = globals()
    dev = torch.device("cuda")
    P = particle_num
    g["solver"] = MGPCG_3(boundary_types=boundary_types, N=list(_res), base_level=3)
    for name in ("particles_pos", "particles_init_imp", "particles_init_imp_grad_m"):
        g[name] = torch.zeros(3, P, device=dev)
    for stem in ("init", "grad_m"):
        buf, rows = _d.vector_rows(3, P, dev)
        g[f"_T_{stem}"] = buf
        g[f"T_x_{stem}"], g[f"T_y_{stem}"], g[f"T_z_{stem}"] = rows
    buf, rows = _d.vector_rows(3, P, dev)
    g["_init_C"] = buf
    g["init_C_x"], g["init_C_y"], g["init_C_z"] = rows
    g["cell_particle_num"] = torch.zeros(_res, dtype=torch.int32, device=dev)
    g["cell_particles_id"] = torch.full(_res + (cell_max_particle_num,), -1, dtype=torch.int32, device=dev)
    g["u"] = torch.zeros(_res + (3,), device=dev)
    g["u_x"], g["u_y"], g["u_z"] = (torch.zeros(s, device=dev) for s in _face_shapes)
    g["p2g_weight_x"], g["p2g_weight_y"], g["p2g_weight_z"] = (torch.zeros(s, device=dev) for s in _face_shapes)
    g["X"] = None  # cell centres (I + 0.5) dx: implied by the grid in the kernels that use them
    g["w"] = torch.zeros(_res + (3,), device=dev)  # curl of u
    g["smoke"] = torch.zeros(_res + (4,), device=dev)
    g["tmp_smoke"] = torch.zeros(_res + (4,), device=dev)


if torch.cuda.is_available():
    _allocate()

# Per-particle smoke fields of the reference (3D/run_3D.py:47-48), allocated on first use: the
# step never touches them (its smoke calls are commented out) and they hold 64 B per particle.
_LAZY = {"particles_smoke": lambda: torch.zeros(4, particle_num, device="cuda"),
         "particles_init_grad_smoke": lambda: torch.zeros(3, 4, particle_num, device="cuda")}


def __getattr__(name):
    if name in _LAZY and torch.cuda.is_available():
        t = _LAZY[name]()
        globals()[name] = t
        return t
    raise AttributeError(name)


# ---------------------------------------------------------------------------------------------
# step phases (3D/run_3D.py:96-552)
# ---------------------------------------------------------------------------------------------
def calc_max_speed(u_x, u_y, u_z):
    """max_speed[None] = max centre-averaged speed, floor 1e-3 (3D/run_3D.py:95-103)."""
    max_speed[None] = _scene().calc_max_speed([u_x, u_y, u_z])


def reset_T_to_identity(T_x, T_y, T_z):
    with _d.Rows((T_x, T_y, T_z), out=True) as T:
        _scene().reset_T(T)


def update_T(T_x_init, T_y_init, T_z_init, T_x_grad_m, T_y_grad_m, T_z_grad_m):
    """T_init <- cols(T_grad_m) @ cols(T_init) (3D/run_3D.py:430-439)."""
    with _d.Rows((T_x_init, T_y_init, T_z_init), out=True) as Ti, _d.Rows((T_x_grad_m, T_y_grad_m, T_z_grad_m)) as Tg:
        _scene().update_T(Ti, Tg, reset_gm=False)


def RK4_T_forward(psi, T_x, T_y, T_z, u_x0, u_y0, u_z0, dt):
    """Forward RK4 of positions psi [3, P] and T (3D/run_3D.py:175-219)."""
    with _d.Rows((T_x, T_y, T_z), out=True) as T:
        _scene().rk4_T_forward(psi, T, [u_x0, u_y0, u_z0], float(np.float32(dt)))


def stretch_T_and_advect_particles(particles_pos, T_x, T_y, T_z, u_x, u_y, u_z, dt):
    RK4_T_forward(particles_pos, T_x, T_y, T_z, u_x, u_y, u_z, dt)


def _family_of(grid):
    shp = tuple(grid.shape[:3])
    for f, s in enumerate(_face_shapes):
        if shp == s:
            return f
    raise ValueError(f"not a face grid of a {_res} grid: {tuple(grid.shape)}")


_midpoint_dt = {}


def reset_to_identity_grid(psi_x, psi_y, psi_z, T_x, T_y, T_z):
    """The midpoint kernels start every face at its own position with T = e_f themselves; nothing
    to do here (3D/run_3D.py:106-120)."""


def RK4_grid(psi_x, T_x, u_x0, u_y0, u_z0, dt):
    """Backward RK4 of one face family's positions and T over dt (3D/run_3D.py:144-173): writes the
    family's psi [F, 3] and T [F, 3] grids."""
    sc = _scene()
    f = _family_of(psi_x)
    scratch = sc.alloc_faces()
    psi_out = [psi_x if a == f else torch.empty(_face_shapes[a] + (3,), device=psi_x.device) for a in range(3)]
    T_out = [T_x if a == f else torch.empty(_face_shapes[a] + (3,), device=psi_x.device) for a in range(3)]
    sc.midpoint([u_x0, u_y0, u_z0], scratch, float(np.float32(dt)), psi_out=psi_out, T_out=T_out)
    _midpoint_dt[f] = float(np.float32(dt))


def advect_u(u_x0, u_y0, u_z0, u_x1, u_y1, u_z1, T_x, T_y, T_z, psi_x, psi_y, psi_z, dx_):
    """u1 = T . u0(psi) on every face (3D/run_3D.py:296-312).  The backward map is recomputed with
    the dt of the preceding RK4_grid calls (the same psi/T, bit for bit, since u0 is the velocity
    those calls integrated)."""
    if len(set(_midpoint_dt.values())) != 1:
        raise RuntimeError("advect_u needs the RK4_grid calls of all three families first")
    _scene().midpoint([u_x0, u_y0, u_z0], [u_x1, u_y1, u_z1], next(iter(_midpoint_dt.values())))


def copy_to(src, dst):
    dst.copy_(src)


def get_particles_id_in_every_cell(cell_particles_id, cell_particle_num, particles_pos):
    """Cell counts and (up to the per-cell capacity) the particle ids of every cell
    (3D/run_3D.py:342-351), from the deterministic counting sort: ids in index order."""
    count, order = _scene().sort_particles(particles_pos)
    cell_particle_num.copy_(count.reshape(cell_particle_num.shape))
    cap = cell_particles_id.shape[-1]
    flat = count.reshape(-1).to(torch.int64)
    start = torch.cumsum(flat, 0) - flat
    slots = torch.arange(cap, device=flat.device)
    idx = start[:, None] + slots[None, :]
    valid = slots[None, :] < flat[:, None]
    ids = torch.where(valid, order[idx.clamp(max=max(order.numel() - 1, 0))].to(torch.int32),
                      torch.full_like(idx, -1, dtype=torch.int32)) if order.numel() else \
        torch.full(idx.shape, -1, dtype=torch.int32, device=flat.device)
    cell_particles_id.copy_(ids.reshape(cell_particles_id.shape))


def P2G(particles_init_imp, particles_init_imp_grad_m, particles_pos, u_x, u_y, u_z, p2g_weight_x, p2g_weight_y,
        p2g_weight_z, T_x_grad_m, T_y_grad_m, T_z_grad_m, T_x_init, T_y_init, T_z_init, cell_particles_id,
        cell_particle_num):
    """APIC impulse P2G with the module's init_C_x/y/z (3D/run_3D.py:441-552); deterministic (the
    cell lists are not needed: libpfm sorts the particles itself)."""
    with _d.Rows((T_x_grad_m, T_y_grad_m, T_z_grad_m)) as Tg, _d.Rows((T_x_init, T_y_init, T_z_init)) as Ti, \
            _d.Rows((init_C_x, init_C_y, init_C_z)) as C:  # noqa: F821
        _scene().p2g3(particles_init_imp, particles_pos, Tg, Ti, C, [u_x, u_y, u_z],
                      [p2g_weight_x, p2g_weight_y, p2g_weight_z])


def split_central_vector(vc, u_x_, u_y_, u_z_):
    _scene().split_central_vector(vc, [u_x_, u_y_, u_z_])


# ---------------------------------------------------------------------------------------------
# smoke transport (3D/run_3D.py:315-334, 554-593) and the alternative "evolve m" dataflow
# (3D/run_3D.py:221-292, 338-340, 353-428); the reference's step loop leaves them commented out
# ---------------------------------------------------------------------------------------------
def advect_smoke(smoke0, smoke1, psi_x, psi_y, psi_z, dx_):
    """smoke1 = smoke0 at the cell-centre average of the face backward maps (3D/run_3D.py:315-323)."""
    _scene().advect_smoke(smoke0, smoke1, [psi_x, psi_y, psi_z], dx=float(dx_))


def clamp_smoke(smoke0, smoke1, psi_x, psi_y, psi_z, dx_):
    """Clamp smoke1 to the range of smoke0's eight corners there (3D/run_3D.py:326-334)."""
    _scene().clamp_smoke(smoke0, smoke1, [psi_x, psi_y, psi_z], dx=float(dx_))


def P2G_smoke(particles_smoke_, particles_init_grad_smoke_, particles_pos_, smoke_, T_x_grad_m_, T_y_grad_m_,
              T_z_grad_m_, T_x_init_, T_y_init_, T_z_init_, p2g_weight):
    """APIC P2G of the particle smoke into smoke_ [nx, ny, nz, 4], normalised and clamped to [0, 1]
    (3D/run_3D.py:554-593), with use_APIC_smoke; deterministic.  p2g_weight is a cell grid."""
    with _d.Rows((T_x_grad_m_, T_y_grad_m_, T_z_grad_m_)) as Tg, _d.Rows((T_x_init_, T_y_init_, T_z_init_)) as Ti:
        _scene().p2g_smoke(particles_smoke_, particles_init_grad_smoke_, particles_pos_, Tg, Ti, smoke_, p2g_weight,
                           use_apic_smoke=use_APIC_smoke)  # noqa: F405


def RK4_T_and_T_grad_m_forward(psi, T_x, T_y, T_z, T_x_grad_m_, T_y_grad_m_, T_z_grad_m_, u_x0, u_y0, u_z0, dt):
    """RK4 of the positions and of both Jacobian sets (3D/run_3D.py:221-292)."""
    with _d.Rows((T_x, T_y, T_z), out=True) as T, _d.Rows((T_x_grad_m_, T_y_grad_m_, T_z_grad_m_), out=True) as T2:
        _scene().rk4_T_and_T_grad_m_forward(psi, T, T2, [u_x0, u_y0, u_z0], float(np.float32(dt)))


def stretch_T_and_T_grad_m_and_advect_particles(particles_pos_, T_x, T_y, T_z, T_x_grad_m_, T_y_grad_m_, T_z_grad_m_,
                                                u_x_, u_y_, u_z_, dt):
    RK4_T_and_T_grad_m_forward(particles_pos_, T_x, T_y, T_z, T_x_grad_m_, T_y_grad_m_, T_z_grad_m_, u_x_, u_y_, u_z_,
                               dt)


def update_particles_imp(particles_imp_, particles_init_imp_, T_x, T_y, T_z):
    """imp = cols(T) @ init_imp (3D/run_3D.py:395-401)."""
    with _d.Rows((T_x, T_y, T_z)) as T:
        _scene().update_imp3(particles_imp_, particles_init_imp_, T)


def update_particles_grad_m(C_x, C_y, C_z, init_C_x_, init_C_y_, init_C_z_, T_x, T_y, T_z, grad_T_init_x,
                            grad_T_init_y, grad_T_init_z, particles_init_imp_):
    """C_r = grad_T_init_r @ init_imp + (T^T init_C T)_r (3D/run_3D.py:412-428); the grad_T_init
    matrices are [3, 3, P] tensors (rows of one [3, 3, 3, P] buffer, or separate)."""
    gT = torch.stack([grad_T_init_x, grad_T_init_y, grad_T_init_z]).contiguous()
    with _d.Rows((C_x, C_y, C_z), out=True) as C, _d.Rows((init_C_x_, init_C_y_, init_C_z_)) as C0, \
            _d.Rows((T_x, T_y, T_z)) as T:
        _scene().update_grad_m3(C, C0, T, gT, particles_init_imp_)


def compute_dT_dx(grad_T_init_x, grad_T_init_y, grad_T_init_z, T_x, T_y, T_z, particles_init_pos, cell_particles_id_,
                  cell_particle_num_, cap=0):
    """compute_dT_dx (3D/run_3D.py:353-390) on the cell lists of the module's particles_pos.  The
    reference's inner loop ti.ndrange(0, n) is an empty two-axis range, so its result is zero: that
    is cap = 0 (the default); cap = cell_max_particle_num computes the neighbourhood sum its body
    describes."""
    with _d.Rows((T_x, T_y, T_z)) as T:
        gT = _scene().compute_dT_dx(particles_pos, particles_init_pos, T, int(cap))  # noqa: F821
    for r, out in enumerate((grad_T_init_x, grad_T_init_y, grad_T_init_z)):
        out.copy_(gT[r])


# ---------------------------------------------------------------------------------------------
# main loop (3D/run_3D.py:618-871)
# ---------------------------------------------------------------------------------------------
def main(from_frame=0, testing=False, logs_root="logs"):
    from_frame = max(0, from_frame)
    logsdir = os.path.join(logs_root, exp_name)  # noqa: F405
    ckptdir = os.path.join(logsdir, "ckpts")
    os.makedirs(ckptdir, exist_ok=True)
    sc = _scene()
    U = [u_x, u_y, u_z]  # noqa: F821
    if from_frame <= 0:
        u.zero_()  # noqa: F821
        init_vorts_leapfrog(X, u, smoke, tmp_smoke)  # noqa: F821
        split_central_vector(u, u_x, u_y, u_z)  # noqa: F821
        solver.Poisson(u_x, u_y, u_z)  # noqa: F821
    else:
        for t, n in zip(U, "xyz"):
            t.copy_(torch.from_numpy(np.load(os.path.join(ckptdir, f"vel_{n}_numpy_{from_frame}.npy"))))
    for t, n in zip(U, "xyz"):
        np.save(os.path.join(ckptdir, f"vel_{n}_numpy_{from_frame}"), t.cpu().numpy())

    W = [p2g_weight_x, p2g_weight_y, p2g_weight_z]  # noqa: F821
    sub_t = 0.
    frame_idx = from_frame
    i, ik = -1, 0
    frame_times = np.zeros(total_steps)  # noqa: F405
    while True:
        start_time = time.time()
        i += 1
        j = i % reinit_every  # noqa: F405
        calc_max_speed(*U)
        curr_dt = CFL * dx / max_speed[None]  # noqa: F405
        if save_frame_each_step:  # noqa: F405
            output_frame = True
            frame_idx += 1
        elif sub_t + curr_dt >= visualize_dt:  # noqa: F405
            curr_dt = visualize_dt - sub_t  # noqa: F405
            sub_t = 0.
            frame_idx += 1
            output_frame = True
        else:
            sub_t += curr_dt
            output_frame = False
        if j == 0:
            if reinit_particle_pos or i == 0:  # noqa: F405
                init_particles_pos_uniform(particles_pos, X, res_x, res_y, particles_per_cell, dx,  # noqa: F405,F821
                                           particles_per_cell_axis, dist_between_neighbor)
                ik = i
            init_particles_imp(particles_init_imp, particles_pos, *U, init_C_x, init_C_y, init_C_z, dx)  # noqa: F821
            reset_T_to_identity(T_x_init, T_y_init, T_z_init)  # noqa: F821
            reset_T_to_identity(T_x_grad_m, T_y_grad_m, T_z_grad_m)  # noqa: F821
        k = (i - ik) % reinit_every_grad_m  # noqa: F405
        if k == 0:
            init_particles_imp_grad_m(particles_init_imp_grad_m, particles_pos, *U, init_C_x, init_C_y,  # noqa: F821
                                      init_C_z, dx)  # noqa: F821
            sc.update_T(_T_init, _T_grad_m, reset_gm=True)  # update_T + reset_T_to_identity  # noqa: F821
        if use_midpoint_vel:  # noqa: F405
            # reset_to_identity_grid + RK4_grid x3 + copy_to + advect_u (3D/run_3D.py:779-788)
            for s, d in zip(U, W):
                d.copy_(s)
            sc.midpoint(W, U, float(np.float32(0.5 * curr_dt)))
            solver.Poisson(*U)  # noqa: F821
        # stretch_T_and_advect_particles + get_particles_id_in_every_cell + P2G (3D/run_3D.py:795-812),
        # as the fused RK4 + P2G call (bitwise the same result)
        sc.rk4_p2g3(particles_pos, _T_grad_m, U, float(np.float32(curr_dt)), particles_init_imp,  # noqa: F821
                    _T_init, _init_C, U, W)  # noqa: F821
        solver.Poisson(*U)  # noqa: F821
        torch.cuda.synchronize()
        frame_time = time.time() - start_time
        if i <= total_steps - 1:  # noqa: F405
            frame_times[i] = frame_time
        print(f"[Simulate] Done with step: {i} / substep: {j}, step time {frame_time:.6f} s, "
              f"MGPCG iterations {solver.last_info.iterations}", flush=True)  # noqa: F821
        done = False
        if output_frame:
            if frame_idx % ckpt_every == 0:  # noqa: F405
                for t, n in zip(U, "xyz"):
                    np.save(os.path.join(ckptdir, f"vel_{n}_numpy_{frame_idx}"), t.cpu().numpy())
                if save_particle_pos_numpy:  # noqa: F405
                    np.save(os.path.join(ckptdir, f"particles_pos_numpy_{frame_idx}"),
                            particles_pos.t().cpu().numpy())  # noqa: F821
            done = frame_idx >= total_frames  # noqa: F405
        if use_total_steps and i >= total_steps - 1:  # noqa: F405
            done = True
        if done:
            ftdir = os.path.join(logsdir, "frame_time")
            os.makedirs(ftdir, exist_ok=True)
            np.save(os.path.join(ftdir, "frame_times.npy"), frame_times)
            break
    return i + 1


if __name__ == "__main__":
    main(from_frame=from_frame)  # noqa: F405
