"""Drop-in for the reference's 2D/run_2D.py: the same module-level fields, the same step-phase
functions with the same arguments, and main(from_frame, testing) with the same schedule
(2D/run_2D.py:14-100, 101-611, 676-976), running libpfm's sm_103a kernels.

Fields are CUDA tensors (allocated at import when a GPU is present): particle vector fields are
SoA [2, P]; T_x/T_y, T_x_init/T_y_init, T_x_grad_m/T_y_grad_m, C_x/C_y and init_C_x/init_C_y are
the rows of one [2, 2, P] tensor each; grids keep the reference's shapes.  main() writes
ckpts/vel_{x,y}_numpy_<frame>.npy and frame_time/frame_times.npy under logs/<exp_name>; the image
writers are not built.
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
                             init_particles_pos_uniform, leapfrog_vel_func, stripe_func)
from mgpcg import MGPCG_2  # noqa: E402
from taichi_utils import curl, get_central_vector  # noqa: E402,F401

dx = 1. / res_y  # noqa: F405
particles_per_cell_axis = int(np.sqrt(particles_per_cell))  # noqa: F405
dist_between_neighbor = dx / particles_per_cell_axis
boundary_types = np.array([[2, 2], [2, 2]], np.int32)  # 1 Dirichlet, 2 Neumann
initial_particle_num = res_x * res_y * particles_per_cell  # noqa: F405
particle_num = initial_particle_num * total_particles_num_ratio  # noqa: F405
cell_max_particle_num = int(cell_max_particle_num_ratio * particles_per_cell)  # noqa: F405
max_speed = _d.Scalar(0.0)
_res = (res_x, res_y)  # noqa: F405
_face_shapes = [(res_x + 1, res_y), (res_x, res_y + 1)]  # noqa: F405


def _scene():
    return _d.scene(2, _res, dx, particle_num, boundary=boundary_types, use_apic=use_APIC)  # noqa: F405


def _allocate():
    g = globals()
    dev = torch.device("cuda")
    P = particle_num
    g["solver"] = MGPCG_2(boundary_types=boundary_types, N=list(_res), base_level=3)
    for name in ("particles_pos", "particles_pos_backup", "particles_imp", "particles_init_imp",
                 "particles_init_imp_grad_m", "psi"):
        g[name] = torch.zeros(2, P, device=dev)
    for stem in ("", "_init", "_grad_m"):
        buf, rows = _d.vector_rows(2, P, dev)
        g[f"_T{stem}"] = buf
        g[f"T_x{stem}"], g[f"T_y{stem}"] = rows
    for stem in ("C", "init_C"):
        buf, rows = _d.vector_rows(2, P, dev)
        g[f"_{stem}"] = buf
        g[f"{stem}_x"], g[f"{stem}_y"] = rows
    g["u"] = torch.zeros(_res + (2,), device=dev)
    g["u_x"], g["u_y"] = (torch.zeros(s, device=dev) for s in _face_shapes)
    g["tmp_u_x"], g["tmp_u_y"] = (torch.zeros(s, device=dev) for s in _face_shapes)
    g["p2g_weight_x"], g["p2g_weight_y"] = (torch.zeros(s, device=dev) for s in _face_shapes)
    g["psi_x_grid"], g["psi_y_grid"] = (torch.zeros(s + (2,), device=dev) for s in _face_shapes)
    g["T_x_grid"], g["T_y_grid"] = (torch.zeros(s + (2,), device=dev) for s in _face_shapes)
    g["cell_particle_num"] = torch.zeros(_res, dtype=torch.int32, device=dev)
    g["X"] = None  # cell centres (I + 0.5) dx: implied by the grid
    g["w"] = torch.zeros(_res, device=dev)  # curl of u
    for name in ("init_smoke", "smoke", "tmp_smoke", "err_smoke"):  # 2D/run_2D.py:95-99
        g[name] = torch.zeros(_res + (3,), device=dev)


if torch.cuda.is_available():
    _allocate()


# ---------------------------------------------------------------------------------------------
# step phases (2D/run_2D.py:101-611)
# ---------------------------------------------------------------------------------------------
def calc_max_speed(u_x, u_y):
    """max_speed[None] = max centre-averaged speed, floor 1e-3 (2D/run_2D.py:101-108)."""
    max_speed[None] = _scene().calc_max_speed([u_x, u_y])


def reset_T_to_identity(T_x, T_y):
    with _d.Rows((T_x, T_y), out=True) as T:
        _scene().reset_T(T)


def reset_to_identity(psi_, T_x, T_y):
    """psi <- particles_pos, T <- I (2D/run_2D.py:133-139)."""
    psi_.copy_(particles_pos)  # noqa: F821
    reset_T_to_identity(T_x, T_y)


def backup_particles_pos(particles_pos_, particles_pos_backup_):
    particles_pos_backup_.copy_(particles_pos_)


def copy_to(src, dst):
    dst.copy_(src)


def RK4_T_forward(psi_, T_x, T_y, u_x0, u_y0, dt, advect_psi):
    """Forward RK4 of positions and T; advect_psi = 0 keeps the positions (2D/run_2D.py:304-341)."""
    with _d.Rows((T_x, T_y), out=True) as T:
        _scene().rk4_T_forward(psi_, T, [u_x0, u_y0], float(np.float32(dt)), advect_psi=bool(advect_psi))


def stretch_T_and_advect_particles(particles_pos_, T_x, T_y, u_x_, u_y_, dt):
    RK4_T_forward(particles_pos_, T_x, T_y, u_x_, u_y_, dt, 1)


def stretch_T(particles_pos_, T_x, T_y, u_x_, u_y_, dt):
    RK4_T_forward(particles_pos_, T_x, T_y, u_x_, u_y_, dt, 0)


def _family_of(grid):
    shp = tuple(grid.shape[:2])
    for f, s in enumerate(_face_shapes):
        if shp == s:
            return f
    raise ValueError(f"not a face grid of a {_res} grid: {tuple(grid.shape)}")


_midpoint_dt = {}


def reset_to_identity_grid(psi_x, psi_y, T_x, T_y):
    """The midpoint kernels start every face at its position with T = e_f (2D/run_2D.py:120-129)."""


def RK4_grid(psi_x, T_x, u_x0, u_y0, dt):
    """Backward RK4 of one face family's positions and T over dt (2D/run_2D.py:233-261)."""
    sc = _scene()
    f = _family_of(psi_x)
    scratch = sc.alloc_faces()
    psi_out = [psi_x if a == f else torch.empty(_face_shapes[a] + (2,), device=psi_x.device) for a in range(2)]
    T_out = [T_x if a == f else torch.empty(_face_shapes[a] + (2,), device=psi_x.device) for a in range(2)]
    sc.midpoint([u_x0, u_y0], scratch, float(np.float32(dt)), psi_out=psi_out, T_out=T_out)
    _midpoint_dt[f] = float(np.float32(dt))


def advect_u(u_x0, u_y0, u_x1, u_y1, T_x, T_y, psi_x, psi_y, dx_):
    """u1 = T . u0(psi) on every face (2D/run_2D.py:429-441), the backward map recomputed with the
    dt of the preceding RK4_grid calls (the same psi/T, bit for bit)."""
    if len(set(_midpoint_dt.values())) != 1:
        raise RuntimeError("advect_u needs the RK4_grid calls of both families first")
    _scene().midpoint([u_x0, u_y0], [u_x1, u_y1], next(iter(_midpoint_dt.values())))


def update_particles_imp(particles_imp_, particles_init_imp_, T_x, T_y):
    """imp = cols(T) @ init_imp (2D/run_2D.py:517-524)."""
    with _d.Rows((T_x, T_y)) as T:
        _scene().update_imp2(particles_imp_, particles_init_imp_, T)


def update_particles_grad_m(C_x_, C_y_, init_C_x_, init_C_y_, T_x, T_y):
    """C = T^T-sandwich of init_C (2D/run_2D.py:526-536)."""
    with _d.Rows((C_x_, C_y_), out=True) as C, _d.Rows((init_C_x_, init_C_y_)) as C0, _d.Rows((T_x, T_y)) as T:
        _scene().update_grad_m2(C, C0, T)


def update_T(T_x_, T_y_, T_x_init_, T_y_init_, T_x_grad_m_, T_y_grad_m_):
    """T = cols(T_grad_m) @ cols(T_init) (2D/run_2D.py:538-546)."""
    with _d.Rows((T_x_, T_y_), out=True) as T, _d.Rows((T_x_init_, T_y_init_)) as Ti, \
            _d.Rows((T_x_grad_m_, T_y_grad_m_)) as Tg:
        _scene().update_T2(T, Ti, Tg)


def P2G(particles_imp_, particles_pos_, u_x_, u_y_, psi_, psi_x_grid_, psi_y_grid_, p2g_weight_x_, p2g_weight_y_):
    """APIC P2G of the impulse (with the module's C_x/C_y) and of the reference map psi
    (2D/run_2D.py:548-611); deterministic."""
    with _d.Rows((C_x, C_y)) as C:  # noqa: F821
        _scene().p2g2(particles_imp_, particles_pos_, C, psi_, [u_x_, u_y_], [p2g_weight_x_, p2g_weight_y_],
                      psi_out=[psi_x_grid_, psi_y_grid_])


def split_central_vector(vc, u_x_, u_y_):
    _scene().split_central_vector(vc, [u_x_, u_y_])


def advect_smoke(smoke0, smoke1, psi_x, psi_y, dx_):
    """smoke1 = smoke0 at the cell-centre average of the face backward maps, bilinear
    (2D/run_2D.py:444-450); smoke grids [nx, ny, 3], psi grids [F, 2]."""
    _scene().advect_smoke(smoke0, smoke1, [psi_x, psi_y], dx=float(dx_))


# ---------------------------------------------------------------------------------------------
# main loop (2D/run_2D.py:676-976)
# ---------------------------------------------------------------------------------------------
def main(from_frame=0, testing=False, logs_root="logs"):
    from_frame = max(0, from_frame)
    logsdir = os.path.join(logs_root, exp_name)  # noqa: F405
    ckptdir = os.path.join(logsdir, "ckpts")
    os.makedirs(ckptdir, exist_ok=True)
    U = [u_x, u_y]  # noqa: F821
    if from_frame <= 0:
        leapfrog_vel_func(u, X)  # noqa: F821
        split_central_vector(u, u_x, u_y)  # noqa: F821
        solver.Poisson(u_x, u_y)  # noqa: F821
        stripe_func(smoke, X, 0.25, 0.48)  # noqa: F821
    else:
        for t, n in zip(U, "xy"):
            t.copy_(torch.from_numpy(np.load(os.path.join(ckptdir, f"vel_{n}_numpy_{from_frame}.npy"))))
        smoke.copy_(torch.from_numpy(np.load(os.path.join(ckptdir, f"smoke_numpy_{from_frame}.npy"))))  # noqa: F821
    # vorticity for the frame output (2D/run_2D.py:741-742); the image writers are not built
    get_central_vector(u_x, u_y, u)  # noqa: F821
    curl(u, w, dx)  # noqa: F821
    if save_ckpt:  # noqa: F405
        for t, n in zip(U, "xy"):
            np.save(os.path.join(ckptdir, f"vel_{n}_numpy_{from_frame}"), t.cpu().numpy())
        np.save(os.path.join(ckptdir, f"smoke_numpy_{from_frame}"), smoke.cpu().numpy())  # noqa: F821

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
                init_particles_pos_uniform(particles_pos, X, res_x, particles_per_cell, dx,  # noqa: F405,F821
                                           particles_per_cell_axis, dist_between_neighbor)
            ik = i
            backup_particles_pos(particles_pos, particles_pos_backup)  # noqa: F821
            init_particles_imp(particles_imp, particles_init_imp, particles_pos, *U, init_C_x, init_C_y, dx)  # noqa: F821
            reset_to_identity(psi, T_x, T_y)  # noqa: F821
            reset_T_to_identity(T_x_init, T_y_init)  # noqa: F821
        k = (i - ik) % reinit_every_grad_m  # noqa: F405
        if k == 0:
            init_particles_imp_grad_m(particles_init_imp_grad_m, particles_pos, *U, init_C_x, init_C_y, dx)  # noqa: F821
            reset_T_to_identity(T_x_grad_m, T_y_grad_m)  # noqa: F821
            _T_init.copy_(_T)  # copy_to(T_x, T_x_init); copy_to(T_y, T_y_init)  # noqa: F821
        if use_midpoint_vel:  # noqa: F405
            # reset_to_identity_grid + RK4_grid x2 + copy_to + advect_u (2D/run_2D.py:866-871)
            tmp_u_x.copy_(u_x)  # noqa: F821
            tmp_u_y.copy_(u_y)  # noqa: F821
            _scene().midpoint([tmp_u_x, tmp_u_y], U, float(np.float32(0.5 * curr_dt)))  # noqa: F821
            solver.Poisson(*U)  # noqa: F821
        stretch_T_and_advect_particles(particles_pos, T_x_grad_m, T_y_grad_m, *U, curr_dt)  # noqa: F821
        update_particles_grad_m(C_x, C_y, init_C_x, init_C_y, T_x_grad_m, T_y_grad_m)  # noqa: F821
        update_T(T_x, T_y, T_x_init, T_y_init, T_x_grad_m, T_y_grad_m)  # noqa: F821
        update_particles_imp(particles_imp, particles_init_imp, T_x, T_y)  # noqa: F821
        P2G(particles_imp, particles_pos, *U, psi, psi_x_grid, psi_y_grid, p2g_weight_x, p2g_weight_y)  # noqa: F821
        solver.Poisson(*U)  # noqa: F821
        torch.cuda.synchronize()
        frame_time = time.time() - start_time
        if i <= total_steps - 1:  # noqa: F405
            frame_times[i] = frame_time
        print(f"[Simulate] Done with step: {i} / substep: {j}, step time {frame_time:.6f} s, "
              f"MGPCG iterations {solver.last_info.iterations}", flush=True)  # noqa: F821
        done = False
        if output_frame:
            get_central_vector(u_x, u_y, u)  # noqa: F821
            curl(u, w, dx)  # noqa: F821
            if save_ckpt and frame_idx % ckpt_every == 0:  # noqa: F405
                for t, n in zip(U, "xy"):
                    np.save(os.path.join(ckptdir, f"vel_{n}_numpy_{frame_idx}"), t.cpu().numpy())
                np.save(os.path.join(ckptdir, f"smoke_numpy_{frame_idx}"), smoke.cpu().numpy())  # noqa: F821
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
