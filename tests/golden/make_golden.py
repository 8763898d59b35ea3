"""Generate the golden vectors by running the reference's own Python/Taichi source.

Run where the reference is checked out, with its root directory (the one holding ``2D/`` and
``3D/``) as the first argument::

    python tests/golden/make_golden.py REFERENCE_ROOT ref3d_kernels   # per-kernel cases, 3D
    python tests/golden/make_golden.py REFERENCE_ROOT ref2d_kernels   # per-kernel cases, 2D
    python tests/golden/make_golden.py REFERENCE_ROOT ref3d_steps     # run_3D.main(): 10 steps at 8^3
    python tests/golden/make_golden.py REFERENCE_ROOT ref3d_steps16   # run_3D.main(): 3 steps at 16^3
    python tests/golden/make_golden.py REFERENCE_ROOT ref2d_steps     # run_2D.main(): 20 steps at 32^2
    python tests/golden/make_golden.py REFERENCE_ROOT ref3d_fields    # smoke transport + curl, 16x12x8
    python tests/golden/make_golden.py REFERENCE_ROOT ref2d_fields    # advect_smoke + curl, 32x24
    python tests/golden/make_golden.py REFERENCE_ROOT ref3d_variants  # the "evolve m" kernels, 12x10x8
    python tests/golden/make_golden.py REFERENCE_ROOT ref3d_mgpcg     # MGPCG_3.Poisson, 32^3, 3 levels

Taichi 1.5.0 is not installable here, so the reference modules are executed through
``oracle/ref_shim`` (a restatement of the Taichi semantics the step uses: f32 arithmetic,
truncating ``int()``, sequential struct-for, in-place atomics).  Every kernel, ``@ti.func`` and
the ``main()`` driver that produces the numbers is the reference's unmodified source; only the
``hyperparameters`` module (grid size, reinit cadence), the image/VTK writers (``io_utils``) and the
2D driver's missing ``single_vortex`` import are replaced.  Each case writes one
``tests/golden/<case>.npz``.
"""
import contextlib
import io
import os
import re
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = None  # the reference checkout, from the command line
sys.path.insert(0, os.path.join(REPO, "oracle", "ref_shim"))
import loader  # noqa: E402

IO_STUB = dict(np=np, os=os, remove_everything_in=lambda d: None,
               write_field=lambda *a, **k: None, write_image=lambda *a, **k: None,
               write_w_and_smoke=lambda *a, **k: None, write_particles=lambda *a, **k: None)


def hp3d(res, **over):
    hp = dict(case=0, dim=3, use_midpoint_vel=True, forward_update_T=True, use_APIC=True,
              use_APIC_smoke=True, save_particle_pos_numpy=False, save_particle_imp_numpy=False,
              save_frame_each_step=False, reinit_particle_pos=True, min_res=(8, 8, 8), num_levels=4,
              feat_dim=4, activate_threshold=0.032, N_iters=1, N_batch=1, success_threshold=2e-7,
              res_x=res[0], res_y=res[1], res_z=res[2], visualize_dt=0.1, reinit_every=20,
              reinit_every_grad_m=1, ckpt_every=1, CFL=0.5, from_frame=0, total_frames=10 ** 6,
              use_total_steps=True, total_steps=1, exp_name="golden3d", particles_per_cell=8,
              total_particles_num_ratio=1, cell_max_particle_num_ratio=1.6)
    hp.update(over)
    return hp


def hp2d(res, **over):
    hp = dict(dim=2, testing=False, use_neural=False, save_ckpt=True, save_frame_each_step=False,
              use_BFECC=False, use_midpoint_vel=True, use_APIC=True, forward_update_T=True,
              plot_particles=False, use_reseed_particles=False, reinit_particle_pos=True, dpi_vor=64,
              min_res=(8, 8), num_levels=4, feat_dim=2, activate_threshold=0.03, N_iters=1, N_batch=1,
              success_threshold=3e-8, res_x=res[0], res_y=res[1], visualize_dt=0.1, reinit_every=12,
              reinit_every_grad_m=8, ckpt_every=1, CFL=0.5, from_frame=0, total_frames=10 ** 6,
              use_total_steps=True, total_steps=1, exp_name="golden2d", particles_per_cell=4,
              total_particles_num_ratio=1, cell_max_particle_num_ratio=2.0,
              min_particles_per_cell_ratio=1, min_particles_per_cell=4,
              max_particles_per_cell_ratio=1.6, max_particles_per_cell=6,
              max_delete_particle_try_num=100000)
    hp.update(over)
    return hp


def load3d(hp):
    loader.install(os.path.join(REF, "3D"), ["taichi_utils", "mgpcg", "init_conditions", "run_3D"],
                   hp, {"io_utils": IO_STUB})
    import run_3D
    return run_3D


def load2d(hp):
    sv = dict(vortex_vel_func_point=None, dvxdx=None, dvxdy=None, dvydx=None, dvydy=None)
    loader.install(os.path.join(REF, "2D"), ["taichi_utils", "mgpcg", "init_conditions", "run_2D"],
                   hp, {"io_utils": IO_STUB, "single_vortex": sv})
    import run_2D
    return run_2D


def smooth_field(shape, rng, amp=1.0, dx=1.0):
    """A smooth random grid field (sum of a few low sine modes) for kernel inputs."""
    idx = np.meshgrid(*[np.arange(s, dtype=np.float64) for s in shape], indexing="ij")
    out = np.zeros(shape)
    for _ in range(4):
        k = rng.uniform(0.5, 2.5, size=len(shape))
        ph = rng.uniform(0, 2 * np.pi, size=len(shape))
        term = rng.uniform(-1, 1)
        for d in range(len(shape)):
            term = term * np.sin(2 * np.pi * k[d] * idx[d] * dx + ph[d])
        out += term
    return (amp * out).astype(np.float32)


def vec_field_np(f):
    return f.to_numpy().astype(np.float32)


def set_vec(f, arr):
    f.from_numpy(np.asarray(arr, dtype=np.float32))


# ------------------------------------------------------------------------------------------------
# 3D per-kernel cases (16^3 grid, so MGPCG runs a 2-level V-cycle)
# ------------------------------------------------------------------------------------------------
def ref3d_kernels():
    import taichi as ti
    res = (16, 16, 16)
    R = load3d(hp3d(res))
    import init_conditions as IC
    import mgpcg as MG
    rng = np.random.default_rng(1234)
    dx = R.dx
    out = {"res": np.array(res), "dx": np.float32(dx)}
    nx, ny, nz = res
    ux = smooth_field((nx + 1, ny, nz), rng, 0.6, 1 / 16)
    uy = smooth_field((nx, ny + 1, nz), rng, 0.6, 1 / 16)
    uz = smooth_field((nx, ny, nz + 1), rng, 0.6, 1 / 16)
    out.update(u_x=ux, u_y=uy, u_z=uz)
    R.u_x.from_numpy(ux); R.u_y.from_numpy(uy); R.u_z.from_numpy(uz)

    R.calc_max_speed(R.u_x, R.u_y, R.u_z)
    out["max_speed"] = np.float32(R.max_speed[None])

    n = 512
    pos = rng.uniform(0.0, 1.0, size=(n, 3)).astype(np.float32)
    pos[:8] = np.array([[0.001, 0.5, 0.5], [0.999, 0.5, 0.5], [0.5, 0.0005, 0.5], [0.5, 0.5, 0.9999],
                        [-0.01, 0.3, 0.3], [1.004, 0.6, 0.7], [0.03, 0.97, 0.02], [0.5, 0.5, 0.5]],
                       dtype=np.float32)
    out["pos"] = pos
    T = (np.eye(3)[None] + 0.05 * rng.standard_normal((n, 3, 3))).astype(np.float32)  # [p, vec, comp]
    out["T_gm"] = T
    T_init = (np.eye(3)[None] + 0.05 * rng.standard_normal((n, 3, 3))).astype(np.float32)
    out["T_init"] = T_init
    C = (0.5 * rng.standard_normal((n, 3, 3))).astype(np.float32)
    out["init_C"] = C
    imp0 = (0.5 * rng.standard_normal((n, 3))).astype(np.float32)
    out["init_imp"] = imp0
    dt = np.float32(0.4 * dx / out["max_speed"])
    out["dt"] = dt

    mk = lambda: ti.Vector.field(3, float, shape=n)  # noqa: E731
    # G2P of impulse and its gradient (init_conditions.py:266-273)
    p_f, imp_f, Cx, Cy, Cz = mk(), mk(), mk(), mk(), mk()
    set_vec(p_f, pos)
    IC.init_particles_imp_grad_m(imp_f, p_f, R.u_x, R.u_y, R.u_z, Cx, Cy, Cz, dx)
    out["g2p_imp"] = vec_field_np(imp_f)
    out["g2p_C"] = np.stack([vec_field_np(Cx), vec_field_np(Cy), vec_field_np(Cz)], axis=1)

    # RK4_T_forward (run_3D.py:175-219)
    p_f = mk(); set_vec(p_f, pos)
    Tx, Ty, Tz = mk(), mk(), mk()
    set_vec(Tx, T[:, 0]); set_vec(Ty, T[:, 1]); set_vec(Tz, T[:, 2])
    R.RK4_T_forward(p_f, Tx, Ty, Tz, R.u_x, R.u_y, R.u_z, dt)
    out["rk4_pos"] = vec_field_np(p_f)
    out["rk4_T"] = np.stack([vec_field_np(Tx), vec_field_np(Ty), vec_field_np(Tz)], axis=1)

    # update_T (run_3D.py:430-439)
    Ti = [mk() for _ in range(3)]
    Tg = [mk() for _ in range(3)]
    for v in range(3):
        set_vec(Ti[v], T_init[:, v]); set_vec(Tg[v], T[:, v])
    R.update_T(*Ti, *Tg)
    out["update_T"] = np.stack([vec_field_np(f) for f in Ti], axis=1)

    # P2G (run_3D.py:441-552); init_C is read from the module globals init_C_[xyz]
    for v, f in enumerate([R.init_C_x, R.init_C_y, R.init_C_z]):
        a = f.to_numpy(); a[:n] = C[:, v]; f.from_numpy(a)
    p_f = mk(); set_vec(p_f, pos)
    imp_f = mk(); set_vec(imp_f, imp0)
    Ti = [mk() for _ in range(3)]
    Tg = [mk() for _ in range(3)]
    for v in range(3):
        set_vec(Ti[v], T_init[:, v]); set_vec(Tg[v], T[:, v])
    ux_f = ti.field(float, shape=(nx + 1, ny, nz)); uy_f = ti.field(float, shape=(nx, ny + 1, nz))
    uz_f = ti.field(float, shape=(nx, ny, nz + 1))
    wx = ti.field(float, shape=(nx + 1, ny, nz)); wy = ti.field(float, shape=(nx, ny + 1, nz))
    wz = ti.field(float, shape=(nx, ny, nz + 1))
    R.P2G(imp_f, mk(), p_f, ux_f, uy_f, uz_f, wx, wy, wz, *Tg, *Ti, R.cell_particles_id,
          R.cell_particle_num)
    out.update(p2g_u_x=ux_f.to_numpy(), p2g_u_y=uy_f.to_numpy(), p2g_u_z=uz_f.to_numpy(),
               p2g_w_x=wx.to_numpy(), p2g_w_y=wy.to_numpy(), p2g_w_z=wz.to_numpy())

    # particle binning (run_3D.py:342-351) on the module's own particle field
    allp = np.zeros((R.particle_num, 3), np.float32)
    allp[:] = rng.uniform(0.0, 1.0, size=(R.particle_num, 3))
    R.particles_pos.from_numpy(allp)
    R.get_particles_id_in_every_cell(R.cell_particles_id, R.cell_particle_num, R.particles_pos)
    out["bin_pos"] = allp
    out["bin_count"] = R.cell_particle_num.to_numpy()

    # midpoint grid step (run_3D.py:779-788 without the projection)
    R.reset_to_identity_grid(R.psi_x_grid, R.psi_y_grid, R.psi_z_grid, R.T_x_grid, R.T_y_grid,
                             R.T_z_grid)
    R.RK4_grid(R.psi_x_grid, R.T_x_grid, R.u_x, R.u_y, R.u_z, 0.5 * float(dt))
    R.RK4_grid(R.psi_y_grid, R.T_y_grid, R.u_x, R.u_y, R.u_z, 0.5 * float(dt))
    R.RK4_grid(R.psi_z_grid, R.T_z_grid, R.u_x, R.u_y, R.u_z, 0.5 * float(dt))
    R.copy_to(R.u_x, R.p2g_weight_x); R.copy_to(R.u_y, R.p2g_weight_y)
    R.copy_to(R.u_z, R.p2g_weight_z)
    R.advect_u(R.p2g_weight_x, R.p2g_weight_y, R.p2g_weight_z, R.u_x, R.u_y, R.u_z, R.T_x_grid,
               R.T_y_grid, R.T_z_grid, R.psi_x_grid, R.psi_y_grid, R.psi_z_grid, dx)
    out.update(mid_u_x=R.u_x.to_numpy(), mid_u_y=R.u_y.to_numpy(), mid_u_z=R.u_z.to_numpy(),
               mid_psi_x=R.psi_x_grid.to_numpy(), mid_T_x=R.T_x_grid.to_numpy(),
               mid_psi_z=R.psi_z_grid.to_numpy(), mid_T_z=R.T_z_grid.to_numpy())

    # MGPCG_3.Poisson (mgpcg.py:425-430) on the midpoint field, 16^3 -> 2 levels
    log = io.StringIO()
    with contextlib.redirect_stdout(log):
        R.solver.Poisson(R.u_x, R.u_y, R.u_z)
    out.update(poisson_u_x=R.u_x.to_numpy(), poisson_u_y=R.u_y.to_numpy(),
               poisson_u_z=R.u_z.to_numpy(), poisson_p=R.solver.p.to_numpy(),
               poisson_iters=np.int32(parse_iters(log.getvalue())[-1]))

    # a non-cubic grid: 32x16x16, 2 levels
    N2 = [32, 16, 16]
    s2 = MG.MGPCG_3(boundary_types=R.boundary_types, N=N2, base_level=3)
    fx = ti.field(float, shape=(33, 16, 16)); fy = ti.field(float, shape=(32, 17, 16))
    fz = ti.field(float, shape=(32, 16, 17))
    a, b, c = (smooth_field(f.shape, rng, 0.3, 1 / 16) for f in (fx, fy, fz))
    fx.from_numpy(a); fy.from_numpy(b); fz.from_numpy(c)
    out.update(poisson2_in_x=a, poisson2_in_y=b, poisson2_in_z=c)
    log = io.StringIO()
    with contextlib.redirect_stdout(log):
        s2.Poisson(fx, fy, fz)
    out.update(poisson2_u_x=fx.to_numpy(), poisson2_u_y=fy.to_numpy(), poisson2_u_z=fz.to_numpy(),
               poisson2_p=s2.p.to_numpy(), poisson2_iters=np.int32(parse_iters(log.getvalue())[-1]))
    return out


def parse_iters(text):
    its = [int(m) for m in re.findall(r"Converged at iter:\s+(\d+)", text)]
    its += [-int(m) for m in re.findall(r"without converging at iter:\s+(\d+)", text)]
    return its or [-1]


# ------------------------------------------------------------------------------------------------
# 2D per-kernel cases (32^2 grid -> 3 MG levels)
# ------------------------------------------------------------------------------------------------
def ref2d_kernels():
    import taichi as ti
    res = (32, 32)
    R = load2d(hp2d(res))
    import init_conditions as IC
    import mgpcg as MG
    rng = np.random.default_rng(4321)
    dx = R.dx
    nx, ny = res
    out = {"res": np.array(res), "dx": np.float32(dx)}
    ux = smooth_field((nx + 1, ny), rng, 0.6, 1 / 32)
    uy = smooth_field((nx, ny + 1), rng, 0.6, 1 / 32)
    out.update(u_x=ux, u_y=uy)
    R.u_x.from_numpy(ux); R.u_y.from_numpy(uy)
    R.calc_max_speed(R.u_x, R.u_y)
    out["max_speed"] = np.float32(R.max_speed[None])
    dt = np.float32(0.4 * dx / out["max_speed"])
    out["dt"] = dt

    n = 512
    pos = rng.uniform(0.0, 1.0, size=(n, 2)).astype(np.float32)
    pos[:6] = np.array([[0.001, 0.5], [0.9995, 0.5], [0.5, 0.0004], [-0.01, 0.3], [1.006, 0.6],
                        [0.5, 0.5]], dtype=np.float32)
    out["pos"] = pos
    T = (np.eye(2)[None] + 0.05 * rng.standard_normal((n, 2, 2))).astype(np.float32)
    T_init = (np.eye(2)[None] + 0.05 * rng.standard_normal((n, 2, 2))).astype(np.float32)
    C = (0.5 * rng.standard_normal((n, 2, 2))).astype(np.float32)
    imp0 = (0.5 * rng.standard_normal((n, 2))).astype(np.float32)
    psi = (pos + 0.01 * rng.standard_normal((n, 2))).astype(np.float32)
    out.update(T_gm=T, T_init=T_init, init_C=C, init_imp=imp0, psi=psi)
    mk = lambda: ti.Vector.field(2, float, shape=n)  # noqa: E731

    # G2P (init_conditions.py:184-210)
    p_f, imp_f, init_f, Cx, Cy = mk(), mk(), mk(), mk(), mk()
    set_vec(p_f, pos)
    IC.init_particles_imp(imp_f, init_f, p_f, R.u_x, R.u_y, Cx, Cy, dx)
    out["g2p_imp"] = vec_field_np(init_f)
    IC.init_particles_imp_grad_m(imp_f, p_f, R.u_x, R.u_y, Cx, Cy, dx)
    out["g2p_C"] = np.stack([vec_field_np(Cx), vec_field_np(Cy)], axis=1)

    # RK4_T_forward with advect_psi=1 (run_2D.py:304-341)
    p_f = mk(); set_vec(p_f, pos)
    Tx, Ty = mk(), mk(); set_vec(Tx, T[:, 0]); set_vec(Ty, T[:, 1])
    R.RK4_T_forward(p_f, Tx, Ty, R.u_x, R.u_y, dt, 1)
    out["rk4_pos"] = vec_field_np(p_f)
    out["rk4_T"] = np.stack([vec_field_np(Tx), vec_field_np(Ty)], axis=1)

    # update_particles_grad_m / update_T / update_particles_imp (run_2D.py:517-546)
    Cx, Cy, iCx, iCy, Tgx, Tgy = mk(), mk(), mk(), mk(), mk(), mk()
    set_vec(iCx, C[:, 0]); set_vec(iCy, C[:, 1]); set_vec(Tgx, T[:, 0]); set_vec(Tgy, T[:, 1])
    R.update_particles_grad_m(Cx, Cy, iCx, iCy, Tgx, Tgy)
    out["grad_m_C"] = np.stack([vec_field_np(Cx), vec_field_np(Cy)], axis=1)
    Tx, Ty, Tix, Tiy = mk(), mk(), mk(), mk()
    set_vec(Tix, T_init[:, 0]); set_vec(Tiy, T_init[:, 1])
    R.update_T(Tx, Ty, Tix, Tiy, Tgx, Tgy)
    out["update_T"] = np.stack([vec_field_np(Tx), vec_field_np(Ty)], axis=1)
    imp_f, init_f = mk(), mk(); set_vec(init_f, imp0)
    R.update_particles_imp(imp_f, init_f, Tx, Ty)
    out["update_imp"] = vec_field_np(imp_f)

    # P2G (run_2D.py:548-611): reads the module globals C_x, C_y
    for v, f in enumerate([R.C_x, R.C_y]):
        a = f.to_numpy(); a[:n] = C[:, v]; f.from_numpy(a)
    p_f = mk(); set_vec(p_f, pos)
    imp_f = mk(); set_vec(imp_f, imp0)
    psi_f = mk(); set_vec(psi_f, psi)
    fx = ti.field(float, shape=(nx + 1, ny)); fy = ti.field(float, shape=(nx, ny + 1))
    wx = ti.field(float, shape=(nx + 1, ny)); wy = ti.field(float, shape=(nx, ny + 1))
    gx = ti.Vector.field(2, float, shape=(nx + 1, ny)); gy = ti.Vector.field(2, float, shape=(nx, ny + 1))
    R.P2G(imp_f, p_f, fx, fy, psi_f, gx, gy, wx, wy)
    out.update(p2g_u_x=fx.to_numpy(), p2g_u_y=fy.to_numpy(), p2g_w_x=wx.to_numpy(),
               p2g_w_y=wy.to_numpy(), p2g_psi_x=gx.to_numpy(), p2g_psi_y=gy.to_numpy())

    # midpoint (run_2D.py:866-871 without the projection)
    R.reset_to_identity_grid(R.psi_x_grid, R.psi_y_grid, R.T_x_grid, R.T_y_grid)
    R.RK4_grid(R.psi_x_grid, R.T_x_grid, R.u_x, R.u_y, 0.5 * float(dt))
    R.RK4_grid(R.psi_y_grid, R.T_y_grid, R.u_x, R.u_y, 0.5 * float(dt))
    R.copy_to(R.u_x, R.tmp_u_x); R.copy_to(R.u_y, R.tmp_u_y)
    R.advect_u(R.tmp_u_x, R.tmp_u_y, R.u_x, R.u_y, R.T_x_grid, R.T_y_grid, R.psi_x_grid,
               R.psi_y_grid, dx)
    out.update(mid_u_x=R.u_x.to_numpy(), mid_u_y=R.u_y.to_numpy(), mid_psi_x=R.psi_x_grid.to_numpy(),
               mid_T_x=R.T_x_grid.to_numpy(), mid_psi_y=R.psi_y_grid.to_numpy(),
               mid_T_y=R.T_y_grid.to_numpy())

    # MGPCG_2.Poisson (mgpcg.py:342-347), 32^2 -> 3 levels
    log = io.StringIO()
    with contextlib.redirect_stdout(log):
        R.solver.Poisson(R.u_x, R.u_y)
    out.update(poisson_u_x=R.u_x.to_numpy(), poisson_u_y=R.u_y.to_numpy(),
               poisson_p=R.solver.p.to_numpy(), poisson_iters=np.int32(parse_iters(log.getvalue())[-1]))

    # 64x32 domain (the reference's 4:1 aspect, shrunk), 3 levels
    s2 = MG.MGPCG_2(boundary_types=R.boundary_types, N=[64, 32], base_level=3)
    fx = ti.field(float, shape=(65, 32)); fy = ti.field(float, shape=(64, 33))
    a, b = smooth_field(fx.shape, rng, 0.3, 1 / 32), smooth_field(fy.shape, rng, 0.3, 1 / 32)
    fx.from_numpy(a); fy.from_numpy(b)
    out.update(poisson2_in_x=a, poisson2_in_y=b)
    log = io.StringIO()
    with contextlib.redirect_stdout(log):
        s2.Poisson(fx, fy)
    out.update(poisson2_u_x=fx.to_numpy(), poisson2_u_y=fy.to_numpy(), poisson2_p=s2.p.to_numpy(),
               poisson2_iters=np.int32(parse_iters(log.getvalue())[-1]))
    return out


# ------------------------------------------------------------------------------------------------
# whole-step runs through the reference's own main()
# ------------------------------------------------------------------------------------------------
def _run_main(R, nsteps, snap_particles_at, particle_fields, grid_fields, extra=None):
    """Run ``R.main()`` and snapshot after every step's final projection."""
    snaps = {}
    state = {"calls": 0, "step": 0, "log": io.StringIO()}
    solver = R.solver
    orig = solver.Poisson
    per_step = 2 if R.use_midpoint_vel else 1

    def hooked(*args, **kw):
        orig(*args, **kw)
        state["calls"] += 1
        c = state["calls"] - 1  # call 0 is the initial-condition projection
        if c == 0:
            for name in grid_fields:
                snaps[f"init_{name}"] = getattr(R, name).to_numpy()
            return
        if (c - 1) % per_step == per_step - 1:
            s = state["step"] + 1
            state["step"] = s
            for name in grid_fields:
                snaps[f"s{s}_{name}"] = getattr(R, name).to_numpy()
            snaps[f"s{s}_p"] = solver.p.to_numpy()
            snaps[f"s{s}_max_speed"] = np.float32(R.max_speed[None])
            if s in snap_particles_at:
                for name in particle_fields:
                    snaps[f"s{s}_{name}"] = getattr(R, name).to_numpy()
            if extra:
                extra(snaps, s)
        else:
            s = state["step"] + 1
            for name in grid_fields:
                snaps[f"s{s}_mid_{name}"] = getattr(R, name).to_numpy()

    solver.Poisson = hooked
    wd = tempfile.mkdtemp()
    cwd = os.getcwd()
    try:
        os.chdir(wd)
        open("hyperparameters.py", "w").write("# golden run\n")
        with contextlib.redirect_stdout(state["log"]):
            R.main(from_frame=0)
    finally:
        os.chdir(cwd)
        shutil.rmtree(wd, ignore_errors=True)
    its = parse_iters(state["log"].getvalue())
    snaps["iters"] = np.array(its, dtype=np.int32)
    dts = [float(m) for m in re.findall(r"Visualize time ([0-9.eE+-]+)/", state["log"].getvalue())]
    snaps["log_sub_t"] = np.array(dts)
    assert state["step"] == nsteps, (state["step"], nsteps)
    return snaps


def ref3d_steps():
    nsteps = 10
    hp = hp3d((8, 8, 8), reinit_every=5, reinit_every_grad_m=2, total_steps=nsteps)
    R = load3d(hp)
    pf = ["particles_pos", "particles_init_imp", "T_x_init", "T_y_init", "T_z_init", "T_x_grad_m",
          "T_y_grad_m", "T_z_grad_m", "init_C_x", "init_C_y", "init_C_z"]
    gf = ["u_x", "u_y", "u_z"]
    snaps = _run_main(R, nsteps, {1, 2, 10}, pf, gf)
    snaps["res"] = np.array([8, 8, 8])
    snaps["hp"] = np.array([hp["reinit_every"], hp["reinit_every_grad_m"]])
    return snaps


def ref3d_steps16():
    """run_3D.main() at 16^3 (a two-level MGPCG inside the loop), 3 steps."""
    nsteps = 3
    hp = hp3d((16, 16, 16), reinit_every=5, reinit_every_grad_m=2, total_steps=nsteps)
    R = load3d(hp)
    snaps = _run_main(R, nsteps, {nsteps}, ["particles_pos", "particles_init_imp"], ["u_x", "u_y", "u_z"])
    snaps["res"] = np.array([16, 16, 16])
    snaps["hp"] = np.array([hp["reinit_every"], hp["reinit_every_grad_m"]])
    return snaps


def ref2d_steps():
    nsteps = 20
    hp = hp2d((32, 32), total_steps=nsteps)
    R = load2d(hp)
    pf = ["particles_pos", "particles_imp", "particles_init_imp", "T_x", "T_y", "T_x_init",
          "T_y_init", "T_x_grad_m", "T_y_grad_m", "init_C_x", "init_C_y", "C_x", "C_y", "psi"]
    gf = ["u_x", "u_y"]
    snaps = _run_main(R, nsteps, {1, 2, 10, 20}, pf, gf)
    snaps["res"] = np.array([32, 32])
    snaps["hp"] = np.array([hp["reinit_every"], hp["reinit_every_grad_m"]])
    return snaps


# ------------------------------------------------------------------------------------------------
# scalar (smoke) transport and diagnostics: the reference's kernels outside the live step loop
# (their call sites in main() are commented out or run only at frame output)
# ------------------------------------------------------------------------------------------------
def _face_psi(shape, fam, rng, dx, amp):
    """Backward-map face grids [F, 3]: face centres moved by a smooth field, some out of range."""
    idx = np.meshgrid(*[np.arange(s, dtype=np.float64) for s in shape], indexing="ij")
    out = np.zeros(shape + (len(shape),), np.float32)
    for d in range(len(shape)):
        x = (idx[d] + (0.0 if d == fam else 0.5)) * dx
        out[..., d] = x + smooth_field(shape, rng, amp, dx)
    return out


def ref3d_fields():
    import taichi as ti
    res = (16, 12, 8)
    R = load3d(hp3d(res))
    import init_conditions as IC
    import taichi_utils as TU
    rng = np.random.default_rng(777)
    dx = R.dx
    nx, ny, nz = res
    out = {"res": np.array(res), "dx": np.float32(dx)}
    ux = smooth_field((nx + 1, ny, nz), rng, 0.6, dx)
    uy = smooth_field((nx, ny + 1, nz), rng, 0.6, dx)
    uz = smooth_field((nx, ny, nz + 1), rng, 0.6, dx)
    out.update(u_x=ux, u_y=uy, u_z=uz)
    R.u_x.from_numpy(ux); R.u_y.from_numpy(uy); R.u_z.from_numpy(uz)

    # get_central_vector + curl (3D/taichi_utils.py:56-85)
    TU.get_central_vector(R.u_x, R.u_y, R.u_z, R.u)
    out["central"] = R.u.to_numpy()
    TU.curl(R.u, R.w, dx)
    out["curl"] = R.w.to_numpy()

    # init_particles_smoke (3D/init_conditions.py:275-279) on a smooth 4-channel smoke field
    smoke = np.stack([np.abs(smooth_field(res, rng, 0.8, dx)) for _ in range(4)], axis=-1).astype(np.float32)
    out["smoke"] = smoke
    n = 512
    pos = (rng.uniform(0.0, 1.0, size=(n, 3)) * np.array([nx, ny, nz]) * dx).astype(np.float32)
    pos[:6] = np.array([[0.001, 0.5, 0.3], [nx * dx - 0.0005, 0.4, 0.2], [0.3, -0.01, 0.3],
                        [0.5, 0.5, nz * dx + 0.004], [0.02, 0.98 * ny * dx, 0.01], [0.5, 0.5, 0.25]],
                       dtype=np.float32)
    out["pos"] = pos
    mk = lambda k: ti.Vector.field(k, float, shape=n)  # noqa: E731
    sm_f = ti.Vector.field(4, float, shape=res); sm_f.from_numpy(smoke)
    p_f = mk(3); set_vec(p_f, pos)
    s_f = mk(4)
    g_f = ti.Matrix.field(3, 4, float, shape=n)
    IC.init_particles_smoke(s_f, g_f, p_f, sm_f, dx)
    out["g2p_smoke"] = s_f.to_numpy()
    out["g2p_grad_smoke"] = g_f.to_numpy()

    # P2G_smoke (3D/run_3D.py:554-593) with T_gm, T_init and a random smoke gradient
    T = (np.eye(3)[None] + 0.05 * rng.standard_normal((n, 3, 3))).astype(np.float32)
    T_init = (np.eye(3)[None] + 0.05 * rng.standard_normal((n, 3, 3))).astype(np.float32)
    s_p = rng.uniform(0.0, 1.0, size=(n, 4)).astype(np.float32)
    G = (2.0 * rng.standard_normal((n, 3, 4))).astype(np.float32)
    out.update(T_gm=T, T_init=T_init, smoke_p=s_p, grad_smoke=G)
    s_f = mk(4); s_f.from_numpy(s_p)
    g_f = ti.Matrix.field(3, 4, float, shape=n); g_f.from_numpy(G)
    Tg = [mk(3) for _ in range(3)]
    Ti = [mk(3) for _ in range(3)]
    for v in range(3):
        set_vec(Tg[v], T[:, v]); set_vec(Ti[v], T_init[:, v])
    out_sm = ti.Vector.field(4, float, shape=res)
    wgt = ti.field(float, shape=res)
    R.P2G_smoke(s_f, g_f, p_f, out_sm, *Tg, *Ti, wgt)
    out["p2g_smoke"] = out_sm.to_numpy()
    out["p2g_smoke_w"] = wgt.to_numpy()

    # advect_smoke / clamp_smoke (3D/run_3D.py:315-334) through perturbed backward maps
    shapes = [(nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1)]
    psi = [_face_psi(shapes[f], f, rng, dx, 2.5 * dx) for f in range(3)]
    out.update(psi_x=psi[0], psi_y=psi[1], psi_z=psi[2])
    pf = [ti.Vector.field(3, float, shape=shapes[f]) for f in range(3)]
    for f in range(3):
        pf[f].from_numpy(psi[f])
    s1 = ti.Vector.field(4, float, shape=res)
    R.advect_smoke(sm_f, s1, *pf, dx)
    out["advect_smoke"] = s1.to_numpy()
    s1_in = (s1.to_numpy() + 0.3 * rng.standard_normal(res + (4,))).astype(np.float32)
    out["clamp_in"] = s1_in
    s1.from_numpy(s1_in)
    R.clamp_smoke(sm_f, s1, *pf, dx)
    out["clamp_smoke"] = s1.to_numpy()

    # add_vortex_ring_and_smoke (3D/init_conditions.py:29-56), 64 samples
    vf = ti.Vector.field(3, float, shape=res)
    smf = ti.Vector.field(4, float, shape=res)
    IC.add_vortex_ring_and_smoke(w=0.02, rad=0.2, delta=0.04, c=ti.Vector([0.45, 0.5, 0.33]),
                                 unit_x=ti.Vector([0., 0., -1.]), unit_y=ti.Vector([0., 1., 0.]),
                                 pf=R.X, vf=vf, smokef=smf, color=ti.Vector([1., 0.5, 0.25]), num_samples=64)
    out["ring_u"] = vf.to_numpy()
    out["ring_smoke"] = smf.to_numpy()
    return out


def ref2d_fields():
    import taichi as ti
    res = (32, 24)
    R = load2d(hp2d(res))
    import taichi_utils as TU
    rng = np.random.default_rng(999)
    dx = R.dx
    nx, ny = res
    out = {"res": np.array(res), "dx": np.float32(dx)}
    ux = smooth_field((nx + 1, ny), rng, 0.6, dx)
    uy = smooth_field((nx, ny + 1), rng, 0.6, dx)
    out.update(u_x=ux, u_y=uy)
    R.u_x.from_numpy(ux); R.u_y.from_numpy(uy)
    # get_central_vector + curl (2D/taichi_utils.py:50-55, 96-104)
    TU.get_central_vector(R.u_x, R.u_y, R.u)
    out["central"] = R.u.to_numpy()
    TU.curl(R.u, R.w, dx)
    out["curl"] = R.w.to_numpy()
    # advect_smoke (2D/run_2D.py:444-450)
    smoke = np.stack([np.abs(smooth_field(res, rng, 0.8, dx)) for _ in range(3)], axis=-1).astype(np.float32)
    out["smoke"] = smoke
    shapes = [(nx + 1, ny), (nx, ny + 1)]
    psi = [_face_psi(shapes[f], f, rng, dx, 2.5 * dx) for f in range(2)]
    out.update(psi_x=psi[0], psi_y=psi[1])
    pf = [ti.Vector.field(2, float, shape=shapes[f]) for f in range(2)]
    for f in range(2):
        pf[f].from_numpy(psi[f])
    s0 = ti.Vector.field(3, float, shape=res); s0.from_numpy(smoke)
    s1 = ti.Vector.field(3, float, shape=res)
    R.advect_smoke(s0, s1, *pf, dx)
    out["advect_smoke"] = s1.to_numpy()
    return out


def ref3d_variants():
    """RK4_T_and_T_grad_m_forward, update_particles_imp, update_particles_grad_m and compute_dT_dx
    (3D/run_3D.py:221-292, 353-428), whose call sites the reference's step has commented out."""
    import taichi as ti
    res = (12, 10, 8)
    R = load3d(hp3d(res))
    rng = np.random.default_rng(4242)
    dx = R.dx
    nx, ny, nz = res
    out = {"res": np.array(res), "dx": np.float32(dx)}
    ux = smooth_field((nx + 1, ny, nz), rng, 0.6, dx)
    uy = smooth_field((nx, ny + 1, nz), rng, 0.6, dx)
    uz = smooth_field((nx, ny, nz + 1), rng, 0.6, dx)
    out.update(u_x=ux, u_y=uy, u_z=uz)
    R.u_x.from_numpy(ux); R.u_y.from_numpy(uy); R.u_z.from_numpy(uz)
    R.calc_max_speed(R.u_x, R.u_y, R.u_z)
    dt = np.float32(0.4 * dx / float(R.max_speed[None]))
    out["dt"] = dt

    # every cell holds 8 particles (a jittered 2x2x2 lattice); interior particles (whose 4x4x4
    # neighbour cells lie in the grid) come first, so compute_dT_dx is evaluated on them only
    cells = np.stack(np.meshgrid(*[np.arange(r) for r in res], indexing="ij"), -1).reshape(-1, 3)
    sub = np.stack(np.meshgrid(*[np.arange(2)] * 3, indexing="ij"), -1).reshape(-1, 3)
    x0 = ((cells[:, None, :] * 2 + sub[None, :, :]).reshape(-1, 3) + rng.uniform(0.05, 0.95, (cells.shape[0] * 8, 3)))
    x0 = (x0 * (dx / 2)).astype(np.float32)
    base = np.floor(x0 / np.float32(dx)).astype(int)
    inner = np.all((base >= 1) & (base <= np.array(res) - 3), axis=1)
    order = np.concatenate([np.nonzero(inner)[0], np.nonzero(~inner)[0]])
    x0 = x0[order]
    n_in = int(inner.sum())
    P = x0.shape[0]
    xc = np.clip(x0 + rng.normal(0, 0.2 * dx, x0.shape), 1e-4, np.array(res) * dx - 1e-4).astype(np.float32)
    T = (np.eye(3)[None] + 0.05 * rng.standard_normal((P, 3, 3))).astype(np.float32)
    T2 = (np.eye(3)[None] + 0.05 * rng.standard_normal((P, 3, 3))).astype(np.float32)
    C0 = (0.5 * rng.standard_normal((P, 3, 3))).astype(np.float32)
    m0 = (0.5 * rng.standard_normal((P, 3))).astype(np.float32)
    out.update(init_pos=x0, pos=xc, T=T, T2=T2, init_C=C0, init_imp=m0, n_inner=np.int32(n_in))
    mk = lambda: ti.Vector.field(3, float, shape=P)  # noqa: E731

    # RK4_T_and_T_grad_m_forward on the current positions
    p_f = mk(); set_vec(p_f, xc)
    Ta = [mk() for _ in range(3)]
    Tb = [mk() for _ in range(3)]
    for v in range(3):
        set_vec(Ta[v], T[:, v]); set_vec(Tb[v], T2[:, v])
    R.RK4_T_and_T_grad_m_forward(p_f, *Ta, *Tb, R.u_x, R.u_y, R.u_z, dt)
    out["rk4_pos"] = vec_field_np(p_f)
    out["rk4_T"] = np.stack([vec_field_np(f) for f in Ta], axis=1)
    out["rk4_T2"] = np.stack([vec_field_np(f) for f in Tb], axis=1)

    # update_particles_imp
    Tf = [mk() for _ in range(3)]
    for v in range(3):
        set_vec(Tf[v], T[:, v])
    imp_f, m_f = mk(), mk(); set_vec(m_f, m0)
    R.update_particles_imp(imp_f, m_f, *Tf)
    out["update_imp"] = vec_field_np(imp_f)

    # compute_dT_dx on the cell lists of the current positions (cap cell_max_particle_num).  Its
    # inner loop ti.ndrange(0, cell_particle_num[..]) is a two-axis range whose first axis is
    # empty, so the reference's kernel accumulates nothing and grad_T_init stays zero.
    pc_f = mk(); set_vec(pc_f, xc)
    R.get_particles_id_in_every_cell(R.cell_particles_id, R.cell_particle_num, pc_f)
    x0_f = mk(); set_vec(x0_f, x0)
    gT = [ti.Matrix.field(3, 3, float, shape=n_in) for _ in range(3)]
    R.compute_dT_dx(*gT, *Tf, x0_f, R.cell_particles_id, R.cell_particle_num)
    gTn = np.stack([f.to_numpy() for f in gT], axis=1)  # [n_in, r, a, b]
    out["dT_dx"] = gTn
    out["cap"] = np.int32(R.cell_max_particle_num)

    # update_particles_grad_m with a random grad_T_init (inner particles)
    n = n_in
    gT_in = (0.5 * rng.standard_normal((n, 3, 3, 3))).astype(np.float32)
    out["grad_T_init"] = gT_in
    for r in range(3):
        gT[r].from_numpy(gT_in[:, r])
    mk_n = lambda: ti.Vector.field(3, float, shape=n)  # noqa: E731
    Cf = [mk_n() for _ in range(3)]
    iC = [mk_n() for _ in range(3)]
    Tn = [mk_n() for _ in range(3)]
    for v in range(3):
        set_vec(iC[v], C0[:n, v]); set_vec(Tn[v], T[:n, v])
    mn = mk_n(); set_vec(mn, m0[:n])
    R.update_particles_grad_m(*Cf, *iC, *Tn, *gT, mn)
    out["grad_m_C"] = np.stack([vec_field_np(f) for f in Cf], axis=1)
    return out


# ------------------------------------------------------------------------------------------------
# 3D MGPCG with a deeper hierarchy: 32^3 -> 3 levels (32, 16, 8)
# ------------------------------------------------------------------------------------------------
def ref3d_mgpcg():
    n = 32
    R = load3d(hp3d((n, n, n)))
    import mgpcg as MG
    import taichi as ti
    rng = np.random.default_rng(7)
    s = MG.MGPCG_3(boundary_types=R.boundary_types, N=[n, n, n], base_level=3)
    fx = ti.field(float, shape=(n + 1, n, n)); fy = ti.field(float, shape=(n, n + 1, n))
    fz = ti.field(float, shape=(n, n, n + 1))
    a, b, c = (smooth_field(f.shape, rng, 0.3, 1 / n) for f in (fx, fy, fz))
    fx.from_numpy(a); fy.from_numpy(b); fz.from_numpy(c)
    out = {"in_x": a, "in_y": b, "in_z": c, "levels": np.int32(s.n_mg_levels)}
    log = io.StringIO()
    with contextlib.redirect_stdout(log):
        s.Poisson(fx, fy, fz)
    out.update(u_x=fx.to_numpy(), u_y=fy.to_numpy(), u_z=fz.to_numpy(), p=s.p.to_numpy(),
               iters=np.int32(parse_iters(log.getvalue())[-1]))
    return out


CASES = dict(ref3d_kernels=ref3d_kernels, ref2d_kernels=ref2d_kernels, ref3d_steps=ref3d_steps,
             ref2d_steps=ref2d_steps, ref3d_fields=ref3d_fields, ref2d_fields=ref2d_fields,
             ref3d_variants=ref3d_variants, ref3d_mgpcg=ref3d_mgpcg, ref3d_steps16=ref3d_steps16)

if __name__ == "__main__":
    if len(sys.argv) != 3 or sys.argv[2] not in CASES:
        sys.exit("usage: make_golden.py REFERENCE_ROOT CASE  (CASE: %s)" % ", ".join(CASES))
    REF = os.path.abspath(sys.argv[1])
    if not (os.path.isdir(os.path.join(REF, "3D")) and os.path.isdir(os.path.join(REF, "2D"))):
        sys.exit(f"{REF} does not hold the reference's 2D/ and 3D/ directories")
    name = sys.argv[2]
    data = CASES[name]()
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in data.items()})
    print("wrote", path, os.path.getsize(path), "bytes")
