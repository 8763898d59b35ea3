"""The 3D drop-in modules (particle-flow-maps_gb300/3D: hyperparameters, init_conditions, mgpcg,
run_3D) keep the reference's names and reproduce pfm.Sim3D / pfm.Scene results bit for bit."""
import importlib
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DROPIN = os.path.join(ROOT, "particle-flow-maps_gb300", "3D")


def _import_3d(**hp):
    """Fresh imports of the drop-in modules with hyperparameters overridden (as a user edits
    hyperparameters.py before running run_3D)."""
    other = os.path.join(ROOT, "particle-flow-maps_gb300", "2D")
    while other in sys.path:
        sys.path.remove(other)
    if DROPIN in sys.path:
        sys.path.remove(DROPIN)
    sys.path.insert(0, DROPIN)
    for m in ("run_3D", "run_2D", "mgpcg", "init_conditions", "taichi_utils", "hyperparameters"):
        sys.modules.pop(m, None)
    h = importlib.import_module("hyperparameters")
    for k, v in hp.items():
        setattr(h, k, v)
    return h, importlib.import_module("run_3D")


def test_dropin_names_match_the_reference_surface():
    h, r = _import_3d()
    for name in ("res_x", "res_y", "res_z", "reinit_every", "reinit_every_grad_m", "CFL", "visualize_dt",
                 "particles_per_cell", "use_midpoint_vel", "use_APIC", "exp_name", "total_steps"):
        assert hasattr(h, name), name
    for name in ("calc_max_speed", "reset_T_to_identity", "RK4_grid", "RK4_T_forward", "advect_u",
                 "stretch_T_and_advect_particles", "get_particles_id_in_every_cell", "update_T", "P2G", "main",
                 "P2G_smoke", "advect_smoke", "clamp_smoke", "RK4_T_and_T_grad_m_forward",
                 "stretch_T_and_T_grad_m_and_advect_particles", "update_particles_imp", "update_particles_grad_m",
                 "compute_dT_dx", "curl", "get_central_vector", "init_particles_smoke"):
        assert callable(getattr(r, name)), name
    tu = importlib.import_module("taichi_utils")
    assert tu.__file__.startswith(DROPIN)
    m = importlib.import_module("mgpcg")
    for name in ("init", "solve", "get_result", "Poisson", "apply_bc", "divergence", "subtract_grad_p",
                 "solve_pressure_MGPCG"):
        assert hasattr(m.MGPCG_3, name), name
    assert r.dx == 1.0 / h.res_y and r.particle_num == h.res_x * h.res_y * h.res_z * h.particles_per_cell


@pytest.mark.gpu
def test_mgpcg3_poisson_equals_its_pieces():
    _, r = _import_3d(res_x=32, res_y=16, res_z=16)
    m = sys.modules["mgpcg"]
    rng = np.random.default_rng(2)
    u = [torch.from_numpy(rng.standard_normal(s).astype(np.float32)).cuda() for s in r._face_shapes]
    a = [t.clone() for t in u]
    b = [t.clone() for t in u]
    s1 = m.MGPCG_3(r.boundary_types, [32, 16, 16])
    s1.Poisson(*a)
    s2 = m.MGPCG_3(r.boundary_types, [32, 16, 16])
    s2.apply_bc(*b)
    s2.divergence(*b)
    s2.init(s2.u_div, -1)
    s2.solve(max_iters=400, tol=1e-12)
    s2.get_result(s2.p)
    s2.subtract_grad_p(*b)
    s2.apply_bc(*b)
    torch.cuda.synchronize()
    assert torch.equal(s1.p, s2.p)
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    div = torch.zeros(32, 16, 16, device="cuda")
    s2.scene.divergence(b, div)
    assert float(div.abs().max()) < 1e-4 * float(torch.cat([t.abs().flatten() for t in u]).max())


@pytest.mark.gpu
def test_rk4_grid_and_advect_u_equal_the_fused_midpoint():
    _, r = _import_3d(res_x=24, res_y=16, res_z=16)
    rng = np.random.default_rng(3)
    u0 = [torch.from_numpy((0.2 * rng.standard_normal(s)).astype(np.float32)).cuda() for s in r._face_shapes]
    psi = [torch.zeros(s + (3,), device="cuda") for s in r._face_shapes]
    T = [torch.zeros(s + (3,), device="cuda") for s in r._face_shapes]
    r.reset_to_identity_grid(*psi, *T)
    for f in range(3):
        r.RK4_grid(psi[f], T[f], *u0, 0.01)
    u1 = [torch.zeros(s, device="cuda") for s in r._face_shapes]
    r.advect_u(*u0, *u1, *T, *psi, r.dx)
    sc = r._scene()
    ref = sc.alloc_faces()
    ps2 = [torch.zeros_like(t) for t in psi]
    T2 = [torch.zeros_like(t) for t in T]
    sc.midpoint(u0, ref, 0.01, psi_out=ps2, T_out=T2)
    torch.cuda.synchronize()
    for f in range(3):
        assert torch.equal(u1[f], ref[f]) and torch.equal(psi[f], ps2[f]) and torch.equal(T[f], T2[f])
    # the backward map starts at the face position with T = e_f
    assert float((psi[0] - psi[0].mean()).abs().max()) > 0


@pytest.mark.gpu
def test_get_particles_id_in_every_cell_matches_numpy():
    _, r = _import_3d(res_x=8, res_y=8, res_z=8, particles_per_cell=8)
    P = r.particle_num
    rng = np.random.default_rng(4)
    pos = (rng.random((3, P)) * np.array([[8.0], [8.0], [8.0]]) * r.dx).astype(np.float32)
    pos_d = torch.from_numpy(pos).cuda()
    r.get_particles_id_in_every_cell(r.cell_particles_id, r.cell_particle_num, pos_d)
    c = np.clip(np.trunc(pos / np.float32(r.dx)).astype(np.int64), 0, 7)
    key = (c[0] * 8 + c[1]) * 8 + c[2]
    counts = np.bincount(key, minlength=512)
    assert np.array_equal(r.cell_particle_num.cpu().numpy().reshape(-1), counts)
    order = np.argsort(key, kind="stable")
    start = np.concatenate([[0], np.cumsum(counts)[:-1]])
    ids = r.cell_particles_id.cpu().numpy().reshape(512, -1)
    cap = ids.shape[1]
    for cell in range(512):
        n = min(counts[cell], cap)
        assert np.array_equal(ids[cell, :n], order[start[cell]:start[cell] + n])
        assert np.all(ids[cell, n:] == -1)


@pytest.mark.gpu
def test_run_3d_main_matches_sim3d(tmp_path):
    import pfm
    h, r = _import_3d(res_x=32, res_y=16, res_z=16, use_total_steps=True, total_steps=5, reinit_every=3,
                      reinit_every_grad_m=1, exp_name="t")
    steps = r.main(logs_root=str(tmp_path))
    assert steps == 5
    ck = tmp_path / "t" / "ckpts"
    assert (ck / "vel_x_numpy_0.npy").exists() and (tmp_path / "t" / "frame_time" / "frame_times.npy").exists()
    # the same run through pfm.Sim3D from the drop-in's initial field
    u0 = [torch.zeros(s, device="cuda") for s in r._face_shapes]
    vc = torch.zeros((32, 16, 16, 3), device="cuda")
    r.init_vorts_leapfrog(None, vc, None, None)
    r.split_central_vector(vc, *u0)
    r.solver.Poisson(*u0)
    seeds = pfm.lattice3((32, 16, 16), r.dx)
    sim = pfm.Sim3D(u0, seeds, (32, 16, 16), r.dx, CFL=h.CFL, visualize_dt=h.visualize_dt, reinit_every=3,
                    reinit_every_grad_m=1)
    for _ in range(5):
        sim.step()
    torch.cuda.synchronize()
    for f, t in enumerate((r.u_x, r.u_y, r.u_z)):
        assert torch.equal(t, sim.u[f]), f
    assert torch.equal(r.particles_pos, sim.pos)


@pytest.mark.gpu
@pytest.mark.parametrize("res", [(20, 16, 12), (20, 12, 16)])
def test_poisson_pieces_match_numpy(res):
    """pfm_divergence / pfm_apply_bc / pfm_subtract_grad_p against their numpy restatement
    (3D/mgpcg.py:359-418), and lap(x) = k r for k = +1 is exactly the negation of k = -1.  With a
    last extent of 16 the x and y faces take the 8-face run form of the subtraction."""
    import pfm
    sc = pfm.Scene(3, res, 1 / res[1], 0)
    rng = np.random.default_rng(8)
    u = [rng.standard_normal(s).astype(np.float32) for s in sc.face_shapes]
    ud = [torch.from_numpy(a).cuda() for a in u]
    div = torch.zeros(res, device="cuda")
    sc.divergence(ud, div)
    want = (u[0][1:] - u[0][:-1]) + (u[1][:, 1:] - u[1][:, :-1]) + (u[2][:, :, 1:] - u[2][:, :, :-1])
    assert np.allclose(div.cpu().numpy(), want, rtol=0, atol=2e-6)
    sc.apply_bc(ud)
    got = [t.cpu().numpy() for t in ud]
    for f in range(3):
        inner = [slice(None)] * 3
        inner[f] = slice(1, -1)
        assert np.array_equal(got[f][tuple(inner)], u[f][tuple(inner)])
        lo = [slice(None)] * 3
        lo[f] = 0
        hi = [slice(None)] * 3
        hi[f] = -1
        assert not got[f][tuple(lo)].any() and not got[f][tuple(hi)].any()
    p = rng.standard_normal(res).astype(np.float32)
    ud = [torch.from_numpy(a).cuda() for a in u]
    sc.subtract_grad_p(ud, torch.from_numpy(p).cuda())
    pp = np.pad(p, 1)  # zero pressure outside the grid
    grads = [pp[1:, 1:-1, 1:-1] - pp[:-1, 1:-1, 1:-1], pp[1:-1, 1:, 1:-1] - pp[1:-1, :-1, 1:-1],
             pp[1:-1, 1:-1, 1:] - pp[1:-1, 1:-1, :-1]]
    for f in range(3):
        assert np.array_equal(ud[f].cpu().numpy(), (u[f] - grads[f]).astype(np.float32))
    r = torch.from_numpy(rng.standard_normal(res).astype(np.float32)).cuda()
    x1, x2 = torch.zeros(res, device="cuda"), torch.zeros(res, device="cuda")
    i1 = sc.mgpcg_solve(r, x1, k=-1.0)
    i2 = sc.mgpcg_solve(r, x2, k=1.0)
    assert i1.iterations == i2.iterations and i1.converged
    assert torch.equal(x1, -x2)


@pytest.mark.gpu
def test_dropin_smoke_and_variants():
    """init_vorts_leapfrog with smoke fields adds the same velocity as without them, colours the
    rings' cells; the drop-in smoke/variant functions equal the Scene calls they wrap."""
    import pfm
    _, r = _import_3d(res_x=32, res_y=16, res_z=16, particles_per_cell=8)
    vc_a = torch.zeros((32, 16, 16, 3), device="cuda")
    vc_b = torch.zeros_like(vc_a)
    s1 = torch.zeros((32, 16, 16, 4), device="cuda")
    s2 = torch.zeros_like(s1)
    r.init_vorts_leapfrog(None, vc_a, s1, s2)
    r.init_vorts_leapfrog(None, vc_b, None, None)
    torch.cuda.synchronize()
    assert torch.equal(vc_a, vc_b)
    vals = {tuple(v) for v in s1.reshape(-1, 4).cpu().numpy().tolist()}
    assert vals <= {(0., 0., 0., 0.), (1., 0., 0., 1.), (0., 0., 1., 1.), (1., 0., 1., 2.)}
    assert (1., 0., 0., 1.) in vals and (0., 0., 1., 1.) in vals
    # advect_smoke through the midpoint's backward map, against the oracle (bitwise)
    import oracle as O
    psi = [torch.zeros(s + (3,), device="cuda") for s in r._face_shapes]
    r._scene().midpoint([r.u_x, r.u_y, r.u_z], [torch.zeros(s, device="cuda") for s in r._face_shapes], 0.01,
                        psi_out=psi)
    out = torch.zeros_like(s1)
    r.advect_smoke(s1, out, *psi, r.dx)
    torch.cuda.synchronize()
    want = O.advect_smoke3(s1.cpu().numpy(), np.zeros((32, 16, 16, 4), np.float32), *(t.cpu().numpy() for t in psi),
                           r.dx)
    assert np.array_equal(out.cpu().numpy(), want)
    # the particle smoke round trip: G2P then P2G_smoke
    P = r.particle_num
    pos = pfm.soa(pfm.jittered((32, 16, 16), r.dx, 8, seed=1))
    sp = r.particles_smoke
    gs = r.particles_init_grad_smoke
    assert tuple(sp.shape) == (4, P) and tuple(gs.shape) == (3, 4, P)
    r.init_particles_smoke(sp, gs, pos, s1, r.dx)
    sm = torch.zeros_like(s1)
    wgt = torch.zeros((32, 16, 16), device="cuda")
    eye = torch.eye(3, device="cuda")[:, :, None].expand(3, 3, P).contiguous()
    r.P2G_smoke(sp, gs, pos, sm, *eye, *eye, wgt)
    ref = torch.zeros_like(s1)
    wref = torch.zeros_like(wgt)
    r._scene().p2g_smoke(sp, gs, pos, eye, eye, ref, wref)
    torch.cuda.synchronize()
    assert torch.equal(sm, ref) and torch.equal(wgt, wref)
    assert float(sm.min()) >= 0 and float(sm.max()) <= 1
    # compute_dT_dx with the reference's own (empty) inner loop gives zero
    gx, gy, gz = (torch.ones(3, 3, P, device="cuda") for _ in range(3))
    r.particles_pos.copy_(pos)
    r.compute_dT_dx(gx, gy, gz, *eye, pos, r.cell_particles_id, r.cell_particle_num)
    torch.cuda.synchronize()
    assert not gx.any() and not gy.any() and not gz.any()


@pytest.mark.gpu
def test_run_3d_restart_from_checkpoint(tmp_path):
    """main(from_frame=k) (3D/run_3D.py:676-680) reloads vel_{x,y,z}_numpy_<k>.npy, the files main()
    writes at every checkpoint frame (3D/run_3D.py:846-853): the reloaded velocity is the saved one
    bit for bit, and because the restart reseeds the particles exactly as the uninterrupted run
    does at a reinitialisation step (reinit every 2 steps, one step per frame), the continued run
    writes the same frames 3 and 4 bit for bit."""
    hp = dict(res_x=32, res_y=16, res_z=16, save_frame_each_step=True, ckpt_every=1, total_frames=4,
              use_total_steps=False, reinit_every=2, reinit_every_grad_m=1, exp_name="rs")
    _, r = _import_3d(**hp)
    assert r.main(logs_root=str(tmp_path)) == 4
    ck = tmp_path / "rs" / "ckpts"
    first = {f: {n: np.load(ck / f"vel_{n}_numpy_{f}.npy") for n in "xyz"} for f in (2, 3, 4)}
    _, r = _import_3d(**hp)
    assert r.main(from_frame=2, logs_root=str(tmp_path)) == 2
    for n, t in zip("xyz", (r.u_x, r.u_y, r.u_z)):
        # main() writes the velocity it loaded back under the restart frame before stepping
        assert np.array_equal(np.load(ck / f"vel_{n}_numpy_2.npy"), first[2][n]), n
        for f in (3, 4):
            assert np.array_equal(np.load(ck / f"vel_{n}_numpy_{f}.npy"), first[f][n]), (f, n)
        assert np.array_equal(t.cpu().numpy(), first[4][n]), n
    # the continued run equals pfm.Sim3D started from the frame-2 velocity with lattice seeds
    import pfm
    u2 = [torch.from_numpy(first[2][n]).cuda() for n in "xyz"]
    sim = pfm.Sim3D(u2, pfm.lattice3((32, 16, 16), r.dx), (32, 16, 16), r.dx, CFL=r.CFL, reinit_every=2,
                    reinit_every_grad_m=1)
    sim.clock.save_frame_each_step = True
    for _ in range(2):
        sim.step()
    torch.cuda.synchronize()
    for n, t in zip("xyz", sim.u):
        assert np.array_equal(t.cpu().numpy(), first[4][n]), n
