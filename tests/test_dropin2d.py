"""The 2D drop-in modules (particle-flow-maps_gb300/2D: hyperparameters, init_conditions, mgpcg,
run_2D) keep the reference's names and reproduce pfm.Sim2D / pfm.Scene results bit for bit."""
import importlib
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DROPIN = os.path.join(ROOT, "particle-flow-maps_gb300", "2D")
OTHER = os.path.join(ROOT, "particle-flow-maps_gb300", "3D")


def _import_2d(**hp):
    while OTHER in sys.path:
        sys.path.remove(OTHER)
    if DROPIN in sys.path:
        sys.path.remove(DROPIN)
    sys.path.insert(0, DROPIN)
    for m in ("run_2D", "run_3D", "mgpcg", "init_conditions", "taichi_utils", "hyperparameters"):
        sys.modules.pop(m, None)
    h = importlib.import_module("hyperparameters")
    for k, v in hp.items():
        setattr(h, k, v)
    return h, importlib.import_module("run_2D")


def test_dropin2d_names_match_the_reference_surface():
    h, r = _import_2d()
    assert h.dim == 2
    for name in ("calc_max_speed", "reset_to_identity", "reset_T_to_identity", "RK4_grid", "RK4_T_forward",
                 "advect_u", "stretch_T_and_advect_particles", "update_particles_imp", "update_particles_grad_m",
                 "update_T", "P2G", "main", "advect_smoke", "curl", "get_central_vector"):
        assert callable(getattr(r, name)), name
    tu = importlib.import_module("taichi_utils")
    assert tu.__file__.startswith(DROPIN)
    m = importlib.import_module("mgpcg")
    assert hasattr(m, "MGPCG_2") and hasattr(m.MGPCG_2, "Poisson")
    ic = importlib.import_module("init_conditions")
    v = ic.angular_vel_func(np.array([0.01, 0.05], np.float32), 0.02, -0.01)
    assert v.dtype == np.float32 and np.all(np.isfinite(v))


@pytest.mark.gpu
def test_mgpcg2_poisson_equals_its_pieces():
    _, r = _import_2d(res_x=64, res_y=32)
    m = sys.modules["mgpcg"]
    rng = np.random.default_rng(6)
    u = [torch.from_numpy(rng.standard_normal(s).astype(np.float32)).cuda() for s in r._face_shapes]
    a = [t.clone() for t in u]
    b = [t.clone() for t in u]
    s1 = m.MGPCG_2(r.boundary_types, [64, 32])
    s1.Poisson(*a)
    s2 = m.MGPCG_2(r.boundary_types, [64, 32])
    s2.apply_bc(*b)
    s2.divergence(*b)
    s2.solve_pressure_MGPCG(verbose=False)
    s2.subtract_grad_p(*b)
    s2.apply_bc(*b)
    torch.cuda.synchronize()
    assert torch.equal(s1.p, s2.p)
    for x, y in zip(a, b):
        assert torch.equal(x, y)


@pytest.mark.gpu
def test_run_2d_main_matches_sim2d(tmp_path):
    import pfm
    h, r = _import_2d(res_x=64, res_y=32, particles_per_cell=4, use_total_steps=True, total_steps=6,
                      reinit_every=4, reinit_every_grad_m=2, CFL=0.5, exp_name="t2")
    assert r.main(logs_root=str(tmp_path)) == 6
    assert (tmp_path / "t2" / "ckpts" / "vel_y_numpy_0.npy").exists()
    u0 = [torch.zeros(s, device="cuda") for s in r._face_shapes]
    vc = torch.zeros((64, 32, 2), device="cuda")
    r.leapfrog_vel_func(vc, None)
    r.split_central_vector(vc, *u0)
    r.solver.Poisson(*u0)
    sim = pfm.Sim2D(u0, pfm.lattice2((64, 32), r.dx, 4), (64, 32), r.dx, CFL=0.5, visualize_dt=h.visualize_dt,
                    reinit_every=4, reinit_every_grad_m=2)
    for _ in range(6):
        sim.step()
    torch.cuda.synchronize()
    assert torch.equal(r.u_x, sim.u[0]) and torch.equal(r.u_y, sim.u[1])
    assert torch.equal(r.particles_pos, sim.pos)


@pytest.mark.gpu
def test_run_2d_restart_from_checkpoint(tmp_path):
    """main(from_frame=k) (2D/run_2D.py:725-728) reloads vel_{x,y}_numpy_<k>.npy and
    smoke_numpy_<k>.npy bit for bit; with a reinitialisation every 2 steps and one step per frame
    the continued run writes the uninterrupted run's frames 3 and 4 bit for bit."""
    hp = dict(res_x=64, res_y=32, particles_per_cell=4, save_frame_each_step=True, ckpt_every=1, total_frames=4,
              use_total_steps=False, reinit_every=2, reinit_every_grad_m=1, CFL=0.5, exp_name="rs2")
    _, r = _import_2d(**hp)
    assert r.main(logs_root=str(tmp_path)) == 4
    ck = tmp_path / "rs2" / "ckpts"
    first = {f: {n: np.load(ck / f"vel_{n}_numpy_{f}.npy") for n in "xy"} for f in (2, 3, 4)}
    smoke2 = np.load(ck / "smoke_numpy_2.npy")
    _, r = _import_2d(**hp)
    assert r.main(from_frame=2, logs_root=str(tmp_path)) == 2
    assert np.array_equal(np.load(ck / "smoke_numpy_2.npy"), smoke2)
    for n, t in zip("xy", (r.u_x, r.u_y)):
        assert np.array_equal(np.load(ck / f"vel_{n}_numpy_2.npy"), first[2][n]), n
        for f in (3, 4):
            assert np.array_equal(np.load(ck / f"vel_{n}_numpy_{f}.npy"), first[f][n]), (f, n)
        assert np.array_equal(t.cpu().numpy(), first[4][n]), n
