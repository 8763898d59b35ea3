"""Pins the CPU oracle to the reference: every golden vector in tests/golden/ was produced by the
reference's own Taichi kernels and main() loop (tests/golden/make_golden.py)."""
import numpy as np
import pytest

import oracle as O


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


def prel(a, b):
    """Relative L2 of the pressure with its all-Neumann null-space constant removed."""
    return rel(np.asarray(a) - np.mean(a), np.asarray(b) - np.mean(b))


# The oracle evaluates each kernel in the reference's expression order; what remains is numpy's
# own rounding in the shim (a few ulp), hence the tight tolerance.
KTOL = 1e-7


def test_oracle_kernels_3d(golden):
    g = golden("ref3d_kernels")
    dx = 1.0 / int(g["res"][1])
    u = (g["u_x"], g["u_y"], g["u_z"])
    assert O.calc_max_speed3(*u) == float(g["max_speed"])
    imp, C = O.g2p3(g["pos"], *u, dx)
    assert rel(imp, g["g2p_imp"]) < KTOL and rel(C, g["g2p_C"]) < KTOL
    pos, T = O.rk4_T_forward3(g["pos"], g["T_gm"], *u, dx, g["dt"])
    assert rel(pos, g["rk4_pos"]) < KTOL and rel(T, g["rk4_T"]) < KTOL
    assert np.array_equal(O.update_T3(g["T_init"], g["T_gm"]), g["update_T"])
    (ux, uy, uz), (wx, wy, wz) = O.p2g3(g["init_imp"], g["pos"], g["T_gm"], g["T_init"], g["init_C"],
                                        tuple(g["res"]), dx)
    for a, n in zip((ux, uy, uz, wx, wy, wz), ("u_x", "u_y", "u_z", "w_x", "w_y", "w_z")):
        assert rel(a, g["p2g_" + n]) < KTOL, n
    assert np.array_equal(O.bin_count3(g["bin_pos"], tuple(g["res"]), dx), g["bin_count"])
    for fam, n in ((0, "x"), (2, "z")):
        psi, T, um = O.midpoint_family3(fam, *u, dx, np.float32(0.5 * float(g["dt"])))
        assert np.array_equal(psi, g[f"mid_psi_{n}"])
        assert rel(T, g[f"mid_T_{n}"]) < KTOL and rel(um, g[f"mid_u_{n}"]) < KTOL


@pytest.mark.parametrize("case", ["poisson", "poisson2"])
def test_oracle_poisson_3d_bitexact(golden, case):
    g = golden("ref3d_kernels")
    ins = ([g["mid_u_x"], g["mid_u_y"], g["mid_u_z"]] if case == "poisson"
           else [g["poisson2_in_x"], g["poisson2_in_y"], g["poisson2_in_z"]])
    ux, uy, uz, p, it, _ = O.poisson3(*ins)
    assert it == int(g[f"{case}_iters"])
    for a, n in zip((ux, uy, uz), "xyz"):
        assert np.array_equal(a, g[f"{case}_u_{n}"])
    assert np.array_equal(p, g[f"{case}_p"])


def test_oracle_poisson_3d_three_levels_bitexact(golden):
    """MGPCG_3.Poisson on a 32^3 grid: a V-cycle of three levels (32, 16, 8; the 16^3 cases above
    have two), the reference's recursion of restriction, bottom sweeps and prolongation one level
    deeper.  Same stopping iteration, bitwise the same velocity and pressure."""
    g = golden("ref3d_mgpcg")
    assert int(g["levels"]) == 3
    ux, uy, uz, p, it, _ = O.poisson3(g["in_x"], g["in_y"], g["in_z"])
    assert it == int(g["iters"])
    for a, n in zip((ux, uy, uz), "xyz"):
        assert np.array_equal(a, g[f"u_{n}"]), n
    assert np.array_equal(p, g["p"])


def test_oracle_kernels_2d(golden):
    g = golden("ref2d_kernels")
    dx = 1.0 / int(g["res"][1])
    u = (g["u_x"], g["u_y"])
    assert O.calc_max_speed2(*u) == float(g["max_speed"])
    imp, C = O.g2p2(g["pos"], *u, dx)
    assert rel(imp, g["g2p_imp"]) < KTOL and rel(C, g["g2p_C"]) < KTOL
    pos, T = O.rk4_T_forward2(g["pos"], g["T_gm"], *u, dx, g["dt"], 1)
    assert rel(pos, g["rk4_pos"]) < KTOL and rel(T, g["rk4_T"]) < KTOL
    assert np.array_equal(O.update_grad_m2(g["init_C"], g["T_gm"]), g["grad_m_C"])
    T2 = O.update_T2(g["T_init"], g["T_gm"])
    assert np.array_equal(T2, g["update_T"])
    assert np.array_equal(O.update_imp2(g["init_imp"], T2), g["update_imp"])
    (ux, uy), (wx, wy), (gx, gy) = O.p2g2(g["init_imp"], g["pos"], g["init_C"], g["psi"], tuple(g["res"]), dx)
    for a, n in zip((ux, uy, wx, wy, gx, gy), ("u_x", "u_y", "w_x", "w_y", "psi_x", "psi_y")):
        assert rel(a, g["p2g_" + n]) < KTOL, n
    for fam, n in ((0, "x"), (1, "y")):
        psi, T, um = O.midpoint_family2(fam, *u, dx, np.float32(0.5 * float(g["dt"])))
        assert np.array_equal(psi, g[f"mid_psi_{n}"])
        assert rel(T, g[f"mid_T_{n}"]) < KTOL and rel(um, g[f"mid_u_{n}"]) < KTOL


@pytest.mark.parametrize("case", ["poisson", "poisson2"])
def test_oracle_poisson_2d_bitexact(golden, case):
    g = golden("ref2d_kernels")
    ins = [g["mid_u_x"], g["mid_u_y"]] if case == "poisson" else [g["poisson2_in_x"], g["poisson2_in_y"]]
    ux, uy, p, it, _ = O.poisson2(*ins)
    assert it == int(g[f"{case}_iters"])
    assert np.array_equal(ux, g[f"{case}_u_x"]) and np.array_equal(uy, g[f"{case}_u_y"])
    assert np.array_equal(p, g[f"{case}_p"])


def test_oracle_steps_2d(golden):
    """run_2D.main() of the reference, 20 steps at 32^2 (reinit 12, grad_m reinit 8)."""
    g = golden("ref2d_steps")
    res = tuple(int(r) for r in g["res"])
    dx = 1.0 / res[1]
    sim = O.Sim2D([g["init_u_x"], g["init_u_y"]], O.lattice2(res, dx, 4), res, dx, CFL=0.5, visualize_dt=0.1,
                  reinit_every=int(g["hp"][0]), reinit_every_grad_m=int(g["hp"][1]))
    for s in range(1, 21):
        sim.step()
        assert rel(sim.u[0], g[f"s{s}_u_x"]) < 1e-5 and rel(sim.u[1], g[f"s{s}_u_y"]) < 1e-5, s
        assert prel(sim.p, g[f"s{s}_p"]) < 1e-5, s
        if f"s{s}_particles_pos" in g:
            assert rel(sim.pos, g[f"s{s}_particles_pos"]) < 1e-6
            assert rel(sim.imp, g[f"s{s}_particles_imp"]) < 1e-5
            assert rel(sim.T, np.stack([g[f"s{s}_T_x"], g[f"s{s}_T_y"]], 1)) < 1e-5
    # iteration counts printed by the reference: IC projection, then (midpoint, final) per step
    assert sim.iters == [int(i) for i in g["iters"][1:]]


@pytest.mark.parametrize("case,nsteps", [("ref3d_steps", 10), ("ref3d_steps16", 3)])
def test_oracle_steps_3d(golden, case, nsteps):
    """run_3D.main() of the reference (reinit 5, grad_m reinit 2): 10 steps at 8^3, where MGPCG has
    one level, and 3 steps at 16^3, where it has two."""
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", f"{case}.npz")
    if not os.path.exists(path):
        pytest.skip("3D step golden not generated")
    g = golden(case)
    res = tuple(int(r) for r in g["res"])
    dx = 1.0 / res[1]
    sim = O.Sim3D([g["init_u_x"], g["init_u_y"], g["init_u_z"]], O.lattice3(res, dx), res, dx, CFL=0.5,
                  visualize_dt=0.1, reinit_every=int(g["hp"][0]), reinit_every_grad_m=int(g["hp"][1]))
    for s in range(1, nsteps + 1):
        sim.step()
        for f, n in enumerate("xyz"):
            assert rel(sim.u[f], g[f"s{s}_u_{n}"]) < 1e-5, (s, n)
        assert prel(sim.p, g[f"s{s}_p"]) < 1e-5, s
        if f"s{s}_particles_pos" in g:
            assert rel(sim.pos, g[f"s{s}_particles_pos"]) < 1e-6
            assert rel(sim.init_imp, g[f"s{s}_particles_init_imp"]) < 1e-5
        if f"s{s}_T_x_init" in g:
            T_init = np.stack([g[f"s{s}_T_{v}_init"] for v in "xyz"], 1)
            assert rel(sim.T_init, T_init) < 1e-5
    assert sim.iters == [int(i) for i in g["iters"][1:]]


def test_oracle_fields_3d(golden):
    """Smoke transport and diagnostics (3D/taichi_utils.py:56-85, 3D/init_conditions.py:275-279,
    3D/run_3D.py:315-334, 554-593) against the reference's kernels on a 16x12x8 grid."""
    g = golden("ref3d_fields")
    dx = float(g["dx"])
    vc = O.central_vector3(g["u_x"], g["u_y"], g["u_z"])
    assert np.array_equal(vc, g["central"])
    assert np.array_equal(O.curl3(vc, dx), g["curl"])
    s, G = O.init_particles_smoke3(g["pos"], g["smoke"], dx)
    assert rel(s, g["g2p_smoke"]) < KTOL and rel(G, g["g2p_grad_smoke"]) < KTOL
    sm, w = O.p2g_smoke3(g["smoke_p"], g["grad_smoke"], g["pos"], g["T_gm"], g["T_init"], tuple(g["res"]), dx)
    assert rel(w, g["p2g_smoke_w"]) < KTOL and rel(sm, g["p2g_smoke"]) < KTOL
    psi = (g["psi_x"], g["psi_y"], g["psi_z"])
    a = O.advect_smoke3(g["smoke"], np.zeros_like(g["smoke"]), *psi, dx)
    assert np.array_equal(a, g["advect_smoke"])
    c = O.advect_smoke3(g["smoke"], g["clamp_in"], *psi, dx, clamp=True)
    assert np.array_equal(c, g["clamp_smoke"])


def test_oracle_fields_2d(golden):
    g = golden("ref2d_fields")
    dx = float(g["dx"])
    vc = O.central_vector2(g["u_x"], g["u_y"])
    assert np.array_equal(vc, g["central"])
    assert np.array_equal(O.curl2(vc, dx), g["curl"])
    assert np.array_equal(O.advect_smoke2(g["smoke"], g["psi_x"], g["psi_y"], dx), g["advect_smoke"])


def test_oracle_variants_3d(golden):
    """RK4_T_and_T_grad_m_forward, update_particles_imp/_grad_m and compute_dT_dx
    (3D/run_3D.py:221-292, 353-428) against the reference's kernels."""
    g = golden("ref3d_variants")
    dx = float(g["dx"])
    u = (g["u_x"], g["u_y"], g["u_z"])
    pos, T, T2 = O.rk4_T_and_T_grad_m_forward3(g["pos"], g["T"], g["T2"], *u, 1.0 / int(g["res"][1]), g["dt"])
    assert rel(pos, g["rk4_pos"]) < KTOL and rel(T, g["rk4_T"]) < KTOL and rel(T2, g["rk4_T2"]) < KTOL
    assert np.array_equal(O.update_imp3(g["init_imp"], g["T"]), g["update_imp"])
    n = int(g["n_inner"])
    # the reference's compute_dT_dx visits no list entry (ti.ndrange(0, n) is an empty 2-D range):
    # its result is the oracle's with cap = 0
    assert not np.any(g["dT_dx"])
    gT = O.compute_dT_dx3(g["pos"], g["init_pos"], g["T"], tuple(g["res"]), dx, 0)
    assert np.array_equal(gT[:n], g["dT_dx"])
    C = O.update_grad_m3(g["init_C"][:n], g["T"][:n], g["grad_T_init"], g["init_imp"][:n])
    assert rel(C, g["grad_m_C"]) < KTOL
