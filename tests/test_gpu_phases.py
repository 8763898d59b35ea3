"""Parity of every step phase on the GPU against the CPU oracle (f32 restatement of the reference).

Tolerance: the reference itself sums taps and P2G scatters in a schedule-dependent order (float
atomics), so results are compared in relative L2: 1e-5 for the step phases (the bar the
reference's port is held to), tighter where the GPU evaluates the same expression.
The cell-sort permutation is compared bit-exactly with numpy's stable argsort of the same keys.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import oracle as O  # noqa: E402
import pfm  # noqa: E402

TOL = 1e-5


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float32))).cuda()


def host(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module")
def g3(golden):
    return golden("ref3d_kernels")


@pytest.fixture(scope="module")
def g2(golden):
    return golden("ref2d_kernels")


def scene3(g, P=None):
    res = tuple(int(x) for x in g["res"])
    return pfm.Scene(3, res, 1.0 / res[1], P if P is not None else g["pos"].shape[0])


def scene2(g, P=None):
    res = tuple(int(x) for x in g["res"])
    return pfm.Scene(2, res, 1.0 / res[1], P if P is not None else g["pos"].shape[0])


# ------------------------------------------------------------------------------------------------
# 3D
# ------------------------------------------------------------------------------------------------
def test_max_speed3(g3):
    sc = scene3(g3)
    u = [dev(g3[k]) for k in ("u_x", "u_y", "u_z")]
    got = sc.calc_max_speed(u)
    assert got == pytest.approx(float(g3["max_speed"]), rel=1e-6)
    assert got == pytest.approx(O.calc_max_speed3(g3["u_x"], g3["u_y"], g3["u_z"]), rel=1e-6)


def test_g2p3(g3):
    sc = scene3(g3)
    u = [dev(g3[k]) for k in ("u_x", "u_y", "u_z")]
    pos = pfm.soa(g3["pos"])
    imp = torch.zeros(3, sc.P, device="cuda")
    C = torch.zeros(3, 3, sc.P, device="cuda")
    sc.g2p(pos, u, imp_out=imp, C_out=C)
    torch.cuda.synchronize()
    assert rel(pfm.aos(imp), g3["g2p_imp"]) < TOL
    assert rel(pfm.aos_T(C), g3["g2p_C"]) < TOL


def test_rk4_T_forward3(g3):
    sc = scene3(g3)
    u = [dev(g3[k]) for k in ("u_x", "u_y", "u_z")]
    pos = pfm.soa(g3["pos"])
    T = pfm.soa_T(g3["T_gm"])
    sc.rk4_T_forward(pos, T, u, float(g3["dt"]))
    assert rel(pfm.aos(pos), g3["rk4_pos"]) < 1e-6
    assert rel(pfm.aos_T(T), g3["rk4_T"]) < TOL


def test_update_T3(g3):
    sc = scene3(g3)
    Ti = pfm.soa_T(g3["T_init"])
    Tg = pfm.soa_T(g3["T_gm"])
    sc.update_T(Ti, Tg, reset_gm=True)
    assert rel(pfm.aos_T(Ti), g3["update_T"]) < 1e-6
    assert np.array_equal(pfm.aos_T(Tg), np.broadcast_to(np.eye(3, dtype=np.float32), (sc.P, 3, 3)))


def test_p2g3(g3):
    sc = scene3(g3)
    u = sc.alloc_faces()
    w = sc.alloc_faces()
    sc.p2g3(pfm.soa(g3["init_imp"]), pfm.soa(g3["pos"]), pfm.soa_T(g3["T_gm"]), pfm.soa_T(g3["T_init"]),
            pfm.soa_T(g3["init_C"]), u, w)
    for f, n in enumerate("xyz"):
        assert rel(host(u[f]), g3[f"p2g_u_{n}"]) < TOL, n
        assert rel(host(w[f]), g3[f"p2g_w_{n}"]) < TOL, n


def test_p2g3_deterministic(g3):
    sc = scene3(g3)
    args = (pfm.soa(g3["init_imp"]), pfm.soa(g3["pos"]), pfm.soa_T(g3["T_gm"]), pfm.soa_T(g3["T_init"]),
            pfm.soa_T(g3["init_C"]))
    outs = []
    for _ in range(3):
        u, w = sc.alloc_faces(), sc.alloc_faces()
        sc.p2g3(*args, u, w)
        outs.append([host(t) for t in u + w])
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert np.array_equal(a, b)


def test_sort_bitexact(g3):
    pos = g3["bin_pos"]
    res = tuple(int(x) for x in g3["res"])
    sc = pfm.Scene(3, res, 1.0 / res[1], pos.shape[0])
    count, order = sc.sort_particles(pfm.soa(pos))
    assert np.array_equal(host(count), g3["bin_count"])
    cells = np.clip((pos / np.float32(1.0 / res[1])).astype(np.int64), 0, np.array(res) - 1)
    key = (cells[:, 0] * res[1] + cells[:, 1]) * res[2] + cells[:, 2]
    assert np.array_equal(host(order), np.argsort(key, kind="stable"))


def test_midpoint3(g3):
    sc = scene3(g3)
    u0 = [dev(g3[k]) for k in ("u_x", "u_y", "u_z")]
    u1 = sc.alloc_faces()
    psi = [torch.zeros(s + (3,), device="cuda") for s in sc.face_shapes]
    T = [torch.zeros(s + (3,), device="cuda") for s in sc.face_shapes]
    sc.midpoint(u0, u1, float(np.float32(0.5 * float(g3["dt"]))), psi_out=psi, T_out=T)
    for f, n in enumerate("xyz"):
        assert rel(host(u1[f]), g3[f"mid_u_{n}"]) < TOL, n
    assert rel(host(psi[0]), g3["mid_psi_x"]) < 1e-6
    assert rel(host(T[2]), g3["mid_T_z"]) < TOL


@pytest.mark.parametrize("case", ["poisson", "poisson2"])
def test_poisson3(g3, case):
    if case == "poisson":
        ins = [g3["mid_u_x"], g3["mid_u_y"], g3["mid_u_z"]]
    else:
        ins = [g3["poisson2_in_x"], g3["poisson2_in_y"], g3["poisson2_in_z"]]
    N = (ins[1].shape[0], ins[0].shape[1], ins[0].shape[2])
    sc = pfm.Scene(3, N, 1.0 / N[1], 0)
    u = [dev(a) for a in ins]
    p = torch.zeros(N, device="cuda")
    info = sc.poisson(u, p)
    assert info.converged
    assert info.iterations == int(g3[f"{case}_iters"])
    for f, n in enumerate("xyz"):
        assert rel(host(u[f]), g3[f"{case}_u_{n}"]) < TOL
    assert rel(host(p), g3[f"{case}_p"]) < TOL


# ------------------------------------------------------------------------------------------------
# 2D
# ------------------------------------------------------------------------------------------------
def test_max_speed2(g2):
    sc = scene2(g2)
    assert sc.calc_max_speed([dev(g2["u_x"]), dev(g2["u_y"])]) == pytest.approx(float(g2["max_speed"]), rel=1e-6)


def test_g2p2(g2):
    sc = scene2(g2)
    u = [dev(g2["u_x"]), dev(g2["u_y"])]
    imp = torch.zeros(2, sc.P, device="cuda")
    C = torch.zeros(2, 2, sc.P, device="cuda")
    sc.g2p(pfm.soa(g2["pos"]), u, imp_out=imp, C_out=C)
    assert rel(pfm.aos(imp), g2["g2p_imp"]) < TOL
    assert rel(pfm.aos_T(C), g2["g2p_C"]) < TOL


def test_rk4_T_forward2(g2):
    sc = scene2(g2)
    u = [dev(g2["u_x"]), dev(g2["u_y"])]
    pos = pfm.soa(g2["pos"])
    T = pfm.soa_T(g2["T_gm"])
    sc.rk4_T_forward(pos, T, u, float(g2["dt"]), advect_psi=True)
    assert rel(pfm.aos(pos), g2["rk4_pos"]) < 1e-6
    assert rel(pfm.aos_T(T), g2["rk4_T"]) < TOL


def test_update_kernels2(g2):
    sc = scene2(g2)
    C = torch.zeros(2, 2, sc.P, device="cuda")
    Tg = pfm.soa_T(g2["T_gm"])
    sc.update_grad_m2(C, pfm.soa_T(g2["init_C"]), Tg)
    assert rel(pfm.aos_T(C), g2["grad_m_C"]) < 1e-6
    T = torch.zeros(2, 2, sc.P, device="cuda")
    sc.update_T2(T, pfm.soa_T(g2["T_init"]), Tg)
    assert rel(pfm.aos_T(T), g2["update_T"]) < 1e-6
    imp = torch.zeros(2, sc.P, device="cuda")
    sc.update_imp2(imp, pfm.soa(g2["init_imp"]), T)
    assert rel(pfm.aos(imp), g2["update_imp"]) < 1e-6


def test_p2g2(g2):
    sc = scene2(g2)
    u, w = sc.alloc_faces(), sc.alloc_faces()
    psi = [torch.zeros(s + (2,), device="cuda") for s in sc.face_shapes]
    sc.p2g2(pfm.soa(g2["init_imp"]), pfm.soa(g2["pos"]), pfm.soa_T(g2["init_C"]), pfm.soa(g2["psi"]), u, w,
            psi_out=psi)
    for f, n in enumerate("xy"):
        assert rel(host(u[f]), g2[f"p2g_u_{n}"]) < TOL
        assert rel(host(w[f]), g2[f"p2g_w_{n}"]) < TOL
        assert rel(host(psi[f]), g2[f"p2g_psi_{n}"]) < TOL


def test_midpoint2(g2):
    sc = scene2(g2)
    u0 = [dev(g2["u_x"]), dev(g2["u_y"])]
    u1 = sc.alloc_faces()
    sc.midpoint(u0, u1, float(np.float32(0.5 * float(g2["dt"]))))
    for f, n in enumerate("xy"):
        assert rel(host(u1[f]), g2[f"mid_u_{n}"]) < TOL


@pytest.mark.parametrize("case", ["poisson", "poisson2"])
def test_poisson2(g2, case):
    ins = [g2["mid_u_x"], g2["mid_u_y"]] if case == "poisson" else [g2["poisson2_in_x"], g2["poisson2_in_y"]]
    N = (ins[1].shape[0], ins[0].shape[1])
    sc = pfm.Scene(2, N, 1.0 / N[1], 0)
    u = [dev(a) for a in ins]
    p = torch.zeros(N, device="cuda")
    info = sc.poisson(u, p)
    assert info.converged and info.iterations == int(g2[f"{case}_iters"])
    for f, n in enumerate("xy"):
        assert rel(host(u[f]), g2[f"{case}_u_{n}"]) < TOL
    assert rel(host(p), g2[f"{case}_p"]) < TOL


# ------------------------------------------------------------------------------------------------
# larger random cases against the oracle (sizes the oracle finishes in seconds)
# ------------------------------------------------------------------------------------------------
def smooth(shape, rng, amp):
    idx = np.meshgrid(*[np.linspace(0, 1, s) for s in shape], indexing="ij")
    out = np.zeros(shape)
    for _ in range(3):
        k = rng.uniform(0.5, 2.0, len(shape))
        ph = rng.uniform(0, 6.3, len(shape))
        t = rng.uniform(-1, 1)
        for d in range(len(shape)):
            t = t * np.sin(2 * np.pi * k[d] * idx[d] + ph[d])
        out += t
    return (amp * out).astype(np.float32)


@pytest.mark.parametrize("res", [(32, 32, 32), (48, 32, 24)])
def test_particle_phases_random3(res):
    rng = np.random.default_rng(7)
    dx = 1.0 / res[1]
    sh = [(res[0] + 1, res[1], res[2]), (res[0], res[1] + 1, res[2]), (res[0], res[1], res[2] + 1)]
    u = [smooth(s, rng, 1.0) for s in sh]
    P = 20000
    hi = np.array(res) * dx
    pos = (rng.uniform(-0.02, 1.02, (P, 3)) * hi).astype(np.float32)
    sc = pfm.Scene(3, res, dx, P)
    ud = [dev(a) for a in u]
    imp = torch.zeros(3, P, device="cuda")
    C = torch.zeros(3, 3, P, device="cuda")
    sc.g2p(pfm.soa(pos), ud, imp_out=imp, C_out=C)
    oi, oC = O.g2p3(pos, *u, dx)
    assert rel(pfm.aos(imp), oi) < TOL and rel(pfm.aos_T(C), oC) < TOL
    T0 = (np.eye(3)[None] + 0.1 * rng.standard_normal((P, 3, 3))).astype(np.float32)
    dt = 0.5 * dx / O.calc_max_speed3(*u)
    p_d, T_d = pfm.soa(pos), pfm.soa_T(T0)
    sc.rk4_T_forward(p_d, T_d, ud, float(np.float32(dt)))
    op, oT = O.rk4_T_forward3(pos, T0, *u, dx, np.float32(dt))
    assert rel(pfm.aos(p_d), op) < 1e-6 and rel(pfm.aos_T(T_d), oT) < TOL
    Ti = (np.eye(3)[None] + 0.1 * rng.standard_normal((P, 3, 3))).astype(np.float32)
    m0 = rng.standard_normal((P, 3)).astype(np.float32)
    uo, wo = sc.alloc_faces(), sc.alloc_faces()
    sc.p2g3(dev(m0.T.copy()), p_d, T_d, pfm.soa_T(Ti), C, uo, wo)
    (gx, gy, gz), (wx, wy, wz) = O.p2g3(m0, op, oT, Ti, oC, res, dx)
    for t, o in zip(uo + wo, [gx, gy, gz, wx, wy, wz]):
        assert rel(host(t), o) < TOL
    mid = sc.alloc_faces()
    sc.midpoint(ud, mid, float(np.float32(0.25 * dt)))
    om = O.midpoint3(*u, dx, np.float32(0.25 * dt))
    for t, o in zip(mid, om):
        assert rel(host(t), o) < TOL


def test_poisson3_random_levels():
    rng = np.random.default_rng(3)
    res = (64, 64, 32)
    sh = [(65, 64, 32), (64, 65, 32), (64, 64, 33)]
    u = [smooth(s, rng, 1.0) for s in sh]
    sc = pfm.Scene(3, res, 1.0 / 64, 0)
    assert sc.mg_levels == 3
    ud = [dev(a) for a in u]
    p = torch.zeros(res, device="cuda")
    info = sc.poisson(ud, p)
    ox, oy, oz, op, oit, _ = O.poisson3(*u)
    assert info.converged and oit >= 0
    assert abs(info.iterations - oit) <= 1
    for t, o in zip(ud, (ox, oy, oz)):
        assert rel(host(t), o) < TOL
    assert rel(host(p), op) < TOL


def test_empty_particles():
    sc = pfm.Scene(3, (8, 8, 8), 1 / 8, 0)
    u, w = sc.alloc_faces(), sc.alloc_faces()
    e3 = torch.zeros(3, 0, device="cuda")
    e33 = torch.zeros(3, 3, 0, device="cuda")
    sc.p2g3(e3, e3, e33, e33, e33, u, w)
    assert all(float(t.abs().sum()) == 0 for t in u + w)
    count, order = sc.sort_particles(e3)
    assert int(count.sum()) == 0 and order.numel() == 0


def test_bad_arguments_raise():
    sc = pfm.Scene(3, (8, 8, 8), 1 / 8, 16)
    with pytest.raises(pfm.PfmError):
        sc.g2p(torch.zeros(3, 15, device="cuda"), sc.alloc_faces(), imp_out=torch.zeros(3, 16, device="cuda"))
    with pytest.raises(pfm.PfmError):
        sc.calc_max_speed([torch.zeros(9, 8, 8, device="cuda")] * 3)
    with pytest.raises(pfm.PfmError):
        sc.g2p(torch.zeros(3, 16), sc.alloc_faces(), imp_out=torch.zeros(3, 16, device="cuda"))


def _clustered_positions(res, dx, rng):
    """Collisions and edges of the cell binning: 5,000 particles in one cell, particles exactly on
    grid planes and at the domain's corners and walls, and a uniform background."""
    hi = np.array(res, np.float64) * dx
    lone = (np.array([5, 6, 7]) + rng.uniform(0.0, 1.0, (5000, 3))) * dx
    planes = np.floor(rng.uniform(0, 1, (600, 3)) * np.array(res)) * dx  # on cell corners and faces
    corners = np.array([[0, 0, 0], hi, [hi[0], 0, 0], [0, hi[1], hi[2]]], np.float64)
    walls = rng.uniform(0, 1, (400, 3)) * hi
    walls[:200, 0] = 0.0
    walls[200:, 2] = hi[2]
    back = rng.uniform(0, 1, (3000, 3)) * hi
    return np.concatenate([lone, planes, corners, walls, back]).astype(np.float32)


def test_p2g3_and_sort_collisions_and_edges():
    rng = np.random.default_rng(11)
    res = (16, 12, 20)
    dx = 1.0 / res[1]
    pos = _clustered_positions(res, dx, rng)
    P = pos.shape[0]
    sc = pfm.Scene(3, res, dx, P)
    count, order = sc.sort_particles(pfm.soa(pos))
    cells = np.clip((pos / np.float32(dx)).astype(np.int64), 0, np.array(res) - 1)
    key = (cells[:, 0] * res[1] + cells[:, 1]) * res[2] + cells[:, 2]
    assert np.array_equal(host(order), np.argsort(key, kind="stable"))
    assert np.array_equal(host(count).ravel(), np.bincount(key, minlength=int(np.prod(res))))
    T_gm = (np.eye(3)[None] + 0.1 * rng.standard_normal((P, 3, 3))).astype(np.float32)
    Ti = (np.eye(3)[None] + 0.1 * rng.standard_normal((P, 3, 3))).astype(np.float32)
    C = (0.3 * rng.standard_normal((P, 3, 3))).astype(np.float32)
    m0 = rng.standard_normal((P, 3)).astype(np.float32)
    u, w = sc.alloc_faces(), sc.alloc_faces()
    sc.p2g3(pfm.soa(m0), pfm.soa(pos), pfm.soa_T(T_gm), pfm.soa_T(Ti), pfm.soa_T(C), u, w)
    (gx, gy, gz), (wx, wy, wz) = O.p2g3(m0, pos, T_gm, Ti, C, res, dx)
    for t, o in zip(u + w, [gx, gy, gz, wx, wy, wz]):
        assert rel(host(t), o) < TOL
    u2, w2 = sc.alloc_faces(), sc.alloc_faces()  # and still bitwise reproducible
    sc.p2g3(pfm.soa(m0), pfm.soa(pos), pfm.soa_T(T_gm), pfm.soa_T(Ti), pfm.soa_T(C), u2, w2)
    for a, b in zip(u + w, u2 + w2):
        assert torch.equal(a, b)


def test_sort_large_bins_bitexact_and_bounded():
    """Bins far beyond the register network's 16 entries: 1.5M particles in one cell, 300K in
    another, 4,000 and 17 in two more, the rest spread, in a shuffled particle order (so the atomic
    slot order inside each bin is scrambled): the permutation equals numpy's stable argsort bit for
    bit, and the sort of 2.1M particles ends within a time bound."""
    import time
    rng = np.random.default_rng(21)
    res = (16, 12, 20)
    dx = 1.0 / res[1]
    parts = [(np.array([5, 6, 7]) + rng.random((1_500_000, 3))) * dx,
             (np.array([0, 0, 0]) + rng.random((300_000, 3))) * dx,
             (np.array([15, 11, 19]) + rng.random((4000, 3))) * dx,
             (np.array([9, 2, 3]) + rng.random((17, 3))) * dx,
             rng.random((300_000, 3)) * np.array(res) * dx]
    pos = np.concatenate(parts).astype(np.float32)
    pos = pos[rng.permutation(pos.shape[0])]
    P = pos.shape[0]
    sc = pfm.Scene(3, res, dx, P)
    pos_d = pfm.soa(pos)
    cells = np.clip((pos / np.float32(dx)).astype(np.int64), 0, np.array(res) - 1)
    key = (cells[:, 0] * res[1] + cells[:, 1]) * res[2] + cells[:, 2]
    want = np.argsort(key, kind="stable")
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        count, order = sc.sort_particles(pos_d)
        torch.cuda.synchronize()
        assert time.perf_counter() - t0 < 2.0
        assert np.array_equal(host(order), want)
        assert np.array_equal(host(count).ravel(), np.bincount(key, minlength=int(np.prod(res))))


def test_p2g2_collisions_and_edges():
    rng = np.random.default_rng(12)
    res = (24, 16)
    dx = 1.0 / res[1]
    hi = np.array(res, np.float64) * dx
    pos = np.concatenate([(np.array([3, 9]) + rng.uniform(0, 1, (4000, 2))) * dx,
                          np.floor(rng.uniform(0, 1, (300, 2)) * np.array(res)) * dx,
                          np.array([[0, 0], hi, [hi[0], 0], [0, hi[1]]]),
                          rng.uniform(0, 1, (1500, 2)) * hi]).astype(np.float32)
    P = pos.shape[0]
    sc = pfm.Scene(2, res, dx, P)
    imp = rng.standard_normal((P, 2)).astype(np.float32)
    C = (0.3 * rng.standard_normal((P, 2, 2))).astype(np.float32)
    psi = (pos + 0.01 * rng.standard_normal((P, 2))).astype(np.float32)
    u, w = sc.alloc_faces(), sc.alloc_faces()
    psi_g = [torch.zeros(s + (2,), device="cuda") for s in sc.face_shapes]
    sc.p2g2(pfm.soa(imp), pfm.soa(pos), pfm.soa_T(C), pfm.soa(psi), u, w, psi_out=psi_g)
    (ox, oy), (owx, owy), (opx, opy) = O.p2g2(imp, pos, C, psi, res, dx)
    for t, o in zip(u + w + psi_g, [ox, oy, owx, owy, opx, opy]):
        assert rel(host(t), o) < TOL


def test_sort_bitexact_512_cube():
    """A 512^3 grid: 134,217,728 cells, 16,384 block sums, so the one-block scan of the block sums
    runs in two chunks with the total carried between them.  2^20 particles spread over the grid,
    a fifth of them in the last eighth of the cells (whose starts the carry offsets): counts and
    permutation bit for bit numpy's."""
    rng = np.random.default_rng(31)
    n = 512
    res = (n, n, n)
    P = 1 << 20
    pos = rng.uniform(0.0, 1.0, (P, 3)).astype(np.float32)
    pos[: P // 5, 0] = rng.uniform(0.875, 1.0, P // 5).astype(np.float32)
    sc = pfm.Scene(3, res, 1.0 / n, P)
    count, order = sc.sort_particles(pfm.soa(pos))
    cells = np.clip((pos / np.float32(1.0 / n)).astype(np.int64), 0, n - 1)
    key = (cells[:, 0] * n + cells[:, 1]) * n + cells[:, 2]
    assert np.array_equal(host(order), np.argsort(key, kind="stable"))
    c = host(count).ravel()
    nz = np.nonzero(c)[0]
    ref = np.bincount(key, minlength=n ** 3)
    assert np.array_equal(nz, np.nonzero(ref)[0]) and np.array_equal(c[nz], ref[nz])
    del sc, count, order
    torch.cuda.empty_cache()
