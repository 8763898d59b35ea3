"""Scalar (smoke) transport and vorticity diagnostics on the GPU, through the C ABI, against the
reference's own kernels (tests/golden/ref3d_fields.npz, ref2d_fields.npz) and the CPU oracle.

Tolerances: the grid stencils (get_central_vector, curl, advect_smoke, clamp_smoke) evaluate the
reference's expressions in its order with rounded products, so they are compared bit for bit.
The particle transfers (init_particles_smoke, P2G_smoke) sum their taps in another association
than the reference's triple loop and are held to 1e-5 relative L2 (TOL); P2G_smoke is also
checked bitwise reproducible from call to call.
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
def f3(golden):
    return golden("ref3d_fields")


@pytest.fixture(scope="module")
def f2(golden):
    return golden("ref2d_fields")


def scene(g, P=0):
    res = tuple(int(x) for x in g["res"])
    return pfm.Scene(len(res), res, 1.0 / res[1], P)


def smooth(shape, seed, amp=1.0):
    rng = np.random.default_rng(seed)
    idx = np.meshgrid(*[np.linspace(0, 1, s) for s in shape], indexing="ij")
    out = np.zeros(shape)
    for _ in range(3):
        term = rng.uniform(-1, 1)
        for x in idx:
            term = term * np.sin(2 * np.pi * rng.uniform(0.5, 2) * x + rng.uniform(0, 6))
        out += term
    return (amp * out).astype(np.float32)


# ------------------------------------------------------------------------------------------------
# diagnostics
# ------------------------------------------------------------------------------------------------
def test_central_curl3_golden(f3):
    sc = scene(f3)
    vc = sc.get_central_vector([dev(f3[k]) for k in ("u_x", "u_y", "u_z")])
    w = sc.curl(vc, dx=float(f3["dx"]))
    torch.cuda.synchronize()
    assert np.array_equal(host(vc), f3["central"])
    assert np.array_equal(host(w), f3["curl"])


def test_central_curl2_golden(f2):
    sc = scene(f2)
    vc = sc.get_central_vector([dev(f2[k]) for k in ("u_x", "u_y")])
    w = sc.curl(vc, dx=float(f2["dx"]))
    torch.cuda.synchronize()
    assert np.array_equal(host(vc), f2["central"])
    assert np.array_equal(host(w), f2["curl"])


def test_central_curl3_oracle_larger():
    res = (40, 32, 24)
    u = [smooth((41, 32, 24), 1), smooth((40, 33, 24), 2), smooth((40, 32, 25), 3)]
    sc = pfm.Scene(3, res, 1.0 / 32, 0)
    vc = sc.get_central_vector([dev(a) for a in u])
    w = sc.curl(vc)
    torch.cuda.synchronize()
    vref = O.central_vector3(*u)
    assert np.array_equal(host(vc), vref)
    assert np.array_equal(host(w), O.curl3(vref, 1.0 / 32))


# ------------------------------------------------------------------------------------------------
# smoke
# ------------------------------------------------------------------------------------------------
def test_init_particles_smoke_golden(f3):
    P = f3["pos"].shape[0]
    sc = scene(f3, P)
    s = torch.zeros(4, P, device="cuda")
    G = torch.zeros(3, 4, P, device="cuda")
    sc.init_particles_smoke(pfm.soa(f3["pos"]), dev(f3["smoke"]), s, G)
    torch.cuda.synchronize()
    assert rel(pfm.aos(s), f3["g2p_smoke"]) < TOL
    assert rel(pfm.aos_T(G), f3["g2p_grad_smoke"]) < TOL


def test_p2g_smoke_golden(f3):
    P = f3["pos"].shape[0]
    sc = scene(f3, P)
    res = tuple(int(x) for x in f3["res"])
    sm = torch.zeros(res + (4,), device="cuda")
    w = torch.zeros(res, device="cuda")
    args = (dev(f3["smoke_p"].T), pfm.soa_T(f3["grad_smoke"]), pfm.soa(f3["pos"]), pfm.soa_T(f3["T_gm"]),
            pfm.soa_T(f3["T_init"]))
    sc.p2g_smoke(*args, sm, w)
    torch.cuda.synchronize()
    assert rel(host(w), f3["p2g_smoke_w"]) < TOL
    assert rel(host(sm), f3["p2g_smoke"]) < TOL
    first = host(sm).copy()
    sc.p2g_smoke(*args, sm, w)
    torch.cuda.synchronize()
    assert np.array_equal(host(sm), first)


@pytest.mark.parametrize("use_apic", [True, False])
def test_p2g_smoke_oracle_jittered(use_apic):
    res = (32, 24, 16)
    dx = 1.0 / 24
    pos = pfm.jittered(res, dx, 8, seed=3)
    P = pos.shape[0]
    rng = np.random.default_rng(5)
    pos = (pos + rng.normal(0, 0.3 * dx, size=pos.shape)).astype(np.float32)  # a few leave the grid
    s_p = rng.uniform(0, 1, size=(P, 4)).astype(np.float32)
    G = rng.normal(0, 2, size=(P, 3, 4)).astype(np.float32)
    Tg = (np.eye(3)[None] + 0.05 * rng.standard_normal((P, 3, 3))).astype(np.float32)
    Ti = (np.eye(3)[None] + 0.05 * rng.standard_normal((P, 3, 3))).astype(np.float32)
    sc = pfm.Scene(3, res, dx, P)
    sm = torch.zeros(res + (4,), device="cuda")
    w = torch.zeros(res, device="cuda")
    sc.p2g_smoke(dev(s_p.T), pfm.soa_T(G), pfm.soa(pos), pfm.soa_T(Tg), pfm.soa_T(Ti), sm, w, use_apic_smoke=use_apic)
    torch.cuda.synchronize()
    ref_sm, ref_w = O.p2g_smoke3(s_p, G, pos, Tg, Ti, res, dx, use_apic=use_apic)
    assert rel(host(w), ref_w) < TOL
    assert rel(host(sm), ref_sm) < TOL
    assert host(sm).min() >= 0.0 and host(sm).max() <= 1.0


def test_advect_clamp_smoke3_golden(f3):
    sc = scene(f3)
    psi = [dev(f3[k]) for k in ("psi_x", "psi_y", "psi_z")]
    s0 = dev(f3["smoke"])
    s1 = torch.zeros_like(s0)
    sc.advect_smoke(s0, s1, psi, dx=float(f3["dx"]))
    torch.cuda.synchronize()
    assert np.array_equal(host(s1), f3["advect_smoke"])
    s1 = dev(f3["clamp_in"])
    sc.clamp_smoke(s0, s1, psi, dx=float(f3["dx"]))
    torch.cuda.synchronize()
    assert np.array_equal(host(s1), f3["clamp_smoke"])


def test_advect_smoke2_golden(f2):
    sc = scene(f2)
    s0 = dev(f2["smoke"])
    s1 = torch.zeros_like(s0)
    sc.advect_smoke(s0, s1, [dev(f2["psi_x"]), dev(f2["psi_y"])], dx=float(f2["dx"]))
    torch.cuda.synchronize()
    assert np.array_equal(host(s1), f2["advect_smoke"])


def test_advect_smoke3_midpoint_map():
    """advect_smoke through the backward map pfm3_midpoint writes (the reference's psi grids)."""
    res = (24, 24, 16)
    dx = 1.0 / 24
    u = [smooth((25, 24, 16), 7, 0.5), smooth((24, 25, 16), 8, 0.5), smooth((24, 24, 17), 9, 0.5)]
    sc = pfm.Scene(3, res, dx, 0)
    ud = [dev(a) for a in u]
    u1 = sc.alloc_faces()
    psi = [torch.empty(s + (3,), device="cuda") for s in sc.face_shapes]
    sc.midpoint(ud, u1, 0.02, psi_out=psi)
    s0 = dev(np.abs(np.stack([smooth(res, 10 + c) for c in range(4)], -1)))
    s1 = torch.zeros_like(s0)
    sc.advect_smoke(s0, s1, psi)
    torch.cuda.synchronize()
    ref = O.advect_smoke3(host(s0), np.zeros(res + (4,), np.float32), *(host(p) for p in psi), dx)
    assert np.array_equal(host(s1), ref)


def test_vortex_ring_and_smoke_golden(f3):
    sc = scene(f3)
    res = tuple(int(x) for x in f3["res"])
    vc = torch.zeros(res + (3,), device="cuda")
    sm = torch.zeros(res + (4,), device="cuda")
    sc.add_vortex_ring_and_smoke(vc, sm, w=0.02, rad=0.2, delta=0.04, c=(0.45, 0.5, 0.33), unit_x=(0., 0., -1.),
                                 unit_y=(0., 1., 0.), color=(1., 0.5, 0.25), num_samples=64)
    torch.cuda.synchronize()
    assert rel(host(vc), f3["ring_u"]) < TOL
    assert np.array_equal(host(sm), f3["ring_smoke"])


def test_smoke_errors():
    sc = pfm.Scene(3, (8, 8, 8), 1.0 / 8, 0)
    s0 = torch.zeros((8, 8, 8, 4), device="cuda")
    with pytest.raises(pfm.PfmError):
        sc.advect_smoke(s0, torch.zeros((8, 8, 8, 3), device="cuda"),
                        [torch.zeros(s + (3,), device="cuda") for s in sc.face_shapes])
    with pytest.raises(pfm.PfmError):  # the kernels read the smoke cells as 16-byte vectors
        sc.clamp_smoke(s0, torch.zeros(8 * 8 * 8 * 4 + 1, device="cuda")[1:].view(8, 8, 8, 4),
                       [torch.zeros(s + (3,), device="cuda") for s in sc.face_shapes])
    s2 = pfm.Scene(2, (8, 8), 1.0 / 8, 0)
    with pytest.raises(pfm.PfmError):
        s2.clamp_smoke(s0, s0, [])


def test_add_fields_and_scale_field_bitwise():
    """add_fields / scale_field (3D/taichi_utils.py:13-21) through the library's elementwise
    kernels: bitwise the f32 expression with the product rounded before the sum."""
    rng = np.random.default_rng(17)
    f1 = rng.standard_normal((33, 17, 9)).astype(np.float32)
    f2 = rng.standard_normal((33, 17, 9)).astype(np.float32)
    m = np.float32(-0.3711)
    dest = torch.empty(f1.shape, device="cuda")
    pfm.add_fields(torch.from_numpy(f1).cuda(), torch.from_numpy(f2).cuda(), dest, float(m))
    res = torch.empty(f1.shape, device="cuda")
    pfm.scale_field(torch.from_numpy(f2).cuda(), float(m), res)
    torch.cuda.synchronize()
    assert np.array_equal(dest.cpu().numpy(), (f1 + (m * f2).astype(np.float32)).astype(np.float32))
    assert np.array_equal(res.cpu().numpy(), (m * f2).astype(np.float32))
    with pytest.raises(pfm.PfmError):
        pfm.add_fields(torch.zeros(3, device="cuda"), torch.zeros(4, device="cuda"), torch.zeros(3, device="cuda"), 1.0)
