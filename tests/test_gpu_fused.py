"""The fused RK4_T_forward + P2G entry points (pfm3_rk4_p2g_records / pfm3_p2g_from_records /
pfm3_rk4_p2g) against the separate calls pfm3_rk4_T_forward then pfm3_p2g: bitwise equal grids,
weights, positions and T, including particles outside the grid."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import pfm  # noqa: E402


def _scene(res=(24, 16, 20), ppc=8, seed=4):
    dx = 1.0 / res[1]
    rng = np.random.default_rng(seed)
    pos = pfm.jittered(res, dx, ppc, seed=seed)
    pos[:11] += np.float32(1.5 * dx)    # some particles leave the grid on the high side
    pos[11:23] -= np.float32(1.2 * dx)  # and on the low side
    P = pos.shape[0]
    dev = torch.device("cuda:0")
    sc = pfm.Scene(3, res, dx, P)
    u = [torch.from_numpy((0.3 * rng.standard_normal(s)).astype(np.float32)).to(dev) for s in sc.face_shapes]
    st = dict(pos=pfm.soa(pos, dev),
              T_gm=torch.from_numpy((np.eye(3)[:, :, None] + 0.05 * rng.standard_normal((3, 3, P))).astype(np.float32)).to(dev),
              init_imp=torch.from_numpy(rng.standard_normal((3, P)).astype(np.float32)).to(dev),
              T_init=torch.from_numpy((np.eye(3)[:, :, None] + 0.05 * rng.standard_normal((3, 3, P))).astype(np.float32)).to(dev),
              init_C=torch.from_numpy(rng.standard_normal((3, 3, P)).astype(np.float32)).to(dev))
    return sc, u, st


def _clone(st):
    return {k: v.clone() for k, v in st.items()}


@pytest.mark.parametrize("mode", ["two_calls", "one_call"])
def test_rk4_p2g_matches_separate_calls(mode):
    sc, u, st = _scene()
    dt = 0.01
    a, b = _clone(st), _clone(st)
    ua, wa = sc.alloc_faces(), sc.alloc_faces()
    sc.rk4_T_forward(a["pos"], a["T_gm"], u, dt)
    sc.p2g3(a["init_imp"], a["pos"], a["T_gm"], a["T_init"], a["init_C"], ua, wa)
    ub, wb = sc.alloc_faces(), sc.alloc_faces()
    if mode == "two_calls":
        sc.rk4_p2g_records3(b["pos"], b["T_gm"], u, dt, b["init_imp"], b["T_init"], b["init_C"])
        sc.p2g_from_records3(ub, wb)
    else:
        sc.rk4_p2g3(b["pos"], b["T_gm"], u, dt, b["init_imp"], b["T_init"], b["init_C"], ub, wb)
    torch.cuda.synchronize()
    assert torch.equal(a["pos"], b["pos"]) and torch.equal(a["T_gm"], b["T_gm"])
    for f in range(3):
        assert torch.equal(ua[f], ub[f]), f
        assert torch.equal(wa[f], wb[f]), f


def test_p2g_from_records_needs_records():
    sc, u, st = _scene(res=(8, 8, 8), ppc=1)
    out, w = sc.alloc_faces(), sc.alloc_faces()
    with pytest.raises(pfm.PfmError, match="no P2G records"):
        sc.p2g_from_records3(out, w)
    sc.rk4_p2g_records3(st["pos"], st["T_gm"], u, 0.01, st["init_imp"], st["T_init"], st["init_C"])
    sc.sort_particles(st["pos"])  # overwrites the keys of the records
    with pytest.raises(pfm.PfmError, match="no P2G records"):
        sc.p2g_from_records3(out, w)


def test_gradm_rk4_records_matches_separate_calls():
    """g2p(C) + update_T(reset) + rk4_p2g_records + p2g_from_records against the fused gradient
    reinitialisation kernel: bitwise equal particle state and grids."""
    sc, u, st = _scene(seed=7)
    rng = np.random.default_rng(9)
    ua = [torch.from_numpy((0.3 * rng.standard_normal(s)).astype(np.float32)).cuda() for s in sc.face_shapes]
    dt = 0.01
    a, b = _clone(st), _clone(st)
    wa, wb = sc.alloc_faces(), sc.alloc_faces()
    oa, ob = sc.alloc_faces(), sc.alloc_faces()
    sc.g2p(a["pos"], u, C_out=a["init_C"])
    sc.update_T(a["T_init"], a["T_gm"], reset_gm=True)
    sc.rk4_p2g_records3(a["pos"], a["T_gm"], ua, dt, a["init_imp"], a["T_init"], a["init_C"])
    sc.p2g_from_records3(oa, wa)
    sc.gradm_rk4_records3(b["pos"], b["T_gm"], b["T_init"], b["init_C"], b["init_imp"], u, ua, dt)
    sc.p2g_from_records3(ob, wb)
    torch.cuda.synchronize()
    for k in ("pos", "T_gm", "T_init", "init_C"):
        assert torch.equal(a[k], b[k]), k
    for f in range(3):
        assert torch.equal(oa[f], ob[f]) and torch.equal(wa[f], wb[f]), f


@pytest.mark.parametrize("n", [64, 128])
def test_cube_instances_equal_runtime_strides(n):
    """PFM_TUNE_CUBE_KERNELS: on an n^3 grid the RK4 kernels (with and without the gradient
    reinitialisation) and the midpoint kernels run instances compiled for the extent n; with the
    tunable off they read the strides at run time.  Same loads and sums: bitwise equal outputs."""
    from pfm import _lib
    sc, u, st = _scene(res=(n, n, n), ppc=1, seed=11)
    rng = np.random.default_rng(12)
    ua = [torch.from_numpy((0.3 * rng.standard_normal(s)).astype(np.float32)).cuda() for s in sc.face_shapes]
    dt = 0.4 / n
    outs = []
    for cube in (1, 0):
        sc.set_tuning(_lib.TUNE_CUBE_KERNELS, cube)
        a, b = _clone(st), _clone(st)
        sc.gradm_rk4_records3(a["pos"], a["T_gm"], a["T_init"], a["init_C"], a["init_imp"], u, ua, dt)
        sc.rk4_T_forward(b["pos"], b["T_gm"], ua, dt)
        mid = sc.alloc_faces()
        sc.midpoint(u, mid, 0.5 * dt)
        torch.cuda.synchronize()
        outs.append([a[k] for k in ("pos", "T_gm", "T_init", "init_C")] + [b["pos"], b["T_gm"]] + list(mid))
    for x, y in zip(*outs):
        assert torch.equal(x, y)


@pytest.mark.parametrize("n", [256, 512])
def test_cube_instance_large_equals_runtime_strides(n):
    """The 256^3 instances (the ones the 256^3 workload runs) and the 512^3 ones (the largest extent
    compiled in; its row offsets reach 2 MB) against the runtime-stride kernels: the RK4 with the
    gradient reinitialisation on 2^20 particles spread over the whole grid, and the three midpoint
    launches over every face.  Bitwise equal."""
    from pfm import _lib
    dx = 1.0 / n
    P = 1 << 20
    rng = np.random.default_rng(13)
    dev = torch.device("cuda:0")
    sc = pfm.Scene(3, (n, n, n), dx, P)
    g = torch.Generator(device=dev).manual_seed(5)
    u = [(0.3 * torch.randn(s, device=dev, generator=g)) for s in sc.face_shapes]
    ua = [(0.3 * torch.randn(s, device=dev, generator=g)) for s in sc.face_shapes]
    pos = torch.from_numpy(rng.uniform(0.0, 1.0, (3, P)).astype(np.float32)).to(dev)
    eye = torch.eye(3, device=dev).reshape(3, 3, 1)
    st = dict(pos=pos, T_gm=eye + 0.05 * torch.randn(3, 3, P, device=dev, generator=g),
              T_init=eye + 0.05 * torch.randn(3, 3, P, device=dev, generator=g),
              init_C=torch.randn(3, 3, P, device=dev, generator=g),
              init_imp=torch.randn(3, P, device=dev, generator=g))
    dt = 0.4 / n
    outs = []
    for cube in (1, 0):
        sc.set_tuning(_lib.TUNE_CUBE_KERNELS, cube)
        a = _clone(st)
        sc.gradm_rk4_records3(a["pos"], a["T_gm"], a["T_init"], a["init_C"], a["init_imp"], u, ua, dt)
        mid = sc.alloc_faces()
        sc.midpoint(u, mid, 0.5 * dt)
        torch.cuda.synchronize()
        outs.append([a[k] for k in ("pos", "T_gm", "T_init", "init_C")] + list(mid))
    for x, y in zip(*outs):
        assert torch.equal(x, y)
    del outs, u, ua, sc
    torch.cuda.empty_cache()


@pytest.mark.parametrize("res", [(64, 64, 64), (40, 32, 48)])
def test_midpoint_face_centre_form_equals_generic_taps(res):
    """PFM_TUNE_MIDPOINT_CENTRE: the midpoint's first RK stage samples the face centre, where every
    axis' weights are the t = 0 or t = -1/2 constants; the constant-weight form leaves the
    zero-weight taps out and is bitwise the generic interpolation (a cube instance and a grid with
    the strides read at run time; boundary faces, where a clamp binds, take the generic taps)."""
    from pfm import _lib
    dx = 1.0 / 32
    sc = pfm.Scene(3, res, dx, 0)
    g = torch.Generator(device="cuda").manual_seed(17)
    u = [0.3 * torch.randn(s, device="cuda", generator=g) for s in sc.face_shapes]
    outs = []
    for centre in (1, 0):
        sc.set_tuning(_lib.TUNE_MIDPOINT_CENTRE, centre)
        mid = sc.alloc_faces()
        psi = [torch.zeros(s + (3,), device="cuda") for s in sc.face_shapes]
        T = [torch.zeros(s + (3,), device="cuda") for s in sc.face_shapes]
        sc.midpoint(u, mid, 0.7 * dx, psi_out=psi, T_out=T)
        torch.cuda.synchronize()
        outs.append(list(mid) + psi + T)
    for x, y in zip(*outs):
        assert torch.equal(x, y)
