"""GPU checks of the plume kernels against oracle/plume_oracle.py and of a short plume run: the
density source and transport, the buoyancy impulse (the impulse P2G forms grows by exactly the
force), and the learned-guess path of the final projection (the solve still reaches its residual
from any initial pressure)."""
import numpy as np
import pytest
import torch

import plume_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    import pfm
    torch.cuda.set_device(0)
    res = (16, 12, 8)
    return pfm.Scene(3, res, 1.0 / 12, 3000), res


def _p(t):
    import ctypes
    return ctypes.c_void_p(t.data_ptr())


def test_source_and_advection(scene):
    sc, res = scene
    dx = sc.dx
    rng = np.random.default_rng(0)
    rho = torch.zeros(res, device="cuda")
    st = None
    sc._check(sc.lib.pfm3_plume_source(sc.h, _p(rho), 0.5, 0.3, 0.3, 0.25, 1.0, st))
    ref = O.plume_source(np.zeros(res, np.float32), dx, (0.5, 0.3, 0.3), 0.25, 1.0)
    np.testing.assert_array_equal(rho.cpu().numpy(), ref)
    assert ref.sum() > 10
    rho0 = rng.random(res).astype(np.float32)
    u = [rng.standard_normal(s).astype(np.float32) for s in sc.face_shapes]
    r0 = torch.as_tensor(rho0).cuda()
    r1 = torch.empty_like(r0)
    ut = [torch.as_tensor(a).cuda() for a in u]
    dt = 0.7 * dx
    sc._check(sc.lib.pfm3_advect_density(sc.h, _p(r0), _p(r1), *map(_p, ut), dt, st))
    ref = O.advect_density(rho0, *u, dx, dt)
    np.testing.assert_allclose(r1.cpu().numpy(), ref, rtol=1e-5, atol=1e-6)


def test_buoyancy_impulse(scene):
    sc, res = scene
    P = sc.P
    dx = sc.dx
    rng = np.random.default_rng(1)
    ext = np.array(res) * dx
    pos = (rng.random((3, P)) * ext[:, None]).astype(np.float32)
    T_gm = (np.eye(3)[:, :, None] + 0.2 * rng.standard_normal((3, 3, P))).astype(np.float32)
    T_in = (np.eye(3)[:, :, None] + 0.2 * rng.standard_normal((3, 3, P))).astype(np.float32)
    imp = rng.standard_normal((3, P)).astype(np.float32)
    rho = rng.random(res).astype(np.float32)
    t = [torch.as_tensor(a).cuda().contiguous() for a in (pos, T_gm, T_in, imp, rho)]
    coef = 0.05
    for axis in (0, 1, 2):
        it = t[3].clone()
        sc._check(sc.lib.pfm3_add_buoyancy_impulse(sc.h, _p(t[0]), _p(t[1]), _p(t[2]), _p(it), _p(t[4]), coef, axis,
                                                   None))
        got = it.cpu().numpy()
        ref = O.buoyancy_impulse(pos, T_gm, T_in, imp, rho, dx, coef, axis)
        M = O.composite(T_gm, T_in)
        cond = np.linalg.cond(M)
        good = cond < 1e3
        np.testing.assert_allclose(got[:, good], ref[:, good], rtol=1e-4, atol=1e-4)
        # the defining property: M (init_imp + delta) = M init_imp + f e_axis
        f = coef * O.sample_cells(rho, dx, *pos)
        lhs = np.einsum("pij,jp->ip", M, got.astype(np.float64)) - np.einsum("pij,jp->ip", M, imp.astype(np.float64))
        want = np.zeros((3, P))
        want[axis] = f
        np.testing.assert_allclose(lhs[:, good], want[:, good], atol=2e-5)


def test_plume_run_and_guess_path():
    import pfm
    from pfm.plume import Plume3D
    res = (32, 32, 32)
    sim = Plume3D(res=res)
    sim.record = []
    for _ in range(6):
        sim.step()
    torch.cuda.synchronize()
    assert all(i.converged for i in sim.infos), [repr(i) for i in sim.infos]
    rho = sim.rho.cpu().numpy()
    n_src = int(O.plume_source(np.zeros(res, np.float32), 1.0 / 32, (0.5, 0.1, 0.5), 0.05, 1.0).sum())
    assert rho.max() == 1.0 and rho.sum() > n_src  # the source cells plus the smoke carried out of them
    uy = sim.u[1].cpu().numpy()
    assert uy[13:19, 3:9, 13:19].mean() > 0  # the plume rises above the source (a closed box: no net flux)
    assert len(sim.record) == 6
    # divergence left after the final projection is at the solver's residual
    d_after = torch.zeros(res, device="cuda")
    sim.scene.divergence(sim.u, d_after)
    d_before = sim.record[-1][0]
    assert d_after.norm().item() < 1e-3 * d_before.norm().item() + 1e-9
    # a callable guess (the network's slot): any initial pressure, same residual at the end
    calls = []

    def guess(div, p_out):
        calls.append(1)
        p_out.copy_(torch.randn_like(p_out))

    sim.pressure_guess = guess
    sim.step()
    torch.cuda.synchronize()
    assert calls and sim.infos[-1].converged
    sim.scene.divergence(sim.u, d_after)
    assert d_after.norm().item() < 1e-3 * sim.div.norm().item() + 1e-9
