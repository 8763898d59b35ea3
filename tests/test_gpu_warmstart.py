"""What the trained network gains over the warm start without it, on a small plume: the network
is trained on (divergence, pressure) pairs of plume runs at 32^3 from three sources and evaluated
on a held-out source.  Its initial pressure must be closer to the converged pressure than the
previous step's pressure (the method without the network) and than zero, and MGPCG must still
reach the same residual from it in no more iterations than from zero."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rel(g, p):
    g = g - g.mean()
    q = p - p.mean()
    return (g - q).norm().item() / q.norm().item()


def test_trained_network_beats_previous_pressure():
    from pfm.nn import UNet3D
    from pfm.plume import Plume3D
    torch.cuda.set_device(0)
    res = (32, 32, 32)
    data = []
    for src in [(0.4, 0.1, 0.4), (0.6, 0.1, 0.5), (0.45, 0.1, 0.6)]:
        sim = Plume3D(res=res, source=src)
        sim.record = []
        for _ in range(45):
            sim.step()
        data += sim.record[5:]
        del sim
    net = UNet3D(seed=0, lr=2e-3)
    rng = np.random.default_rng(0)
    for it in range(800):
        d, p = data[int(rng.integers(len(data)))]
        net.train_step(d, p, lr=2e-3 * 0.5 * (1 + np.cos(np.pi * it / 800)))
    torch.cuda.synchronize()
    net.check()
    sim = Plume3D(res=res, source=(0.55, 0.1, 0.42))
    for _ in range(5):
        sim.step()
    err_prev, err_net, it_zero, it_net, it_prev = [], [], [], [], []

    def compare():  # inside the step, before its final projection: the divergence P2G left
        sim.divergence()
        div = sim.div.clone()
        prev = sim.p.clone()
        u0 = [a.clone() for a in sim.u]
        p0 = torch.zeros_like(prev)
        i0 = sim.scene.poisson([a.clone() for a in u0], p0, **sim.poisson_opts)
        guess = net.predict(div)
        pn = guess.clone()
        i1 = sim.scene.poisson([a.clone() for a in u0], pn, warm_start=True, **sim.poisson_opts)
        pp = prev.clone()
        i2 = sim.scene.poisson([a.clone() for a in u0], pp, warm_start=True, **sim.poisson_opts)
        assert i0.converged and i1.converged and i2.converged
        err_prev.append(_rel(prev, p0))
        err_net.append(_rel(guess, p0))
        it_zero.append(i0.iterations)
        it_net.append(i1.iterations)
        it_prev.append(i2.iterations)
        return {"warm_start": True}

    sim.before_poisson = compare
    for _ in range(15):
        sim.step()
    torch.cuda.synchronize()
    # the guess is clearly closer than the previous pressure (measured: 0.075 against 0.142 with the
    # line-grouped seeding order, 8x closer at 192^3 in the study)
    assert np.mean(err_net) < 0.6 * np.mean(err_prev), (np.mean(err_net), np.mean(err_prev))
    assert np.mean(err_net) < 0.5
    assert np.mean(it_net) <= np.mean(it_zero), (it_net, it_zero)
