"""Drop-in for the reference's 2D/init_conditions.py: the leapfrog initial velocity and the
particle initialisation under the same names and arguments (2D/init_conditions.py:5-60,
139-212), on CUDA tensors.  Particle vector fields are SoA tensors [2, P]; C_x/C_y are the rows of
one [2, 2, P] tensor (``pfm.dropin.vector_rows``).  The initial velocity is one-time set-up and
is evaluated on the host in f32 (the Taichi kernel's expression order) and copied to the device."""
import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from pfm import dropin as _d  # noqa: E402


def angular_vel_func(r, rad, strength):
    """Gaussian-core vortex profile divided by r (2D/init_conditions.py:5-9), f32."""
    f = np.float32
    r = (r + f(1e-6)).astype(np.float32)
    linear_vel = ((f(strength) * f(1.)) / r * (f(1.) - np.exp(-(r ** 2) / f(rad ** 2)).astype(np.float32))).astype(np.float32)
    return ((f(1.) / r) * linear_vel).astype(np.float32)


def leapfrog_vel_func(vf, pf):
    """Two counter-rotating vortex pairs at x = 0.25 (2D/init_conditions.py:29-60) into the
    cell-centred field vf [nx, ny, 2]; pf (the cell centres (I + 0.5) dx, dx = 1 / ny) is implied
    by vf's grid."""
    nx, ny = int(vf.shape[0]), int(vf.shape[1])
    dxf = np.float32(1.0 / ny)
    ii, jj = np.meshgrid(np.arange(nx, dtype=np.float32), np.arange(ny, dtype=np.float32), indexing="ij")
    px = ((ii + np.float32(0.5)) * dxf).astype(np.float32)
    py = ((jj + np.float32(0.5)) * dxf).astype(np.float32)
    out = np.zeros((nx, ny, 2), np.float32)
    for (cx, cy), wv in (((0.25, 0.62), -0.5), ((0.25, 0.38), 0.5), ((0.25, 0.74), -0.5), ((0.25, 0.26), 0.5)):
        dxp = (px - np.float32(cx)).astype(np.float32)
        dyp = (py - np.float32(cy)).astype(np.float32)
        r = np.sqrt(dxp * dxp + dyp * dyp).astype(np.float32)
        s = (angular_vel_func(r, 0.02, -0.01) * np.float32(wv)).astype(np.float32)
        out[..., 0] += (s * -dyp).astype(np.float32)
        out[..., 1] += (s * dxp).astype(np.float32)
    vf.copy_(torch.from_numpy(out))


def stripe_func(qf, pf, x_start, x_end):
    """Smoke stripe (2D/init_conditions.py:108-113): qf [nx, ny, 3] = 0 where the cell centre lies in
    x_start <= x <= x_end and 0.15 <= y <= 0.85, else 1.  pf (the cell centres (I + 0.5) dx,
    dx = 1 / ny) is implied by qf's grid; the centres are formed in f32 as the reference's."""
    nx, ny = int(qf.shape[0]), int(qf.shape[1])
    dxf = np.float32(1.0 / ny)
    x = (np.arange(nx, dtype=np.float32) + np.float32(0.5)) * dxf
    y = (np.arange(ny, dtype=np.float32) + np.float32(0.5)) * dxf
    inside = ((x[:, None] >= np.float32(x_start)) & (x[:, None] <= np.float32(x_end))
              & (y[None, :] >= np.float32(0.15)) & (y[None, :] <= np.float32(0.85)))
    out = np.where(inside[..., None], np.float32(0.0), np.float32(1.0)) * np.ones((1, 1, 3), np.float32)
    qf.copy_(torch.from_numpy(out.astype(np.float32)))


def init_particles_pos_uniform(particles_pos, X, res_x, particles_per_cell, dx, particles_per_cell_axis,
                               dist_between_neighbor):
    """Particles on the x-fastest lattice at (index + 0.5) * dist_between_neighbor
    (2D/init_conditions.py:139-166); particles_pos is [2, P]."""
    _d.check_soa(particles_pos, 2, "particles_pos")
    P = particles_pos.shape[1]
    a = int(particles_per_cell_axis)
    res_y = P // (res_x * a * a)
    lat = _d.lattice_device((res_x, res_y), float(dist_between_neighbor) * a, a, particles_pos.device)
    particles_pos.copy_(lat)


def _g2p(particles_pos, u_x, u_y, imp_out, C_rows, dx):
    _d.check_soa(particles_pos, 2, "particles_pos")
    res = (u_x.shape[0] - 1, u_x.shape[1])
    sc = _d.scene(2, res, float(dx), particles_pos.shape[1])
    if C_rows is None:
        sc.g2p(particles_pos, [u_x, u_y], imp_out=imp_out)
        return
    with _d.Rows(C_rows, out=True) as C:
        sc.g2p(particles_pos, [u_x, u_y], imp_out=imp_out, C_out=C)


def init_particles_imp(particles_imp, particles_init_imp, particles_pos, u_x, u_y, C_x, C_y, dx):
    """G2P of the velocity into particles_imp and particles_init_imp (2D/init_conditions.py:183-192)."""
    _g2p(particles_pos, u_x, u_y, particles_imp, None, dx)
    particles_init_imp.copy_(particles_imp)


def init_particles_imp_grad_m(particles_imp, particles_pos, u_x, u_y, C_x, C_y, dx):
    """G2P of the velocity and its gradient rows C_x/C_y (2D/init_conditions.py:203-211)."""
    _g2p(particles_pos, u_x, u_y, particles_imp, (C_x, C_y), dx)
