"""Drop-in for the reference's 3D/init_conditions.py: initial velocity fields and particle
initialisation under the same names and arguments (3D/init_conditions.py:10-22, 79-118,
238-273), on CUDA tensors.  Particle vector fields are SoA tensors [3, P]; the per-row fields
C_x/C_y/C_z are the rows of one [3, 3, P] tensor (``pfm.dropin.vector_rows``); particle smoke is [4, P] and its gradient
[3, 4, P]; smoke grids are [nx, ny, nz, 4]."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from pfm import dropin as _d  # noqa: E402


def _scene_for_cells(vf):
    res = tuple(int(n) for n in vf.shape[:3])
    return _d.scene(3, res, 1.0 / res[1], 0)


def add_vortex_ring(w, rad, delta, c, unit_x, unit_y, pf, vf, num_samples):
    """Biot-Savart velocity of a sampled vortex ring added to the cell-centred field vf [nx, ny, nz, 3]
    (3D/init_conditions.py:10-22).  pf (the cell centres (I + 0.5) dx) is implied by vf's grid with
    dx = 1 / ny, as in the reference's solver."""
    sc = _scene_for_cells(vf)
    sc.add_vortex_ring(vf, w=float(w), rad=float(rad), delta=float(delta), c=[float(v) for v in c],
                       unit_x=[float(v) for v in unit_x], unit_y=[float(v) for v in unit_y],
                       num_samples=int(num_samples))


def add_vortex_ring_and_smoke(w, rad, delta, c, unit_x, unit_y, pf, vf, smokef, color, num_samples):
    """Ring velocity into vf and its smoke marker into smokef [nx, ny, nz, 4]: cells whose marker
    exceeds 0.002 become (color, 1), the others 0 (3D/init_conditions.py:29-56).  With smokef None
    only the velocity is added (the same velocity, bit for bit)."""
    if smokef is None:
        add_vortex_ring(w, rad, delta, c, unit_x, unit_y, pf, vf, num_samples)
        return
    sc = _scene_for_cells(vf)
    sc.add_vortex_ring_and_smoke(vf, smokef, w=float(w), rad=float(rad), delta=float(delta),
                                 c=[float(v) for v in c], unit_x=[float(v) for v in unit_x],
                                 unit_y=[float(v) for v in unit_y], color=[float(v) for v in color],
                                 num_samples=int(num_samples))


def init_vorts_leapfrog(X, u, smoke1, smoke2):
    """Two coaxial rings, 'front and back revised' (3D/init_conditions.py:79-118): red smoke in
    smoke1, blue in smoke2, then smoke1 += smoke2."""
    radius = 0.21
    x_gap = 0.625 * radius
    x_start = 0.16
    delta = 0.08 * radius
    w = radius * 0.1
    for cx, sm, color in ((x_start, smoke1, (1., 0., 0.)), (x_start + x_gap, smoke2, (0., 0., 1.))):
        add_vortex_ring_and_smoke(w=w, rad=radius, delta=delta, c=(cx, 0.5, 0.5), unit_x=(0., 0., -1.),
                                  unit_y=(0., 1., 0.), pf=X, vf=u, smokef=sm, color=color, num_samples=2000)
    if smoke1 is not None and smoke2 is not None:
        smoke1.add_(smoke2)  # add_fields(smoke1, smoke2, smoke1, 1.0)


def init_particles_smoke(particles_smoke, particles_grad_smoke, particles_pos, smoke, dx):
    """Particle smoke [4, P] and its gradient [3, 4, P] from the smoke grid [nx, ny, nz, 4]
    (3D/init_conditions.py:275-279)."""
    _d.check_soa(particles_pos, 3, "particles_pos")
    res = tuple(int(n) for n in smoke.shape[:3])
    _d.scene(3, res, float(dx), particles_pos.shape[1]).init_particles_smoke(particles_pos, smoke, particles_smoke,
                                                                             particles_grad_smoke)


def init_particles_pos_uniform(particles_pos, X, res_x, res_y, particles_per_cell, dx, particles_per_cell_axis,
                               dist_between_neighbor):
    """Particles on the x-fastest lattice at (index + 0.5) * dist_between_neighbor
    (3D/init_conditions.py:238-252); particles_pos is [3, P]."""
    _d.check_soa(particles_pos, 3, "particles_pos")
    P = particles_pos.shape[1]
    a = int(particles_per_cell_axis)
    res_z = P // (res_x * res_y * a ** 3)
    lat = _d.lattice_device((res_x, res_y, res_z), float(dist_between_neighbor) * a, a, particles_pos.device)
    particles_pos.copy_(lat)


def _g2p(particles_pos, u_x, u_y, u_z, imp_out, C_rows, dx):
    _d.check_soa(particles_pos, 3, "particles_pos")
    res = (u_x.shape[0] - 1, u_x.shape[1], u_x.shape[2])
    sc = _d.scene(3, res, float(dx), particles_pos.shape[1])
    if C_rows is None:
        sc.g2p(particles_pos, [u_x, u_y, u_z], imp_out=imp_out)
        return
    with _d.Rows(C_rows, out=True) as C:
        sc.g2p(particles_pos, [u_x, u_y, u_z], imp_out=imp_out, C_out=C)


def init_particles_imp(particles_init_imp, particles_pos, u_x, u_y, u_z, C_x, C_y, C_z, dx):
    """G2P of the velocity (3D/init_conditions.py:254-263; the reference leaves C untouched)."""
    _g2p(particles_pos, u_x, u_y, u_z, particles_init_imp, None, dx)


def init_particles_imp_grad_m(particles_imp, particles_pos, u_x, u_y, u_z, C_x, C_y, C_z, dx):
    """G2P of the velocity and its gradient rows C_x/C_y/C_z (3D/init_conditions.py:265-273)."""
    _g2p(particles_pos, u_x, u_y, u_z, particles_imp, (C_x, C_y, C_z), dx)
