"""CPU oracle of the plume kernels (test infrastructure: only tests use it).

NumPy restatements of ``pfm3_plume_source``, ``pfm3_advect_density`` and
``pfm3_add_buoyancy_impulse``.  The reference has no plume or external force, so these follow the
definitions in ``include/pfm.h``; the impulse update is checked against its defining property
(the impulse P2G forms, ``cols(T_gm) cols(T_init) init_imp``, grows by exactly ``f``) in
tests/test_gpu_plume.py as well as against this restatement.
Cell fields are ``[nx][ny][nz]``; particle fields SoA ``[3][P]`` and ``[3][3][P]`` (vector,
component, particle) as in the C ABI.
"""
import numpy as np


def plume_source(rho, dx, c, radius, value):
    nx, ny, nz = rho.shape
    f32 = np.float32
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    x = (i.astype(f32) + f32(0.5)) * f32(dx) - f32(c[0])
    y = (j.astype(f32) + f32(0.5)) * f32(dx) - f32(c[1])
    z = (k.astype(f32) + f32(0.5)) * f32(dx) - f32(c[2])
    out = rho.copy()
    out[x * x + y * y + z * z < f32(radius) * f32(radius)] = f32(value)
    return out


def sample_cells(f, dx, x, y, z):
    """trilinear sample of the cell-centred f at world positions, clamped to the cell centres"""
    N = f.shape
    idx, t = [], []
    for a, p in enumerate((x, y, z)):
        s = np.asarray(p, np.float64) / dx - 0.5
        c = np.clip(s, 0.0, N[a] - 1)
        b = np.clip(np.floor(c).astype(np.int64), 0, max(N[a] - 2, 0))
        idx.append(b)
        t.append(c - b if N[a] > 1 else np.zeros_like(c))
    i0, j0, k0 = idx
    i1, j1, k1 = np.minimum(i0 + 1, N[0] - 1), np.minimum(j0 + 1, N[1] - 1), np.minimum(k0 + 1, N[2] - 1)
    tx, ty, tz = t
    f = np.asarray(f, np.float64)
    c00 = f[i0, j0, k0] * (1 - tz) + f[i0, j0, k1] * tz
    c01 = f[i0, j1, k0] * (1 - tz) + f[i0, j1, k1] * tz
    c10 = f[i1, j0, k0] * (1 - tz) + f[i1, j0, k1] * tz
    c11 = f[i1, j1, k0] * (1 - tz) + f[i1, j1, k1] * tz
    return (c00 * (1 - ty) + c01 * ty) * (1 - tx) + (c10 * (1 - ty) + c11 * ty) * tx


def advect_density(rho0, ux, uy, uz, dx, dt):
    nx, ny, nz = rho0.shape
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    vx = 0.5 * (ux[:-1].astype(np.float64) + ux[1:])
    vy = 0.5 * (uy[:, :-1].astype(np.float64) + uy[:, 1:])
    vz = 0.5 * (uz[:, :, :-1].astype(np.float64) + uz[:, :, 1:])
    return sample_cells(rho0, dx, (i + 0.5) * dx - dt * vx, (j + 0.5) * dx - dt * vy, (k + 0.5) * dx - dt * vz)


def composite(T_gm, T_init):
    """M[q] = cols(T_gm) cols(T_init) per particle, [P][3][3] (float64)."""
    A = np.transpose(np.asarray(T_gm, np.float64), (2, 1, 0))  # [P][component][vector] = cols
    B = np.transpose(np.asarray(T_init, np.float64), (2, 1, 0))
    return A @ B


def buoyancy_impulse(pos, T_gm, T_init, init_imp, rho, dx, coef, axis):
    P = pos.shape[1]
    f = coef * sample_cells(rho, dx, pos[0], pos[1], pos[2])
    M = composite(T_gm, T_init)
    rhs = np.zeros((P, 3))
    rhs[:, axis] = f
    det = np.linalg.det(M)
    ok = (np.abs(det) > 1e-20) & (f != 0)
    delta = np.zeros((P, 3))
    delta[ok] = np.linalg.solve(M[ok], rhs[ok][..., None])[..., 0]
    return np.asarray(init_imp, np.float64) + delta.T
