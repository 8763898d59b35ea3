"""The particle-flow-map step loops on the GPU: run_3D.main() / run_2D.main() loop bodies.

Phase order, reinitialisation cadence and the CFL/frame clock follow 3D/run_3D.py:716-822 and
2D/run_2D.py:772-909; every phase is one libpfm entry point (see core.Scene).
"""
import numpy as np
import torch

from . import _lib
from ._lib import PfmError
from .core import Scene

__all__ = ["DtClock", "Sim3D", "Sim2D", "soa", "aos", "soa_T", "aos_T", "lattice3", "lattice2",
           "jittered"]


# ------------------------------------------------------------------------------------------------
# layout helpers: the reference's Taichi AoS [P, n] / [P, nv, nc]  <->  device SoA [n, P] / [nv, nc, P]
# ------------------------------------------------------------------------------------------------
def soa(a, device="cuda"):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float32).T)).to(device)


def aos(t):
    return t.detach().cpu().numpy().T.copy()


def soa_T(a, device="cuda"):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float32).transpose(1, 2, 0))).to(device)


def aos_T(t):
    return t.detach().cpu().numpy().transpose(2, 0, 1).copy()


# ------------------------------------------------------------------------------------------------
# particle seeding
# ------------------------------------------------------------------------------------------------
def lattice3(res, dx, ppc_axis=2):
    """init_particles_pos_uniform (3D/init_conditions.py:238-252): the reference's x-fastest lattice."""
    nx, ny, nz = res
    P = nx * ny * nz * ppc_axis ** 3
    i = np.arange(P, dtype=np.int64)
    px, py = ppc_axis * nx, ppc_axis * ny
    idx = np.stack([i % px, (i // px) % py, (i // px) // py], axis=1)
    dist = np.float32(dx / ppc_axis)
    return ((idx.astype(np.float32) + np.float32(0.5)) * dist).astype(np.float32)


def lattice2(res, dx, ppc):
    """init_particles_pos_uniform (2D/init_conditions.py:139-166)."""
    nx, ny = res
    axis = int(np.sqrt(ppc))
    P = nx * ny * ppc
    i = np.arange(P, dtype=np.int64)
    px = axis * nx
    idx = np.stack([i % px, i // px], axis=1)
    dist = np.float32(dx / axis)
    return ((idx.astype(np.float32) + np.float32(0.5)) * dist).astype(np.float32)


def _hash_uniform(seed, n):
    """Counter-based uniform in [0, 1) (24 bits): splitmix64 finaliser of (seed, n)."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) * np.uint64(0xD1B54A32D192ED03) + n.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)


SEED_GROUP = 16  # cells of a line along the last axis that the seeding order interleaves


def jittered(res, dx, ppc, seed=0):
    """Stratified jittered seeding, bit-identical to the device kernel pfm_seed_jittered.

    Each cell holds ppc particles, one per sub-cell of a ppc_axis^d lattice, at
    (sub-lattice index + U) * dx / ppc_axis, U a splitmix64 hash of (seed, particle, axis).
    Order: the lines of cells along the last axis in turn, each in groups of 16 cells (the last
    group takes the remainder), inside a group [leading sub-indices][cell][last sub-index]; with 8
    particles per cell, 32 consecutive particles are 16 neighbouring cells with the same leading
    sub-cell, so a warp's interpolation stencils share their rows."""
    d = len(res)
    axis = int(round(ppc ** (1.0 / d)))
    if axis ** d != ppc:
        raise ValueError("particles per cell must be a perfect square (2D) or cube (3D)")
    cells = int(np.prod(res))
    P = cells * ppc
    nl = int(res[-1])
    q = np.arange(P, dtype=np.int64)
    line_len = nl * ppc
    line, rem = q // line_len, q % line_len
    gi = rem // (SEED_GROUP * ppc)
    r = rem % (SEED_GROUP * ppc)
    k0 = gi * SEED_GROUP
    gsz = np.minimum(SEED_GROUP, nl - k0)
    s_last = r % axis
    t = r // axis
    kk = t % gsz
    o = t // gsz
    lead = np.stack(np.unravel_index(line, tuple(res[:-1])), axis=1) if d > 1 else np.zeros((P, 0), np.int64)
    ci = np.concatenate([lead, (k0 + kk)[:, None]], axis=1)
    si_lead = np.stack(np.unravel_index(o, (axis,) * (d - 1)), axis=1)
    si = np.concatenate([si_lead, s_last[:, None]], axis=1)
    lat = (ci * axis + si).astype(np.float32)
    u = _hash_uniform(seed, (q[:, None] * d + np.arange(d)[None, :]))
    return ((lat + u) * np.float32(dx / axis)).astype(np.float32)


def vortex_blobs2(res, dx, seed):
    """Face velocity of 2-8 Gaussian-core point vortices for one scene of the batched workload:
    centres uniform in [0.2, 0.8]^2 (of the unit-height domain), circulation uniform in
    +-[0.5, 1.5], core sigma uniform in [0.01, 0.04], all drawn from numpy default_rng(seed).  Each
    blob adds u = G / (2 pi) (1 - exp(-r^2 / sigma^2)) / r^2 (-(y - yc), x - xc) (the Gaussian-core
    profile of 2D/init_conditions.py:5-9), evaluated in f64 at the face centres and cast to f32."""
    rng = np.random.default_rng(seed)
    nb = int(rng.integers(2, 9))
    c = rng.uniform(0.2, 0.8, size=(nb, 2))
    g = rng.uniform(0.5, 1.5, size=nb) * rng.choice([-1.0, 1.0], size=nb)
    sig = rng.uniform(0.01, 0.04, size=nb)
    nx, ny = res
    out = []
    for fam in range(2):
        shp = (nx + (fam == 0), ny + (fam == 1))
        ii, jj = np.meshgrid(np.arange(shp[0], dtype=np.float64), np.arange(shp[1], dtype=np.float64), indexing="ij")
        x = (ii + (0.0 if fam == 0 else 0.5)) * dx
        y = (jj + (0.0 if fam == 1 else 0.5)) * dx
        u = np.zeros(shp)
        for k in range(nb):
            rx, ry = x - c[k, 0], y - c[k, 1]
            r2 = rx * rx + ry * ry + 1e-12
            f = g[k] / (2 * np.pi) * (1.0 - np.exp(-r2 / sig[k] ** 2)) / r2
            u += f * (-ry if fam == 0 else rx)
        out.append(u.astype(np.float32))
    return out


class DtClock:
    """CFL step with the frame clamp of run_3D.py:725-743 / run_2D.py:782-799 (Python doubles)."""

    def __init__(self, CFL, dx, visualize_dt, save_frame_each_step=False):
        self.CFL, self.dx, self.visualize_dt = CFL, dx, visualize_dt
        self.save_frame_each_step = save_frame_each_step
        self.sub_t = 0.0
        self.frame_idx = 0

    def next(self, max_speed):
        curr_dt = self.CFL * self.dx / max_speed
        if self.save_frame_each_step:
            self.frame_idx += 1
            return curr_dt, True
        if self.sub_t + curr_dt >= self.visualize_dt:
            curr_dt = self.visualize_dt - self.sub_t
            self.sub_t = 0.0
            self.frame_idx += 1
            return curr_dt, True
        self.sub_t += curr_dt
        return curr_dt, False


class Sim3D:
    """GPU state and step of the 3D solver (3D/run_3D.py:716-822).

    ``u``: the three face grids (numpy arrays or CUDA tensors); ``seeds``: reinit positions, AoS
    numpy [P, 3] or a device SoA tensor [3, P].  Pass ``timer`` (a callable taking a phase name and
    returning a context manager) to bracket the phases with CUDA events.  ``fused_rk4_p2g`` runs
    the step's particle work as one RK4 kernel (gradient reinitialisation, RK4, P2G records) and
    the P2G tiles (the same results as the separate calls, particle state read once)."""

    def __init__(self, u, seeds, res, dx, CFL=0.5, visualize_dt=0.1, reinit_every=20,
                 reinit_every_grad_m=1, use_midpoint_vel=True, reinit_particle_pos=True, use_apic=True,
                 base_level=3, mg_levels=0, poisson_opts=None, device="cuda", fused_rk4_p2g=True, graph=False):
        self.fused_rk4_p2g = bool(fused_rk4_p2g)  # RK4_T_forward + P2G through pfm3_rk4_p2g
        self.graph = bool(graph)  # step() = one pfm3_step graph launch, no host synchronization
        if isinstance(seeds, torch.Tensor):
            self.P = int(seeds.shape[1])
        else:
            seeds = np.asarray(seeds, np.float32)
            self.P = seeds.shape[0]
        self.scene = Scene(3, res, dx, self.P, base_level=base_level, mg_levels=mg_levels, use_apic=use_apic,
                           device=device)
        sc = self.scene
        self.res, self.dx = tuple(res), dx
        self.clock = DtClock(CFL, dx, visualize_dt)
        self.reinit_every, self.grad_m = reinit_every, reinit_every_grad_m
        self.use_midpoint_vel, self.reinit_particle_pos = use_midpoint_vel, reinit_particle_pos
        self.poisson_opts = dict(poisson_opts or {})
        dev = sc.device
        self.u = [(a.to(dev).contiguous() if isinstance(a, torch.Tensor)
                   else torch.as_tensor(np.asarray(a, np.float32)).to(dev).contiguous()) for a in u]
        self.u_mid = sc.alloc_faces()
        self.w = sc.alloc_faces()
        self.seeds = seeds.to(dev).contiguous() if isinstance(seeds, torch.Tensor) else soa(seeds, dev)
        P = self.P
        self.pos = torch.zeros(3, P, device=dev)
        self.init_imp = torch.zeros(3, P, device=dev)
        self.T_init = torch.zeros(3, 3, P, device=dev)
        self.T_gm = torch.zeros(3, 3, P, device=dev)
        self.init_C = torch.zeros(3, 3, P, device=dev)
        sc.reset_T(self.T_init)
        sc.reset_T(self.T_gm)
        self.p = torch.zeros(sc.cell_shape, device=dev)
        self.p_mid = torch.zeros(sc.cell_shape, device=dev)  # the midpoint solve's pressure (warm starts)
        self.i, self.ik = -1, 0
        self.infos = []
        self.last_dt = None
        self.timer = None
        # optional callbacks of scenes built on this step (pfm.plume): before_rk4(dt) after the
        # midpoint solve, before_poisson() -> overrides of the final solve's options, after_step(dt)
        self.before_rk4 = self.before_poisson = self.after_step = None
        self.poisson_mid_opts = None  # options of the midpoint solve if they differ (eager steps)

    def _t(self, name):
        import contextlib
        return self.timer(name) if self.timer is not None else contextlib.nullcontext()

    def _graph_args(self):
        if getattr(self, "_gargs", None) is None:
            f = _lib.Step3Fields()
            for a in range(3):
                f.u[a], f.u_mid[a], f.w[a] = self.u[a].data_ptr(), self.u_mid[a].data_ptr(), self.w[a].data_ptr()
            f.p, f.p_mid = self.p.data_ptr(), self.p_mid.data_ptr()
            for name in ("seeds", "pos", "init_imp", "T_init", "T_gm", "init_C"):
                setattr(f, name, getattr(self, name).data_ptr())
            o = {k: v for k, v in self.poisson_opts.items() if k != "raise_on_limit"}
            prm = Scene.step_params(CFL=self.clock.CFL, visualize_dt=self.clock.visualize_dt,
                                    save_frame_each_step=self.clock.save_frame_each_step,
                                    reinit_every=self.reinit_every, reinit_every_grad_m=self.grad_m,
                                    use_midpoint_vel=self.use_midpoint_vel,
                                    reinit_particle_pos=self.reinit_particle_pos, **o)
            self._gargs = (f, prm)
            self.scene.step_reset(self.i, self.ik, self.clock.sub_t, self.clock.frame_idx)
        return self._gargs

    def step_info(self):
        """Graph mode: the device step state after the last step (a host sync)."""
        return self.scene.step_info()

    def set_graph(self, on):
        """Switches between graph steps and eager phase calls, handing the frame clock and the
        reinitialisation schedule over between the device and the host."""
        on = bool(on)
        if on == self.graph:
            return
        if not on and getattr(self, "_gargs", None) is not None:
            info = self.scene.step_info()
            self.ik, self.clock.sub_t, self.clock.frame_idx = info.ik, info.sub_t, info.frame_idx
            self.last_dt = info.dt if info.step >= 0 else self.last_dt
        elif on and getattr(self, "_gargs", None) is not None:
            self.scene.step_reset(self.i, self.ik, self.clock.sub_t, self.clock.frame_idx)
        self.graph = on

    def step(self):
        if self.graph:  # the whole step as one graph launch; dt and the solves stay on the device
            if self.before_rk4 or self.before_poisson or self.after_step:
                raise PfmError(7, "step callbacks run only with eager steps (graph=False)")
            f, prm = self._graph_args()
            self.scene.step_graph(f, prm)
            self.i += 1
            return None
        sc = self.scene
        self.i += 1
        i = self.i
        j = i % self.reinit_every
        with self._t("max_speed"):
            max_speed = sc.calc_max_speed(self.u)
        curr_dt, _ = self.clock.next(max_speed)
        self.last_dt = curr_dt
        if j == 0:
            with self._t("reinit"):
                if self.reinit_particle_pos or i == 0:
                    self.pos.copy_(self.seeds)
                    self.ik = i
                sc.g2p(self.pos, self.u, imp_out=self.init_imp)
                sc.reset_T(self.T_init)
                sc.reset_T(self.T_gm)
        k = (i - self.ik) % self.grad_m
        # with fused_rk4_p2g the gradient reinitialisation runs inside the RK4 kernel after the
        # midpoint solve (it reads the same positions and the pre-midpoint velocity)
        if k == 0 and not self.fused_rk4_p2g:
            with self._t("g2p"):
                sc.g2p(self.pos, self.u, C_out=self.init_C)
            with self._t("update_T"):
                sc.update_T(self.T_init, self.T_gm, reset_gm=True)
        adv = self.u
        if self.use_midpoint_vel:
            with self._t("midpoint"):
                sc.midpoint(self.u, self.u_mid, float(np.float32(0.5 * curr_dt)))
            with self._t("poisson_mid"):
                self.infos.append(sc.poisson(self.u_mid, self.p_mid, **(self.poisson_mid_opts or self.poisson_opts)))
            adv = self.u_mid
        if self.before_rk4 is not None:
            self.before_rk4(curr_dt)
        if self.fused_rk4_p2g:
            with self._t("rk4"):
                if k == 0:
                    sc.gradm_rk4_records3(self.pos, self.T_gm, self.T_init, self.init_C, self.init_imp, self.u, adv,
                                          float(np.float32(curr_dt)))
                else:
                    sc.rk4_p2g_records3(self.pos, self.T_gm, adv, float(np.float32(curr_dt)), self.init_imp,
                                        self.T_init, self.init_C)
            with self._t("p2g"):
                sc.p2g_from_records3(self.u, self.w)
        else:
            with self._t("rk4"):
                sc.rk4_T_forward(self.pos, self.T_gm, adv, float(np.float32(curr_dt)))
            with self._t("p2g"):
                sc.p2g3(self.init_imp, self.pos, self.T_gm, self.T_init, self.init_C, self.u, self.w)
        opts = self.poisson_opts
        if self.before_poisson is not None:
            opts = dict(opts, **(self.before_poisson() or {}))
        with self._t("poisson"):
            self.infos.append(sc.poisson(self.u, self.p, **opts))
        if self.after_step is not None:
            self.after_step(curr_dt)
        return curr_dt


class Sim2D:
    """GPU state and step of the 2D solver (2D/run_2D.py:772-909)."""

    def __init__(self, u, seeds, res, dx, CFL=0.5, visualize_dt=0.1, reinit_every=12,
                 reinit_every_grad_m=8, use_midpoint_vel=True, reinit_particle_pos=True, use_apic=True,
                 base_level=3, mg_levels=0, poisson_opts=None, device="cuda", graph=False):
        self.graph = bool(graph)  # step() = one pfm2_step graph launch, no host synchronization
        seeds = np.asarray(seeds, np.float32)
        self.P = seeds.shape[0]
        self.scene = Scene(2, res, dx, self.P, base_level=base_level, mg_levels=mg_levels, use_apic=use_apic,
                           device=device)
        sc = self.scene
        self.res, self.dx = tuple(res), dx
        self.clock = DtClock(CFL, dx, visualize_dt)
        self.reinit_every, self.grad_m = reinit_every, reinit_every_grad_m
        self.use_midpoint_vel, self.reinit_particle_pos = use_midpoint_vel, reinit_particle_pos
        self.poisson_opts = dict(poisson_opts or {})
        dev = sc.device
        self.u = [(a.to(dev).float().contiguous() if isinstance(a, torch.Tensor)
                   else torch.as_tensor(np.asarray(a, np.float32)).to(dev).contiguous()) for a in u]
        self.u_mid = sc.alloc_faces()
        self.w = sc.alloc_faces()
        self.psi_grid = [torch.zeros(s + (2,), device=dev) for s in sc.face_shapes]
        self.seeds = soa(seeds, dev)
        P = self.P
        self.pos = self.seeds.clone()
        self.imp = torch.zeros(2, P, device=dev)
        self.init_imp = torch.zeros(2, P, device=dev)
        self.psi = self.seeds.clone()
        self.T = torch.zeros(2, 2, P, device=dev)
        self.T_init = torch.zeros(2, 2, P, device=dev)
        self.T_gm = torch.zeros(2, 2, P, device=dev)
        for t in (self.T, self.T_init, self.T_gm):
            sc.reset_T(t)
        self.init_C = torch.zeros(2, 2, P, device=dev)
        self.C = torch.zeros(2, 2, P, device=dev)
        self.p = torch.zeros(sc.cell_shape, device=dev)
        self.i, self.ik = -1, 0
        self.infos = []
        self.last_dt = None

    def _graph_args(self):
        if getattr(self, "_gargs", None) is None:
            f = _lib.Step2Fields()
            for a in range(2):
                f.u[a], f.u_mid[a], f.w[a] = self.u[a].data_ptr(), self.u_mid[a].data_ptr(), self.w[a].data_ptr()
                f.psi_grid[a] = self.psi_grid[a].data_ptr()
            f.p, f.p_mid = self.p.data_ptr(), None  # the midpoint solve has no pressure buffer (as step())
            for name in ("seeds", "pos", "imp", "init_imp", "psi", "T", "T_init", "T_gm", "init_C", "C"):
                setattr(f, name, getattr(self, name).data_ptr())
            o = {k: v for k, v in self.poisson_opts.items() if k != "raise_on_limit"}
            prm = Scene.step_params(CFL=self.clock.CFL, visualize_dt=self.clock.visualize_dt,
                                    save_frame_each_step=self.clock.save_frame_each_step,
                                    reinit_every=self.reinit_every, reinit_every_grad_m=self.grad_m,
                                    use_midpoint_vel=self.use_midpoint_vel,
                                    reinit_particle_pos=self.reinit_particle_pos, **o)
            self._gargs = (f, prm)
            self.scene.step_reset(self.i, self.ik, self.clock.sub_t, self.clock.frame_idx)
        return self._gargs

    def step_info(self):
        """Graph mode: the device step state after the last step (a host sync)."""
        return self.scene.step_info()

    def set_graph(self, on):
        """Switches between graph steps and eager phase calls, handing the frame clock and the
        reinitialisation schedule over between the device and the host."""
        on = bool(on)
        if on == self.graph:
            return
        if not on and getattr(self, "_gargs", None) is not None:
            info = self.scene.step_info()
            self.ik, self.clock.sub_t, self.clock.frame_idx = info.ik, info.sub_t, info.frame_idx
            self.last_dt = info.dt if info.step >= 0 else self.last_dt
        elif on and getattr(self, "_gargs", None) is not None:
            self.scene.step_reset(self.i, self.ik, self.clock.sub_t, self.clock.frame_idx)
        self.graph = on

    def step(self):
        if self.graph:
            f, prm = self._graph_args()
            self.scene.step_graph(f, prm)
            self.i += 1
            return None
        sc = self.scene
        self.i += 1
        i = self.i
        j = i % self.reinit_every
        max_speed = sc.calc_max_speed(self.u)
        curr_dt, _ = self.clock.next(max_speed)
        self.last_dt = curr_dt
        if j == 0:
            if self.reinit_particle_pos or i == 0:
                self.pos.copy_(self.seeds)
            self.ik = i
            sc.g2p(self.pos, self.u, imp_out=self.imp)
            self.init_imp.copy_(self.imp)
            self.psi.copy_(self.pos)
            sc.reset_T(self.T)
            sc.reset_T(self.T_init)
        k = (i - self.ik) % self.grad_m
        if k == 0:
            sc.g2p(self.pos, self.u, C_out=self.init_C)
            sc.reset_T(self.T_gm)
            self.T_init.copy_(self.T)
        adv = self.u
        if self.use_midpoint_vel:
            sc.midpoint(self.u, self.u_mid, float(np.float32(0.5 * curr_dt)))
            self.infos.append(sc.poisson(self.u_mid, **self.poisson_opts))
            adv = self.u_mid
        sc.rk4_T_forward(self.pos, self.T_gm, adv, float(np.float32(curr_dt)), advect_psi=True)
        sc.update_grad_m2(self.C, self.init_C, self.T_gm)
        sc.update_T2(self.T, self.T_init, self.T_gm)
        sc.update_imp2(self.imp, self.init_imp, self.T)
        sc.p2g2(self.imp, self.pos, self.C, self.psi, self.u, self.w, psi_out=self.psi_grid)
        self.infos.append(sc.poisson(self.u, self.p, **self.poisson_opts))
        return curr_dt
