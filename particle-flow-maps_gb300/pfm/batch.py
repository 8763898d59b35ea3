"""Batches of independent scenes advanced with one CUDA graph launch per step (pfm_batch_*).

Each scene is a :class:`pfm.Sim2D` or :class:`pfm.Sim3D` (its handle, workspace and fields).  In
the branch form the batch graph holds every scene's whole step as an independent branch, so the
GPU runs the scenes concurrently.  In the work-list form (``worklist=True``) the branches join at
each MGPCG solve and one device loop advances every scene's solver iterations with persistent
kernels over a (scene, block) work list -- one launch per kernel of the iteration for the whole
batch.  Either way the results are bitwise those of stepping each scene alone.
"""
import ctypes

import torch

from . import _lib
from ._lib import PfmError

__all__ = ["Batch"]


class Batch:
    def __init__(self, sims, worklist=False):
        self.lib = _lib.load()
        self.sims = list(sims)
        if not self.sims:
            raise PfmError(7, "a batch needs at least one scene")
        b = ctypes.c_void_p()
        st = self.lib.pfm_batch_create(ctypes.byref(b))
        if st != 0:
            raise PfmError(st, "pfm_batch_create failed")
        self.b = b
        self._args = []
        for sim in self.sims:
            f, prm = sim._graph_args()  # also hands the host clock to the scene's device clock
            self._args.append((f, prm))
            fn = self.lib.pfm_batch_add3 if sim.scene.dim == 3 else self.lib.pfm_batch_add2
            self._check(fn(self.b, sim.scene.h, ctypes.byref(f), ctypes.byref(prm)))
            sim.graph = True
        self.set_worklist(worklist)

    def set_worklist(self, on):
        """Switches between the branch form and the work-list form (from the next step on)."""
        self._check(self.lib.pfm_batch_set_worklist(self.b, int(bool(on))))
        self.worklist = bool(on)

    def _check(self, status):
        if status != 0:
            raise PfmError(status, (self.lib.pfm_batch_last_error(self.b) or b"").decode())

    def step(self):
        """Every scene advances one step: one graph launch on the current stream, no host sync."""
        dev = self.sims[0].scene.device
        self._check(self.lib.pfm_batch_step(self.b, ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
        for sim in self.sims:
            sim.i += 1

    def __del__(self):
        b = getattr(self, "b", None)
        if b is not None and getattr(self, "lib", None) is not None:
            self.lib.pfm_batch_destroy(b)
            self.b = None
