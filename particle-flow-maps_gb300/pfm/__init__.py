"""pfm: GB300 (sm_103a) particle-flow-map time step behind a C ABI (libpfm.so).

Host-side mirror of the reference solver's step phases (zjw49246/particle-flow-maps,
3D/run_3D.py, 2D/run_2D.py, */mgpcg.py).  Every phase runs hand-written CUDA kernels through
ctypes; torch tensors are only device buffers.  There is no CPU fallback.
"""
from ._lib import PfmError, exported_symbols, lib_path, load
from .core import Scene, SolveInfo, add_fields, measure_fp32_peak, scale_field, sort_particles_noalloc
from .batch import Batch
from .sim import (DtClock, Sim2D, Sim3D, aos, aos_T, jittered, lattice2, lattice3, soa, soa_T, vortex_blobs2)

__all__ = ["PfmError", "Scene", "SolveInfo", "Sim2D", "Sim3D", "DtClock", "soa", "aos", "soa_T", "aos_T",
           "lattice2", "lattice3", "jittered", "load", "lib_path", "exported_symbols",
           "sort_particles_noalloc", "measure_fp32_peak", "Batch", "vortex_blobs2", "add_fields", "scale_field"]
