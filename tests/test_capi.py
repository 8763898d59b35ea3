"""The C ABI: libpfm.so builds, loads and exports every entry point include/pfm.h declares, and
the ctypes mirrors of the public structs match the C layout.  No compute calls (CPU only)."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

import pfm
from pfm import _lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "pfm.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(pfm\w*)\s*\(", src, flags=re.M)))


def test_header_declares_the_step_phases():
    names = declared_functions()
    for must in ("pfm_create", "pfm_destroy", "pfm_workspace_size", "pfm_set_workspace", "pfm3_g2p",
                 "pfm3_rk4_T_forward", "pfm3_p2g", "pfm3_poisson", "pfm2_p2g", "pfm_mgpcg_solve"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = pfm.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_status_strings_without_gpu():
    lib = pfm.load()
    assert lib.pfm_status_string(0) == b"ok"
    assert b"converge" in lib.pfm_status_string(4)


def test_create_rejects_bad_config_without_gpu():
    lib = pfm.load()
    cfg = _lib.Config()
    cfg.dim = 4
    h = ctypes.c_void_p()
    assert lib.pfm_create(ctypes.byref(cfg), ctypes.byref(h)) == 7  # PFM_ERR_ARG
    assert lib.pfm_create(None, ctypes.byref(h)) == 1


def _c_layout():
    code = r"""
#include <stddef.h>
#include <stdio.h>
#include "pfm.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(pfm_config), offsetof(pfm_config, dx), offsetof(pfm_config, particles),
         offsetof(pfm_config, boundary), offsetof(pfm_config, use_apic));
  printf("%zu %zu %zu %zu\n", sizeof(pfm_solve_opts), offsetof(pfm_solve_opts, tol), offsetof(pfm_solve_opts, check_every),
         offsetof(pfm_solve_opts, true_residual_every));
  printf("%zu %zu %zu %zu\n", sizeof(pfm_solve_stats), offsetof(pfm_solve_stats, rTr0), offsetof(pfm_solve_stats, bTb),
         offsetof(pfm_solve_stats, rTr_true));
  printf("%zu %zu %zu\n", sizeof(pfm_step_params), offsetof(pfm_step_params, reinit_particle_pos),
         offsetof(pfm_step_params, poisson));
  printf("%zu %zu %zu\n", sizeof(pfm3_step_fields), offsetof(pfm3_step_fields, p), offsetof(pfm3_step_fields, init_C));
  printf("%zu %zu %zu\n", sizeof(pfm2_step_fields), offsetof(pfm2_step_fields, psi_grid), offsetof(pfm2_step_fields, C));
  printf("%zu %zu %zu %zu %zu\n", sizeof(pfm_step_info_t), offsetof(pfm_step_info_t, dt),
         offsetof(pfm_step_info_t, max_speed), offsetof(pfm_step_info_t, rTr), offsetof(pfm_step_info_t, history));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        open(c, "w").write(code)
        subprocess.check_call(["gcc", "-I", os.path.join(REPO, "include"), c, "-o", exe])
        out = subprocess.check_output([exe]).decode().split()
    return [int(x) for x in out]


def test_struct_layouts_match_header():
    if not subprocess.run(["which", "gcc"], capture_output=True).returncode == 0:
        pytest.skip("gcc not available")
    c = _c_layout()
    C = _lib.Config
    assert c[:5] == [ctypes.sizeof(C), C.dx.offset, C.particles.offset, C.boundary.offset, C.use_apic.offset]
    O = _lib.SolveOpts
    assert c[5:9] == [ctypes.sizeof(O), O.tol.offset, O.check_every.offset, O.true_residual_every.offset]
    S = _lib.SolveStats
    assert c[9:13] == [ctypes.sizeof(S), S.rTr0.offset, S.bTb.offset, S.rTr_true.offset]
    P = _lib.StepParams
    assert c[13:16] == [ctypes.sizeof(P), P.reinit_particle_pos.offset, P.poisson.offset]
    F3, F2 = _lib.Step3Fields, _lib.Step2Fields
    assert c[16:19] == [ctypes.sizeof(F3), F3.p.offset, F3.init_C.offset]
    assert c[19:22] == [ctypes.sizeof(F2), F2.psi_grid.offset, F2.C.offset]
    I = _lib.StepInfo
    assert c[22:27] == [ctypes.sizeof(I), I.dt.offset, I.max_speed.offset, I.rTr.offset, I.history.offset]


def test_scene_fails_loudly_without_cuda():
    import torch
    if torch.cuda.is_available():
        pytest.skip("this container-side check needs a machine without a GPU")
    with pytest.raises(pfm.PfmError):
        pfm.Scene(3, (8, 8, 8), 1 / 8, 16)
