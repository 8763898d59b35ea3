"""ctypes binding of libpfm.so (declarations in include/pfm.h).

The library is the only compute path: if it is missing or CUDA is unavailable, loading raises
:class:`PfmError` -- there is no CPU fallback.
"""
import ctypes
import os

from . import build as _build

PFM_OK = 0
PFM_ERR_NOT_CONVERGED = 4
STATUS_NAMES = {0: "PFM_OK", 1: "PFM_ERR_NULL", 2: "PFM_ERR_SHAPE", 3: "PFM_ERR_WORKSPACE",
                4: "PFM_ERR_NOT_CONVERGED", 5: "PFM_ERR_NONFINITE", 6: "PFM_ERR_CUDA", 7: "PFM_ERR_ARG"}


class PfmError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("res", ctypes.c_int * 3), ("dx", ctypes.c_double),
                ("particles", ctypes.c_int64), ("base_level", ctypes.c_int), ("mg_levels", ctypes.c_int),
                ("pre_post_smoothing", ctypes.c_int), ("bottom_smoothing", ctypes.c_int),
                ("boundary", (ctypes.c_int * 2) * 3), ("use_apic", ctypes.c_int)]


class SolveOpts(ctypes.Structure):
    _fields_ = [("max_iters", ctypes.c_int), ("eps", ctypes.c_double), ("tol", ctypes.c_double),
                ("tol_mode", ctypes.c_int), ("check_every", ctypes.c_int), ("precision", ctypes.c_int),
                ("warm_start", ctypes.c_int), ("true_residual_every", ctypes.c_int),
                ("true_residual_replace", ctypes.c_int)]


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("rTr", ctypes.c_double),
                ("rTr0", ctypes.c_double), ("bTb", ctypes.c_double),
                ("rTr_true", ctypes.c_double)]


class StepParams(ctypes.Structure):
    _fields_ = [("CFL", ctypes.c_double), ("visualize_dt", ctypes.c_double), ("save_frame_each_step", ctypes.c_int),
                ("reinit_every", ctypes.c_int), ("reinit_every_grad_m", ctypes.c_int),
                ("use_midpoint_vel", ctypes.c_int), ("reinit_particle_pos", ctypes.c_int), ("poisson", SolveOpts)]


class Step3Fields(ctypes.Structure):
    _fields_ = [("u", ctypes.c_void_p * 3), ("u_mid", ctypes.c_void_p * 3), ("w", ctypes.c_void_p * 3),
                ("p", ctypes.c_void_p), ("p_mid", ctypes.c_void_p), ("seeds", ctypes.c_void_p),
                ("pos", ctypes.c_void_p), ("init_imp", ctypes.c_void_p), ("T_init", ctypes.c_void_p),
                ("T_gm", ctypes.c_void_p), ("init_C", ctypes.c_void_p)]


class Step2Fields(ctypes.Structure):
    _fields_ = [("u", ctypes.c_void_p * 2), ("u_mid", ctypes.c_void_p * 2), ("w", ctypes.c_void_p * 2),
                ("psi_grid", ctypes.c_void_p * 2), ("p", ctypes.c_void_p), ("p_mid", ctypes.c_void_p),
                ("seeds", ctypes.c_void_p), ("pos", ctypes.c_void_p), ("imp", ctypes.c_void_p),
                ("init_imp", ctypes.c_void_p), ("psi", ctypes.c_void_p), ("T", ctypes.c_void_p),
                ("T_init", ctypes.c_void_p), ("T_gm", ctypes.c_void_p), ("init_C", ctypes.c_void_p),
                ("C", ctypes.c_void_p)]


class StepInfo(ctypes.Structure):
    _fields_ = [("step", ctypes.c_int), ("ik", ctypes.c_int), ("frame_idx", ctypes.c_int),
                ("output_frame", ctypes.c_int), ("reinit", ctypes.c_int), ("reseed", ctypes.c_int),
                ("gradm_reinit", ctypes.c_int), ("dt", ctypes.c_double), ("sub_t", ctypes.c_double),
                ("max_speed", ctypes.c_float), ("iterations", ctypes.c_int * 2), ("converged", ctypes.c_int * 2),
                ("rTr", ctypes.c_double * 2), ("history", (ctypes.c_int * 2) * 64)]


class Conv3Args(ctypes.Structure):
    _fields_ = [("d0", ctypes.c_int), ("d1", ctypes.c_int), ("d2", ctypes.c_int), ("x1", ctypes.c_void_p),
                ("c1", ctypes.c_int), ("x2", ctypes.c_void_p), ("c2", ctypes.c_int), ("w", ctypes.c_void_p),
                ("bias", ctypes.c_void_p), ("cout", ctypes.c_int), ("relu", ctypes.c_int), ("y1", ctypes.c_void_p),
                ("cy1", ctypes.c_int), ("y2", ctypes.c_void_p), ("yf", ctypes.c_void_p),
                ("yf_scale", ctypes.c_void_p), ("err", ctypes.c_void_p)]


class Conv3WgradArgs(ctypes.Structure):
    _fields_ = [("d0", ctypes.c_int), ("d1", ctypes.c_int), ("d2", ctypes.c_int), ("x1", ctypes.c_void_p),
                ("c1", ctypes.c_int), ("x2", ctypes.c_void_p), ("c2", ctypes.c_int), ("dy", ctypes.c_void_p),
                ("cdy", ctypes.c_int), ("cout", ctypes.c_int), ("dw", ctypes.c_void_p),
                ("partial", ctypes.c_void_p), ("partial_bytes", ctypes.c_size_t), ("err", ctypes.c_void_p)]


# name -> argument types (all return int status unless listed in _RESTYPE)
_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
SIGNATURES = {
    "pfm_create": [ctypes.POINTER(Config), ctypes.POINTER(_P)],
    "pfm_destroy": [_P],
    "pfm_workspace_size": [_P, ctypes.POINTER(ctypes.c_size_t)],
    "pfm_set_workspace": [_P, _P, ctypes.c_size_t],
    "pfm_last_error": [_P],
    "pfm_status_string": [_I],
    "pfm_mg_levels": [_P, ctypes.POINTER(_I)],
    "pfm_launch_count": [_P, ctypes.POINTER(ctypes.c_uint64)],
    "pfm_measure_fp32_peak": [_P, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_double), _P],
    "pfm3_add_vortex_ring": [_P, _F, _F, _F, ctypes.POINTER(_F), ctypes.POINTER(_F), ctypes.POINTER(_F), _I, _P, _P],
    "pfm_split_central_vector": [_P, _P, _P, _P, _P, _P],
    "pfm_seed_jittered": [_P, ctypes.c_uint64, _I, _P, _P],
    "pfm3_calc_max_speed": [_P, _P, _P, _P, _P, _P],
    "pfm3_g2p": [_P, _P, _P, _P, _P, _P, _P, _P],
    "pfm3_update_T": [_P, _P, _P, _I, _P],
    "pfm3_reset_T": [_P, _P, _P],
    "pfm3_rk4_T_forward": [_P, _P, _P, _P, _P, _P, _F, _P],
    "pfm3_midpoint": [_P, _P, _P, _P, _P, _P, _P, _F, _P, _P, _P],
    "pfm3_sort_particles": [_P, _P, _P, _P, _P],
    "pfm3_p2g": [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "pfm3_rk4_p2g": [_P, _P, _P, _P, _P, _P, _F, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "pfm3_rk4_p2g_records": [_P, _P, _P, _P, _P, _P, _F, _P, _P, _P, _P],
    "pfm3_p2g_from_records": [_P, _P, _P, _P, _P, _P, _P, _P],
    "pfm3_gradm_rk4_p2g_records": [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _F, _P],
    "pfm3_poisson": [_P, _P, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats), _P],
    "pfm2_calc_max_speed": [_P, _P, _P, _P, _P],
    "pfm2_g2p": [_P, _P, _P, _P, _P, _P, _P],
    "pfm2_rk4_T_forward": [_P, _P, _P, _P, _P, _F, _I, _P],
    "pfm2_update_grad_m": [_P, _P, _P, _P, _P],
    "pfm2_update_T": [_P, _P, _P, _P, _P],
    "pfm2_update_imp": [_P, _P, _P, _P, _P],
    "pfm2_reset_T": [_P, _P, _P],
    "pfm2_midpoint": [_P, _P, _P, _P, _P, _F, _P, _P, _P],
    "pfm2_sort_particles": [_P, _P, _P, _P, _P],
    "pfm2_p2g": [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "pfm2_poisson": [_P, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats), _P],
    "pfm_mgpcg_solve": [_P, _P, _F, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats), _P],
    "pfm_apply_bc": [_P, _P, _P, _P, _P],
    "pfm_divergence": [_P, _P, _P, _P, _P, _P],
    "pfm_subtract_grad_p": [_P, _P, _P, _P, _P, _P],
    "pfm_sort_particles_noalloc": [_I, ctypes.POINTER(_I), ctypes.c_double, ctypes.c_int64, _P, _P, _P, _P],
    "pfm_add_fields": [_P, _P, _F, _P, ctypes.c_int64, _P],
    "pfm_scale_field": [_P, _F, _P, ctypes.c_int64, _P],
    "pfm3_get_central_vector": [_P, _P, _P, _P, _P, _P],
    "pfm3_curl": [_P, _P, _P, _F, _P],
    "pfm2_get_central_vector": [_P, _P, _P, _P, _P],
    "pfm2_curl": [_P, _P, _P, _F, _P],
    "pfm3_init_particles_smoke": [_P, _P, _P, _P, _P, _P],
    "pfm3_p2g_smoke": [_P, _P, _P, _P, _P, _P, _I, _P, _P, _P],
    "pfm3_advect_smoke": [_P, _P, _P, _P, _P, _P, _F, _P],
    "pfm3_clamp_smoke": [_P, _P, _P, _P, _P, _P, _F, _P],
    "pfm2_advect_smoke": [_P, _P, _P, _P, _P, _F, _P],
    "pfm3_add_vortex_ring_and_smoke": [_P, _F, _F, _F, ctypes.POINTER(_F), ctypes.POINTER(_F), ctypes.POINTER(_F),
                                       ctypes.POINTER(_F), _I, _P, _P, _P],
    "pfm3_rk4_T_and_T_grad_m_forward": [_P, _P, _P, _P, _P, _P, _P, _F, _P],
    "pfm3_update_imp": [_P, _P, _P, _P, _P],
    "pfm3_update_grad_m": [_P, _P, _P, _P, _P, _P, _P],
    "pfm3_compute_dT_dx": [_P, _P, _P, _P, _I, _P, _P],
    "pfm3_step": [_P, ctypes.POINTER(Step3Fields), ctypes.POINTER(StepParams), _P],
    "pfm2_step": [_P, ctypes.POINTER(Step2Fields), ctypes.POINTER(StepParams), _P],
    "pfm_step_reset": [_P, _I, _I, ctypes.c_double, _I, _P],
    "pfm_reset_warm_history": [_P, _P],
    "pfm_step_info": [_P, ctypes.POINTER(StepInfo), _P],
    "pfm_batch_create": [ctypes.POINTER(_P)],
    "pfm_batch_destroy": [_P],
    "pfm_batch_add3": [_P, _P, ctypes.POINTER(Step3Fields), ctypes.POINTER(StepParams)],
    "pfm_batch_add2": [_P, _P, ctypes.POINTER(Step2Fields), ctypes.POINTER(StepParams)],
    "pfm_batch_step": [_P, _P],
    "pfm_batch_set_worklist": [_P, _I],
    "pfm_batch_last_error": [_P],
    "pfm_set_tuning": [_P, _I, _I],
    "pfm_get_tuning": [_P, _I, ctypes.POINTER(_I)],
    "pfm3_plume_source": [_P, _P, _F, _F, _F, _F, _F, _P],
    "pfm3_advect_density": [_P, _P, _P, _P, _P, _P, _F, _P],
    "pfm3_add_buoyancy_impulse": [_P, _P, _P, _P, _P, _P, _F, _I, _P],
    "pfm_nn_conv3": [ctypes.POINTER(Conv3Args), _P],
    "pfm_nn_conv3_wgrad": [ctypes.POINTER(Conv3WgradArgs), _P],
    "pfm_nn_wgrad_workspace": [ctypes.POINTER(Conv3WgradArgs), ctypes.POINTER(ctypes.c_size_t)],
    "pfm_nn_pack_weights": [_P, _I, _I, _I, _I, _I, _P, _P],
    "pfm_nn_pack_scalar": [_P, _I, _I, _I, _P, _P, _P],
    "pfm_nn_resample": [_P, _P, _I, _I, _I, _I, _I, _P],
    "pfm_nn_elementwise": [_P, _P, ctypes.c_size_t, _I, _P],
    "pfm_nn_scratch_floats": [_I],
    "pfm_nn_bias_grad": [_P, _I, _I, _I, _I, _I, _P, _P, _P],
    "pfm_nn_loss": [_P, _P, _P, _I, _I, _I, _P, _P, _P, _P],
    "pfm_nn_adam": [_P, _P, _P, _P, ctypes.c_size_t, _F, _F, _F, _F, _I, _F, _P],
}
# tuning keys (include/pfm.h)
TUNE_P2G2_COLUMN = 1
TUNE_MG_TAIL_CELLS = 2
TUNE_SMOOTH_TMA = 3
TUNE_CUBE_KERNELS = 4
TUNE_MIDPOINT_CENTRE = 5
# scratch limits of pfm_sort_particles_noalloc (include/pfm.h)
NOALLOC_MAX_PARTICLES = 1 << 21
NOALLOC_MAX_CELLS = 1 << 18
_RESTYPE = {"pfm_last_error": ctypes.c_char_p, "pfm_status_string": ctypes.c_char_p,
            "pfm_batch_last_error": ctypes.c_char_p, "pfm_nn_scratch_floats": ctypes.c_size_t}

_lib = None


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing=True):
    """Load libpfm.so (building it first when absent).  Raises PfmError if that fails."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise PfmError(6, f"libpfm.so not built at {path}")
        try:
            _build.build()
        except Exception as e:  # noqa: BLE001
            raise PfmError(6, f"cannot build libpfm.so: {e}") from e
    L = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = _RESTYPE.get(name, ctypes.c_int)
    _lib = L
    return L


def exported_symbols():
    return list(SIGNATURES)
