"""ctypes binding of the C ABI declared in include/mmf_gb300.h.

Loading fails loudly when the CUDA library is missing: there is no CPU
fallback behind these functions.
"""
import ctypes as C
import os

from . import _build

MMF_OK = 0
MMF_ERR_ARG, MMF_ERR_CUDA, MMF_ERR_STATE, MMF_ERR_UNSUPPORTED, MMF_ERR_NOMEM = -1, -2, -3, -4, -5
BC_NONE, BC_FREE_FLOW, BC_REFLECTING, BC_WALL, BC_DIRICHLET, BC_PERIODIC = -1, 0, 1, 2, 3, 16
ARITH_REFERENCE, ARITH_FAST = 0, 1

# every symbol the header declares (checked by the CPU test suite)
EXPORTS = [
    "mmf_create", "mmf_destroy", "mmf_last_error", "mmf_abi_version", "mmf_launch_count",
    "mmf_set_cell_map", "mmf_upload_state", "mmf_download_state", "mmf_upload_state_device",
    "mmf_download_state_device", "mmf_compute_rhs", "mmf_compute_polynomials", "mmf_time_setup",
    "mmf_advance", "mmf_advance_async", "mmf_time_info", "mmf_get_stream", "mmf_advance_host", "mmf_last_step_info", "mmf_get_status", "mmf_synchronize",
    "mmf_rk_stage", "mmf_cons2prim", "mmf_prim2cons", "mmf_eval_fluxes", "mmf_eval_splitting",
    "mmf_eval_bc_values", "mmf_fp64_rate", "mmf_newton_selftest", "mmf_o2_screen_selftest", "mmf_compute_rhs_noalloc", "mmf_set_limiter",
    "mmf_set_limiter_flags_device", "mmf_get_limiter_activity",
    "mmf_batch_create", "mmf_batch_destroy", "mmf_batch_cell_count", "mmf_batch_launch_count",
    "mmf_batch_get_stream", "mmf_batch_upload", "mmf_batch_download", "mmf_batch_time_setup",
    "mmf_batch_advance_async", "mmf_batch_synchronize", "mmf_batch_case_info", "mmf_batch_set_shape",
    "mmf_batch_get_shape", "mmf_batch_autotune", "mmf_batch_set_limiter", "mmf_batch_set_indicator", "mmf_batch_set_indicator_period",
    "mmf_mlp_create", "mmf_mlp_destroy", "mmf_mlp_num_params", "mmf_mlp_input_width", "mmf_mlp_get_params",
    "mmf_mlp_set_params", "mmf_mlp_set_wait_limits", "mmf_mlp_gradients", "mmf_mlp_train_batch", "mmf_mlp_predict", "mmf_features",
    "mmf_indicator", "mmf_set_indicator", "mmf_set_indicator_period", "mmf_limiter_labels",
    "mmf_umesh_create", "mmf_umesh_destroy", "mmf_umesh_launch_count", "mmf_umesh_upload", "mmf_umesh_download",
    "mmf_umesh_compute_rhs", "mmf_umesh_time_setup", "mmf_umesh_advance",
    "mmf_autotune", "mmf_set_shape", "mmf_set_step_log", "mmf_get_step_log", "mmf_init_state", "mmf_l1_density_error", "mmf_write_vtk", "mmf_save_checkpoint", "mmf_load_checkpoint",
]
LIMIT_ALL, LIMIT_NONE, LIMIT_FLAGGED = 0, 1, 2
NOALLOC_MAX_CELLS = 65536


class Grid(C.Structure):
    _fields_ = [("dim", C.c_int), ("n", C.c_int * 3), ("origin", C.c_double * 3), ("h", C.c_double),
                ("bc_lo", C.c_int * 3), ("bc_hi", C.c_int * 3), ("dirichlet_prim", C.c_double * 5),
                ("order", C.c_int), ("arith", C.c_int), ("chunk", C.c_int)]


class UMeshDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("n_cells", C.c_int64), ("n_faces", C.c_int64),
                ("cell_volume", C.c_void_p), ("cell_size", C.c_void_p), ("solved", C.c_void_p),
                ("owner", C.c_void_p), ("neigh", C.c_void_p), ("area", C.c_void_p), ("normal", C.c_void_p),
                ("bc", C.c_void_p), ("dirichlet_prim", C.c_double * 5), ("arith", C.c_int)]


class Problem(C.Structure):
    _fields_ = [("problem", C.c_int), ("vortex_beta", C.c_double), ("sod_radius", C.c_double),
                ("sod_rho_in", C.c_double), ("sod_p_in", C.c_double), ("sod_rho_out", C.c_double),
                ("sod_p_out", C.c_double), ("periodic_exact", C.c_int)]


class MMFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("mmf error %d: %s" % (code, msg))
        self.code = code


_lib = None
_P = C.c_void_p
_D = C.POINTER(C.c_double)


def load(build_if_missing=True):
    """Load libmmf_gb300.so (building it in-tree first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB_PATH) or not _build.up_to_date():
        if not build_if_missing:
            raise RuntimeError("libmmf_gb300.so is not built")
        _build.build()
    L = C.CDLL(_build.LIB_PATH)
    L.mmf_last_error.restype = C.c_char_p
    L.mmf_launch_count.restype = C.c_int64
    L.mmf_launch_count.argtypes = [_P]
    L.mmf_create.argtypes = [C.POINTER(Grid), C.c_int, C.POINTER(_P)]
    L.mmf_destroy.argtypes = [_P]
    L.mmf_set_cell_map.argtypes = [_P, C.c_int64, C.POINTER(C.c_int64)]
    for name in ("mmf_upload_state", "mmf_download_state", "mmf_upload_state_device", "mmf_download_state_device"):
        getattr(L, name).argtypes = [_P, _P, C.c_int64]
    L.mmf_compute_rhs.argtypes = [_P, _P, _P, _D, C.c_int64]
    L.mmf_compute_polynomials.argtypes = [_P, _P, _P, _P, C.c_int64]
    L.mmf_set_limiter.argtypes = [_P, C.c_int, _P, C.c_int64]
    L.mmf_set_limiter_flags_device.argtypes = [_P, _P]
    L.mmf_get_limiter_activity.argtypes = [_P, _P, C.c_int64]
    L.mmf_time_setup.argtypes = [_P, C.c_double, C.c_double, C.c_double, C.c_int64]
    L.mmf_advance.argtypes = [_P, C.c_int64, _D, C.POINTER(C.c_int64)]
    L.mmf_advance_async.argtypes = [_P, C.c_int64]
    L.mmf_time_info.argtypes = [_P, _D, C.POINTER(C.c_int64)]
    L.mmf_get_stream.argtypes = [_P]
    L.mmf_get_stream.restype = C.c_void_p
    L.mmf_advance_host.argtypes = [_P, _P, C.c_int64, C.c_int64, _D]
    L.mmf_last_step_info.argtypes = [_P, _D, _D]
    L.mmf_get_status.argtypes = [_P, C.POINTER(C.c_uint)]
    L.mmf_synchronize.argtypes = [_P]
    L.mmf_rk_stage.argtypes = [_P, C.c_int]
    L.mmf_cons2prim.argtypes = [C.c_int64, _P, _P]
    L.mmf_prim2cons.argtypes = [C.c_int64, _P, _P]
    L.mmf_eval_fluxes.argtypes = [C.c_int64, _P, _P, _P, _P]
    L.mmf_eval_splitting.argtypes = [C.c_int64, _P, _P, _P, _P, _P]
    L.mmf_eval_bc_values.argtypes = [C.c_int64, C.c_int, _P, _P, _P, _P]
    L.mmf_newton_selftest.argtypes = [C.c_int64, _P, _P, _P]
    L.mmf_fp64_rate.argtypes = [C.c_int, _D]
    L.mmf_o2_screen_selftest.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, _P, _P, _P, _P]
    L.mmf_batch_create.argtypes = [C.c_int, C.POINTER(Grid), C.c_int, C.POINTER(_P)]
    L.mmf_batch_destroy.argtypes = [_P]
    L.mmf_batch_cell_count.argtypes = [_P]
    L.mmf_batch_cell_count.restype = C.c_int64
    L.mmf_batch_launch_count.argtypes = [_P]
    L.mmf_batch_launch_count.restype = C.c_int64
    L.mmf_batch_get_stream.argtypes = [_P]
    L.mmf_batch_get_stream.restype = C.c_void_p
    L.mmf_batch_upload.argtypes = [_P, _P, C.c_int64]
    L.mmf_batch_download.argtypes = [_P, _P, C.c_int64]
    L.mmf_batch_time_setup.argtypes = [_P, _P, _P, C.c_int64]
    L.mmf_batch_advance_async.argtypes = [_P, C.c_int64]
    L.mmf_batch_synchronize.argtypes = [_P]
    L.mmf_batch_case_info.argtypes = [_P, C.c_int, _D, C.POINTER(C.c_int64), C.POINTER(C.c_uint)]
    L.mmf_batch_set_shape.argtypes = [_P, C.c_int, C.c_int]
    L.mmf_batch_get_shape.argtypes = [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.mmf_batch_set_limiter.argtypes = [_P, C.c_int]
    L.mmf_batch_set_indicator.argtypes = [_P, _P, C.c_float]
    L.mmf_batch_autotune.argtypes = [_P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.mmf_mlp_create.argtypes = [C.c_int, C.c_uint64, C.c_int, C.POINTER(_P)]
    L.mmf_mlp_destroy.argtypes = [_P]
    L.mmf_mlp_num_params.argtypes = [_P]
    L.mmf_mlp_num_params.restype = C.c_int64
    L.mmf_mlp_input_width.argtypes = [_P]
    L.mmf_mlp_get_params.argtypes = [_P, _P, C.c_int64]
    L.mmf_mlp_set_params.argtypes = [_P, _P, C.c_int64]
    L.mmf_mlp_gradients.argtypes = [_P, _P, _P, C.c_int64, _P, C.POINTER(C.c_float)]
    L.mmf_mlp_train_batch.argtypes = [_P, _P, _P, C.c_int64, C.c_float, C.POINTER(C.c_float)]
    L.mmf_mlp_predict.argtypes = [_P, _P, C.c_int64, _P]
    L.mmf_mlp_set_wait_limits.argtypes = [_P, C.c_int64, C.c_int64]
    L.mmf_features.argtypes = [_P, _P]
    L.mmf_indicator.argtypes = [_P, _P, C.c_float, _P, _P]
    L.mmf_set_indicator.argtypes = [_P, _P, C.c_float]
    L.mmf_set_indicator_period.argtypes = [_P, C.c_int]
    L.mmf_batch_set_indicator_period.argtypes = [_P, C.c_int]
    L.mmf_limiter_labels.argtypes = [_P, _P]
    L.mmf_umesh_create.argtypes = [C.POINTER(UMeshDesc), C.c_int, C.POINTER(_P)]
    L.mmf_umesh_destroy.argtypes = [_P]
    L.mmf_umesh_launch_count.argtypes = [_P]
    L.mmf_umesh_launch_count.restype = C.c_int64
    L.mmf_umesh_upload.argtypes = [_P, _P, C.c_int64]
    L.mmf_umesh_download.argtypes = [_P, _P, C.c_int64]
    L.mmf_umesh_compute_rhs.argtypes = [_P, _P, _P, _D, C.c_int64]
    L.mmf_umesh_time_setup.argtypes = [_P, C.c_double, C.c_double, C.c_double, C.c_int64]
    L.mmf_umesh_advance.argtypes = [_P, C.c_int64, _D, C.POINTER(C.c_int64)]
    L.mmf_autotune.argtypes = [_P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.mmf_set_shape.argtypes = [_P, C.c_int, C.c_int]
    L.mmf_set_step_log.argtypes = [_P, C.c_int64]
    L.mmf_get_step_log.argtypes = [_P, _P, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.mmf_init_state.argtypes = [_P, C.POINTER(Problem)]
    L.mmf_l1_density_error.argtypes = [_P, C.POINTER(Problem), C.c_double, _D]
    L.mmf_write_vtk.argtypes = [_P, C.c_char_p]
    L.mmf_save_checkpoint.argtypes = [_P, C.c_char_p]
    L.mmf_load_checkpoint.argtypes = [_P, C.c_char_p]
    L.mmf_compute_rhs_noalloc.argtypes = [C.POINTER(Grid), _P, _P, _P, _P, _P]
    _lib = L
    return L


def check(rc):
    if rc != MMF_OK:
        raise MMFError(rc, load().mmf_last_error().decode(errors="replace"))
    return rc


def fp64_rate(device=0):
    """Measured FP64 instruction rate of a GPU (thread-level instructions/s):
    (DFMA with reused operands, DADD/DMUL/DFMA with varying operands)."""
    out = (C.c_double * 2)()
    check(load().mmf_fp64_rate(device, out))
    return out[0], out[1]


def ptr(a):
    """Raw pointer of a numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a.ctypes.data)
