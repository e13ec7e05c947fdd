"""ctypes binding of ``libpanopaea_gpu.so`` (the C ABI of include/panopaea_gpu.h).

The library is built in-tree by ``panopaea_gb300.build``.  There is no CPU
fallback: if the library is missing or no CUDA device is present, calls
raise instead of computing anything on the host.
"""

import ctypes as C
import os

from . import build as _build

PG_OK = 0
PG_NOT_CONVERGED = 1
PG_NAN_DETECTED = 2
PG_TIMEOUT = 3
PG_BAD_ARG = 4
PG_CUDA_ERROR = 5
PG_NO_DEVICE = 6
PG_OUT_OF_MEMORY = 7
PG_BREAKDOWN = 8

PG_F32, PG_F64 = 0, 1
PG_FACES, PG_CELLS = 1, 2
PG_PRECOND_NONE, PG_PRECOND_JACOBI, PG_PRECOND_MG = 0, 1, 2


class PgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (_STATUS.get(status, status), msg))
        self.status = status


_STATUS = {
    0: "PG_OK", 1: "PG_NOT_CONVERGED", 2: "PG_NAN_DETECTED", 3: "PG_TIMEOUT", 4: "PG_BAD_ARG",
    5: "PG_CUDA_ERROR", 6: "PG_NO_DEVICE", 7: "PG_OUT_OF_MEMORY", 8: "PG_BREAKDOWN",
}


class PcgStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int64),
        ("refinements", C.c_int64),
        ("residual_max", C.c_double),
        ("b_max", C.c_double),
        ("threshold", C.c_double),
        ("true_residual_max", C.c_double),
        ("status", C.c_int32),
        ("reserved", C.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class SolverParams(C.Structure):
    _fields_ = [
        ("precond", C.c_int32),
        ("rel_stop", C.c_int32),
        ("threshold", C.c_double),
        ("rel_tol", C.c_double),
        ("max_iter", C.c_int64),
        ("refine", C.c_int32),
        ("check_every", C.c_int32),
        ("inner_rel_tol", C.c_double),
        ("mg_levels", C.c_int32),
        ("mg_smooth", C.c_int32),
        ("fp64_native", C.c_int32),
        ("initial_guess", C.c_int32),
    ]


class StepParams(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("buoyancy", C.c_double),
        ("source_enabled", C.c_int32),
        ("walls_after_advect", C.c_int32),
        ("source_lo", C.c_int64 * 3),
        ("source_hi", C.c_int64 * 3),
        ("source_density", C.c_double),
        ("source_vy", C.c_double),
        ("source_field", C.c_void_p),
        ("zero_solid_after_project", C.c_int32),
        ("advect_scheme", C.c_int32),
        ("solver", SolverParams),
    ]


class AdamParams(C.Structure):
    _fields_ = [("lr", C.c_double), ("beta1", C.c_double), ("beta2", C.c_double), ("eps", C.c_double),
                ("grad_scale", C.c_double)]


_P = C.c_void_p
_I64 = C.c_int64
_D = C.c_double
_I = C.c_int

# name -> (restype, argtypes)
_SIGS = {
    "pg_status_string": (C.c_char_p, [_I]),
    "pg_debug_set_stage_wait_polls": (_I, [C.c_uint32]),
    "pg_debug_stage_wait_polls_default": (C.c_uint32, []),
    "pg_debug_mg_vcycle_ms": (C.c_int, [C.c_void_p, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]),
    "pg_debug_sym_pinv": (C.c_int, [C.c_int, C.c_void_p]),
    "pg_last_error": (C.c_char_p, []),
    "pg_version": (_I, []),
    "pg_grid_create_2d": (_I, [_I64, _I64, C.POINTER(_P)]),
    "pg_grid_create_3d": (_I, [_I64, _I64, _I64, C.POINTER(_P)]),
    "pg_grid_destroy": (_I, [_P]),
    "pg_grid_dim": (_I, [_P, C.POINTER(_I64)]),
    "pg_grid_num_elem_1": (_I64, [_P]),
    "pg_grid_num_elem_2": (_I64, [_P]),
    "pg_grid_set_stream": (_I, [_P, _P]),
    "pg_grid_synchronize": (_I, [_P]),
    "pg_grid_set_solid_faces": (_I, [_P, _P]),
    "pg_grid_set_solid_cells": (_I, [_P, _P]),
    "pg_field_alloc": (_I, [_P, _I, _I, C.POINTER(_P)]),
    "pg_field_free": (_I, [_P]),
    "pg_copy_h2d": (_I, [_P, _P, _P, C.c_size_t]),
    "pg_copy_d2h": (_I, [_P, _P, _P, C.c_size_t]),
    "pg_solve_pressure_f32": (_I, [_P, C.POINTER(SolverParams), _P, _P, _D, C.POINTER(PcgStats)]),
    "pg_pcg_noalloc_f32": (_I, [C.c_int32, _I64, _I64, _I64, _P, _I, _P, _P, _I64, _D, _P, _P, _P, _D, _P,
                                C.POINTER(PcgStats)]),
    "pg_batch_create_2d": (_I, [C.c_int32, _P, _P, C.POINTER(_P)]),
    "pg_batch_destroy": (_I, [_P]),
    "pg_batch_set_stream": (_I, [_P, _P]),
    "pg_batch_layout": (_I, [_P, _P, _P]),
    "pg_batch_set_solid_cells": (_I, [_P, _P]),
    "pg_batch_tile": (_I, [_P, _P, _P, _P]),
    "pg_batch_set_tile": (_I, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "pg_batch_autotune": (_I, [_P, C.c_char_p]),
    "pg_batch_step_f32": (_I, [_P, C.POINTER(StepParams), _P, _P, _P, _P]),
    "pg_advect_bf16": (_I, [_P, _P, _P, _D, _P]),
    "pg_step_bf16rho_f32": (_I, [_P, C.POINTER(StepParams), _P, _P, _P, C.POINTER(PcgStats)]),
    "pg_wavelet_fwt_1d": (_I, [_I, _P, _I64, _I, _P, _P]),
    "pg_wavelet_ifwt_1d": (_I, [_I, _P, _I64, _I, _P, _P]),
    "pg_wavelet_fwt_2d": (_I, [_I, _I, _I, _P, _I64, _I64, _I, _P, _P]),
    "pg_wavelet_ifwt_2d": (_I, [_I, _I, _I, _P, _I64, _I64, _I, _P, _P]),
    "pg_wavelet_div_coeff_2d": (_I, [_I, _P, _P, _P, _P, _I64, _I64, _P]),
    "pg_wavelet_inv_div_coeff_2d": (_I, [_I, _P, _P, _P, _P, _I64, _I64, _P]),
    "pg_wavelet_border_sizes_1d": (_I, [_I, _I64, _I, C.POINTER(_I64), C.POINTER(_I64), C.POINTER(_I64)]),
    "pg_wavelet_border_sizes_2d": (_I, [_I, _I, _I64, _I64, _I, C.POINTER(_I64), C.POINTER(_I64), C.POINTER(_I64),
                                        C.POINTER(_I64)]),
    "pg_wavelet_fwt_1d_border": (_I, [_I, _P, _I64, _I, _P, _P, _P]),
    "pg_wavelet_ifwt_1d_border": (_I, [_I, _P, _I64, _I, _P, _P, _P]),
    "pg_wavelet_fwt_2d_border": (_I, [_I, _I, _P, _I64, _I64, _I, _P, _P, _P]),
    "pg_wavelet_ifwt_2d_border": (_I, [_I, _I, _P, _I64, _I64, _I, _P, _P, _P]),
    "pg_wavelet_div_coeff_2d_border": (_I, [_I, _I, _P, _P, _I64, _I64, _I, _P, _P, _P]),
    "pg_unet_num_params": (_I64, []),
    "pg_unet_create": (_I, [_I64, _I64, _I64, C.POINTER(_P)]),
    "pg_unet_destroy": (_I, [_P]),
    "pg_unet_set_stream": (_I, [_P, _P]),
    "pg_unet_set_params": (_I, [_P, _P, _D]),
    "pg_unet_get_params": (_I, [_P, _P, C.POINTER(_D)]),
    "pg_unet_get_grads": (_I, [_P, _P]),
    "pg_unet_zero_grads": (_I, [_P]),
    "pg_unet_accumulate_f32": (_I, [_P, _P, _P, _P, _D, C.POINTER(_D)]),
    "pg_unet_adam_step": (_I, [_P, C.POINTER(AdamParams)]),
    "pg_unet_guess_f32": (_I, [_P, _P, _P, _D, _I, _P]),
    "pg_unet_check": (_I, [_P]),
    "pg_solve_pressure_learned_f32": (_I, [_P, C.POINTER(SolverParams), _P, _P, _P, _D, C.POINTER(PcgStats)]),
    "pg_unet_forward_f32": (_I, [_P, _P, _P, _D, _P]),
    "pg_unet_set_loss": (_I, [_P, _I]),
    "pg_kernel_launches": (_I64, []),
    "pg_profile_enable": (_I, [_I]),
    "pg_profile_reset": (_I, []),
    "pg_profile_num_kinds": (_I, []),
    "pg_profile_kind_name": (C.c_char_p, [_I]),
    "pg_profile_read": (_I, [_I, C.POINTER(_D), C.POINTER(_I64)]),
    "pg_profile_read_active": (_I, [_I, C.POINTER(_D), C.POINTER(_I64)]),
}
for _sfx in ("f32", "f64"):
    _SIGS.update({
        "pg_hodge_1_dual_" + _sfx: (_I, [_P, _P, _P]),
        "pg_hodge_1_primal_" + _sfx: (_I, [_P, _P, _P]),
        "pg_hodge_2_primal_" + _sfx: (_I, [_P, _P, _P]),
        "pg_derivative_1_primal_" + _sfx: (_I, [_P, _P, _P]),
        "pg_derivative_0_dual_" + _sfx: (_I, [_P, _P, _P]),
        "pg_mask_solid_faces_" + _sfx: (_I, [_P, _P]),
        "pg_laplacian_" + _sfx: (_I, [_P, _P, _P, _D]),
        "pg_divergence_rhs_" + _sfx: (_I, [_P, _P, _P]),
        "pg_advect_" + _sfx: (_I, [_P, _P, _P, _D, _P]),
        "pg_advect_mac_" + _sfx: (_I, [_P, _P, _P, _D, _P]),
        "pg_advect2_" + _sfx: (_I, [_P, _P, _P, _D, _P, _I]),
        "pg_project_" + _sfx: (_I, [_P, _P, _P, _D, _I]),
        "pg_walls_" + _sfx: (_I, [_P, _P]),
        "pg_pcg_" + _sfx: (_I, [_P, _I, _P, _P, _I64, _D, _P, _P, _P, _D, C.POINTER(PcgStats)]),
        "pg_step_" + _sfx: (_I, [_P, C.POINTER(StepParams), _P, _P, _P, C.POINTER(PcgStats)]),
        "pg_csr_mul_vec_" + _sfx: (_I, [_I64, _P, _P, _P, _P, _P, _P]),
        "pg_diag_mul_vec_" + _sfx: (_I, [_I64, _P, _P, _P, _P]),
        "pg_transfer_rgb8_" + _sfx: (_I, [_I64, _I64, _P, _D, _D, _P, _P]),
    })

_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load the library (building it first if needed) and bind every symbol."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("libpanopaea_gpu.so is not built (%s); run panopaea_gb300.build" % path)
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return sorted(_SIGS)


def last_error():
    return load().pg_last_error().decode(errors="replace")


def check(status, allow=(PG_OK,)):
    """Raise PgError unless `status` is in `allow`; returns the status."""
    if status not in allow:
        raise PgError(status, last_error())
    return status
