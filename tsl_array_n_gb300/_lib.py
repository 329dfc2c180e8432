"""ctypes binding of libff.so (the C ABI declared in include/ff.h).

The library is built in-tree by ``tsl_array_n_gb300.build``.  Loading fails
loudly when it is missing: there is no CPU fallback for any entry point.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libff.so")
_lib = None


class FFError(RuntimeError):
    """A libff call returned a negative status."""


class PressureDesc(C.Structure):
    _fields_ = [
        ("resolution", C.c_int * 3), ("grid_spacing", C.c_double * 3), ("origin", C.c_double * 3),
        ("preconditioner", C.c_int), ("tolerance", C.c_double), ("max_iterations", C.c_int),
        ("max_iterations_factor", C.c_double), ("relative_tolerance", C.c_int),
        ("max_plausible_pressure", C.c_double),
        ("mg_levels", C.c_int), ("mg_down", C.c_int), ("mg_up", C.c_int), ("mg_coarsest", C.c_int),
        ("mg_final", C.c_int), ("mg_sor", C.c_double), ("mg_coarsen_mask", C.c_int),
        ("mg_coarsen_weights", C.c_int), ("mg_coarse_mode", C.c_int),
        ("vcycle_storage", C.c_int), ("iterate", C.c_int),
    ]


class Shape(C.Structure):
    _fields_ = [("type", C.c_int), ("has_rotation", C.c_int), ("center", C.c_double * 3),
                ("radius", C.c_double), ("half_extents", C.c_double * 3),
                ("rotation_axis", C.c_double * 3), ("rotation_angle", C.c_double)]


class AdvectDesc(C.Structure):
    _fields_ = [("resolution", C.c_int * 3), ("grid_spacing", C.c_double * 3), ("origin", C.c_double * 3),
                ("dt", C.c_double), ("max_substeps", C.c_int), ("order", C.c_int)]


class FlipDesc(C.Structure):
    _fields_ = [("resolution", C.c_int * 3), ("grid_spacing", C.c_double * 3), ("origin", C.c_double * 3),
                ("max_particles", C.c_int), ("dt", C.c_double), ("gravity", C.c_double * 3),
                ("reduced_pressure", C.c_int), ("flip_ratio", C.c_double), ("velocity_damping", C.c_double),
                ("p2g_atomic_scale", C.c_double), ("weight_epsilon", C.c_double), ("closed_flags", C.c_int),
                ("max_substeps", C.c_int), ("collider_push_thresh", C.c_double),
                ("collider_push_shift", C.c_double), ("carry_concentration", C.c_int), ("mixing", C.c_double),
                ("fade", C.c_double), ("concentration_atomic_scale", C.c_double),
                ("ambient_density", C.c_double), ("component_density", C.c_double),
                ("extrapolation_depth", C.c_int), ("pressure", PressureDesc), ("resample_enabled", C.c_int),
                ("min_particles_per_cell", C.c_int), ("max_particles_per_cell", C.c_int)]


class TwoPhaseDesc(C.Structure):
    _fields_ = [("resolution", C.c_int * 2), ("grid_spacing", C.c_double * 2), ("origin", C.c_double * 2),
                ("max_particles", C.c_int), ("dt", C.c_double), ("gravity", C.c_double * 2),
                ("ambient_density", C.c_double), ("component_density", C.c_double), ("mixing", C.c_double),
                ("fade", C.c_double), ("concentration_atomic_scale", C.c_double), ("flip_ratio", C.c_double),
                ("gas_flip_ratio", C.c_double), ("velocity_damping", C.c_double), ("p2g_atomic_scale", C.c_double),
                ("weight_epsilon", C.c_double), ("closed_flags", C.c_int), ("max_substeps", C.c_int),
                ("collider_push_thresh", C.c_double), ("collider_push_shift", C.c_double),
                ("pin_cell", C.c_int * 2), ("resample_enabled", C.c_int), ("min_particles_per_cell", C.c_int),
                ("max_particles_per_cell", C.c_int), ("extrapolation_depth", C.c_int), ("pressure", PressureDesc)]


class TwoPhase3Desc(C.Structure):
    _fields_ = [("resolution", C.c_int * 3), ("grid_spacing", C.c_double * 3), ("origin", C.c_double * 3),
                ("max_particles", C.c_int), ("dt", C.c_double), ("gravity", C.c_double * 3),
                ("ambient_density", C.c_double), ("component_density", C.c_double), ("mixing", C.c_double),
                ("fade", C.c_double), ("concentration_atomic_scale", C.c_double), ("flip_ratio", C.c_double),
                ("gas_flip_ratio", C.c_double), ("velocity_damping", C.c_double), ("p2g_atomic_scale", C.c_double),
                ("weight_epsilon", C.c_double), ("closed_flags", C.c_int), ("max_substeps", C.c_int),
                ("collider_push_thresh", C.c_double), ("collider_push_shift", C.c_double),
                ("pin_cell", C.c_int * 3), ("resample_enabled", C.c_int), ("min_particles_per_cell", C.c_int),
                ("max_particles_per_cell", C.c_int), ("extrapolation_depth", C.c_int), ("pressure", PressureDesc)]


class Diag(C.Structure):
    _fields_ = [("converged", C.c_int), ("rejected", C.c_int), ("iterations", C.c_int),
                ("stopped_by", C.c_int), ("residual", C.c_double), ("b_norm", C.c_double),
                ("bad_cells", C.c_int), ("max_iterations", C.c_int), ("kernel_launches", C.c_int),
                ("warm_start", C.c_int), ("report_floor", C.c_int), ("tolerance_below_floor", C.c_int),
                ("max_residual", C.c_double), ("noise_floor", C.c_double),
                ("noise_floor_relative", C.c_double), ("floor_threshold", C.c_double)]


# every symbol include/ff.h declares, with (restype, argtypes)
_P, _I, _D, _S = C.c_void_p, C.c_int, C.c_double, C.c_size_t
_PP = C.POINTER(C.c_void_p)
_IP = C.POINTER(C.c_int)
_FP = C.POINTER(C.c_float)
_U8P = C.POINTER(C.c_uint8)
PROTOTYPES = {
    "ff_last_error": (C.c_char_p, []),
    "ff_version": (C.c_char_p, []),
    "ff_ctx_create": (_I, [_I, _PP]),
    "ff_ctx_destroy": (_I, [_P]),
    "ff_ctx_synchronize": (_I, [_P]),
    "ff_ctx_join_copies": (_I, [_P]),
    "ff_host_alloc": (_I, [_S, _PP]),
    "ff_host_free": (_I, [_P]),
    "ff_ctx_event_record": (_I, [_P, _I]),
    "ff_ctx_event_elapsed": (_I, [_P, _I, _I, _FP]),
    "ff_field_create": (_I, [_P, _I, _I, _IP, _PP]),
    "ff_field_destroy": (_I, [_P]),
    "ff_field_upload": (_I, [_P, _P, _S]),
    "ff_field_download": (_I, [_P, _P, _S]),
    "ff_field_upload_async": (_I, [_P, _P, _S]),
    "ff_field_download_async": (_I, [_P, _P, _S]),
    "ff_field_fill": (_I, [_P, C.c_float]),
    "ff_field_copy": (_I, [_P, _P]),
    "ff_field_info": (_I, [_P, _IP, _IP, _IP, C.POINTER(C.c_int64)]),
    "ff_field_device_ptr": (_P, [_P]),
    "ff_pressure_desc_default": (None, [C.POINTER(PressureDesc), _IP, C.POINTER(C.c_double)]),
    "ff_pressure3_create": (_I, [_P, C.POINTER(PressureDesc), _PP]),
    "ff_pressure3_destroy": (_I, [_P]),
    "ff_pressure3_set_collider_weights": (_I, [_P, _P, _P, _P]),
    "ff_pressure3_set_face_weights": (_I, [_P, _P, _P, _P]),
    "ff_pressure3_set_dirichlet": (_I, [_P, _P, _P]),
    "ff_pressure3_set": (_I, [_P, C.c_char_p, _D]),
    "ff_pressure3_project": (_I, [_P, _P, _P, _P, _P, _P, _P, C.POINTER(Diag)]),
    "ff_pressure3_project_host": (_I, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, C.POINTER(Diag)]),
    "ff_pressure3_solve": (_I, [_P, _P, C.POINTER(Diag)]),
    "ff_pressure3_fields": (_I, [_P, _PP, _PP, _PP, _PP]),
    "ff_pressure3_prepare": (_I, [_P, _P, _P, _P]),
    "ff_collider3_bake": (_I, [_P, C.POINTER(Shape), _I, _I, _IP, C.POINTER(C.c_double),
                               C.POINTER(C.c_double), _P, _P, _P, _P]),
    "ff_collider3_bake_noalloc": (_I, [_P, C.POINTER(Shape), _I, _I, _IP, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), _P, _P, _P, _P]),
    "ff_advect3_create": (_I, [_P, C.POINTER(AdvectDesc), _PP]),
    "ff_advect3_destroy": (_I, [_P]),
    "ff_advect3_set_dt": (_I, [_P, _D]),
    "ff_advect3_set_collider": (_I, [_P, _P]),
    "ff_advect3_faces": (_I, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "ff_advect3_scalar": (_I, [_P, _P, _P, _P, _P, _P]),
    "ff_advect3_trace": (_I, [_P, _P, _P, _P, _P, _P, _I]),
    "ff_bc3_create": (_I, [_P, _IP, C.POINTER(C.c_double), C.POINTER(C.c_double), _PP]),
    "ff_bc3_destroy": (_I, [_P]),
    "ff_bc3_set_collider": (_I, [_P, _P, _P, _P, _P]),
    "ff_bc3_set_closed": (_I, [_P, _I]),
    "ff_bc3_set_inflows": (_I, [_P, _I, _PP, C.POINTER(C.c_double), _IP]),
    "ff_bc3_constrain": (_I, [_P, _P, _P, _P, _I]),
    "ff_viscosity3_apply": (_I, [_P, _IP, C.POINTER(C.c_double), _P, _P, _P, _D, _D, _P, _P, _P]),
    "ff_velocity3_add_force": (_I, [_P, _IP, _P, _P, _P, _D, _D, _D, _D]),
    "ff_flip_desc_default": (None, [C.POINTER(FlipDesc), _IP, C.POINTER(C.c_double), _I, _D]),
    "ff_outflow3_create": (_I, [_P, _IP, C.POINTER(C.c_double), C.POINTER(C.c_double), _I, _PP, _IP,
                                C.POINTER(C.c_double), C.POINTER(C.c_double), _D, _I, _PP]),
    "ff_outflow3_destroy": (_I, [_P]),
    "ff_outflow3_set_dt": (_I, [_P, _D]),
    "ff_outflow3_apply_velocity_bc": (_I, [_P, _P, _P, _P]),
    "ff_outflow3_clear_scalar": (_I, [_P, _P, _IP, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ff_outflow3_dirichlet": (_I, [_P, _IP, C.POINTER(C.c_double), C.POINTER(C.c_double), _D, _P, _P]),
    "ff_flip3_create": (_I, [_P, C.POINTER(FlipDesc), _P, _P, _P, _PP]),
    "ff_flip3_destroy": (_I, [_P]),
    "ff_flip3_set_collider": (_I, [_P, _P]),
    "ff_flip3_set_count": (_I, [_P, _I]),
    "ff_flip3_fields": (_I, [_P, _PP, _PP, _PP, _PP, _PP]),
    "ff_flip3_grid_fields": (_I, [_P, _PP, _PP, _PP, _PP, _PP, _PP, _PP]),
    "ff_flip3_stage": (_I, [_P, _I]),
    "ff_flip3_step": (_I, [_P, C.POINTER(Diag)]),
    "ff_twophase_desc_default": (None, [C.POINTER(TwoPhaseDesc), _IP, C.POINTER(C.c_double), _I, _D]),
    "ff_twophase2_create": (_I, [_P, C.POINTER(TwoPhaseDesc), _P, _P, _PP]),
    "ff_twophase2_destroy": (_I, [_P]),
    "ff_twophase2_set_collider": (_I, [_P, _P]),
    "ff_twophase2_set_count": (_I, [_P, _I]),
    "ff_twophase2_set_particles": (_I, [_P, _I, _FP, _FP, _FP]),
    "ff_twophase2_get_particles": (_I, [_P, _I, _FP, _FP, _FP]),
    "ff_twophase2_fields": (_I, [_P, _PP, _PP, _PP, _PP, _PP, _PP]),
    "ff_twophase2_stage": (_I, [_P, _I]),
    "ff_twophase2_step": (_I, [_P, C.POINTER(Diag)]),
    "ff_twophase2_resample_stats": (_I, [_P, C.POINTER(C.c_int64)]),
    "ff_twophase3_desc_default": (None, [C.POINTER(TwoPhase3Desc), _IP, C.POINTER(C.c_double), _I, _D]),
    "ff_twophase3_create": (_I, [_P, C.POINTER(TwoPhase3Desc), _P, _P, _P, _PP]),
    "ff_twophase3_set_particles": (_I, [_P, _I, _FP, _FP, _FP]),
    "ff_twophase3_get_particles": (_I, [_P, _I, _FP, _FP, _FP]),
    "ff_twophase3_fields": (_I, [_P, _PP, _PP, _PP, _PP, _PP, _PP, _PP]),
    "ff_twophase3_cell_counts": (_I, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "ff_flip3_resample_stats": (_I, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "ff_flip_box_seed3": (_I, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double), _I, _D,
                               C.c_uint32, _FP, C.c_int64, C.POINTER(C.c_int64)]),
    "ff_jitter_random": (_I, [C.c_uint32, _I, C.POINTER(C.c_double)]),
    "ff_unet_create": (_I, [_P, C.c_uint32, _PP]),
    "ff_unet_destroy": (_I, [_P]),
    "ff_unet_param_count": (_I, [_P, C.POINTER(C.c_int64)]),
    "ff_unet_get_params": (_I, [_P, _FP, C.c_int64]),
    "ff_unet_set_params": (_I, [_P, _FP, C.c_int64]),
    "ff_unet_get_grads": (_I, [_P, _FP, C.c_int64]),
    "ff_unet_forward": (_I, [_P, _IP, _D, _P, _P, _P, _P]),
    "ff_unet_loss_backward": (_I, [_P, _IP, _D, _P, _P, _P, _P, C.POINTER(C.c_double)]),
    "ff_unet_adam_step": (_I, [_P, _D, _D, _D, _D]),
    "ff_pressure3_set_warm_start": (_I, [_P, _P]),
    "ff_laplacian_apply": (_I, [_P, _P, _P]),
    "ff_precondition_apply": (_I, [_P, _P, _P]),
    "ff_mg_restrict": (_I, [_P, _I, _P, _P]),
    "ff_mg_prolong_add": (_I, [_P, _I, _P, _P]),
    "ff_mg_level_info": (_I, [_P, _I, _IP]),
    "ff_pressure3_profile": (_I, [_P, _I, _I, _FP]),
    "ff_mg_level_download": (_I, [_P, _I, _U8P, _FP, _FP, _FP]),
}


def declare(lib):
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def load(path=LIB_PATH):
    """Load libff.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise FFError(f"libff.so not built at {path}: run tsl_array_n_gb300.build.build()")
        _lib = declare(C.CDLL(path))
    return _lib


def check(status):
    if status != 0:
        raise FFError(f"libff status {status}: {load().ff_last_error().decode()}")
    return status
