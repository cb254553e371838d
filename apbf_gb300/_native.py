"""ctypes binding of the C ABI declared in include/apbf_gb300.h.

Loading fails loudly when libapbf_gb300.so has not been built: there is no
CPU fallback anywhere in the product path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libapbf_gb300.so"

APBF_OK = 0
STATUS_NAMES = {
    0: "APBF_OK",
    1: "APBF_ERR_INVALID_ARG",
    2: "APBF_ERR_CAPACITY",
    3: "APBF_ERR_NONFINITE",
    4: "APBF_ERR_SPIN_LIMIT",
    5: "APBF_ERR_CUDA",
    6: "APBF_ERR_NOT_BUILT",
}
FLAG_NEIGHBOR_OVERFLOW = 0x1
FLAG_TRANSFER_OVERFLOW = 0x2
FLAG_PARTICLE_OVERFLOW = 0x4
FLAG_SPIN_LIMIT = 0x8
FLAG_NONFINITE = 0x10
MAX_BOXES = 64
MAX_TRANSFERS = 10000
MLP_PARAMS = 4824  # apbf_mlp_param_count()
WARM_LEARNED = 1    # APBF_WARM_LEARNED
WARM_PROJECTED = 2  # APBF_WARM_PROJECTED
NEIGHBORHOOD_GREEN = 1  # APBF_NEIGHBORHOOD_GREEN
NEIGHBORHOOD_BINARY_SEARCH = 3  # APBF_NEIGHBORHOOD_BINARY_SEARCH


class ApbfError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} {detail}".strip())


class Settings(C.Structure):
    _fields_ = [
        ("height_kernel_id", C.c_int32),
        ("gradient_kernel_id", C.c_int32),
        ("merge", C.c_int32),
        ("split", C.c_int32),
        ("base_kernel_width_on_target_radius", C.c_int32),
        ("base_kernel_width_on_boundary_distance", C.c_int32),
        ("update_target_radius", C.c_int32),
        ("update_boundariness", C.c_int32),
        ("boundariness_calculation_method", C.c_int32),
        ("basic_pbf", C.c_int32),
        ("solver_iterations", C.c_int32),
        ("pad0", C.c_int32),
        ("boundariness_adaption_speed", C.c_float),
        ("kernel_width_adaption_speed", C.c_float),
        ("boundariness_self_grad_length_factor", C.c_float),
        ("boundariness_underpressure_factor", C.c_float),
        ("merge_duration", C.c_float),
        ("split_duration", C.c_float),
        ("smallest_target_radius", C.c_float),
        ("target_radius_offset", C.c_float),
        ("target_radius_scale_factor", C.c_float),
        ("density_error_target", C.c_float),
        ("pad1", C.c_float * 2),
    ]


class Config(C.Structure):
    _fields_ = [
        ("particle_capacity", C.c_uint32),
        ("max_neighbors", C.c_uint32),
        ("transfer_capacity", C.c_uint32),
        ("max_log2res", C.c_uint32),
        ("device", C.c_int32),
        ("reserved", C.c_uint32 * 3),
    ]


class Scene(C.Structure):
    _fields_ = [
        ("min_pos", C.c_float * 3),
        ("max_pos", C.c_float * 3),
        ("log2res", C.c_uint32),
        ("acceleration", C.c_float * 3),
    ]


class FluidView(C.Structure):
    _fields_ = [
        ("capacity", C.c_uint32),
        ("d_length", C.c_void_p),
        ("position", C.c_void_p),
        ("velocity", C.c_void_p),
        ("inverse_mass", C.c_void_p),
        ("radius", C.c_void_p),
        ("pos_backup", C.c_void_p),
        ("transferring", C.c_void_p),
        ("target_radius", C.c_void_p),
        ("kernel_width", C.c_void_p),
        ("boundariness", C.c_void_p),
        ("boundary_distance", C.c_void_p),
    ]


class TransfersView(C.Structure):
    _fields_ = [
        ("capacity", C.c_uint32),
        ("d_length", C.c_void_p),
        ("source", C.c_void_p),
        ("target", C.c_void_p),
        ("time_left", C.c_void_p),
    ]


class NeighborsView(C.Structure):
    _fields_ = [
        ("row_stride", C.c_uint32),
        ("max_per_row", C.c_uint32),
        ("count", C.c_void_p),
        ("index", C.c_void_p),
        ("d_total", C.c_void_p),
    ]


class HostFluid(C.Structure):
    """apbf_host_fluid: host pointers of the particle lists (null fields are skipped)."""
    _fields_ = [(name, C.c_void_p) for name in (
        "position", "velocity", "inverse_mass", "radius", "pos_backup", "transferring", "target_radius",
        "kernel_width", "boundariness", "boundary_distance", "lambda_prev")]


class StatusInfo(C.Structure):
    _fields_ = [
        ("flags", C.c_uint32),
        ("required_neighbors", C.c_uint32),
        ("required_transfers", C.c_uint32),
        ("required_particles", C.c_uint32),
        ("pairs", C.c_ulonglong),
        ("density_passes", C.c_uint32),
        ("converged_substeps", C.c_uint32),
        ("spin_where", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class Emitter(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("radius", C.c_float), ("nx", C.c_uint32), ("nz", C.c_uint32),
                ("speed", C.c_float), ("jitter", C.c_float), ("seed", C.c_uint32), ("max_particles", C.c_uint32),
                ("enabled", C.c_uint32), ("pad", C.c_uint32)]


class Tuning(C.Structure):
    _fields_ = [("gather_lanes", C.c_uint32), ("pass_block", C.c_uint32), ("pass_blocks_per_sm", C.c_uint32),
                ("reserved0", C.c_uint32), ("filter_in_density", C.c_uint32), ("sort_digit_bits", C.c_uint32),
                ("search_log2res", C.c_uint32), ("reserved", C.c_uint32)]


class KernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_uint32), ("pad", C.c_uint32), ("total_ms", C.c_double)]


_P = C.c_void_p
_F3 = C.POINTER(C.c_float)
_ST = C.c_int

# name -> (restype, argtypes); exactly the functions declared in include/apbf_gb300.h
SIGNATURES = {
    "apbf_abi_version": (C.c_uint32, []),
    "apbf_last_error": (C.c_char_p, []),
    "apbf_default_settings": (None, [C.POINTER(Settings)]),
    "apbf_create": (_ST, [C.POINTER(Config), C.POINTER(_P)]),
    "apbf_destroy": (_ST, [_P]),
    "apbf_set_settings": (_ST, [_P, C.POINTER(Settings)]),
    "apbf_set_scene": (_ST, [_P, C.POINTER(Scene)]),
    "apbf_set_emitter": (_ST, [_P, _P]),
    "apbf_set_oriented_boxes": (_ST, [_P, _P, _P, _P, C.c_uint32]),
    "apbf_get_box_rotations": (_ST, [_P, _P, C.c_uint32]),
    "apbf_set_boxes": (_ST, [_P, _F3, _F3, C.c_uint32]),
    "apbf_fluid_get_view": (_ST, [_P, C.POINTER(FluidView)]),
    "apbf_transfers_get_view": (_ST, [_P, C.POINTER(TransfersView)]),
    "apbf_neighbors_get_view": (_ST, [_P, C.POINTER(NeighborsView)]),
    "apbf_set_wait_limit": (_ST, [_P, C.c_uint32, C.c_int]),
    "apbf_bind_lists": (_ST, [_P, C.POINTER(FluidView), C.POINTER(TransfersView), C.POINTER(NeighborsView)]),
    "apbf_unbind_lists": (_ST, [_P]),
    "apbf_neighbors_get_reverse_view": (_ST, [_P, C.POINTER(NeighborsView), C.POINTER(C.c_uint32), _P]),
    "apbf_set_lengths": (_ST, [_P, C.c_uint32, C.c_uint32, _P]),
    "apbf_get_lengths": (_ST, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), _P]),
    "apbf_velocity_handling_apply": (_ST, [_P, C.c_float, _F3, _P]),
    "apbf_neighborhood_green_apply": (_ST, [_P, C.c_float, _F3, _F3, C.c_uint32, _P]),
    "apbf_neighborhood_binary_search_apply": (_ST, [_P, C.c_float, _P]),
    "apbf_calculate_position_code": (_ST, [_P, _P, C.c_uint32, _P, _P]),
    "apbf_set_neighborhood_search": (_ST, [_P, C.c_int]),
    "apbf_box_collision_apply": (_ST, [_P, _P]),
    "apbf_incompressibility_apply": (_ST, [_P, _P]),
    "apbf_kernel_width_from_boundary_distance_apply": (_ST, [_P, _P]),
    "apbf_spread_kernel_width_apply": (_ST, [_P, _P]),
    "apbf_update_transfers_apply": (_ST, [_P, _P]),
    "apbf_particle_transfer_apply": (_ST, [_P, C.c_float, _P]),
    "apbf_substep": (_ST, [_P, C.c_float, _P]),
    "apbf_reduce_fp64": (_ST, [_P, C.POINTER(C.c_double), _P]),
    "apbf_get_status": (_ST, [_P, C.POINTER(StatusInfo), C.c_int, _P]),
    "apbf_export_pairs": (_ST, [_P, _P, C.c_uint32, _P, _P]),
    "apbf_set_debug": (_ST, [_P, C.c_int]),
    "apbf_debug_incompressibility": (_ST, [_P, _P, _P, _P, _P, _P]),
    "apbf_debug_sort": (_ST, [_P, _P, _P, _P]),
    "apbf_profile_enable": (_ST, [_P, C.c_int, C.c_uint32]),
    "apbf_profile_read": (_ST, [_P, C.POINTER(KernelTime), C.c_uint32, C.POINTER(C.c_uint32),
                                C.POINTER(C.c_ulonglong), _P]),
    "apbf_launch_count": (_ST, [_P, C.POINTER(C.c_ulonglong)]),
    "apbf_mlp_param_count": (_ST, [C.POINTER(C.c_uint32)]),
    "apbf_mlp_partials_size": (_ST, [C.c_uint32, C.POINTER(C.c_uint32)]),
    "apbf_mlp_load": (_ST, [_P, _P, _P]),
    "apbf_set_warm_start": (_ST, [_P, C.c_int]),
    "apbf_set_solve_graph": (_ST, [_P, C.c_int]),
    "apbf_set_persistent_solve": (_ST, [_P, C.c_int]),
    "apbf_fluid_write": (_ST, [_P, _P, C.c_uint32, _P]),
    "apbf_autotune_search": (_ST, [_P, _P, _P, _P]),
    "apbf_batch_set_persistent_solve": (_ST, [_P, C.c_int]),
    "apbf_fluid_read": (_ST, [_P, _P, C.c_uint32, _P, _P]),
    "apbf_batch_create": (_ST, [_P, C.c_uint32, _P]),
    "apbf_batch_substep": (_ST, [_P, C.c_float, _P]),
    "apbf_batch_destroy": (_ST, [_P]),
    "apbf_set_tuning": (_ST, [_P, _P]),
    "apbf_get_tuning": (_ST, [_P, _P]),
    "apbf_autotune": (_ST, [_P, _P, _P, _P]),
    "apbf_record_samples": (_ST, [_P, C.c_uint32, _P, _P, C.c_uint32, _P]),
    "apbf_mlp_forward": (_ST, [_P, _P, C.c_uint32, _P, _P]),
    "apbf_mlp_train_step": (_ST, [_P, _P, _P, _P, _P, _P, C.c_uint32, C.c_float, C.c_float, C.c_uint32, _P, _P,
                                  _P]),
    "apbf_sphere_collision_apply": (_ST, [_P, _F3, C.c_float, C.c_int, _P]),
    "apbf_inter_particle_collision_apply": (_ST, [_P, _P]),
    "apbf_glue_generate": (_ST, [_P, C.c_uint32, _P]),
    "apbf_glue_apply": (_ST, [_P, C.c_float, C.c_float, _P]),
    "apbf_glue_get_view": (_ST, [_P, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                 C.POINTER(C.c_void_p), C.POINTER(C.c_uint32)]),
    "apbf_save_particle_info": (_ST, [_P, C.c_char_p, _F3, _P]),
    "apbf_list_apply_edit": (_ST, [_P, C.c_uint32, _P, _P, C.c_uint32, _P, _P]),
    "apbf_list_delete_edit": (_ST, [_P, _P, _P, C.c_uint32, C.c_uint32, _P, _P, _P]),
    "apbf_list_remap_index": (_ST, [_P, _P, _P, C.c_uint32, _P, _P, C.c_uint32, C.c_uint32, _P, _P, C.c_uint32, _P,
                                    _P, _P]),
    "apbf_list_append": (_ST, [_P, _P, C.c_uint32, _P, _P, C.c_uint32, C.c_uint32, _P, _P]),
    "apbf_sort_pairs": (_ST, [_P, _P, _P, _P, C.c_uint32, C.c_uint32, _P, _P, _P]),
    "apbf_sort_pairs_noalloc": (_ST, [_P, _P, _P, C.c_uint32, C.c_uint32, _P, _P, _P]),
    "apbf_prefix_sum": (_ST, [_P, _P, _P, C.c_uint32, _P]),
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Loads libapbf_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is missing: build the CUDA library first (python -m apbf_gb300.build); "
            "apbf_gb300 has no CPU fallback"
        )
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, where: str) -> None:
    if status != APBF_OK:
        detail = ""
        if _lib is not None:
            msg = _lib.apbf_last_error()
            detail = msg.decode() if msg else ""
        raise ApbfError(status, where, detail)


def f3(v) -> C.Array:
    return (C.c_float * 3)(*[float(x) for x in v])
