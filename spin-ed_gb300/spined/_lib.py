"""ctypes binding of libsed.so (the C ABI declared in include/sed.h).

This is the same binding a Haskell maintainer writes with ``foreign import
ccall`` in src/SpinED/Internal.hs: plain pointers, sizes and int statuses.
There is no fallback: if libsed.so is missing, importing fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libsed.so")

# Status codes (include/sed.h)
LS_SUCCESS = 0
LS_OUT_OF_MEMORY = 1
LS_INVALID_ARGUMENT = 2
LS_INVALID_HAMMING_WEIGHT = 3
LS_INVALID_SPIN_INVERSION = 4
LS_INVALID_NUMBER_SPINS = 5
LS_INVALID_PERMUTATION = 6
LS_INVALID_SECTOR = 7
LS_INVALID_STATE = 8
LS_INVALID_DATATYPE = 9
LS_PERMUTATION_TOO_LONG = 10
LS_INCOMPATIBLE_SYMMETRIES = 11
LS_NOT_A_REPRESENTATIVE = 12
LS_CACHE_NOT_BUILT = 14
LS_OPERATOR_IS_COMPLEX = 18
LS_DIMENSION_MISMATCH = 19
LS_GROUP_TOO_BIG = 20
LS_CUDA_ERROR = 21
LS_NOT_CONVERGED = 22
LS_DEVICE_TIMEOUT = 23

SED_FORM_AUTO, SED_FORM_STREAM, SED_FORM_ON_THE_FLY = 0, 1, 2
SED_PRECISION_FP64, SED_PRECISION_MIXED = 0, 1
SED_ROTATE_AUTO, SED_ROTATE_FP64, SED_ROTATE_TENSOR = 0, 1, 2
SED_START_RANDOM, SED_START_GIVEN = 0, 1
SED_MLP_PATH_AUTO, SED_MLP_PATH_SIMT = 0, 1
SED_RECORD_AUTO, SED_RECORD_CANONICALISE = 0, 1

PROGRESS_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_uint64, C.POINTER(C.c_double),
                          C.POINTER(C.c_double), C.c_uint)


class EighOptions(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("nev", C.c_uint32),
        ("tol", C.c_double),
        ("max_iter", C.c_uint32),
        ("max_basis", C.c_uint32),
        ("block_size", C.c_uint32),
        ("precision", C.c_uint32),
        ("start", C.c_uint32),
        ("form", C.c_uint32),
        ("seed", C.c_uint64),
        ("start_vectors", C.c_void_p),
        ("start_stride", C.c_uint64),
        ("progress", PROGRESS_FN),
        ("progress_user", C.c_void_p),
    ]


class EighInfo(C.Structure):
    _fields_ = [
        ("iterations", C.c_uint64),
        ("matvecs", C.c_uint64),
        ("restarts", C.c_uint64),
        ("fp32_iterations", C.c_uint64),
        ("seconds_total", C.c_double),
        ("seconds_setup", C.c_double),
        ("seconds_solve", C.c_double),
    ]


class BatchInfo(C.Structure):
    _fields_ = [
        ("block_steps_max", C.c_uint64),
        ("restarts_max", C.c_uint64),
        ("seconds_total", C.c_double),
        ("seconds_setup", C.c_double),
        ("seconds_solve", C.c_double),
        ("kernel_ms", C.c_double),
        ("grid", C.c_uint32),
        ("ctas_per_sm", C.c_uint32),
        ("threads_per_cta", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


# (name, restype, argtypes)
_P, _U, _I, _U64, _D, _B = C.c_void_p, C.c_uint, C.c_int, C.c_uint64, C.c_double, C.c_bool
SIGNATURES = [
    ("ls_error_to_string", C.c_void_p, [_I]),
    ("ls_destroy_string", None, [_P]),
    ("ls_enable_logging", None, []),
    ("ls_disable_logging", None, []),
    ("ls_create_symmetry", _I, [C.POINTER(_P), _U, _P, _U]),
    ("ls_destroy_symmetry", None, [_P]),
    ("ls_get_sector", _U, [_P]),
    ("ls_get_phase", _D, [_P]),
    ("ls_get_periodicity", _U, [_P]),
    ("ls_create_group", _I, [C.POINTER(_P), _U, _P]),
    ("ls_destroy_group", None, [_P]),
    ("ls_get_group_size", _U, [_P]),
    ("ls_create_spin_basis", _I, [C.POINTER(_P), _P, _U, _I, _I]),
    ("ls_destroy_spin_basis", None, [_P]),
    ("ls_build", _I, [_P]),
    ("ls_build_unsafe", _I, [_P, _U64, _P]),
    ("ls_get_number_states", _I, [_P, C.POINTER(_U64)]),
    ("ls_get_states", _I, [C.POINTER(_P), _P]),
    ("ls_states_get_data", _P, [_P]),
    ("ls_states_get_size", _U64, [_P]),
    ("ls_destroy_states", None, [_P]),
    ("ls_create_interaction1", _I, [C.POINTER(_P), _P, _U, _P]),
    ("ls_create_interaction2", _I, [C.POINTER(_P), _P, _U, _P]),
    ("ls_create_interaction3", _I, [C.POINTER(_P), _P, _U, _P]),
    ("ls_create_interaction4", _I, [C.POINTER(_P), _P, _U, _P]),
    ("ls_interaction_is_real", _B, [_P]),
    ("ls_destroy_interaction", None, [_P]),
    ("ls_create_operator", _I, [C.POINTER(_P), _P, _U, _P]),
    ("ls_destroy_operator", None, [_P]),
    ("ls_operator_matmat", _I, [_P, _I, _U64, _U64, _P, _U64, _P, _U64]),
    ("ls_operator_expectation", _I, [_P, _I, _U64, _U64, _P, _U64, _P]),
    ("ls_operator_is_real", _B, [_P]),
    ("sed_eigh_options_init", None, [C.POINTER(EighOptions)]),
    ("sed_eigh", _I, [_P, _I, C.POINTER(EighOptions), _P, _P, _U64, _P, C.POINTER(EighInfo)]),
    ("sed_eigh_batched", _I, [_U, _P, C.POINTER(EighOptions), _P, _P, _P, _P, C.POINTER(BatchInfo)]),
    ("sed_operator_prepare", _I, [_P, _I]),
    ("sed_operator_stream_bytes", _U64, [_P]),
    ("sed_operator_stream_elements", _U64, [_P]),
    ("sed_operator_matmat_device", _I, [_P, _I, _U64, _U64, _P, _U64, _P, _U64, _P]),
    ("sed_operator_expectation_noalloc", _I, [_P, _I, _U64, _U64, _P, _U64, _P, _U64, _P, _P]),
    ("sed_basis_get_norms", _I, [_P, _P]),
    ("sed_basis_device_states", _P, [_P]),
    ("sed_basis_index", _I, [_P, _U64, C.POINTER(_U64)]),
    ("sed_basis_state_info", _I, [_P, _U64, C.POINTER(_U64), C.POINTER(_U), C.POINTER(_U)]),
    ("sed_mlp_create", _I, [C.POINTER(_P), _U, _U, _U64, _U64]),
    ("sed_mlp_destroy", None, [_P]),
    ("sed_mlp_num_params", _U64, [_P]),
    ("sed_mlp_get_params", _I, [_P, _P]),
    ("sed_mlp_set_params", _I, [_P, _P]),
    ("sed_mlp_forward", _I, [_P, _P, _U64, _P]),
    ("sed_mlp_loss_grad", _I, [_P, _P, _P, _P, _U64, C.POINTER(_D), _P]),
    ("sed_mlp_train", _I, [_P, _P, _P, _P, _U64, _U, _U, C.c_float, _U64, C.POINTER(_D)]),
    ("sed_mlp_sample", _I, [_P, _P, _U64, _U64, _U64, _P, _P, _P]),
    ("sed_mlp_start_vector", _I, [_P, _P, _P]),
    ("sed_mlp_set_path", _I, [_P, _I]),
    ("sed_mlp_create_patch", _I, [C.POINTER(_P), _U, _U, _P, _U, _U64, _U64]),
    ("sed_mlp_set_patch_sites", _I, [_P, _U, _P, _U64]),
    ("sed_release_workspace", None, []),
    ("sed_set_batched_launch", None, [C.c_uint, C.c_uint]),
    ("sed_rotate_vectors", _I, [_P, _U64, C.c_uint32, _P, C.c_uint32, _U64, _I, _P]),
    ("sed_set_rotate_path", None, [_I]),
    ("sed_operator_time_matvec", _I, [_P, _P, _P, C.c_uint, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("sed_set_device_memory_limit", None, [_U64]),
    ("sed_device_memory_in_use", _U64, []),
    ("sed_set_device_wait_limit", None, [C.c_double]),
    ("sed_debug_barrier_extra_arrivals", None, [C.c_uint]),
    ("sed_debug_batched_layout", C.c_uint, [C.c_uint, C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.c_double,
                                           C.c_uint, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    ("sed_set_record_mode", None, [_I]),
    ("sed_operator_recorded_with_table", _I, [_P]),
    ("sed_mlp_uses_tensor_cores", _I, [_P]),
    ("sed_kernel_launches", _U64, []),
    ("sed_version", C.c_char_p, []),
]

_lib: C.CDLL | None = None


def load() -> C.CDLL:
    """Load libsed.so; raises if it has not been built (no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build libsed first (spin-ed_gb300/build_lib.py)")
        lib = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def error_message(code: int) -> str:
    lib = load()
    p = lib.ls_error_to_string(code)
    try:
        return C.string_at(p).decode()
    finally:
        lib.ls_destroy_string(p)
