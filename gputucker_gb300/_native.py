"""ctypes binding of include/gputucker_gb300.h (the library's C ABI).

Loads the in-tree build gputucker_gb300/lib/libgputucker_gb300.so.  There is no
fallback: if the library is missing, importing a compute entry point raises.
"""

from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libgputucker_gb300.so")

GTK_OK = 0
GTK_ERR_ARG = 1
GTK_ERR_IO = 2
GTK_ERR_PARSE = 3
GTK_ERR_PARTITION = 4
GTK_ERR_CUDA = 5
GTK_ERR_OOM = 6
GTK_ERR_STATE = 7
GTK_ERR_UNSUPPORTED = 8
GTK_ERR_NUMERIC = 9

GTK_F32 = 0
GTK_F64 = 1
GTK_PREC_PLAIN = 0
GTK_PREC_BF16 = 1
GTK_PREC_TF32 = 2
GTK_GEN_UNIFORM = 0
GTK_GEN_ZIPF = 1
GTK_VAL_UNIFORM = 0
GTK_VAL_LOGNORMAL = 1
GTK_VAL_PLANTED = 2
GTK_MAX_ORDER = 8
GTK_MAX_RANK = 64
GTK_VALIDATE_CHECKS = 8

STATUS_NAMES = {
    GTK_ERR_ARG: "GTK_ERR_ARG", GTK_ERR_IO: "GTK_ERR_IO", GTK_ERR_PARSE: "GTK_ERR_PARSE",
    GTK_ERR_PARTITION: "GTK_ERR_PARTITION", GTK_ERR_CUDA: "GTK_ERR_CUDA", GTK_ERR_OOM: "GTK_ERR_OOM",
    GTK_ERR_STATE: "GTK_ERR_STATE", GTK_ERR_UNSUPPORTED: "GTK_ERR_UNSUPPORTED", GTK_ERR_NUMERIC: "GTK_ERR_NUMERIC",
}


class GTKError(RuntimeError):
    """A GTK_ERR_* status returned by the native library."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code
        self.message = message


class TensorInfo(C.Structure):
    _fields_ = [
        ("order", C.c_int), ("rank", C.c_int), ("dtype", C.c_int), ("device", C.c_int),
        ("nnz", C.c_uint64), ("block_count", C.c_uint64),
        ("dims", C.c_uint32 * GTK_MAX_ORDER), ("partition_dims", C.c_uint32 * GTK_MAX_ORDER),
        ("block_dims", C.c_uint32 * GTK_MAX_ORDER), ("norm", C.c_double), ("device_bytes", C.c_uint64),
        ("streamed", C.c_uint32), ("stream_chunk", C.c_uint64), ("host_direct", C.c_uint32),
    ]


class Plan(C.Structure):
    _fields_ = [
        ("partition_dims", C.c_uint32 * GTK_MAX_ORDER), ("block_dims", C.c_uint32 * GTK_MAX_ORDER),
        ("block_count", C.c_uint64), ("dimension_based", C.c_int), ("streams", C.c_int),
        ("avail_nnz_per_task", C.c_uint64), ("required_bytes", C.c_uint64), ("block_bytes", C.c_uint64),
    ]


P = C.c_void_p
U32P = C.POINTER(C.c_uint32)
U64P = C.POINTER(C.c_uint64)

# name -> (restype, argtypes)
SIGNATURES = {
    "gtk_last_error": (C.c_char_p, []),
    "gtk_version": (C.c_int, []),
    "gtk_parse_file": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_uint32, C.POINTER(P)]),
    "gtk_parse_buffer": (C.c_int, [C.c_char_p, C.c_size_t, C.c_int, C.c_int, C.c_uint32, C.POINTER(P)]),
    "gtk_coo_from_arrays": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(P), P, C.c_int, P, C.POINTER(P)]),
    "gtk_coo_info": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), U64P, U32P, U64P]),
    "gtk_coo_export": (C.c_int, [P, C.POINTER(P), P]),
    "gtk_coo_free": (None, [P]),
    "gtk_coo_pin": (C.c_int, [P]),
    "gtk_create_blocks": (C.c_int, [P, U32P, C.c_int, C.c_int, C.POINTER(P)]),
    "gtk_tensor_info_get": (C.c_int, [P, C.POINTER(TensorInfo)]),
    "gtk_block_info": (C.c_int, [P, C.c_uint64, U32P, U64P]),
    "gtk_block_data": (C.c_int, [P, C.c_uint64, C.POINTER(P), P]),
    "gtk_block_segments": (C.c_int, [P, C.c_uint64, C.c_int, P, P]),
    "gtk_destroy": (None, [P]),
    "gtk_init_random": (C.c_int, [P, C.c_uint32, C.c_uint64]),
    "gtk_set_factor": (C.c_int, [P, C.c_int, P]),
    "gtk_get_factor": (C.c_int, [P, C.c_int, P]),
    "gtk_set_core": (C.c_int, [P, P]),
    "gtk_get_core": (C.c_int, [P, P]),
    "gtk_set_precision": (C.c_int, [P, C.c_int]),
    "gtk_update_mode": (C.c_int, [P, C.c_int]),
    "gtk_update_factor_matrices": (C.c_int, [P]),
    "gtk_update_core": (C.c_int, [P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "gtk_validate": (C.c_int, [P, U64P]),
    "gtk_reconstruction": (C.c_int, [P, C.POINTER(C.c_double)]),
    "gtk_tucker_decomposition": (C.c_int, [P, C.c_int, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "gtk_compute_delta": (C.c_int, [P, C.c_int, P]),
    "gtk_sweep": (C.c_int, [P, C.POINTER(C.c_double)]),
    "gtk_set_graph": (C.c_int, [P, C.c_int]),
    "gtk_generate": (C.c_int, [C.c_int, U32P, C.c_uint64, C.c_int, C.c_double, C.c_int, C.c_int, C.c_uint64,
                               C.POINTER(P)]),
    "gtk_generate_planted": (C.c_int, [C.c_int, U32P, C.c_uint64, C.c_int, C.c_double, C.c_int, C.c_uint64,
                                       C.POINTER(P)]),
    "gtk_write_text": (C.c_int, [P, C.c_char_p]),
    "gtk_reconstruction_error_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_uint64, C.POINTER(P), P, C.POINTER(P), P, P,
                                                   P]),
    "gtk_plan_partition": (C.c_int, [C.c_int, U32P, C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_uint64,
                                     C.POINTER(Plan)]),
    "gtk_device_memory": (C.c_int, [C.c_int, U64P, U64P]),
    "gtk_release_cached_memory": (None, []),
    "gtk_checkpoint_save": (C.c_int, [P, C.c_char_p, C.POINTER(C.c_double), C.c_int]),
    "gtk_checkpoint_load": (C.c_int, [P, C.c_char_p, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_int)]),
    "gtk_checkpoint_info": (C.c_int, [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), U32P,
                                      U32P, C.POINTER(C.c_int)]),
    "gtk_ws_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_int, C.POINTER(P)]),
    "gtk_ws_destroy": (None, [P]),
    "gtk_ws_info": (C.c_int, [P, C.POINTER(C.c_int), U64P, U64P]),
    "gtk_ws_save": (C.c_int, [P, C.c_char_p]),
    "gtk_ws_load": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(P)]),
    "gtk_ws_get_params": (C.c_int, [P, P, P, P]),
    "gtk_ws_set_params": (C.c_int, [P, P, P, P]),
    "gtk_ws_features": (C.c_int, [P, C.c_int, P]),
    "gtk_ws_add_example": (C.c_int, [P, P]),
    "gtk_ws_train": (C.c_int, [P, C.c_int, C.c_int, C.c_float, C.POINTER(C.c_double)]),
    "gtk_ws_apply": (C.c_int, [P, P]),
    "gtk_ws_loss_grad": (C.c_int, [P, P, P, C.c_int, C.POINTER(C.c_double), P]),
    "gtk_ws_predict": (C.c_int, [P, P, C.c_int, P]),
    "gtk_set_kernel_variant": (C.c_int, [P, C.c_int]),
    "gtk_get_kernel_variant": (C.c_int, [P, C.POINTER(C.c_int)]),
    "gtk_autotune": (C.c_int, [P, C.POINTER(C.c_int)]),
    "gtk_random_sequence": (C.c_int, [C.c_uint32, C.c_uint64, C.c_uint64, C.c_void_p]),
    "gtk_set_ctas_per_sm": (C.c_int, [P, C.c_int]),
    "gtk_get_ctas_per_sm": (C.c_int, [P, C.POINTER(C.c_int)]),
    "gtk_batch_create": (C.c_int, [C.POINTER(P), C.c_int, C.POINTER(P)]),
    "gtk_batch_sweep": (C.c_int, [P, C.POINTER(C.c_double)]),
    "gtk_batch_kernels": (C.c_int, [P, U64P]),
    "gtk_batch_destroy": (None, [P]),
    "gtk_profile_enable": (C.c_int, [P, C.c_int]),
    "gtk_profile_read": (C.c_int, [P, C.c_int, C.POINTER(C.c_double), U64P]),
    "gtk_solve_counters": (C.c_int, [P, U64P, U64P, C.c_int]),
    "gtk_profile_reset": (C.c_int, [P]),
    "gtk_timer_begin": (C.c_int, [P]),
    "gtk_timer_end": (C.c_int, [P, C.POINTER(C.c_double)]),
    "gtk_synchronize": (C.c_int, [P]),
}

_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Load the native library (once) and declare every signature."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(
            f"gputucker_gb300 native library not built: {path} is missing "
            "(run `python -m gputucker_gb300.build`)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != GTK_OK:
        msg = load().gtk_last_error()
        raise GTKError(rc, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
