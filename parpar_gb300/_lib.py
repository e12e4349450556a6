"""ctypes binding of libpar2cuda.so (include/par2cuda.h).

The CUDA library is the only implementation: if it is missing or fails to
load, every entry point raises — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libpar2cuda.so")

DONE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int)
PROGRESS_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_uint)

ADD_OK, ADD_OK_BUSY, ADD_FULL = 0, 1, 2
METHOD_AUTO, METHOD_COMB, METHOD_XOR, METHOD_NIBBLE, METHOD_TENSOR, METHOD_TENSOR_FP4 = 0, 1, 2, 3, 4, 5
METHOD_NAMES = {"auto": METHOD_AUTO, "comb": METHOD_COMB, "xor": METHOD_XOR, "nibble": METHOD_NIBBLE,
                "tensor": METHOD_TENSOR, "tensor_fp4": METHOD_TENSOR_FP4}


def comb_kernel_name(shape: int) -> str:
    """Kernel behind a comb CTA shape id (par2cuda_set_comb_shape)."""
    if 10 <= shape <= 15:
        return "k_comb_ws"
    if shape >= 26:
        return "k_comb_pair_rr"
    if shape >= 16:
        return "k_comb_pair"
    return "k_comb_muladd"


class Info(ctypes.Structure):
    _fields_ = [
        ("device", ctypes.c_int),
        ("device_name", ctypes.c_char * 128),
        ("method_desc", ctypes.c_char * 64),
        ("staging_count", ctypes.c_uint),
        ("staging_size", ctypes.c_uint),
        ("min_staging_size", ctypes.c_uint),
        ("chunk_size", ctypes.c_size_t),
        ("slice_mem", ctypes.c_size_t),
        ("slice_size", ctypes.c_size_t),
        ("num_output_slices", ctypes.c_uint),
        ("batches_started", ctypes.c_uint),
        ("device_bytes", ctypes.c_size_t),
    ]


# every exported symbol of include/par2cuda.h: (name, restype, argtypes)
_vp, _sz, _i, _u, _u16, _u64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint, ctypes.c_uint16, ctypes.c_uint64
SIGNATURES = [
    ("par2cuda_version", ctypes.c_char_p, []),
    ("par2cuda_last_error", ctypes.c_char_p, []),
    ("par2cuda_device_count", _i, []),
    ("par2cuda_create", _i, [_i, _u, ctypes.POINTER(_vp)]),
    ("par2cuda_init", _i, [_vp, _i, _u]),
    ("par2cuda_set_slice_size", _i, [_vp, _sz]),
    ("par2cuda_set_current_slice_size", _i, [_vp, _sz]),
    ("par2cuda_set_recovery_slices", _i, [_vp, _u, _vp]),
    ("par2cuda_set_min_input_batch", _i, [_vp, _u]),
    ("par2cuda_set_progress_cb", _i, [_vp, PROGRESS_FN, _vp]),
    ("par2cuda_can_add", _i, [_vp]),
    ("par2cuda_wait_for_add", _i, [_vp]),
    ("par2cuda_add_input", _i, [_vp, _vp, _sz, _u16, _i, DONE_FN, _vp]),
    ("par2cuda_add_input_coeffs", _i, [_vp, _vp, _sz, _vp, _i, DONE_FN, _vp]),
    ("par2cuda_dummy_input", _i, [_vp, _u16, _i]),
    ("par2cuda_fill_input", _i, [_vp, _vp]),
    ("par2cuda_flush", _i, [_vp]),
    ("par2cuda_end_input", _i, [_vp, DONE_FN, _vp]),
    ("par2cuda_get_output", _i, [_vp, _u, _vp, DONE_FN, _vp]),
    ("par2cuda_output_valid", _i, [_vp, _u]),
    ("par2cuda_discard_output", _i, [_vp]),
    ("par2cuda_has_added", _i, [_vp]),
    ("par2cuda_is_empty", _i, [_vp]),
    ("par2cuda_sync", _i, [_vp]),
    ("par2cuda_free_processing_mem", _i, [_vp]),
    ("par2cuda_info_get", _i, [_vp, ctypes.POINTER(Info)]),
    ("par2cuda_destroy", _i, [_vp]),
    ("par2cuda_row_pitch_bytes", _sz, [_sz]),
    ("par2cuda_coeff", _u16, [_u16, _u16]),
    ("par2cuda_set_comb_shape", _i, [_i]),
    ("par2cuda_set_tc4_shape", _i, [_i]),
    ("par2cuda_set_tc4_group", _i, [_i]),
    ("par2cuda_tc4_shape_for", _i, [_u]),
    ("par2cuda_device_error", _i, []),
    ("par2cuda_lop3_rate", _i, [ctypes.POINTER(ctypes.c_double), _vp]),
    ("par2cuda_comb_shape_for", _i, [_u]),
    ("par2cuda_md5_chain_rate", _i, [ctypes.POINTER(ctypes.c_double), _vp]),
    ("par2cuda_muladd_scratch_bytes", _sz, [_u, _u]),
    ("par2cuda_muladd_launches", _i, [_u, _u, _sz, _i, _sz]),
    ("par2cuda_muladd", _i, [_vp, _sz, _u, _vp, _vp, _sz, _u, _sz, _i, _i, _vp, _sz, _vp]),
    ("par2cuda_muladd_noalloc", _i, [_vp, _sz, _u, _vp, _vp, _sz, _u, _sz, _i, _vp]),
    ("par2cuda_rows_checksum", _i, [_vp, _sz, _u, _vp, _sz, _i, _vp, _vp, _vp]),
    ("par2cuda_slice_hash", _i, [_vp, _sz, _u, _vp, _sz, _vp, _vp]),
    ("par2cuda_file_md5", _i, [_vp, _sz, _u, _vp, _vp, _sz, _vp, _vp]),
    ("par2cuda_file_md5_packed", _i, [_vp, _sz, _u, _vp, _vp, _sz, _vp, _vp]),
    ("par2cuda_file_md5_pooled", _i, [_vp, _sz, _u, _vp, _vp, _sz, _vp, _u, _vp]),
    ("par2cuda_file_md5_staged", _i, [_vp, _sz, _u, _vp, _vp, _sz, _vp, _u, _vp]),
    ("par2cuda_file_md5_staged_indexed", _i, [_vp, _sz, _u, _vp, _vp, _vp, _sz, _vp, _u, _vp]),
    ("par2cuda_copy_rows", _i, [_vp, _sz, _vp, _sz, _sz, _u, _vp]),
    ("par2cuda_tensor_fp4_scratch_bytes", _sz, [_u, _u, _sz]),
    ("par2cuda_tensor_fp4_rate", _i, [ctypes.POINTER(ctypes.c_double), _vp]),
    ("par2cuda_wait_selftest", _i, [_u, ctypes.POINTER(_i), ctypes.POINTER(ctypes.c_double)]),
    ("par2cuda_rows_md5", _i, [_vp, _sz, _u, _sz, _vp, _u, _vp, _vp]),
    ("par2cuda_synth_fill", _i, [_vp, _sz, _u, _sz, _u64, _u64, _vp]),
    ("par2cuda_synth_fill_at", _i, [_vp, _sz, _u, _sz, _u64, _u64, _u64, _vp]),
    ("par2cuda_coeff_index_bytes", _sz, [_u, _u]),
    ("par2cuda_coeff_index", _i, [_vp, _u, _u, _vp, _vp]),
    ("par2cuda_par2_index", _i, [_vp, _u, _vp, _u, _vp, _vp]),
    ("par2cuda_par2_coeffs", _i, [_vp, _u, _vp, _u, _vp, _vp]),
    ("par2cuda_batch_units", ctypes.c_ulonglong, [_u, _sz, _i]),
    ("par2cuda_batch_muladd", _i, [_vp, _u, ctypes.c_ulonglong, _vp, _i, _vp]),
    ("par2cuda_muladd_index", _i, [_vp, _sz, _u, _vp, _vp, _sz, _u, _sz, _i, _vp]),
]


class BatchJob(ctypes.Structure):
    """par2cuda_batch_job (include/par2cuda.h)."""
    _fields_ = [
        ("d_in", ctypes.c_void_p), ("in_pitch_words", ctypes.c_size_t), ("num_in", ctypes.c_uint),
        ("d_index", ctypes.c_void_p),
        ("d_rec", ctypes.c_void_p), ("rec_pitch_words", ctypes.c_size_t), ("num_rec", ctypes.c_uint),
        ("accumulate", ctypes.c_int),
        ("unit_base", ctypes.c_ulonglong),
    ]

_lib = None


class Par2CudaError(RuntimeError):
    pass


def load(path: str | None = None):
    """Loads libpar2cuda.so (building it first if the toolkit is present)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str = "") -> int:
    if rc < 0:
        msg = load().par2cuda_last_error().decode(errors="replace")
        raise Par2CudaError("%s failed: %s" % (what or "par2cuda call", msg))
    return rc
