"""CPU-side checks of the C-ABI library: it loads, exports every symbol that
include/par2cuda.h declares, and the pure host helpers agree with the oracle."""
import ctypes
import os
import re

import numpy as np

from parpar_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(par2cuda_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    # and the Python binding covers the same set
    assert names == {s[0] for s in _lib.SIGNATURES}


def test_host_helpers_without_gpu():
    lib = _lib.load()
    from oracle import oracle as O
    assert lib.par2cuda_version().startswith(b"par2cuda")
    for i, e in [(0, 1), (1, 1), (2, 1), (32767, 65534), (100, 0), (7, 12345)]:
        assert lib.par2cuda_coeff(i, e) == O.coeff(i, e)
    # pitch: data padded to 8 bytes + 8-byte checksum, rounded to 128 bytes
    for s, p in [(2, 128), (120, 128), (121, 256), (1 << 20, (1 << 20) + 128)]:
        assert lib.par2cuda_row_pitch_bytes(s) == p
    assert lib.par2cuda_muladd_scratch_bytes(10, 100) == (max(10 * 13 * 16, 10 * 100 * 32) + 255) // 256 * 256


def test_launch_counts_without_gpu():
    lib = _lib.load()
    assert lib.par2cuda_muladd_launches(200, 2000, 1 << 20, _lib.METHOD_COMB, 0) == 2
    assert lib.par2cuda_muladd_launches(200, 2000, 1 << 20, _lib.METHOD_XOR, 0) == 1
    assert lib.par2cuda_muladd_launches(0, 2000, 1 << 20, _lib.METHOD_COMB, 0) == 0
    # tensor_fp4: coefficient expansion, then per word chunk the input planes
    # and the GEMM; a chunk holds what the scratch leaves after the fixed part
    R, N, nw = 200, 2000, 1048580
    kbytes = (N + 15) // 16 * 16 * 8
    one_tile = (128 * kbytes + 1023) // 1024 * 1024
    fixed = lib.par2cuda_tensor_fp4_scratch_bytes(R, N, 1) - one_tile
    full = lib.par2cuda_tensor_fp4_scratch_bytes(R, N, nw)
    chunk_words = (full - fixed) // kbytes // 128 * 128
    assert lib.par2cuda_muladd_launches(R, N, nw, _lib.METHOD_TENSOR_FP4, full) == 1 + 2 * -(-nw // chunk_words)
    assert lib.par2cuda_muladd_launches(R, N, nw, _lib.METHOD_TENSOR_FP4, fixed + 128 * kbytes) == 1 + 2 * -(-nw // 128)
    assert lib.par2cuda_muladd_launches(R, N, nw, _lib.METHOD_TENSOR_FP4, fixed) == 0   # too small: the call fails


def test_create_fails_cleanly_without_device():
    lib = _lib.load()
    h = ctypes.c_void_p()
    if lib.par2cuda_device_count() > 0:
        return
    assert lib.par2cuda_create(0, 2, ctypes.byref(h)) < 0
    assert lib.par2cuda_last_error()
