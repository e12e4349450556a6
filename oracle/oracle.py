"""ORACLE loader — test infrastructure, not product code.

Compiles and loads the plain-C restatement of the reference algorithm
(oracle/par2_oracle.c) and, where it has been built, the reference's own CPU
implementation (oracle/_ref/libparref.so, see oracle/ref.mk).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "par2_oracle.c")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libpar2oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libparref.so")

_lib = None
_ref = None


def build(force: bool = False) -> str:
    """Compiles the oracle with gcc (portable C, no ISA-specific flags)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        os.makedirs(BUILD_DIR, exist_ok=True)
        tmp = LIB + ".tmp.%d" % os.getpid()
        base = ["gcc", "-O3", "-fPIC", "-shared", "-pthread", "-std=gnu11", "-fno-strict-aliasing", "-o", tmp, SRC]
        if os.uname().machine == "aarch64":
            # CRC32 instructions; the SVE2 carry-less multiply baseline only if
            # this compiler accepts it (the library checks the CPU at run time)
            r = subprocess.run(base + ["-march=armv8-a+crc", "-DOR_ENABLE_SVE2"], capture_output=True)
            if r.returncode != 0:
                subprocess.check_call(base + ["-march=armv8-a+crc"])
        else:
            subprocess.check_call(base)
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        u16, sz, vp, i32 = ctypes.c_uint16, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int
        L.or_exp.restype = u16; L.or_exp.argtypes = [ctypes.c_uint32]
        L.or_mul.restype = u16; L.or_mul.argtypes = [u16, u16]
        L.or_mul_slow.restype = u16; L.or_mul_slow.argtypes = [u16, u16]
        L.or_input_log.restype = u16; L.or_input_log.argtypes = [u16]
        L.or_coeff.restype = u16; L.or_coeff.argtypes = [u16, u16]
        L.or_coeff_from_log.restype = u16; L.or_coeff_from_log.argtypes = [u16, u16]
        L.or_recover.restype = i32
        L.or_recover.argtypes = [vp, vp, vp, ctypes.c_uint, sz, vp, ctypes.c_uint, vp, i32]
        L.or_recover_coeffs.restype = i32
        L.or_recover_coeffs.argtypes = [vp, vp, vp, ctypes.c_uint, sz, ctypes.c_uint, vp, i32]
        L.or_cksum.restype = ctypes.c_uint64; L.or_cksum.argtypes = [vp, sz, sz]
        L.or_cksum_check.restype = i32; L.or_cksum_check.argtypes = [vp, sz, ctypes.c_uint64]
        L.or_md5.restype = None; L.or_md5.argtypes = [vp, sz, ctypes.c_uint64, vp]
        L.or_crc32.restype = ctypes.c_uint32; L.or_crc32.argtypes = [vp, sz, ctypes.c_uint64]
        L.or_hash_file.restype = None; L.or_hash_file.argtypes = [vp, sz, sz, vp, vp]
        L.or_recover_fast.restype = i32
        L.or_recover_fast.argtypes = [vp, ctypes.c_uint, sz, vp, ctypes.c_uint, vp, i32]
        L.or_fast_method.restype = ctypes.c_char_p
        L.or_clmul_method.restype = ctypes.c_char_p
        L.or_recover_clmul.restype = i32
        L.or_recover_clmul.argtypes = [vp, ctypes.c_uint, sz, vp, ctypes.c_uint, vp, i32]
        L.or_crc32_fast.restype = ctypes.c_uint32; L.or_crc32_fast.argtypes = [vp, sz, ctypes.c_uint64]
        L.or_hash_rows.restype = None
        L.or_hash_rows.argtypes = [vp, sz, sz, vp, ctypes.c_uint, vp, vp, i32]
        L.or_synth_fill.restype = None
        L.or_synth_fill.argtypes = [vp, sz, ctypes.c_uint, sz, ctypes.c_uint64, ctypes.c_uint64, i32]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref():
    """The reference's own compiled CPU core (only where oracle/ref.mk ran)."""
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError(REF_LIB)
        L = ctypes.CDLL(REF_LIB)
        u16, sz, vp, i32 = ctypes.c_uint16, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int
        L.ref_gf_exp.restype = u16; L.ref_gf_exp.argtypes = [u16]
        L.ref_input_log.restype = u16; L.ref_input_log.argtypes = [u16]
        L.ref_coeff.restype = u16; L.ref_coeff.argtypes = [u16, u16]
        L.ref_cksum_copy.restype = None; L.ref_cksum_copy.argtypes = [vp, vp, sz, sz]
        L.ref_cksum_copy_check.restype = i32; L.ref_cksum_copy_check.argtypes = [vp, vp, sz]
        L.ref_create.restype = i32
        L.ref_create.argtypes = [vp, vp, vp, ctypes.c_uint, sz, vp, ctypes.c_uint, vp, vp, i32, i32,
                                 ctypes.c_uint, ctypes.POINTER(ctypes.c_double)]
        L.ref_create_coeffs.restype = i32
        L.ref_create_coeffs.argtypes = [vp, vp, vp, ctypes.c_uint, sz, ctypes.c_uint, vp, vp, i32]
        L.ref_last_method_name.restype = ctypes.c_char_p
        L.ref_hash_file.restype = None; L.ref_hash_file.argtypes = [vp, sz, sz, sz, vp, vp]
        L.ref_crc32.restype = ctypes.c_uint32; L.ref_crc32.argtypes = [vp, sz]
        L.ref_md5crc.restype = ctypes.c_uint32; L.ref_md5crc.argtypes = [vp, sz, sz, vp]
        L.ref_md5multi.restype = None; L.ref_md5multi.argtypes = [vp, ctypes.c_uint, sz, vp]
        L.ref_job.restype = i32
        L.ref_job.argtypes = [vp, sz, vp, vp, ctypes.c_uint, sz, vp, ctypes.c_uint, vp, vp, vp, vp, ctypes.c_uint,
                              vp, vp, i32, ctypes.POINTER(ctypes.c_double)]
        L.ref_host_info.restype = i32
        L.ref_host_info.argtypes = [ctypes.c_char_p, sz]
        _ref = L
    return _ref


def ref_job(x: np.ndarray, lens, input_nums, exps, file_lens=None, first_rows=None, threads: int = 0):
    """One whole create job through the reference's own CPU core
    (oracle/ref_shim.cpp ref_job: PAR2Proc + PAR2ProcCPU with GF16_AUTO, and
    HasherInput per file concurrently).  x: uint8 [n, S] rows, row i holding
    lens[i] bytes.  Returns (recovery [r, S], valid [r], ifsc bytes, file MD5
    bytes, (wall, gf, hash) seconds)."""
    L = ref()
    x = np.ascontiguousarray(x, dtype=np.uint8)
    n, S = x.shape
    lens = np.ascontiguousarray(lens, dtype=np.uint64)
    nums = np.ascontiguousarray(input_nums, dtype=np.uint16)
    e = np.ascontiguousarray(exps, dtype=np.uint16)
    nf = 0 if file_lens is None else len(file_lens)
    fl = np.ascontiguousarray(file_lens if nf else [0], dtype=np.uint64)
    fr = np.ascontiguousarray(first_rows if nf else [0], dtype=np.uint32)
    out = np.zeros((len(e), S), dtype=np.uint8)
    valid = np.zeros(len(e), dtype=np.int32)
    ifsc = np.zeros(max(n, 1) * 20, dtype=np.uint8)
    fmd5 = np.zeros(max(nf, 1) * 16, dtype=np.uint8)
    t = (ctypes.c_double * 3)()
    rc = L.ref_job(_p(x), S, _p(lens), _p(nums), n, S, _p(e), len(e), _p(out), _p(valid), _p(fl), _p(fr), nf,
                   _p(ifsc), _p(fmd5), threads, t)
    if rc:
        raise RuntimeError("reference job failed: %d" % rc)
    return out, valid, ifsc[: n * 20].tobytes(), fmd5[: nf * 16].tobytes(), (t[0], t[1], t[2])


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


# ---------------------------------------------------------------- helpers
def recover(inputs: np.ndarray, lens, input_nums, exps, threads: int = 1) -> np.ndarray:
    """inputs: uint8 [n, slice]; returns uint8 [r, slice] recovery slices."""
    inputs = np.ascontiguousarray(inputs, dtype=np.uint8)
    n, S = inputs.shape
    lens = np.ascontiguousarray(lens, dtype=np.uint64)
    nums = np.ascontiguousarray(input_nums, dtype=np.uint16)
    exps = np.ascontiguousarray(exps, dtype=np.uint16)
    out = np.zeros((len(exps), S), dtype=np.uint8)
    rc = lib().or_recover(_p(inputs), _p(lens), _p(nums), n, S, _p(exps), len(exps), _p(out), threads)
    if rc:
        raise RuntimeError("oracle recover failed: %d" % rc)
    return out


def recover_coeffs(inputs: np.ndarray, lens, coeffs_rn: np.ndarray, threads: int = 1) -> np.ndarray:
    inputs = np.ascontiguousarray(inputs, dtype=np.uint8)
    n, S = inputs.shape
    lens = np.ascontiguousarray(lens, dtype=np.uint64)
    c = np.ascontiguousarray(coeffs_rn, dtype=np.uint16)
    r = c.shape[0]
    out = np.zeros((r, S), dtype=np.uint8)
    rc = lib().or_recover_coeffs(_p(inputs), _p(lens), _p(c), n, S, r, _p(out), threads)
    if rc:
        raise RuntimeError("oracle recover failed: %d" % rc)
    return out


def recover_fast(inputs: np.ndarray, coeffs_rn: np.ndarray, threads: int = 1) -> np.ndarray:
    """Baseline-speed CPU recovery of zero-padded rows (see or_recover_fast)."""
    inputs = np.ascontiguousarray(inputs, dtype=np.uint8)
    n, S = inputs.shape
    c = np.ascontiguousarray(coeffs_rn, dtype=np.uint16)
    out = np.zeros((c.shape[0], S), dtype=np.uint8)
    rc = lib().or_recover_fast(_p(inputs), n, S, _p(c), c.shape[0], _p(out), threads)
    if rc:
        raise RuntimeError("oracle recover_fast failed: %d" % rc)
    return out


def recover_clmul(inputs: np.ndarray, coeffs_rn: np.ndarray, threads: int = 1):
    """The carry-less multiply restatement (aarch64: SVE2 where the CPU has it,
    else NEON); None where unavailable."""
    inputs = np.ascontiguousarray(inputs, dtype=np.uint8)
    n, S = inputs.shape
    c = np.ascontiguousarray(coeffs_rn, dtype=np.uint16)
    out = np.zeros((c.shape[0], S), dtype=np.uint8)
    rc = lib().or_recover_clmul(_p(inputs), n, S, _p(c), c.shape[0], _p(out), threads)
    if rc == -3:
        return None
    if rc:
        raise RuntimeError("oracle recover_clmul failed: %d" % rc)
    return out


def synth_rows(seed: int, first: int, count: int, nbytes: int, threads: int = 0) -> np.ndarray:
    """uint8[count, nbytes]: the bytes of parpar_gb300.synth.slices(seed, first, count, nbytes),
    generated in C over `threads` threads (all host cores by default)."""
    out = np.empty((count, nbytes), dtype=np.uint8)
    lib().or_synth_fill(_p(out), nbytes, count, nbytes, seed, first, threads or (os.cpu_count() or 1))
    return out


def par2_coeff_matrix(input_nums, exps) -> np.ndarray:
    """[R][N] uint16 PAR2 coefficients 2^(log_i * e) from the oracle's tables."""
    L = lib()
    logs = np.array([L.or_input_log(int(i)) for i in input_nums], dtype=np.int64)
    expt = np.array([L.or_exp(k) for k in range(65535)], dtype=np.uint16)
    e = np.asarray(exps, dtype=np.int64)
    return expt[(e[:, None] * logs[None, :]) % 65535]


def coeff(i: int, e: int) -> int:
    return lib().or_coeff(i, e)


def cksum(data: bytes | np.ndarray, slice_len: int | None = None) -> int:
    a = np.frombuffer(bytes(data), dtype=np.uint8) if not isinstance(data, np.ndarray) else np.ascontiguousarray(data, dtype=np.uint8)
    if slice_len is None:
        slice_len = a.size
    return lib().or_cksum(_p(a), a.size, slice_len)


def md5(data, zero_pad: int = 0) -> bytes:
    a = np.frombuffer(bytes(data), dtype=np.uint8) if not isinstance(data, np.ndarray) else np.ascontiguousarray(data, dtype=np.uint8)
    out = np.zeros(16, dtype=np.uint8)
    lib().or_md5(_p(a), a.size, zero_pad, _p(out))
    return out.tobytes()


def crc32(data, zero_pad: int = 0) -> int:
    a = np.frombuffer(bytes(data), dtype=np.uint8) if not isinstance(data, np.ndarray) else np.ascontiguousarray(data, dtype=np.uint8)
    return lib().or_crc32(_p(a), a.size, zero_pad)


def hash_file(data: np.ndarray, slice_size: int):
    a = np.ascontiguousarray(data, dtype=np.uint8)
    ns = (a.size + slice_size - 1) // slice_size
    ifsc = np.zeros(max(ns, 1) * 20, dtype=np.uint8)
    fmd5 = np.zeros(16, dtype=np.uint8)
    lib().or_hash_file(_p(a), a.size, slice_size, _p(ifsc), _p(fmd5))
    return ifsc[: ns * 20].tobytes(), fmd5.tobytes()


def hash_rows(rows: np.ndarray, lens=None, threads: int = 1):
    """MD5 + CRC32 of each row of a uint8 [n, S] array (row i zero-padded from lens[i])."""
    rows = np.ascontiguousarray(rows, dtype=np.uint8)
    n, S = rows.shape
    md5s = np.zeros((n, 16), dtype=np.uint8)
    crcs = np.zeros(n, dtype=np.uint32)
    lp = None
    if lens is not None:
        lens = np.ascontiguousarray(lens, dtype=np.uint64)
        lp = _p(lens)
    lib().or_hash_rows(_p(rows), S, S, lp, n, _p(md5s), _p(crcs), threads)
    return md5s, crcs
