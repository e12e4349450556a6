"""PAR2ProcCUDA (parpar_gb300/adapter/controller_cuda.{h,cpp}) driven by the
reference's own PAR2Proc (gf16/controller.cpp), compiled together with the
reference core from its staged sources (oracle/_ref/libparref_cuda.so, built by
oracle/ref.mk through oracle/refsrc.py).

The GPU cases run the CUDA backend alone and beside the reference's
PAR2ProcCPU over split byte ranges of every slice (PAR2Proc's static split,
gf16/controller.cpp:13-130, 171-226, 335-399), in one pass and in chunked
passes (lib/par2.js PAR2Chunked), with PAR2 and explicit coefficients; every
recovery slice must equal the oracle's bit for bit and every verdict be valid.
"""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle import refsrc
from parpar_gb300 import synth


def _lib():
    if not refsrc.staged():
        pytest.skip("reference sources are not staged on this host (oracle/_ref/src)")
    if not os.path.exists(refsrc.REF_CUDA_LIB):
        err = os.path.join(refsrc.REF_OUT, "build_error.txt")
        pytest.fail("adapter library missing: %s" % (open(err).read() if os.path.exists(err) else "not built"))
    L = ctypes.CDLL(refsrc.REF_CUDA_LIB)
    vp, sz, u = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint
    L.adapter_create.restype = ctypes.c_int
    L.adapter_create.argtypes = [vp, sz, vp, vp, vp, u, sz, vp, u, vp, vp, sz, sz, ctypes.c_int, u, vp]
    L.adapter_probe.restype = ctypes.c_int
    L.adapter_probe.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_char_p, sz]
    return L


def run_adapter(x, lens, nums, exps, coeffs=None, cpu_bytes=0, chunk=0, method=0, batch=0):
    L = _lib()
    x = np.ascontiguousarray(x, dtype=np.uint8)
    n, S = x.shape
    lens = np.ascontiguousarray(lens, dtype=np.uint64)
    nums = np.ascontiguousarray(nums, dtype=np.uint16)
    R = len(exps) if coeffs is None else coeffs.shape[1]
    e = np.ascontiguousarray(exps if exps is not None else np.zeros(R), dtype=np.uint16)
    c = None if coeffs is None else np.ascontiguousarray(coeffs, dtype=np.uint16)
    out = np.zeros((R, S), dtype=np.uint8)
    valid = np.zeros(R, dtype=np.int32)
    stats = np.zeros(2, dtype=np.uint32)
    p = O._p
    rc = L.adapter_create(p(x), S, p(lens), p(nums), None if c is None else p(c), n, S,
                          None if coeffs is not None else p(e), R, p(out), p(valid), cpu_bytes, chunk, method, batch,
                          p(stats))
    assert rc == 0, "adapter_create failed: %d" % rc
    return out, valid, stats


def ragged(seed, n, S, short=()):
    x = synth.slices(seed, 0, n, S)
    lens = np.full(n, S)
    for i, ln in short:
        lens[i] = ln
        x[i, ln:] = 0
    return x, lens


def test_adapter_builds_against_the_reference_controller():
    """CPU: the adapter compiled against the reference's gf16/controller.h and
    linked with its PAR2Proc; init reports failure (false, as the addon's
    "Failed to allocate memory" path expects) for a device that does not
    exist and for a staging count of 0, with the library's message."""
    L = _lib()
    msg = ctypes.create_string_buffer(256)
    assert L.adapter_probe(4096, 2, msg, 256) == 0
    assert msg.value
    assert L.adapter_probe(0, 0, msg, 256) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("n,S,exps,short", [
    (20, 4100, list(range(6)), [(3, 1001)]),
    (3, 4, [0, 1], []),
    (37, 65536 + 2, [0, 5, 65534, 300], [(0, 2), (36, 12345)]),
    (130, 12224, list(range(13)), [(129, 5000)]),
])
def test_adapter_alone_matches_oracle(n, S, exps, short):
    x, lens = ragged(n * 7 + S, n, S, short)
    nums = np.arange(n)
    out, valid, stats = run_adapter(x, lens, nums, exps, batch=16)
    assert valid.all()
    assert np.array_equal(out, O.recover(x, lens, nums, exps))
    assert stats[1] == 16 and stats[0] >= (n + 15) // 16


@pytest.mark.gpu
@pytest.mark.parametrize("cpu_bytes", [2, 2048, 4096])
def test_adapter_split_with_reference_cpu_backend(cpu_bytes):
    """PAR2Proc splits every slice: bytes [0, cpu_bytes) to PAR2ProcCPU, the
    rest to PAR2ProcCUDA; the output is assembled by PAR2Proc::getOutput."""
    n, S = 25, 4100
    x, lens = ragged(91, n, S, [(2, 3000), (7, 2048), (24, 100)])
    nums = np.arange(100, 100 + n)
    exps = [0, 1, 2, 77, 1000]
    out, valid, _ = run_adapter(x, lens, nums, exps, cpu_bytes=cpu_bytes, batch=8)
    assert valid.all()
    assert np.array_equal(out, O.recover(x, lens, nums, exps))


@pytest.mark.gpu
@pytest.mark.parametrize("cpu_bytes,chunk", [(0, 4096), (1000, 3000), (2600, 3000)])
def test_adapter_chunked_passes(cpu_bytes, chunk):
    """Byte-window passes (setCurrentSliceSize per window, discardOutput after
    each end); with chunk 3000 and 2600 CPU bytes the last window (1100 bytes)
    gives the CUDA backend 0 bytes, which PAR2Proc skips."""
    n, S = 18, 7100
    x, lens = ragged(5, n, S, [(4, 2500), (17, 6000)])
    nums = np.arange(n)
    exps = list(range(1, 8))
    out, valid, _ = run_adapter(x, lens, nums, exps, cpu_bytes=cpu_bytes, chunk=chunk, batch=4)
    assert valid.all()
    assert np.array_equal(out, O.recover(x, lens, nums, exps))


@pytest.mark.gpu
def test_adapter_explicit_coefficients():
    n, S, R = 11, 3000, 4
    x, lens = ragged(17, n, S, [(5, 1234)])
    rng = np.random.default_rng(4)
    coeffs = rng.integers(0, 65536, size=(n, R), dtype=np.uint16)   # [input][rec]
    out, valid, _ = run_adapter(x, lens, np.zeros(n), None, coeffs=coeffs, cpu_bytes=1000, batch=4)
    assert valid.all()
    assert np.array_equal(out, O.recover_coeffs(x, lens, coeffs.T.copy()))
