"""Autotuner: the multiply method and the comb kernel's CTA shape.

Method: for each bucket of recovery counts the tuner times every
multiply-accumulate method of the library (comb XOR-combination tables, the
LOP3 bit-plane form, split-nibble tables, the tcgen05 e4m3 and block-scaled
4-bit tensor-core forms) on a small resident problem through par2cuda_muladd,
and keeps the fastest (best_method).

Shape: the comb kernel's cost per word mul-add depends on how many recovery
rows one CTA serves (the 256-row XOR table is built once per 8 inputs and
shared by those rows, while accumulator registers bound the rows per CTA).
For each bucket the tuner times the candidate shapes with the real kernel
and keeps the fastest (best_shape).

Results are cached per device for the process.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib

# batched shape id -> recovery rows per CTA: 1..4 one-phase tables (8 rows
# per warp x 1, 4, 8, 12 warps), 5..7 paired tables with table-building warps
SHAPES = {1: 8, 2: 32, 3: 64, 4: 96, 5: 72, 6: 64, 7: 32}
# the single-job kernel with the same CTA configuration (timed in its place)
SINGLE = {1: 1, 2: 2, 3: 3, 4: 4, 5: 16, 6: 18, 7: 23}
BUCKETS = [8, 16, 32, 64, 96, 128, 192, 100000]

_cache: dict = {}


def _bucket(R: int) -> int:
    for b in BUCKETS:
        if R <= b:
            return b
    return BUCKETS[-1]


def _time_shape(shape: int, R: int, n: int = 256, slice_bytes: int = 262144, reps: int = 3) -> float:
    L = _lib.load()
    pitch = L.par2cuda_row_pitch_bytes(slice_bytes)
    pw = pitch // 2
    d_in = torch.empty((n, pw), dtype=torch.int16, device="cuda")
    _lib.check(L.par2cuda_synth_fill(d_in.data_ptr(), pitch, n, slice_bytes, 99, 0, None), "synth")
    coeff = torch.from_numpy(np.random.default_rng(R).integers(0, 65536, size=(R, n), dtype=np.uint16).view(np.int16)).cuda()
    d_rec = torch.empty((R, pw), dtype=torch.int16, device="cuda")
    sb = L.par2cuda_muladd_scratch_bytes(R, n)
    scratch = torch.empty(max(sb, 256), dtype=torch.uint8, device="cuda")
    nw = ((slice_bytes + 7) // 8 * 8 + 8) // 2
    prev = L.par2cuda_set_comb_shape(SINGLE[shape])
    try:
        def once():
            _lib.check(L.par2cuda_muladd(d_in.data_ptr(), pw, n, coeff.data_ptr(), d_rec.data_ptr(), pw, R, nw, 0,
                                         _lib.METHOD_COMB, scratch.data_ptr(), sb, None), "muladd")
        once()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            once()
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best
    finally:
        L.par2cuda_set_comb_shape(prev)


METHODS = {"comb": _lib.METHOD_COMB, "xor": _lib.METHOD_XOR, "nibble": _lib.METHOD_NIBBLE,
           "tensor": _lib.METHOD_TENSOR, "tensor_fp4": _lib.METHOD_TENSOR_FP4}
# word-chunk scratch of the 4-bit tensor method per job (it needs the
# coefficient bit matrix plus at least one 128-word tile of input planes;
# more scratch only means fewer, larger chunks)
FP4_CHUNK_BYTES = 256 << 20


def scratch_bytes(method: str, R: int, N: int, n_words: int) -> int:
    """Scratch par2cuda_muladd needs for `method` on an R x N job."""
    L = _lib.load()
    if method == "tensor_fp4":
        full = L.par2cuda_tensor_fp4_scratch_bytes(R, N, n_words)
        # one 128-word tile of expanded input planes (8 bytes per input, 16-input steps)
        one_tile = ((N + 15) // 16 * 16 * 8 * 128 + 1023) // 1024 * 1024
        fixed = L.par2cuda_tensor_fp4_scratch_bytes(R, N, 1) - one_tile   # tile counter + coefficient bit matrix
        return min(full, fixed + (max(FP4_CHUNK_BYTES, one_tile) + 1023) // 1024 * 1024)
    return L.par2cuda_muladd_scratch_bytes(R, N)


def _time_method(method: int, R: int, n: int = 256, slice_bytes: int = 262144, reps: int = 3) -> float:
    L = _lib.load()
    pitch = L.par2cuda_row_pitch_bytes(slice_bytes)
    pw = pitch // 2
    d_in = torch.empty((n, pw), dtype=torch.int16, device="cuda")
    _lib.check(L.par2cuda_synth_fill(d_in.data_ptr(), pitch, n, slice_bytes, 98, 0, None), "synth")
    coeff = torch.from_numpy(np.random.default_rng(R + 1).integers(0, 65536, size=(R, n), dtype=np.uint16).view(np.int16)).cuda()
    d_rec = torch.empty((R, pw), dtype=torch.int16, device="cuda")
    nw = ((slice_bytes + 7) // 8 * 8 + 8) // 2
    name = [k for k, v in METHODS.items() if v == method][0]
    sb = scratch_bytes(name, R, n, nw)
    scratch = torch.empty(max(sb, 256), dtype=torch.uint8, device="cuda")

    def once():
        _lib.check(L.par2cuda_muladd(d_in.data_ptr(), pw, n, coeff.data_ptr(), d_rec.data_ptr(), pw, R, nw, 0,
                                     method, scratch.data_ptr(), sb, None), "muladd")
    once()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        once()
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def best_method(R: int) -> str:
    """Fastest multiply-accumulate method ("comb", "xor", "nibble", "tensor"
    or "tensor_fp4") for R recovery rows on this device."""
    dev = torch.cuda.current_device()
    key = (dev, "method", _bucket(R))
    if key not in _cache:
        Rb = min(_bucket(R), 384)
        times = {name: _time_method(m, Rb) for name, m in METHODS.items()}
        _cache[key] = min(times, key=times.get)
        _cache[(dev, "method_times", key[2])] = times
    return _cache[key]


def method_table() -> dict:
    """{recovery bucket: (best method, {method: ms})} measured so far."""
    return {k[2]: (v, _cache.get((k[0], "method_times", k[2]))) for k, v in _cache.items()
            if len(k) == 3 and k[1] == "method"}


def best_shape(R: int) -> int:
    """Fastest batched comb shape (1..7) for R recovery rows on this device."""
    dev = torch.cuda.current_device()
    key = (dev, _bucket(R))
    if key not in _cache:
        Rb = min(_bucket(R), 384)
        times = {s: _time_shape(s, Rb) for s in SHAPES}
        _cache[key] = min(times, key=times.get)
        _cache[(dev, "times", key[1])] = times
    return _cache[key]


def warm(methods: bool = True):
    """Measures every bucket up front (a serving loop must not stop to tune)."""
    for b in BUCKETS:
        best_shape(min(b, 384))
        if methods:
            best_method(min(b, 384))


def table() -> dict:
    """{recovery bucket: (best shape, {shape: ms})} measured so far."""
    out = {}
    for k, v in _cache.items():
        if len(k) == 2 and k[1] != "times":
            out[k[1]] = (v, _cache.get((k[0], "times", k[1])))
    return out
