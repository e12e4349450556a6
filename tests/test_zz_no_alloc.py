"""par2cuda_muladd_noalloc against par2cuda_muladd and the oracle, through the C ABI.

The no-alloc entry point serves callers that cannot hand the library a
scratch buffer or let it allocate one (a fixed device-memory budget, or a
submission loop that must not call cudaMalloc because an allocation may
synchronise the device).  It keeps its scratch in a fixed device array inside
the library.  This file is collected last so that a failing run stops only
after every other test has run; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from parpar_gb300 import _lib

pytestmark = pytest.mark.gpu


def _bind(L):
    fn = L.par2cuda_muladd_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_size_t, ctypes.c_uint, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]
    return fn


def _case(torch, L, n, R, S, seed):
    pitch = L.par2cuda_row_pitch_bytes(S)
    pw = pitch // 2
    d_in = torch.zeros((n, pw), dtype=torch.int16, device="cuda")
    _lib.check(L.par2cuda_synth_fill(d_in.data_ptr(), pitch, n, S, seed, 0, None), "synth")
    rng = np.random.default_rng(seed)
    coeff = torch.from_numpy(rng.integers(0, 65536, size=(R, n), dtype=np.uint16).view(np.int16)).cuda()
    nw = ((S + 7) // 8 * 8 + 8) // 2
    return d_in, pw, coeff, nw


def _reference_muladd(torch, L, d_in, pw, n, coeff, R, nw, rec, accumulate):
    """The existing entry point, with caller-provided scratch."""
    sb = L.par2cuda_muladd_scratch_bytes(R, n)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_muladd(d_in.data_ptr(), pw, n, coeff.data_ptr(), rec.data_ptr(), pw, R, nw, accumulate,
                                 _lib.METHOD_COMB, scratch.data_ptr(), sb, None), "muladd")
    torch.cuda.synchronize()


def test_noalloc_matches_existing_entry_point_twice_in_a_row():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    noalloc = _bind(L)
    # two calls in a row with different shapes: the second call must not be
    # affected by what the first left in the shared scratch
    for (n, R, S, seed, acc) in [(37, 150, 10000, 5, 0), (300, 45, 4100, 6, 1)]:
        d_in, pw, coeff, nw = _case(torch, L, n, R, S, seed)
        start = torch.from_numpy(np.random.default_rng(seed + 7).integers(-32768, 32767, size=(R, pw), dtype=np.int16)).cuda()
        want = start.clone()
        got = start.clone()
        _reference_muladd(torch, L, d_in, pw, n, coeff, R, nw, want, acc)
        rc = noalloc(d_in.data_ptr(), pw, n, coeff.data_ptr(), got.data_ptr(), pw, R, nw, acc, None)
        assert rc == 0, L.par2cuda_last_error()
        torch.cuda.synchronize()
        # bit-exact over the words the call covers
        assert torch.equal(got[:, :nw], want[:, :nw])
        # and against the oracle over the slice bytes
        from oracle import oracle as O
        from parpar_gb300 import synth
        prod = O.recover_coeffs(synth.slices(seed, 0, n, S), np.full(n, S), coeff.cpu().numpy().view(np.uint16))
        expect = prod.view(np.int16) ^ (start[:, : S // 2].cpu().numpy() if acc else 0)
        assert np.array_equal(got[:, : S // 2].cpu().numpy(), expect)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    noalloc = _bind(L)
    n, R, S = 4096, 1024, 64  # 1024 * 512 * 16 bytes = 8 MiB > 4 MiB
    # buffers of the full size, so the call would stay in bounds even if it ran
    d_in, pw, coeff, nw = _case(torch, L, n, R, S, 1)
    rec = torch.zeros((R, pw), dtype=torch.int16, device="cuda")
    rc = noalloc(d_in.data_ptr(), pw, n, coeff.data_ptr(), rec.data_ptr(), pw, R, nw, 0, None)
    assert rc < 0
    msg = L.par2cuda_last_error().decode()
    assert "limit" in msg and "scratch" in msg
