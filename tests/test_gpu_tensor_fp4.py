"""The block-scaled 4-bit tcgen05 form of the contraction (par2cuda_muladd with
PAR2CUDA_METHOD_TENSOR_FP4, k_tc4.cu) against the oracle, bit-exact: one tile,
padded recovery and input counts, several word chunks (small scratch), and
accumulate mode."""
import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


def run_fp4(n, R, S, seed, accumulate=False, scratch_bytes=None):
    import torch
    L = _lib.load()
    pitch = L.par2cuda_row_pitch_bytes(S)
    pw = pitch // 2
    x = synth.slices(seed, 0, n, S)
    d_in = torch.zeros((n, pw), dtype=torch.int16, device="cuda")
    d_in.view(torch.uint8)[:, :S].copy_(torch.from_numpy(x))
    rng = np.random.default_rng(seed)
    coeff = rng.integers(0, 65536, size=(R, n), dtype=np.uint16)
    d_coeff = torch.from_numpy(coeff.view(np.int16)).cuda()
    start = rng.integers(-32768, 32767, size=(R, pw), dtype=np.int16)
    d_rec = torch.from_numpy(start.copy()).cuda()
    nw = S // 2
    sb = scratch_bytes or L.par2cuda_tensor_fp4_scratch_bytes(R, n, nw)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    rc = L.par2cuda_muladd(d_in.data_ptr(), pw, n, d_coeff.data_ptr(), d_rec.data_ptr(), pw, R, nw, int(accumulate),
                           _lib.METHOD_TENSOR_FP4, scratch.data_ptr(), sb, None)
    assert rc == 0, L.par2cuda_last_error()
    torch.cuda.synchronize()
    assert L.par2cuda_device_error() == 0
    got = d_rec.cpu().numpy()[:, :nw]
    want = O.recover_coeffs(x, np.full(n, S), coeff).view(np.int16)
    if accumulate:
        want = want ^ start[:, :nw]
    return got, want


@pytest.mark.parametrize("n,R,S", [
    (16, 16, 256),        # one 128-word x 16-slice tile, one K block
    (3, 2, 256),          # padded inputs and recovery slices
    (37, 20, 10000),      # two recovery tiles, ragged words
    (200, 33, 65536),     # several K blocks, three recovery tiles
])
def test_fp4_matches_oracle(n, R, S):
    got, want = run_fp4(n, R, S, seed=n * 31 + R)
    assert np.array_equal(got, want)


def test_fp4_accumulate_and_word_chunks():
    from parpar_gb300 import _lib as lib
    L = lib.load()
    n, R, S = 48, 24, 40000
    kbytes = ((n + 15) // 16 * 16) * 8
    bbytes = ((R + 15) // 16 * 16) * 16 * kbytes
    # room for 2 tiles of words only: 40000-byte rows take 79 chunks
    small = (bbytes + 1023) // 1024 * 1024 + 2 * 128 * kbytes
    got, want = run_fp4(n, R, S, seed=5, accumulate=True, scratch_bytes=small)
    assert np.array_equal(got, want)
    assert L.par2cuda_tensor_fp4_scratch_bytes(R, n, S // 2) >= small
