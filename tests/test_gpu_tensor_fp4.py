"""The block-scaled 4-bit tcgen05 form of the contraction (par2cuda_muladd with
PAR2CUDA_METHOD_TENSOR_FP4, k_tc4.cu) against the oracle, bit-exact: one tile,
padded recovery and input counts, several word chunks (small scratch), and
accumulate mode."""
import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


def run_fp4(n, R, S, seed, accumulate=False, scratch_bytes=None, shape=0, pitch_pad=0):
    import torch
    L = _lib.load()
    prev = L.par2cuda_set_tc4_shape(shape)
    pitch = L.par2cuda_row_pitch_bytes(S)
    # pitch_pad words more per row: a pitch that is not a multiple of 16 bytes
    # takes the input expansion's 2-byte-load path
    pw = pitch // 2 + pitch_pad
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
    try:
        rc = L.par2cuda_muladd(d_in.data_ptr(), pw, n, d_coeff.data_ptr(), d_rec.data_ptr(), pw, R, nw, int(accumulate),
                               _lib.METHOD_TENSOR_FP4, scratch.data_ptr(), sb, None)
    finally:
        L.par2cuda_set_tc4_shape(prev)
    assert rc == 0, L.par2cuda_last_error()
    torch.cuda.synchronize()
    assert L.par2cuda_device_error() == 0
    got = d_rec.cpu().numpy()[:, :nw]
    want = O.recover_coeffs(x, np.full(n, S), coeff).view(np.int16)
    if accumulate:
        want = want ^ start[:, :nw]
    return got, want


@pytest.mark.parametrize("shape", [1, 2])
@pytest.mark.parametrize("n,R,S", [
    (16, 12, 256),        # one 128-word x 12-slice tile, one K block
    (16, 16, 256),        # one 16-slice tile; two 12-slice tiles, the second padded
    (3, 2, 256),          # padded inputs and recovery slices
    (37, 20, 10000),      # two recovery tiles, ragged words
    (200, 33, 65536),     # several K blocks, three recovery tiles
    (40, 100, 131072),    # 7 or 9 recovery tiles x 512 word tiles: accumulators reused, many tiles per CTA
    (1100, 30, 20000),    # 69 k-blocks (the automatic choice takes the 16-slice tile)
    (37, 20, 4100),       # 2050 words: the last 8-word load segment is partly past the words
])
def test_fp4_matches_oracle(n, R, S, shape):
    got, want = run_fp4(n, R, S, seed=n * 31 + R, shape=shape)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("n,R,S", [(37, 20, 4100), (70, 33, 10002)])
def test_fp4_unaligned_pitch(n, R, S):
    got, want = run_fp4(n, R, S, seed=n + R, pitch_pad=2)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("shape", [1, 2])
def test_fp4_accumulate_and_word_chunks(shape):
    from parpar_gb300 import _lib as lib
    L = lib.load()
    n, R, S = 48, 24, 40000
    kbytes = ((n + 15) // 16 * 16) * 8
    one_tile = (128 * kbytes + 1023) // 1024 * 1024
    # the scratch for one 128-word tile, less that tile: the tile counter and
    # the coefficient bit matrix
    fixed = L.par2cuda_tensor_fp4_scratch_bytes(R, n, 1) - one_tile
    # room for 2 tiles of words only: 40000-byte rows take 79 chunks
    small = fixed + 2 * 128 * kbytes
    got, want = run_fp4(n, R, S, seed=5, accumulate=True, scratch_bytes=small, shape=shape)
    assert np.array_equal(got, want)
    assert L.par2cuda_tensor_fp4_scratch_bytes(R, n, S // 2) >= small
