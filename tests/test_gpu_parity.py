"""CUDA path vs the oracle, bit-exact, through the C ABI (libpar2cuda.so).

Small cases compare whole recovery slices against the oracle and the golden
vectors recorded from the reference; the large cases use size-independent
properties (every carried checksum verifies; sampled words equal the
oracle's sum over all inputs at that word position).
"""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import _lib, synth
from parpar_gb300.gfproc import GfProc, GfProcError, create_recovery

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
METHODS = ["comb", "xor", "nibble", "tensor", "tensor_fp4"]


def golden_inputs(c):
    x = synth.slices(c["seed"], 0, c["n"], c["slice"])
    for i, l in enumerate(c["lens"]):
        x[i, l:] = 0
    return x, np.array(c["lens"])


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("case", GOLDEN["recovery"], ids=lambda c: c["name"])
def test_golden_recovery(case, method):
    x, lens = golden_inputs(case)
    out, valid = create_recovery(x, lens, case["nums"], case["exps"], method=method, input_batchsize=8)
    assert valid.all()
    assert [hashlib.md5(out[j].tobytes()).hexdigest() for j in range(len(case["exps"]))] == case["md5"]


def test_golden_custom_coefficients():
    c = GOLDEN["recovery_coeffs"]
    x, lens = golden_inputs(c)
    coeffs = np.array(c["coeffs_in_rec"], dtype=np.uint16)  # [input][rec]
    g = GfProc(c["slice"], input_batchsize=4)
    g.set_recovery_slices([1] * coeffs.shape[1])
    evs = [g.add_sync(0, x[i, : lens[i]], coeffs=coeffs[i]) for i in range(c["n"])]
    g.end_sync()
    [e.wait() for e in evs]
    out = np.zeros((coeffs.shape[1], c["slice"]), np.uint8)
    for r in range(coeffs.shape[1]):
        assert g.get_sync(r, out[r])
    assert [hashlib.md5(out[j].tobytes()).hexdigest() for j in range(coeffs.shape[1])] == c["md5"]
    g.close()


def test_mixed_par2_and_custom_in_one_batch():
    rng = np.random.default_rng(3)
    n, S, R = 9, 2000, 4
    x = synth.slices(44, 0, n, S)
    exps = [0, 3, 7, 100]
    coeffs = np.array([[O.coeff(i, e) for e in exps] for i in range(n)], dtype=np.uint16)
    coeffs[2] = rng.integers(0, 65536, size=R)
    g = GfProc(S, input_batchsize=16)
    g.set_recovery_slices(exps)
    evs = []
    for i in range(n):
        evs.append(g.add_sync(i, x[i], coeffs=coeffs[i] if i in (2, 5) else None))
    g.end_sync()
    [e.wait() for e in evs]
    ref = O.recover_coeffs(x, np.full(n, S), coeffs.T)
    for r in range(R):
        out = np.zeros(S, np.uint8)
        assert g.get_sync(r, out)
        assert np.array_equal(out, ref[r])
    g.close()


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("batch,areas", [(8, 1), (8, 2), (16, 3), (3, 2), (64, 2)])
def test_batching_and_staging(method, batch, areas):
    rng = np.random.default_rng(batch * 10 + areas)
    n, S = 37, 3002
    x = synth.slices(batch + 100 * areas, 0, n, S)
    lens = rng.integers(0, S + 1, size=n)
    lens[lens % 2 == 1] -= 1  # any length is allowed; keep some even, some odd below
    lens[5] = 1
    lens[6] = 0
    for i in range(n):
        x[i, lens[i]:] = 0
    nums = rng.choice(32768, size=n, replace=False)
    exps = [0, 1, 2, 65534, 12345]
    out, valid = create_recovery(x, lens, nums, exps, method=method, input_batchsize=batch, staging_areas=areas)
    assert valid.all()
    assert np.array_equal(out, O.recover(x, lens, nums, exps))


@pytest.mark.parametrize("S", [2, 4, 6, 8, 10, 126, 128, 130, 65521 * 4 + 2])
def test_slice_size_edges(S):
    n, R = 11, 7
    x = synth.slices(S, 0, n, S)
    out, valid = create_recovery(x, np.full(n, S), np.arange(n), list(range(R)), input_batchsize=8)
    assert valid.all()
    assert np.array_equal(out, O.recover(x, np.full(n, S), np.arange(n), list(range(R))))


def test_more_recovery_than_inputs_and_many_rows():
    n, S, R = 3, 64, 300
    x = synth.slices(5, 0, n, S)
    exps = list(range(R))
    out, valid = create_recovery(x, np.full(n, S), np.arange(n), exps)
    assert valid.all()
    assert np.array_equal(out, O.recover(x, np.full(n, S), np.arange(n), exps))


def test_chunked_passes_and_zero_output_without_input():
    # PAR2Chunked: the same GfProc processes byte windows of each slice
    # (lib/par2.js:847-867), smaller than the declared slice size.
    n, S, R, chunk = 10, 10000, 5, 4000
    x = synth.slices(77, 0, n, S)
    ref = O.recover(x, np.full(n, S), np.arange(n), list(range(R)))
    g = GfProc(S, input_batchsize=4)
    g.set_recovery_slices(list(range(R)))
    got = np.zeros((R, S), np.uint8)
    for off in range(0, S, chunk):
        size = min(chunk, S - off)
        g.set_current_slice_size(size)
        evs = [g.add_sync(i, np.ascontiguousarray(x[i, off:off + size])) for i in range(n)]
        g.end_sync()
        [e.wait() for e in evs]
        for r in range(R):
            buf = np.zeros(size, np.uint8)
            assert g.get_sync(r, buf)
            got[r, off:off + size] = buf
    assert np.array_equal(got, ref)
    # end without adding anything -> the controller reports zeros
    g.end_sync()
    buf = np.full(size, 0xAB, np.uint8)
    assert g.get_sync(0, buf) and not buf.any()
    g.close()


def test_addon_error_behaviour():
    with pytest.raises(GfProcError, match="Slice size is invalid"):
        GfProc(3)
    g = GfProc(100)
    with pytest.raises(GfProcError, match="setRecoverySlices not yet called"):
        g.add(0, np.zeros(100, np.uint8))
    with pytest.raises(GfProcError, match="Invalid recovery index"):
        g.set_recovery_slices([65535])
    g.set_recovery_slices([1])
    with pytest.raises(GfProcError, match="Input index not valid"):
        g.add(32768, np.zeros(100, np.uint8))
    with pytest.raises(GfProcError, match="Input buffer too large"):
        g.add(0, np.zeros(102, np.uint8))
    with pytest.raises(GfProcError, match="No finalized output"):
        g.get(0, np.zeros(100, np.uint8))
    info = g.info()
    assert info["num_output_slices"] == 1 and info["device_name"]
    g.close()
    with pytest.raises(GfProcError, match="Already closed"):
        g.close()


# ------------------------------------------------------------ device level
def _dev_rows(torch, n, S, seed, first=0):
    L = _lib.load()
    pitch = L.par2cuda_row_pitch_bytes(S)
    t = torch.zeros((n, pitch // 2), dtype=torch.int16, device="cuda")
    _lib.check(L.par2cuda_synth_fill(t.data_ptr(), pitch, n, S, seed, first, None), "synth")
    return t, pitch // 2


@pytest.mark.parametrize("method", [0, 1, 2, 3, 4])
def test_device_muladd_accumulate(method):
    torch = pytest.importorskip("torch")
    L = _lib.load()
    n, R, S = 29, 13, 5000
    d_in, pw = _dev_rows(torch, n, S, 9)
    host_in = synth.slices(9, 0, n, S)
    assert np.array_equal(d_in.cpu().numpy().view(np.uint8)[:, :S], host_in)  # generator parity
    rng = np.random.default_rng(method)
    coeff = rng.integers(0, 65536, size=(R, n), dtype=np.uint16)
    d_coeff = torch.from_numpy(coeff.view(np.int16)).cuda()
    d_rec = torch.zeros((R, pw), dtype=torch.int16, device="cuda")
    sb = L.par2cuda_muladd_scratch_bytes(R, n)
    scratch = torch.zeros(sb, dtype=torch.uint8, device="cuda")
    nw = S // 2
    half = 16
    # two launches: overwrite with the first 16 inputs, then accumulate the rest
    c1 = d_coeff[:, :half].contiguous()
    _lib.check(L.par2cuda_muladd(d_in.data_ptr(), pw, half, c1.data_ptr(), d_rec.data_ptr(), pw, R,
                                 nw, 0, method, scratch.data_ptr(), sb, None), "muladd")
    c2 = d_coeff[:, half:].contiguous()
    _lib.check(L.par2cuda_muladd(d_in[half:].data_ptr(), pw, n - half, c2.data_ptr(), d_rec.data_ptr(), pw, R,
                                 nw, 1, method, scratch.data_ptr(), sb, None), "muladd")
    torch.cuda.synchronize()
    assert L.par2cuda_device_error() == 0
    got = d_rec.cpu().numpy().view(np.uint8)[:, :S]
    assert np.array_equal(got, O.recover_coeffs(host_in, np.full(n, S), coeff))


@pytest.mark.parametrize("n,R,S", [(1, 1, 2), (8, 16, 512), (100, 40, 3000), (257, 17, 4100)])
def test_tensor_core_variant(n, R, S):
    """The tcgen05 variant: pipeline wrap (more stages than the 3-stage ring),
    partial recovery blocks and word tiles, one input, many inputs."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    d_in, pw = _dev_rows(torch, n, S, 77 + n)
    host_in = synth.slices(77 + n, 0, n, S)
    coeff = np.random.default_rng(n).integers(0, 65536, size=(R, n), dtype=np.uint16)
    d_coeff = torch.from_numpy(coeff.view(np.int16)).cuda()
    d_rec = torch.zeros((R, pw), dtype=torch.int16, device="cuda")
    sb = L.par2cuda_muladd_scratch_bytes(R, n)
    scratch = torch.zeros(sb, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_muladd(d_in.data_ptr(), pw, n, d_coeff.data_ptr(), d_rec.data_ptr(), pw, R, S // 2, 0,
                                 _lib.METHOD_TENSOR, scratch.data_ptr(), sb, None), "muladd")
    torch.cuda.synchronize()
    assert L.par2cuda_device_error() == 0
    got = d_rec.cpu().numpy().view(np.uint8)[:, :S]
    assert np.array_equal(got, O.recover_coeffs(host_in, np.full(n, S), coeff))


def test_device_checksum_detects_corruption():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    n, S = 6, 3000
    rows, pw = _dev_rows(torch, n, S, 31)
    lens = torch.tensor([3000, 2999, 1, 0, 1500, 2998], dtype=torch.int32, device="cuda")
    ck = torch.zeros(n * 8, dtype=torch.uint8, device="cuda")
    flags = torch.zeros(n, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_rows_checksum(rows.data_ptr(), pw, n, lens.data_ptr(), S, 0, None, ck.data_ptr(), None), "ck")
    torch.cuda.synchronize()
    host = synth.slices(31, 0, n, S)
    got = rows.cpu().numpy().view(np.uint8)
    for i, l in enumerate(lens.tolist()):
        assert not got[i, l:S].any()  # zero padded
        assert int.from_bytes(got[i, (S + 7) // 8 * 8:][:8].tobytes(), "little") == O.cksum(host[i, :l], S)
    _lib.check(L.par2cuda_rows_checksum(rows.data_ptr(), pw, n, None, S, 1, flags.data_ptr(), ck.data_ptr(), None), "verify")
    torch.cuda.synchronize()
    assert flags.tolist() == [1] * n
    # flip one bit of row 4's data: its verdict turns false, the others stay true
    rows[4, 100] ^= 4
    _lib.check(L.par2cuda_rows_checksum(rows.data_ptr(), pw, n, None, S, 1, flags.data_ptr(), ck.data_ptr(), None), "verify")
    torch.cuda.synchronize()
    assert flags.tolist() == [1, 1, 1, 1, 0, 1]


# ------------------------------------------------------------ full-size properties
def _sampled_check(torch, d_in, pw, n, d_rec, R, S, exps, samples=48, seed=0):
    """rec[r][w] == sum_i c(i, e_r) * in[i][w] at sampled (r, w)."""
    rng = np.random.default_rng(seed)
    rs = rng.integers(0, R, size=samples)
    ws = rng.integers(0, S // 2, size=samples)
    col = d_in[:, torch.from_numpy(ws).cuda()].cpu().numpy().view(np.uint16)  # [n, samples]
    got = d_rec[torch.from_numpy(rs).cuda(), torch.from_numpy(ws).cuda()].cpu().numpy().view(np.uint16)
    Lo = O.lib()
    for k in range(samples):
        acc = 0
        for i in range(n):
            acc ^= Lo.or_mul(O.coeff(i, exps[rs[k]]), int(col[i, k]))
        assert acc == got[k], (rs[k], ws[k])


@pytest.mark.parametrize("n,R,S", [(4096, 4096, 262144 // 16), (2000, 200, 2 * 1048576 // 16)])
def test_large_shapes_sampled(n, R, S):
    """The dense (4096 x 4096) and bandwidth (2000 x 200) workloads' counts
    (inputs x recovery) at reduced slice size:
    every checksum verifies and sampled words match the oracle."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    d_in, pw = _dev_rows(torch, n, S, 1234)
    exps = list(range(R))
    coeff = np.array([[O.coeff(i, e) for i in range(n)] for e in exps], dtype=np.uint16) if R * n <= 1 << 20 else None
    if coeff is None:
        # vectorised coefficients: 2^((log_i * e) mod 65535)
        logs = np.array([O.lib().or_input_log(i) for i in range(n)], dtype=np.int64)
        expt = np.array([O.lib().or_exp(v) for v in range(65535)], dtype=np.uint16)
        coeff = expt[(np.array(exps, dtype=np.int64)[:, None] * logs[None, :]) % 65535]
    d_coeff = torch.from_numpy(coeff.view(np.int16)).cuda()
    d_rec = torch.zeros((R, pw), dtype=torch.int16, device="cuda")
    ck = torch.zeros(max(n, R) * 8, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_rows_checksum(d_in.data_ptr(), pw, n, None, S, 0, None, ck.data_ptr(), None), "ck")
    sb = L.par2cuda_muladd_scratch_bytes(R, n)
    scratch = torch.zeros(sb, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_muladd(d_in.data_ptr(), pw, n, d_coeff.data_ptr(), d_rec.data_ptr(), pw, R,
                                 ((S + 7) // 8 * 8 + 8) // 2, 0, 1, scratch.data_ptr(), sb, None), "muladd")
    flags = torch.zeros(R, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_rows_checksum(d_rec.data_ptr(), pw, R, None, S, 1, flags.data_ptr(), ck.data_ptr(), None), "verify")
    torch.cuda.synchronize()
    assert int(flags.sum()) == R
    _sampled_check(torch, d_in, pw, n, d_rec, R, S, exps)


@pytest.mark.parametrize("shape", list(range(0, 29)))
def test_comb_every_cta_shape(shape):
    """Every comb CTA shape (rows per warp x warps) gives the oracle's result,
    including partial recovery blocks and a ragged input group."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    prev = L.par2cuda_set_comb_shape(shape)
    try:
        n, R, S = 43, 101, 3000
        d_in, pw = _dev_rows(torch, n, S, 21 + shape)
        host_in = synth.slices(21 + shape, 0, n, S)
        rng = np.random.default_rng(shape)
        coeff = rng.integers(0, 65536, size=(R, n), dtype=np.uint16)
        d_coeff = torch.from_numpy(coeff.view(np.int16)).cuda()
        d_rec = torch.zeros((R, pw), dtype=torch.int16, device="cuda")
        sb = L.par2cuda_muladd_scratch_bytes(R, n)
        scratch = torch.zeros(sb, dtype=torch.uint8, device="cuda")
        _lib.check(L.par2cuda_muladd(d_in.data_ptr(), pw, n, d_coeff.data_ptr(), d_rec.data_ptr(), pw, R, S // 2, 0,
                                     1, scratch.data_ptr(), sb, None), "muladd")
        torch.cuda.synchronize()
        got = d_rec.cpu().numpy().view(np.uint8)[:, :S]
        assert L.par2cuda_device_error() == 0
        assert np.array_equal(got, O.recover_coeffs(host_in, np.full(n, S), coeff))
    finally:
        L.par2cuda_set_comb_shape(prev)


def test_lop3_rate_calibration():
    """The integer-ALU roofline denominator: a positive, plausible LOP3 rate
    (between 32 and 256 lanes per SM per clock at 1-2.2 GHz)."""
    torch = pytest.importorskip("torch")
    import ctypes
    L = _lib.load()
    v = ctypes.c_double(0)
    _lib.check(L.par2cuda_lop3_rate(ctypes.byref(v), None), "lop3_rate")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    per_sm_clk = v.value / sms / 2.0e9
    assert 16 < per_sm_clk < 300, v.value


def test_muladd_index_matches_oracle():
    """par2cuda_muladd_index (grid launch from resident index bytes) over
    chunks of one job: accumulate mode and the device-computed PAR2 index."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    n, R, S = 45, 77, 5000
    d_in, pw = _dev_rows(torch, n, S, 4242)
    host_in = synth.slices(4242, 0, n, S)
    exps = list(range(3, 3 + R))
    d_nums = torch.arange(n, dtype=torch.int16, device="cuda")
    d_exps = torch.tensor(np.asarray(exps, dtype=np.uint16).view(np.int16), device="cuda")
    d_idx = torch.zeros(L.par2cuda_coeff_index_bytes(R, n), dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_par2_index(d_nums.data_ptr(), n, d_exps.data_ptr(), R, d_idx.data_ptr(), None), "index")
    want = O.recover(host_in, np.full(n, S), np.arange(n), exps)
    d_rec = torch.zeros((R, pw), dtype=torch.int16, device="cuda")
    nw = S // 2
    # two halves of the inputs, the second accumulating
    h = 24
    idx_a = torch.zeros(L.par2cuda_coeff_index_bytes(R, h), dtype=torch.uint8, device="cuda")
    idx_b = torch.zeros(L.par2cuda_coeff_index_bytes(R, n - h), dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_par2_index(d_nums[:h].data_ptr(), h, d_exps.data_ptr(), R, idx_a.data_ptr(), None), "ia")
    _lib.check(L.par2cuda_par2_index(d_nums[h:].data_ptr(), n - h, d_exps.data_ptr(), R, idx_b.data_ptr(), None), "ib")
    _lib.check(L.par2cuda_muladd_index(d_in.data_ptr(), pw, h, idx_a.data_ptr(), d_rec.data_ptr(), pw, R, nw, 0, None), "a")
    _lib.check(L.par2cuda_muladd_index(d_in[h:].data_ptr(), pw, n - h, idx_b.data_ptr(), d_rec.data_ptr(), pw, R, nw, 1,
                                       None), "b")
    torch.cuda.synchronize()
    assert np.array_equal(d_rec.cpu().numpy().view(np.uint8)[:, :S], want)
    # whole job in one call
    d_rec.zero_()
    _lib.check(L.par2cuda_muladd_index(d_in.data_ptr(), pw, n, d_idx.data_ptr(), d_rec.data_ptr(), pw, R, nw, 0, None), "w")
    torch.cuda.synchronize()
    assert np.array_equal(d_rec.cpu().numpy().view(np.uint8)[:, :S], want)
    assert L.par2cuda_device_error() == 0
    # pitch below roundup(n_words, 64) is rejected
    assert L.par2cuda_muladd_index(d_in.data_ptr(), 32, n, d_idx.data_ptr(), d_rec.data_ptr(), pw, R, nw, 0, None) < 0


def test_md5_chain_rate_calibration():
    """The hash kernels' latency bound: one MD5 chain on one thread runs at
    tens to hundreds of MB/s."""
    pytest.importorskip("torch")
    import ctypes
    L = _lib.load()
    v = ctypes.c_double(0)
    _lib.check(L.par2cuda_md5_chain_rate(ctypes.byref(v), None), "md5_chain_rate")
    assert 20e6 < v.value < 2e9, v.value


def test_output_valid_matches_get_output_verdicts():
    """par2cuda_output_valid (synchronous verdict) agrees with the get_output
    callbacks, after outputs fetched without callbacks, and against the oracle."""
    n, S, R = 23, 3000, 7
    x = synth.slices(77, 0, n, S)
    g = GfProc(S, input_batchsize=8)
    g.set_recovery_slices(list(range(R)))
    L = _lib.load()
    assert L.par2cuda_output_valid(g._ctx, R) < 0          # index out of range
    for i in range(n):
        g.add_sync(i, x[i]).wait()
    g.end_sync()
    out = np.zeros((R, S), np.uint8)
    null_cb = _lib.DONE_FN()
    for r in range(R):
        _lib.check(L.par2cuda_get_output(g._ctx, r, out[r].ctypes.data_as(ctypes.c_void_p), null_cb, None), "get")
    _lib.check(L.par2cuda_sync(g._ctx), "sync")
    assert [L.par2cuda_output_valid(g._ctx, r) for r in range(R)] == [1] * R
    assert np.array_equal(out, O.recover(x, np.full(n, S), np.arange(n), list(range(R))))
    other = np.zeros(S, np.uint8)
    assert g.get_sync(3, other) and np.array_equal(other, out[3])
    g.close()


def test_max_recovery_count():
    """32768 recovery slices (par-compare's large-recovery shape), exponents
    spread up to 65534, a few small inputs."""
    n, S = 3, 32
    rng = np.random.default_rng(32768)
    exps = sorted(rng.choice(65535, size=32768, replace=False).tolist())
    x = synth.slices(9, 0, n, S)
    out, valid = create_recovery(x, np.full(n, S), np.arange(n), exps)
    assert valid.all()
    assert np.array_equal(out, O.recover(x, np.full(n, S), np.arange(n), exps))


def test_max_input_count():
    """32768 inputs (input numbers 0..32767, the PAR2 maximum), short slices."""
    n, S, R = 32768, 8, 3
    x = synth.slices(11, 0, n, S)
    exps = [0, 1, 65534]
    out, valid = create_recovery(x, np.full(n, S), np.arange(n), exps, input_batchsize=4096)
    assert valid.all()
    assert np.array_equal(out, O.recover(x, np.full(n, S), np.arange(n), exps))


def test_device_par2_coefficient_matrix():
    """par2cuda_par2_coeffs = the oracle's PAR2 coefficients, including the
    largest input number and exponent."""
    import torch
    L = _lib.load()
    nums = np.array([0, 1, 2, 3, 100, 4095, 32767], dtype=np.uint16)
    exps = np.array([0, 1, 2, 300, 12345, 65534], dtype=np.uint16)
    d_nums = torch.from_numpy(nums.view(np.int16)).cuda()
    d_exps = torch.from_numpy(exps.view(np.int16)).cuda()
    out = torch.zeros((len(exps), len(nums)), dtype=torch.int16, device="cuda")
    _lib.check(L.par2cuda_par2_coeffs(d_nums.data_ptr(), len(nums), d_exps.data_ptr(), len(exps), out.data_ptr(), None),
               "coeffs")
    got = out.cpu().numpy().view(np.uint16)
    want = np.array([[O.coeff(int(i), int(e)) for i in nums] for e in exps], dtype=np.uint16)
    assert np.array_equal(got, want)
