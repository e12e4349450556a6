"""GPU hashing (IFSC slice MD5+CRC32, file MD5, packet MD5) vs the golden
vectors recorded from the reference hasher and vs the oracle."""
import hashlib
import json
import os
import zlib

import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import _lib, synth

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def _rows_from_files(torch, files, S):
    """Lays files out as consecutive rows of S bytes (row pitch from the library)."""
    L = _lib.load()
    pitch = L.par2cuda_row_pitch_bytes(S)
    nrows = sum((len(f) + S - 1) // S for f in files)
    host = np.zeros((max(nrows, 1), pitch), np.uint8)
    lens, first, r = [], [], 0
    for f in files:
        first.append(r)
        for off in range(0, len(f), S):
            chunk = f[off:off + S]
            host[r, :len(chunk)] = chunk
            lens.append(len(chunk))
            r += 1
    d = torch.from_numpy(host).cuda()
    return d, pitch, np.array(lens, np.uint32), np.array(first, np.uint32), nrows


def _hash(torch, files, S):
    L = _lib.load()
    d, pitch, lens, first, nrows = _rows_from_files(torch, files, S)
    d_lens = torch.from_numpy(lens.view(np.int32)).cuda()
    ifsc = torch.zeros(max(nrows, 1) * 20, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_slice_hash(d.data_ptr(), pitch, nrows, d_lens.data_ptr(), S, ifsc.data_ptr(), None), "slice_hash")
    flen = torch.tensor([len(f) for f in files], dtype=torch.int64, device="cuda")
    d_first = torch.from_numpy(first.view(np.int32)).cuda()
    md5 = torch.zeros(16 * len(files), dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_file_md5(d.data_ptr(), pitch, len(files), flen.data_ptr(), d_first.data_ptr(), S, md5.data_ptr(), None), "file_md5")
    torch.cuda.synchronize()
    return ifsc.cpu().numpy()[: nrows * 20].tobytes(), md5.cpu().numpy().tobytes()


@pytest.mark.parametrize("case", GOLDEN["hash"], ids=lambda c: c["name"])
def test_golden_ifsc_and_file_md5(case):
    torch = pytest.importorskip("torch")
    data = synth.slice_bytes(case["seed"], 0, case["len"])
    ifsc, md5 = _hash(torch, [data], case["slice"])
    assert ifsc.hex() == case["ifsc"]
    assert md5.hex() == case["file_md5"]


def test_many_files_uneven():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    S = 4096
    files = [synth.slice_bytes(100 + k, 0, int(l)) for k, l in enumerate(rng.integers(1, 5 * S, size=23))]
    files.append(synth.slice_bytes(999, 0, 3 * S))  # exact multiple
    ifsc, md5 = _hash(torch, files, S)
    exp_ifsc = b"".join(O.hash_file(f, S)[0] for f in files)
    assert ifsc == exp_ifsc
    assert md5 == b"".join(hashlib.md5(f.tobytes()).digest() for f in files)


@pytest.mark.parametrize("S", [4, 8, 60, 64, 68, 1000, 65536 + 4])
def test_slice_sizes_not_block_aligned(S):
    torch = pytest.importorskip("torch")
    files = [synth.slice_bytes(S, 0, 3 * S + S // 2 + 2), synth.slice_bytes(S + 1, 0, 2)]
    ifsc, md5 = _hash(torch, files, S)
    assert ifsc == b"".join(O.hash_file(f, S)[0] for f in files)
    assert md5 == b"".join(hashlib.md5(f.tobytes()).digest() for f in files)
    # each IFSC CRC equals zlib's CRC of the zero-padded slice
    d = files[0]
    blk = d[:S].tobytes()
    assert int.from_bytes(ifsc[16:20], "little") == zlib.crc32(blk)


@pytest.mark.parametrize("case", GOLDEN["md5multi"], ids=lambda c: "n%d_len%d" % (c["n"], c["len"]))
def test_rows_md5_golden(case):
    torch = pytest.importorskip("torch")
    L = _lib.load()
    n, ln = case["n"], case["len"]
    bufs = synth.slices(case["seed"], 0, n, ln)
    pitch = L.par2cuda_row_pitch_bytes(ln)
    host = np.zeros((n, pitch), np.uint8)
    host[:, :ln] = bufs
    d = torch.from_numpy(host).cuda()
    out = torch.zeros(16 * n, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_rows_md5(d.data_ptr(), pitch, n, ln, None, 0, out.data_ptr(), None), "rows_md5")
    torch.cuda.synchronize()
    assert out.cpu().numpy().tobytes().hex() == case["md5"]


def test_rows_md5_with_packet_prefix():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    n, ln, pl = 5, 4100, 36
    bufs = synth.slices(3, 0, n, ln)
    pre = synth.slices(4, 0, n, pl)
    pitch = L.par2cuda_row_pitch_bytes(ln)
    host = np.zeros((n, pitch), np.uint8)
    host[:, :ln] = bufs
    d = torch.from_numpy(host).cuda()
    dp = torch.from_numpy(np.ascontiguousarray(pre)).cuda()
    out = torch.zeros(16 * n, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_rows_md5(d.data_ptr(), pitch, n, ln, dp.data_ptr(), pl, out.data_ptr(), None), "rows_md5")
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(n, 16)
    for i in range(n):
        assert got[i].tobytes() == hashlib.md5(pre[i].tobytes() + bufs[i].tobytes()).digest()


def test_packed_file_md5_matches_unpacked():
    """par2cuda_file_md5_packed (32 chains per warp) gives the same digests as
    the one-chain-per-block launch, for 40 uneven files including a 1-byte one."""
    torch = pytest.importorskip("torch")
    from parpar_gb300 import _lib
    from parpar_gb300.job import ResidentJob
    S = 4096
    rng = np.random.default_rng(40)
    lens = [int(x) for x in rng.integers(1, 40 * S, size=39)] + [1]
    job = ResidentJob(S, lens, [0])
    job.fill_synthetic(5)
    L = _lib.load()
    outs = []
    for fn in (L.par2cuda_file_md5, L.par2cuda_file_md5_packed):
        d = torch.zeros(16 * len(lens), dtype=torch.uint8, device="cuda")
        _lib.check(fn(job.d_in.data_ptr(), job.pitch, len(lens), job.d_flen.data_ptr(), job.d_first.data_ptr(), S,
                      d.data_ptr(), None), "md5")
        outs.append(d.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
    rows = job.d_in.view(torch.uint8).cpu().numpy()
    f = 7
    a = int(job.first_row[f])
    data = rows[a:a + (lens[f] + S - 1) // S, :S].reshape(-1)[:lens[f]]
    assert outs[0][16 * f:16 * f + 16].tobytes() == O.md5(data)
