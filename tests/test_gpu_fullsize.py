"""The two full-size workloads, every byte, against the reference's own CPU core.

  bandwidth: 2000 input slices x 2 MiB over 40 seeded uneven files (the last
             slice of each zero-padded), 200 recovery slices (exponents
             0..199), IFSC entries and file MD5s;
  dense:     4096 input slices x 256 KiB, 4096 recovery slices (0..4095).

The GPU path (parpar_gb300.job.ResidentJob, the C ABI) and ParPar's PAR2Proc +
PAR2ProcCPU (GF16_AUTO) with its HasherInput per file (oracle/_ref, built on
this host from the staged reference sources) run on the same seeded bytes;
recovery slices, checksum verdicts, IFSC entries and file MD5s must be equal.
Where the reference core is not built, the oracle's multi-threaded
restatement stands in (it is pinned to the reference by tests/golden/).
"""
import hashlib
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from parpar_gb300.layout import file_layout, file_lengths

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8


def cpu_expected(x, lens, exps, file_lens, first):
    nums = np.arange(x.shape[0])
    if O.ref_available():
        out, valid, ifsc, fmd5, _ = O.ref_job(x, lens, nums, exps, file_lens, first, THREADS)
        assert valid.all()
        return out, ifsc, fmd5
    xz = x.copy()
    for i, ln in enumerate(lens):
        xz[i, ln:] = 0
    out = O.recover_clmul(xz, O.par2_coeff_matrix(nums, exps), threads=THREADS)
    if out is None:
        out = O.recover_fast(xz, O.par2_coeff_matrix(nums, exps), threads=THREADS)
    ifsc, fmd5 = b"", b""
    if file_lens is not None:
        S = x.shape[1]
        for f, ln in enumerate(file_lens):
            a = int(first[f])
            i_, m_ = O.hash_file(x[a:a + max(1, (ln + S - 1) // S)].reshape(-1)[:ln], S)
            ifsc += i_
            fmd5 += m_
    return out, ifsc, fmd5


def run_gpu(S, file_lens, exps, seed, hashes):
    from parpar_gb300.job import ResidentJob
    job = ResidentJob(S, file_lens, exps)
    job.fill_synthetic(seed)
    job.run(hashes=hashes)
    rec = job.d_rec.view(torch.uint8)[:, :S].cpu().numpy()
    res = (rec, job.d_flags.cpu().numpy(), job.d_ifsc.cpu().numpy().tobytes(), job.d_fmd5.cpu().numpy().tobytes())
    del job
    torch.cuda.empty_cache()
    return res


def row_digests(a):
    return [hashlib.md5(r.tobytes()).digest() for r in a]


def test_bandwidth_workload_every_byte():
    S, N, R = 2 * 1048576, 2000, 200
    file_lens = file_lengths(N, 40, S, seed=2000)
    first, lens = file_layout(file_lens, S)
    exps = list(range(R))
    rec, flags, ifsc, fmd5 = run_gpu(S, file_lens, exps, seed=1, hashes=True)
    x = O.synth_rows(1, 0, N, S)
    want, want_ifsc, want_fmd5 = cpu_expected(x, lens, exps, file_lens, first)
    assert flags.all()
    assert row_digests(rec) == row_digests(want)
    assert np.array_equal(rec, want)
    assert ifsc == want_ifsc
    assert fmd5 == want_fmd5


def test_dense_workload_every_byte():
    S, N, R = 262144, 4096, 4096
    exps = list(range(R))
    rec, flags, _, _ = run_gpu(S, [N * S], exps, seed=7, hashes=False)
    x = O.synth_rows(7, 0, N, S)
    want, _, _ = cpu_expected(x, np.full(N, S), exps, None, None)
    assert flags.all()
    assert np.array_equal(rec, want)
