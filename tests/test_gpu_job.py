"""The device-resident job path (bench.py's step) against the oracle: recovery
slices, IFSC entries, file MD5s and checksum verdicts for a multi-file job."""
import hashlib

import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("S,file_lens,R", [
    (65536, [65536 * 3 + 1000, 5, 65536, 200001], 7),
    (4100, [4100 * 10, 4100 * 2 - 2, 1], 12),
])
def test_resident_job_matches_oracle(S, file_lens, R):
    torch = pytest.importorskip("torch")
    from parpar_gb300.job import ResidentJob, file_layout
    first, lens = file_layout(file_lens, S)
    N = len(lens)
    host = np.zeros((N, S), np.uint8)
    files = []
    for f, ln in enumerate(file_lens):
        data = synth.slice_bytes(50 + f, 0, ln)
        files.append(data)
        for k in range((ln + S - 1) // S):
            chunk = data[k * S:(k + 1) * S]
            host[first[f] + k, :len(chunk)] = chunk
    exps = list(range(3, 3 + R))
    job = ResidentJob(S, file_lens, exps)
    pinned = torch.from_numpy(host).pin_memory()
    job.upload(pinned)
    # twice through upload + run, then twice through run_from_host (per-file
    # copies overlapped with the file MD5s, in launch groups of 2 files)
    for it in range(4):
        if it < 2:
            job.run()
        else:
            job.d_in.zero_()
            job.d_fmd5.zero_()
            job.run_from_host(pinned, group=2)
        rec, ifsc, fmd5, flags = job.download()
        torch.cuda.synchronize()
        assert flags.numpy().tolist() == [1] * R
        ref = O.recover(host, lens, np.arange(N), exps)
        assert np.array_equal(rec.numpy(), ref)
        exp_ifsc = b"".join(O.hash_file(d, S)[0] for d in files)
        assert ifsc.numpy().tobytes() == exp_ifsc
        assert fmd5.numpy().tobytes() == b"".join(hashlib.md5(d.tobytes()).digest() for d in files)
