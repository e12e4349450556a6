"""The job stream (parpar_gb300.stream.JobStream): many create jobs in flight,
file MD5 chains of several jobs pooled in one launch.  Every job's recovery
slices, IFSC entries, file MD5s and verdicts must equal the oracle's for that
job's inputs, with resident inputs and with inputs copied from (and results
copied to) pinned host buffers, including partial groups and slot reuse."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from parpar_gb300 import synth
from parpar_gb300.layout import file_layout

pytestmark = pytest.mark.gpu

S = 65536
FILE_LENS = [5 * S + 123, 3 * S, 1, 7 * S + 65535, 2 * S + 2, 40000]
EXPS = [0, 1, 2, 300, 65534]


def expected(x):
    """Oracle results for one job's rows x (uint8 [N, S], tails beyond each row's length ignored)."""
    first, lens = file_layout(FILE_LENS, S)
    xz = x.copy()
    for i, ln in enumerate(lens):
        xz[i, ln:] = 0
    rec = O.recover(xz, lens, np.arange(len(lens)), EXPS)
    ifsc, fmd5 = b"", b""
    for f, ln in enumerate(FILE_LENS):
        a = int(first[f])
        n = max(1, (ln + S - 1) // S)
        i_, m_ = O.hash_file(x[a:a + n].reshape(-1)[:ln], S)
        ifsc += i_
        fmd5 += m_
    return rec, ifsc, fmd5


def make_stream(slots=4, group=2):
    from parpar_gb300.stream import JobStream
    return JobStream(S, FILE_LENS, EXPS, slots=slots, group=group)


def test_stream_resident_jobs_match_oracle():
    js = make_stream()
    js.fill_synthetic(seed0=50)
    js.run(7, first_job=0, timing=True)       # 3 full groups + a partial one, slots reused
    js.run(3, first_job=7)                    # continues mid-group
    torch.cuda.synchronize()
    for s in range(js.slots):
        x = synth.slices(50 + s, 0, js.N, S)
        rec, ifsc, fmd5 = expected(x)
        got_rec, got_ifsc, got_fmd5, flags = js.slot_results(s)
        assert flags.all()
        assert np.array_equal(got_rec, rec)
        assert got_ifsc.tobytes() == ifsc
        assert got_fmd5.tobytes() == fmd5
    lat = js.latencies()
    assert len(lat) == 7 and min(lat) > 0


def test_stream_host_buffers_match_oracle():
    js = make_stream(slots=4, group=2)
    hosts = [torch.from_numpy(synth.slices(70 + k, 0, js.N, S)).pin_memory() for k in range(3)]
    outs = js.host_out_buffers(5)
    js.run(9, first_job=0, host_in=hosts, host_out=outs)
    torch.cuda.synchronize()
    want = [expected(h.numpy()) for h in hosts]
    # job k read hosts[k % 3] and wrote outs[k % 5]; the last 5 jobs (4..8) hold the outputs
    for k in range(4, 9):
        rec, ifsc, fmd5 = want[k % 3]
        o = outs[k % 5]
        assert o[3].numpy().all()
        assert np.array_equal(o[0].numpy(), rec)
        assert o[1].numpy().tobytes() == ifsc
        assert o[2].numpy().tobytes() == fmd5


def test_pooled_file_md5_matches_per_file_launch():
    """par2cuda_file_md5_pooled (several block sizes) = par2cuda_file_md5."""
    from parpar_gb300 import _lib
    L = _lib.load()
    first, lens = file_layout(FILE_LENS * 7, S)
    N = len(lens)
    pitch = L.par2cuda_row_pitch_bytes(S)
    d = torch.empty((N, pitch), dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.par2cuda_synth_fill(d.data_ptr(), pitch, N, S, 9, 0, st), "synth")
    flen = torch.tensor(FILE_LENS * 7, dtype=torch.int64, device="cuda")
    fr = torch.from_numpy(first.view(np.int32)).cuda()
    nf = len(FILE_LENS) * 7
    ref = torch.empty(nf * 16, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_file_md5(d.data_ptr(), pitch, nf, flen.data_ptr(), fr.data_ptr(), S, ref.data_ptr(), st), "md5")
    for per in (1, 32, 64, 512):
        out = torch.zeros(nf * 16, dtype=torch.uint8, device="cuda")
        _lib.check(L.par2cuda_file_md5_pooled(d.data_ptr(), pitch, nf, flen.data_ptr(), fr.data_ptr(), S,
                                             out.data_ptr(), per, st), "pooled")
        assert torch.equal(out, ref), per
    assert L.par2cuda_file_md5_pooled(d.data_ptr(), pitch, nf, flen.data_ptr(), fr.data_ptr(), S,
                                      ref.data_ptr(), 48, st) < 0
    for per in (32, 64):
        out = torch.zeros(nf * 16, dtype=torch.uint8, device="cuda")
        _lib.check(L.par2cuda_file_md5_staged(d.data_ptr(), pitch, nf, flen.data_ptr(), fr.data_ptr(), S,
                                             out.data_ptr(), per, st), "staged")
        assert torch.equal(out, ref), per
    assert L.par2cuda_device_error() == 0
    # the staged form needs whole MD5 blocks per slice and 32 or 64 files per block
    assert L.par2cuda_file_md5_staged(d.data_ptr(), pitch, nf, flen.data_ptr(), fr.data_ptr(), S - 4,
                                      ref.data_ptr(), 64, st) < 0
    assert L.par2cuda_file_md5_staged(d.data_ptr(), pitch, nf, flen.data_ptr(), fr.data_ptr(), S,
                                      ref.data_ptr(), 128, st) < 0


def test_staged_file_md5_against_oracle_odd_lengths():
    """Files ending at every residue of the 1 KiB chunk and the 64-byte block."""
    from parpar_gb300 import _lib
    L = _lib.load()
    S = 4096
    lens = [0, 1, 15, 16, 63, 64, 65, 1023, 1024, 1025, 4095, 4096, 4097, 3 * 4096 + 1000, 20000]
    first, _ = file_layout(lens, S)
    N = int(first[-1]) + max(1, -(-lens[-1] // S))
    pitch = L.par2cuda_row_pitch_bytes(S)
    d = torch.empty((N, pitch), dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.par2cuda_synth_fill(d.data_ptr(), pitch, N, S, 21, 0, st), "synth")
    flen = torch.tensor(lens, dtype=torch.int64, device="cuda")
    fr = torch.from_numpy(first.view(np.int32)).cuda()
    out = torch.zeros(len(lens) * 16, dtype=torch.uint8, device="cuda")
    _lib.check(L.par2cuda_file_md5_staged(d.data_ptr(), pitch, len(lens), flen.data_ptr(), fr.data_ptr(), S,
                                         out.data_ptr(), 32, st), "staged")
    x = synth.slices(21, 0, N, S)
    got = out.cpu().numpy().reshape(-1, 16)
    for f, ln in enumerate(lens):
        a = int(first[f])
        data = x[a:a + max(1, -(-ln // S))].reshape(-1)[:ln]
        assert got[f].tobytes() == O.md5(data), ln


def test_stream_size_classes_and_mixed_runs():
    """Three size classes of copies from host buffers (neighbouring files of
    a class copied together), windows that reuse
    slots, and resident runs in between on the rows the copies left."""
    from parpar_gb300.stream import JobStream
    js = JobStream(S, FILE_LENS, EXPS, slots=4, group=2, size_classes=(0.95, 0.5))
    assert js.classes == [[3], [0], [1, 2, 4, 5]]
    assert js.class_runs[2] == [[6, 4], [18, 4]]   # files 1+2 and 4+5: neighbouring rows merged
    hosts = [torch.from_numpy(synth.slices(90 + k, 0, js.N, S)).pin_memory() for k in range(3)]
    outs = js.host_out_buffers(5)
    js.run(6, first_job=0, host_in=hosts, host_out=outs, timing=True)   # windows of 4 + 2 jobs
    torch.cuda.synchronize()
    assert js.upload_span_ms() > 0 and len(js.latencies()) == 6
    js.run(2, first_job=6)                                              # resident, slots 2 and 3
    js.run(3, first_job=8, host_in=hosts, host_out=outs)                # slots 0, 1, 2
    torch.cuda.synchronize()
    want = [expected(h.numpy()) for h in hosts]
    for k, o in ((1, outs[1]), (2, outs[2]), (8, outs[3]), (9, outs[4]), (10, outs[0])):
        rec, ifsc, fmd5 = want[k % 3]
        assert o[3].numpy().all(), k
        assert np.array_equal(o[0].numpy(), rec), k
        assert o[1].numpy().tobytes() == ifsc, k
        assert o[2].numpy().tobytes() == fmd5, k
    # slot 3 ran job 7 on the rows job 3 copied in (hosts[0]); slot 2 ran job 10 (hosts[1])
    for s, h in ((3, 0), (2, 1)):
        rec, ifsc, fmd5 = want[h]
        got_rec, got_ifsc, got_fmd5, flags = js.slot_results(s)
        assert flags.all() and np.array_equal(got_rec, rec)
        assert got_ifsc.tobytes() == ifsc and got_fmd5.tobytes() == fmd5


def test_indexed_file_md5_places_digests():
    """par2cuda_file_md5_staged_indexed over a permuted subset of files puts
    each digest in its file's place; a null index is the plain staged form."""
    from parpar_gb300 import _lib
    L = _lib.load()
    first, lens = file_layout(FILE_LENS * 5, S)
    N = len(lens)
    pitch = L.par2cuda_row_pitch_bytes(S)
    d = torch.empty((N, pitch), dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.par2cuda_synth_fill(d.data_ptr(), pitch, N, S, 11, 0, st), "synth")
    nf = len(FILE_LENS) * 5
    flen_all = np.array(FILE_LENS * 5, dtype=np.int64)
    ref = torch.zeros(nf * 16, dtype=torch.uint8, device="cuda")
    # device tables held in names: a pointer taken from a temporary tensor
    # would outlive its memory
    flen = torch.from_numpy(flen_all).cuda()
    fr = torch.from_numpy(first.view(np.int32)).cuda()
    _lib.check(L.par2cuda_file_md5_staged_indexed(d.data_ptr(), pitch, nf, flen.data_ptr(), fr.data_ptr(), None, S,
                                                 ref.data_ptr(), 64, st), "indexed")
    x = synth.slices(11, 0, N, S)
    for f in range(nf):
        a, ln = int(first[f]), int(flen_all[f])
        assert ref[16 * f:16 * f + 16].cpu().numpy().tobytes() == O.md5(x[a:a + max(1, -(-ln // S))].reshape(-1)[:ln])
    rng = np.random.default_rng(4)
    pick = rng.permutation(nf)[: nf - 7]            # a subset, in shuffled order
    out = torch.full((nf * 16,), 0xAB, dtype=torch.uint8, device="cuda")
    tl = torch.from_numpy(flen_all[pick]).cuda()
    tf = torch.from_numpy(first[pick].astype(np.uint32).view(np.int32)).cuda()
    ti = torch.from_numpy(pick.astype(np.uint32).view(np.int32)).cuda()
    _lib.check(L.par2cuda_file_md5_staged_indexed(d.data_ptr(), pitch, len(pick), tl.data_ptr(), tf.data_ptr(),
                                                 ti.data_ptr(), S, out.data_ptr(), 32, st), "indexed")
    got, want = out.cpu().numpy().reshape(nf, 16), ref.cpu().numpy().reshape(nf, 16)
    for f in range(nf):
        if f in set(pick.tolist()):
            assert got[f].tobytes() == want[f].tobytes(), f
        else:
            assert (got[f] == 0xAB).all(), f
    assert L.par2cuda_device_error() == 0
