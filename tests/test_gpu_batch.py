"""Batched jobs (persistent comb launches, graph capture, byte-window passes)
against the oracle, and each job's result alone vs in the mix."""
import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import synth

pytestmark = pytest.mark.gpu


def small_mix(seed=3, n=7):
    from parpar_gb300.batch import make_job_mix
    return make_job_mix(n_jobs=n, seed=seed, n_range=(3, 60), s_range=(64, 6000), r_frac=(0.05, 0.6))


def oracle_rec(spec):
    x = synth.slices(spec.seed, 0, spec.N, spec.S)
    return O.recover(x, np.full(spec.N, spec.S), np.arange(spec.N), spec.exps)


@pytest.mark.parametrize("fixed_shape,mode", [(None, "persistent"), (None, "grid")] +
                         [(s, "persistent") for s in range(1, 8)])
def test_batched_passes_match_oracle(fixed_shape, mode):
    torch = pytest.importorskip("torch")
    from parpar_gb300.batch import BatchRunner
    jobs = small_mix()
    total = sum((j.N + j.R) * j.S for j in jobs)
    runner = BatchRunner(jobs, budget_bytes=total // 3 + 4096,
                         shape_of=(lambda R: fixed_shape) if fixed_shape else None, mode=mode)
    assert runner.P >= 3
    refs = {id(b.spec): oracle_rec(b.spec) for b in runner.bufs}
    seen = []

    def check(b, p):
        off, n = b.window(p)
        torch.cuda.synchronize()
        got = b.d_rec.cpu().numpy().view(np.uint8)[:, :n]
        assert np.array_equal(got, refs[id(b.spec)][:, off:off + n]), (b.spec, p)
        assert bool(b.d_flags.all())
        seen.append((id(b.spec), p))

    runner._issue_batched(verify_cb=check)
    assert len(seen) == sum(1 for b in runner.bufs for p in range(runner.P) if b.window(p)[1])


@pytest.mark.parametrize("mode", ["persistent", "grid", "tuned"])
def test_graph_replay_and_alone_vs_mix(mode):
    torch = pytest.importorskip("torch")
    from parpar_gb300.batch import BatchRunner
    jobs = small_mix(seed=9, n=9)
    runner = BatchRunner(jobs, budget_bytes=1 << 30, mode="persistent" if mode == "tuned" else mode)  # one pass
    if mode == "tuned":
        times = runner.tune_mode()
        assert set(times) == {"persistent", "grid"} and runner.mode in times
    assert runner.P == 1
    runner.run_per_job()
    torch.cuda.synchronize()
    alone = [b.d_rec.clone() for b in runner.bufs]
    for b in runner.bufs:
        b.d_rec.zero_()
    runner.capture()
    for _ in range(2):
        runner.run_batched()
    torch.cuda.synchronize()
    assert runner.all_valid()
    for b, a in zip(runner.bufs, alone):
        S = b.spec.S
        mix = b.d_rec.cpu().numpy().view(np.uint8)[:, :S]
        assert np.array_equal(mix, a.cpu().numpy().view(np.uint8)[:, :S])
        assert np.array_equal(mix, oracle_rec(b.spec))


@pytest.mark.parametrize("shape", [1, 4, 5, 6, 7])
def test_batch_descriptors_edge_jobs(shape):
    """One persistent launch over jobs that exercise the unit stream: a job
    without inputs (zero result), accumulation onto existing rows, R spanning
    several recovery blocks with a ragged last one, an input count that is not
    a multiple of 16, and jobs with a single unit."""
    torch = pytest.importorskip("torch")
    import ctypes
    from parpar_gb300 import _lib
    L = _lib.load()
    specs = [(0, 5, 0, 640), (13, 80, 1, 1280), (200, 3, 0, 192), (37, 150, 0, 64), (8, 1, 1, 4096)]
    rng = np.random.default_rng(shape)
    arr = (_lib.BatchJob * len(specs))()
    keep, want = [], []
    base = 0
    for k, (n, R, acc, S) in enumerate(specs):
        pitch = L.par2cuda_row_pitch_bytes(S)
        pw = pitch // 2
        x = rng.integers(0, 256, size=(max(n, 1), S), dtype=np.uint8)
        d_in = torch.zeros((max(n, 1), pw), dtype=torch.int16, device="cuda")
        d_in.view(torch.uint8)[:, :S] = torch.from_numpy(x).cuda()
        c = rng.integers(0, 65536, size=(R, max(n, 1)), dtype=np.uint16)
        d_c = torch.from_numpy(c.view(np.int16)).cuda()
        d_idx = torch.zeros(max(L.par2cuda_coeff_index_bytes(R, n), 16), dtype=torch.uint8, device="cuda")
        if n:
            _lib.check(L.par2cuda_coeff_index(d_c.data_ptr(), R, n, d_idx.data_ptr(), None), "index")
        prior = rng.integers(0, 256, size=(R, S), dtype=np.uint8)
        d_rec = torch.zeros((R, pw), dtype=torch.int16, device="cuda")
        d_rec.view(torch.uint8)[:, :S] = torch.from_numpy(prior).cuda()
        expect = O.recover_coeffs(x[:n], np.full(n, S), c[:, :n]) if n else np.zeros((R, S), np.uint8)
        if acc:
            expect = expect ^ prior
        want.append((d_rec, S, expect))
        keep += [d_in, d_c, d_idx]
        nw = (S // 2 + 7) // 8 * 8
        arr[k].d_in = d_in.data_ptr(); arr[k].in_pitch_words = pw; arr[k].num_in = n
        arr[k].d_index = d_idx.data_ptr(); arr[k].d_rec = d_rec.data_ptr(); arr[k].rec_pitch_words = pw
        arr[k].num_rec = R; arr[k].accumulate = acc; arr[k].unit_base = base
        base += L.par2cuda_batch_units(R, nw, shape)
    d_jobs = torch.frombuffer(bytearray(arr), dtype=torch.uint8).cuda()
    counter = torch.zeros(1, dtype=torch.int64, device="cuda")
    _lib.check(L.par2cuda_batch_muladd(d_jobs.data_ptr(), len(specs), base, counter.data_ptr(), shape, None), "batch")
    torch.cuda.synchronize()
    assert L.par2cuda_device_error() == 0
    for d_rec, S, expect in want:
        got = d_rec.cpu().numpy().view(np.uint8)[:, :S]
        assert np.array_equal(got, expect)


@pytest.mark.parametrize("method", ["xor", "nibble", "tensor", "tensor_fp4"])
def test_grid_mode_with_each_method_matches_oracle(method):
    """The batched grid path with the autotuner's choice forced to each
    non-comb method (the choice the tuner may make for some recovery count)."""
    torch = pytest.importorskip("torch")
    from parpar_gb300.batch import BatchRunner
    jobs = small_mix(seed=5, n=5)
    runner = BatchRunner(jobs, budget_bytes=1 << 30, mode="grid", method_of=lambda R: method)
    runner.capture()
    runner.run_batched()
    torch.cuda.synchronize()
    for b in runner.bufs:
        got = b.d_rec.cpu().numpy().view(np.uint8)[:, : b.spec.S]
        assert np.array_equal(got, oracle_rec(b.spec)), (method, b.spec)
        assert bool(b.d_flags.all())


def test_autotuner_weighs_every_method():
    pytest.importorskip("torch")
    from parpar_gb300 import autotune
    m = autotune.best_method(24)
    assert m in autotune.METHODS
    best, times = autotune.method_table()[autotune._bucket(24)]
    assert best == m and set(times) == set(autotune.METHODS) and min(times.values()) == times[m]
