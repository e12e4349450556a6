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


@pytest.mark.parametrize("fixed_shape", [None, 1, 2, 3, 4, 5, 6, 7])
def test_batched_passes_match_oracle(fixed_shape):
    torch = pytest.importorskip("torch")
    from parpar_gb300.batch import BatchRunner
    jobs = small_mix()
    total = sum((j.N + j.R) * j.S for j in jobs)
    runner = BatchRunner(jobs, budget_bytes=total // 3 + 4096,
                         shape_of=(lambda R: fixed_shape) if fixed_shape else None)
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


def test_graph_replay_and_alone_vs_mix():
    torch = pytest.importorskip("torch")
    from parpar_gb300.batch import BatchRunner
    jobs = small_mix(seed=9, n=9)
    runner = BatchRunner(jobs, budget_bytes=1 << 30)  # one pass
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
