"""Serving loop: continuous admission by free HBM, overlapping jobs, chunked
requests; every result is the same alone and in the mix, and equals the oracle."""
import hashlib

import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import synth

pytestmark = pytest.mark.gpu


def _oracle_digest(spec, window):
    x = synth.slices(spec.seed, 0, spec.N, spec.S)
    rec = O.recover(x, np.full(spec.N, spec.S), np.arange(spec.N), spec.exps)
    h = hashlib.md5()
    for off in range(0, spec.S, window):
        h.update(np.ascontiguousarray(rec[:, off:off + window]).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("chunk_share,persistent", [(0.5, False), (0.02, False), (0.5, True), (0.02, True)])
def test_serving_alone_equals_mix(chunk_share, persistent):
    pytest.importorskip("torch")
    from parpar_gb300.serve import Request, Server, make_requests
    reqs = make_requests(12, rate=2000.0, seed=7, n_range=(3, 80), s_range=(64, 20000), r_frac=(0.05, 0.5))
    mk = lambda: Server(budget_bytes=3 * 10**6, slots=3, digests=True, chunk_share=chunk_share, persistent=persistent)
    srv = mk()
    done = srv.run(reqs)
    assert len(done) == len(reqs)
    assert all(r.valid for r in done)
    # requests overlapped: some were admitted before an earlier one finished
    order = sorted(done, key=lambda r: r.admitted)
    assert any(b.admitted < a.done for a, b in zip(order, order[1:]))
    mix = {r.rid: r.digest for r in done}
    for r in reqs:
        alone = mk().run([Request(r.rid, r.spec, 0.0)])[0]
        assert alone.valid and alone.digest == mix[r.rid]
        assert alone.digest == _oracle_digest(r.spec, srv._window(r.spec))
