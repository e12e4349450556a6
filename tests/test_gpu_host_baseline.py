"""The CPU baseline's fast multiply on the GPU host's own cores.

The GPU host is aarch64, where the oracle compiles its NEON restatement of
the reference's split-nibble shuffle method (or_recover_fast) and the ARMv8
CRC32 instructions.  This container is x86, so that code only runs here: it
is checked against the plain oracle over ragged sizes, odd word tails and
more threads than work units.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,r,S,threads", [
    (7, 3, 64, 1), (33, 5, 8192 + 34, 4), (3, 1, 30, 16), (64, 9, 3 * 8192, 16), (2, 2, 2, 3),
])
def test_fast_recover_matches_oracle(n, r, S, threads):
    rng = np.random.default_rng(n * 100 + r)
    x = rng.integers(0, 256, size=(n, S), dtype=np.uint8)
    c = rng.integers(0, 65536, size=(r, n), dtype=np.uint16)
    assert np.array_equal(O.recover_fast(x, c, threads=threads), O.recover_coeffs(x, np.full(n, S), c))


def test_fast_crc_matches_oracle():
    rng = np.random.default_rng(3)
    L = O.lib()
    for ln, pad in [(0, 0), (7, 9), (4096, 0), (10007, 123)]:
        d = rng.integers(0, 256, size=ln, dtype=np.uint8)
        assert L.or_crc32_fast(O._p(d), ln, pad) == O.crc32(d, pad)


def test_method_name():
    import platform
    name = O.lib().or_fast_method().decode()
    if platform.machine() == "aarch64":
        assert "NEON" in name
        assert "carry-less" in O.lib().or_clmul_method().decode()
    print(O.lib().or_clmul_method().decode())


@pytest.mark.parametrize("n,r,S,threads", [
    (7, 3, 4096, 1), (33, 5, 2048 * 2 * 3 + 34, 4), (5, 2, 30, 2), (64, 9, 2048 * 2 * 5, 16), (1, 1, 4096, 3),
])
def test_clmul_recover_matches_oracle(n, r, S, threads):
    """The carry-less multiply restatement (SVE2 or NEON form, whichever the
    host runs) against the plain oracle: ragged input groups, word tails,
    one input."""
    rng = np.random.default_rng(n * 7 + r)
    x = rng.integers(0, 256, size=(n, S), dtype=np.uint8)
    c = rng.integers(0, 65536, size=(r, n), dtype=np.uint16)
    got = O.recover_clmul(x, c, threads=threads)
    if got is None:
        pytest.skip("not an aarch64 host")
    assert np.array_equal(got, O.recover_coeffs(x, np.full(n, S), c))
