"""The oracle restatement (oracle/par2_oracle.c) against the golden vectors
recorded from the reference's own compiled CPU code (tests/golden/golden.json)."""
import hashlib
import json
import os
import zlib

import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import synth

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def case_inputs(c):
    x = synth.slices(c["seed"], 0, c["n"], c["slice"])
    lens = np.array(c["lens"], dtype=np.uint64)
    for i, l in enumerate(c["lens"]):
        x[i, l:] = 0
    return x, lens


def test_known_answers():
    # gfmat_coeff.c known answers and standard hash vectors
    assert [O.coeff(0, 1), O.coeff(1, 1), O.coeff(2, 1)] == [0x0002, 0x0004, 0x0010]
    assert O.crc32(b"abc") == 0x352441C2
    assert O.md5(b"abc").hex() == "900150983cd24fb0d6963f7d28e17f72"


def test_coefficients():
    for i, e, c in GOLDEN["coeffs"]:
        assert O.coeff(i, e) == c, (i, e)
    logs = np.array([O.lib().or_input_log(i) for i in range(32768)], dtype="<u2")
    assert hashlib.md5(logs.tobytes()).hexdigest() == GOLDEN["input_log_md5"]


def test_gf_mul_tables_match_shift_xor():
    rng = np.random.default_rng(0)
    L = O.lib()
    for a, b in rng.integers(0, 65536, size=(3000, 2)):
        assert L.or_mul(int(a), int(b)) == L.or_mul_slow(int(a), int(b))


@pytest.mark.parametrize("case", GOLDEN["recovery"], ids=lambda c: c["name"])
def test_recovery(case):
    x, lens = case_inputs(case)
    out = O.recover(x, lens, case["nums"], case["exps"], threads=2)
    got = [hashlib.md5(out[j].tobytes()).hexdigest() for j in range(len(case["exps"]))]
    assert got == case["md5"]
    if "hex" in case:
        assert [out[j].tobytes().hex() for j in range(len(case["exps"]))] == case["hex"]


def test_recovery_custom_coeffs():
    c = GOLDEN["recovery_coeffs"]
    x, lens = case_inputs(c)
    coeffs = np.array(c["coeffs_in_rec"], dtype=np.uint16).T  # [rec][input]
    out = O.recover_coeffs(x, lens, coeffs)
    assert [hashlib.md5(out[j].tobytes()).hexdigest() for j in range(out.shape[0])] == c["md5"]


@pytest.mark.parametrize("case", GOLDEN["cksum"], ids=lambda c: "%d_%d" % (c["src_len"], c["slice_len"]))
def test_checksum(case):
    src = synth.slice_bytes(case["seed"], 0, case["src_len"])
    ck = O.cksum(src, case["slice_len"])
    assert ck.to_bytes(8, "little").hex() == case["cksum"]
    full = np.zeros(case["slice_len"], np.uint8)
    full[: case["src_len"]] = src
    assert O.lib().or_cksum_check(O._p(full), full.size, ck) == 1
    if full.size:
        full[full.size // 2] ^= 0x10  # a flipped bit must fail the check
        assert O.lib().or_cksum_check(O._p(full), full.size, ck) == 0


@pytest.mark.parametrize("case", GOLDEN["hash"], ids=lambda c: c["name"])
def test_ifsc_and_file_md5(case):
    data = synth.slice_bytes(case["seed"], 0, case["len"])
    ifsc, fmd5 = O.hash_file(data, case["slice"])
    assert ifsc.hex() == case["ifsc"]
    assert fmd5.hex() == case["file_md5"] == hashlib.md5(data.tobytes()).hexdigest()
    # every IFSC entry equals MD5/CRC32 of the zero-padded slice
    S = case["slice"]
    for s in range(len(ifsc) // 20):
        blk = data[s * S:(s + 1) * S].tobytes()
        blk += bytes(S - len(blk))
        assert ifsc[20 * s:20 * s + 16] == hashlib.md5(blk).digest()
        assert int.from_bytes(ifsc[20 * s + 16:20 * s + 20], "little") == zlib.crc32(blk)


@pytest.mark.parametrize("case", GOLDEN["md5multi"], ids=lambda c: "n%d_len%d" % (c["n"], c["len"]))
def test_md5multi(case):
    bufs = synth.slices(case["seed"], 0, case["n"], case["len"])
    md5s, _ = O.hash_rows(bufs)
    assert md5s.tobytes().hex() == case["md5"]


def test_fast_baseline_path_matches_oracle():
    """The CPU baseline's fast path (NEON on aarch64, the plain method
    elsewhere) computes the same recovery and CRCs as the oracle."""
    rng = np.random.default_rng(8)
    for n, r, S in [(5, 3, 64), (17, 5, 8192 + 34), (3, 1, 32), (9, 4, 2)]:
        x = rng.integers(0, 256, size=(n, S), dtype=np.uint8)
        c = rng.integers(0, 65536, size=(r, n), dtype=np.uint16)
        assert np.array_equal(O.recover_fast(x, c, threads=3), O.recover_coeffs(x, np.full(n, S), c))
    L = O.lib()
    for ln, pad in [(0, 5), (13, 0), (1000, 77), (64, 4096)]:
        d = rng.integers(0, 256, size=ln, dtype=np.uint8)
        assert L.or_crc32_fast(O._p(d), ln, pad) == O.crc32(d, pad)
