"""Generates tests/golden/golden.json from the reference's own CPU code.

Run in a container that has the reference tree: it builds oracle/_ref/libparref.so
with oracle/ref.mk (the reference's gf16/ + hasher/ sources compiled in place)
and records its outputs on seeded synthetic inputs (parpar_gb300.synth), so the
oracle restatement and the CUDA path can be checked against them anywhere.

    PARPAR_REFERENCE=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import argparse
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from parpar_gb300 import synth  # noqa: E402

# Recovery cases: shapes from the reference's par-compare edge list
# (test/par-compare.js:341-540): odd/prime sizes, 4- and 8-byte slices,
# exponent 0, more recovery than inputs, ragged (short) inputs, high input
# numbers and exponents.
RECOVERY_CASES = [
    # name, seed, n, S, r, exps, input numbering, ragged
    ("tiny4", 1, 3, 4, 2, "seq0", "seq", False),
    ("tiny8_r_gt_n", 2, 2, 8, 5, "seq0", "seq", False),
    ("plain_100x10_small", 3, 100, 4096, 10, "seq0", "seq", False),
    ("prime_65521x4_ragged", 4, 7, 65521 * 4, 3, "seq0", "seq", True),
    ("odd_12224", 5, 11, 12224, 13, "seq1", "seq", True),
    ("high_exps", 6, 9, 1000, 6, "random", "random", True),
    ("single_in_single_out", 7, 1, 65540, 1, "seq0", "seq", False),
    ("r_gt_n_64", 8, 5, 2048, 64, "seq0", "seq", True),
    ("batch_boundary_25x", 9, 25, 6000, 4, "seq0", "seq", True),
]

HASH_CASES = [
    # name, seed, file length, slice size, feed piece size
    ("empty_tail_exact", 11, 4096, 1024, 333),
    ("one_byte", 12, 1, 1024, 1),
    ("eight_bytes", 13, 8, 4, 3),
    ("prime_65521", 14, 65521, 65536, 4000),
    ("multi_slice_ragged", 15, 1000003, 65536, 65536),
    ("big_slice", 16, 3 * 1048576 + 12345, 1048576, 1 << 20),
]

CKSUM_CASES = [(0, 8), (5, 8), (6, 10), (100, 100), (99, 1000), (1000, 1000), (4, 4), (13, 4096),
               (65521 * 4, 65521 * 4), (12224, 12224), (777, 1 << 20)]


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def case_inputs(seed, n, S, ragged):
    x = synth.slices(seed, 0, n, S)
    lens = np.full(n, S, dtype=np.uint64)
    if ragged:
        rng = np.random.default_rng(seed)
        for i in range(0, n, 2):
            lens[i] = int(rng.integers(1, S + 1))
    return x, lens


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference checkout (default: $PARPAR_REFERENCE)")
    args = ap.parse_args()
    from oracle import refsrc
    if not refsrc.stage(args.ref):
        sys.exit("no reference tree: pass --ref or set PARPAR_REFERENCE")
    res = refsrc.build(with_cuda=False)
    if res["error"]:
        sys.exit(res["error"])
    R = O.ref()
    out = {"generator": "tests/golden/make_golden.py", "reference": "ParPar gf16/ + hasher/ (compiled by oracle/ref.mk)",
           "coeffs": [], "recovery": [], "cksum": [], "hash": [], "md5multi": []}

    rng = np.random.default_rng(1234)
    pairs = [(0, 0), (0, 1), (1, 1), (2, 1), (32767, 65534), (100, 0), (5, 65535 - 1)]
    pairs += [(int(rng.integers(32768)), int(rng.integers(65535))) for _ in range(500)]
    out["coeffs"] = [[i, e, R.ref_coeff(i, e)] for i, e in pairs]
    out["input_log_md5"] = hashlib.md5(np.array([R.ref_input_log(i) for i in range(32768)], dtype="<u2").tobytes()).hexdigest()

    for name, seed, n, S, r, exps_kind, nums_kind, ragged in RECOVERY_CASES:
        x, lens = case_inputs(seed, n, S, ragged)
        crng = np.random.default_rng(seed + 1000)
        if exps_kind == "seq0":
            exps = np.arange(r, dtype=np.uint16)
        elif exps_kind == "seq1":
            exps = np.arange(1, r + 1, dtype=np.uint16)
        else:
            exps = crng.choice(65535, size=r, replace=False).astype(np.uint16)
        nums = np.arange(n, dtype=np.uint16) if nums_kind == "seq" else crng.choice(32768, size=n, replace=False).astype(np.uint16)
        res = np.zeros((r, S), dtype=np.uint8)
        valid = np.zeros(r, dtype=np.int32)
        sec = ctypes.c_double()
        rc = R.ref_create(P(x), P(lens), P(nums), n, S, P(exps), r, P(res), P(valid), 0, 0, 0, ctypes.byref(sec))
        assert rc == 0 and valid.all(), (name, rc, valid)
        entry = {"name": name, "seed": seed, "n": n, "slice": S, "lens": [int(v) for v in lens],
                 "nums": [int(v) for v in nums], "exps": [int(v) for v in exps],
                 "method": R.ref_last_method_name().decode(),
                 "md5": [hashlib.md5(res[j].tobytes()).hexdigest() for j in range(r)]}
        if S * r <= 256:
            entry["hex"] = [res[j].tobytes().hex() for j in range(r)]
        out["recovery"].append(entry)

    # custom-coefficient path: PAR2Proc::addInput(buf, size, coeffs, flush)
    x, lens = case_inputs(21, 6, 3000, True)
    crng = np.random.default_rng(21)
    coeffs = crng.integers(0, 65536, size=(6, 5), dtype=np.uint16)  # [input][rec]
    res = np.zeros((5, 3000), dtype=np.uint8)
    valid = np.zeros(5, dtype=np.int32)
    assert R.ref_create_coeffs(P(x), P(lens), P(np.ascontiguousarray(coeffs)), 6, 3000, 5, P(res), P(valid), 0) == 0
    out["recovery_coeffs"] = {"seed": 21, "n": 6, "slice": 3000, "lens": [int(v) for v in lens],
                              "coeffs_in_rec": coeffs.tolist(),
                              "md5": [hashlib.md5(res[j].tobytes()).hexdigest() for j in range(5)]}

    for k, (srcLen, sliceLen) in enumerate(CKSUM_CASES):
        src = synth.slice_bytes(500 + k, 0, srcLen) if srcLen else np.zeros(0, np.uint8)
        dst = np.zeros(sliceLen + 8, dtype=np.uint8)
        R.ref_cksum_copy(P(dst), P(src), srcLen, sliceLen)
        out["cksum"].append({"seed": 500 + k, "src_len": srcLen, "slice_len": sliceLen,
                             "cksum": dst[sliceLen:].tobytes().hex()})

    for name, seed, ln, S, feed in HASH_CASES:
        data = synth.slice_bytes(seed, 0, ln)
        ns = (ln + S - 1) // S
        ifsc = np.zeros(ns * 20, dtype=np.uint8)
        fm = np.zeros(16, dtype=np.uint8)
        R.ref_hash_file(P(data), ln, S, feed, P(ifsc), P(fm))
        out["hash"].append({"name": name, "seed": seed, "len": ln, "slice": S,
                            "ifsc": ifsc.tobytes().hex(), "file_md5": fm.tobytes().hex()})

    for k, (n, ln) in enumerate([(1, 100), (3, 4096), (7, 65536 + 20), (16, 1000)]):
        bufs = synth.slices(900 + k, 0, n, ln)
        ptrs = (ctypes.c_void_p * n)(*[bufs[j].ctypes.data for j in range(n)])
        md5s = np.zeros(16 * n, dtype=np.uint8)
        R.ref_md5multi(ctypes.cast(ptrs, ctypes.c_void_p), n, ln, P(md5s))
        out["md5multi"].append({"seed": 900 + k, "n": n, "len": ln, "md5": md5s.tobytes().hex()})

    with open(os.path.join(ROOT, "tests", "golden", "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote golden.json:", len(out["recovery"]), "recovery cases")


if __name__ == "__main__":
    main()
