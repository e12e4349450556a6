"""Host-side logic that feeds the GPU paths, on CPU: PAR2 packet assembly and
parsing, PAR2 coefficients from input numbers, the job layout of files in
slices, and the HBM pass planner of the batched path."""
import hashlib
import struct

import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import par2packets as P
from parpar_gb300.job import file_layout, par2_coefficients


def test_packet_header_and_parse_roundtrip():
    sid = bytes(range(16))
    body = b"abcd" * 3
    pkt = P.packet(sid, P.T_CREATOR, body)
    assert pkt[:8] == b"PAR2\0PKT" and struct.unpack_from("<Q", pkt, 8)[0] == 64 + len(body)
    assert pkt[16:32] == hashlib.md5(pkt[32:]).digest()
    assert list(P.parse(pkt + pkt)) == [(P.T_CREATOR, sid, body)] * 2
    with pytest.raises(ValueError):
        P.packet(sid, P.T_CREATOR, b"abc")                 # body not a multiple of 4
    bad = bytearray(pkt)
    bad[-1] ^= 1
    with pytest.raises(ValueError, match="MD5"):
        list(P.parse(bytes(bad)))
    with pytest.raises(ValueError, match="magic"):
        list(P.parse(b"X" + pkt[1:]))


def test_main_packet_sorts_ids_as_little_endian_integers():
    ids = [bytes([0] * 15 + [1]), bytes([2] + [0] * 15), bytes([1] + [0] * 15)]
    pkt, sid = P.main_packet(4096, ids)
    (ptype, got_sid, body), = list(P.parse(pkt))
    assert ptype == P.T_MAIN and got_sid == sid == hashlib.md5(body).digest()
    assert struct.unpack_from("<QI", body) == (4096, 3)
    assert [body[12 + 16 * k: 28 + 16 * k] for k in range(3)] == [ids[2], ids[1], ids[0]]


def test_file_id_and_descriptions_with_unicode_name():
    m16, md5 = bytes(16), bytes(range(16, 32))
    fid = P.file_id(m16, 12345, "déjà.bin")
    assert fid == hashlib.md5(m16 + struct.pack("<Q", 12345) + "déjà.bin".encode("utf-8")).digest()
    blob = P.filedesc_packets(b"S" * 16, fid, md5, m16, 12345, "déjà.bin")
    (t1, _, b1), (t2, _, b2) = list(P.parse(blob))
    assert t1 == P.T_DESC and b1[:16] == fid and b1[16:32] == md5 and b1[32:48] == m16
    assert struct.unpack_from("<Q", b1, 48)[0] == 12345 and b1[56:].rstrip(b"\0") == "déjà.bin".encode("utf-8")
    assert t2 == P.T_UNI and b2[16:].decode("utf-16-le").rstrip("\0") == "déjà.bin"
    assert len(list(P.parse(P.filedesc_packets(b"S" * 16, fid, md5, m16, 1, "plain.bin")))) == 1   # ASCII: no UniFileN


def test_recovery_header_matches_full_packet():
    sid, data = b"\x07" * 16, bytes(range(256)) * 4
    full = P.recovery_packet(sid, 513, data)
    assert P.recovery_header(sid, 513, len(data), full[16:32]) + data == full
    pre = P.recovery_prefixes(sid, [513])
    assert hashlib.md5(pre[0].tobytes() + data).digest() == full[16:32]


def test_par2_coefficients_match_oracle():
    nums, exps = [0, 1, 2, 100, 32767], [0, 1, 7, 65534]
    c = par2_coefficients(np.array(nums), exps)
    assert c.shape == (len(exps), len(nums))
    for r, e in enumerate(exps):
        for k, i in enumerate(nums):
            assert int(c[r, k]) == O.coeff(i, e)


def test_file_layout_rows_and_lengths():
    first, lens = file_layout([10, 0, 8192, 8193], 4096)
    assert first.tolist() == [0, 1, 2, 4]
    assert lens.tolist() == [10, 0, 4096, 4096, 4096, 4096, 1]


def test_plan_passes_fits_budget():
    from parpar_gb300 import _lib
    from parpar_gb300.batch import make_job_mix, plan_passes
    jobs = make_job_mix(16, seed=3, n_range=(10, 300), s_range=(64 * 1024, 1 << 20))
    L = _lib.load()
    for budget in (1 << 30, 256 << 20, 64 << 20):
        P_, wins = plan_passes(jobs, budget)
        need = sum((j.N + j.R) * L.par2cuda_row_pitch_bytes(w) for j, w in zip(jobs, wins))
        assert need <= budget
        assert all(w % 64 == 0 and w * P_ >= j.S for j, w in zip(jobs, wins))   # every byte is in some pass


def test_stream_upload_order_staircase():
    """The job stream's copy order from host buffers: every (job, size class)
    once; job 0 whole first; class c of jobs past c before class c+1 of any
    job past c+1; a job's classes in order."""
    from parpar_gb300.stream import JobStream
    for n in range(1, 30):
        for C in range(1, 5):
            o = JobStream.upload_order(n, C)
            assert sorted(o) == [(i, c) for i in range(n) for c in range(C)]
            assert o[:C] == [(0, c) for c in range(C)]
            pos = {u: k for k, u in enumerate(o)}
            for i in range(n):
                assert [pos[i, c] for c in range(C)] == sorted(pos[i, c] for c in range(C))
            for c in range(C - 1):
                for i in range(c + 1, n):
                    for j in range(c + 2, n):
                        assert pos[i, c] < pos[j, c + 1]
