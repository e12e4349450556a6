"""Files on disk -> finished .par2 files through the GPU backend, checked
packet by packet: every packet MD5, the set ID, file IDs and descriptions,
IFSC entries against the oracle's hashes, recovery slices against the oracle
with the inputs numbered in file-ID order, and ParPar's default file layout."""
import hashlib
import struct

import numpy as np
import pytest

from oracle import oracle as O
from parpar_gb300 import par2packets as P

pytestmark = pytest.mark.gpu


def _files(tmp_path, sizes, names, seed):
    rng = np.random.default_rng(seed)
    paths = []
    for n, sz in zip(names, sizes):
        p = tmp_path / n
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_bytes(rng.integers(0, 256, size=sz, dtype=np.uint8).tobytes())
        paths.append(str(p))
    return paths


@pytest.mark.parametrize("S,R,sizes,names", [
    (4100, 10, [10000, 4100, 0, 123457, 40000], ["a.bin", "b.bin", "empty", "sub/c.bin", "déjà.bin"]),
    (65536, 3, [65536 * 5 + 7, 20000], ["x", "y"]),
    (1024, 1, [16384 + 3000], ["only"]),
    (2048, 0, [5000, 9000], ["m", "n"]),
    # par-compare's file sizes with its 65521*4-byte slices and 200 recovery slices
    (65521 * 4, 200, [1, 8, 65521, 13631477], ["f1", "f8", "f65521", "f13631477"]),
    # par-compare's 40000-byte slices with 10000 recovery slices (pow2 volumes up to 4096)
    (40000, 10000, [400000], ["big.bin"]),
])
def test_create_par2_files(tmp_path, S, R, sizes, names):
    pytest.importorskip("torch")
    from parpar_gb300.create import create, plan_files
    paths = _files(tmp_path / "in", sizes, names, seed=S + R)
    out = create(paths, S, R, str(tmp_path / "set"))
    data = [open(p, "rb").read() for p in paths]

    # per-file facts from the bytes themselves and the oracle
    m16 = [hashlib.md5(d[:16384]).digest() for d in data]
    ids = [P.file_id(m16[i], sizes[i], names[i]) for i in range(len(paths))]
    order = sorted(range(len(paths)), key=lambda i: int.from_bytes(ids[i], "little"))
    main_body = struct.pack("<QI", S, len(ids)) + b"".join(ids[i] for i in order)
    set_id = hashlib.md5(main_body).digest()

    # recovery reference: input slices numbered in file-ID order, zero-padded
    rows, lens = [], []
    for i in order:
        for k in range((sizes[i] + S - 1) // S):
            chunk = data[i][k * S:(k + 1) * S]
            rows.append(np.frombuffer(chunk + bytes(S - len(chunk)), dtype=np.uint8))
            lens.append(len(chunk))
    x = np.stack(rows)
    rec = O.recover(x, np.array(lens), np.arange(len(rows)), list(range(R)), threads=8) if R else None

    n_crit = sum(1 + (1 if sizes[i] else 0) for i in range(len(paths))) + 1
    plan = plan_files(str(tmp_path / "set"), n_crit, R)
    assert out == [f.name for f in plan]
    seen_rec = set()
    for of in plan:
        buf = open(of.name, "rb").read()
        pkts = list(P.parse(buf))          # validates every packet MD5 and length
        assert all(sid == set_id for _, sid, _ in pkts)
        kinds = []
        for ptype, _, body in pkts:
            if ptype == P.T_RECV:
                e = struct.unpack_from("<I", body)[0]
                assert body[4:] == rec[e].tobytes()
                seen_rec.add(e)
                kinds.append("R")
            elif ptype == P.T_DESC:
                fid = body[:16]
                i = ids.index(fid)
                assert body[16:32] == hashlib.md5(data[i]).digest()
                assert body[32:48] == m16[i]
                assert struct.unpack_from("<Q", body, 48)[0] == sizes[i]
                assert body[56:].rstrip(b"\0") == names[i].encode("utf-8")
                kinds.append("d")
            elif ptype == P.T_UNI:
                i = ids.index(body[:16])
                assert body[16:].decode("utf-16-le").rstrip("\0") == names[i]
            elif ptype == P.T_IFSC:
                i = ids.index(body[:16])
                ifsc, _ = O.hash_file(np.frombuffer(data[i], dtype=np.uint8), S)
                assert body[16:] == ifsc
                kinds.append("i")
            elif ptype == P.T_MAIN:
                assert body == main_body
                kinds.append("m")
            elif ptype == P.T_CREATOR:
                kinds.append("C")
            else:
                raise AssertionError(ptype)
        # the layout: critical packets in file-ID order (desc, ifsc), main last
        crit_seq = []
        for i in order:
            crit_seq.append("d")
            if sizes[i]:
                crit_seq.append("i")
        crit_seq.append("m")
        want = []
        for kind, k in of.packets:
            want.append("R" if kind == "recovery" else ("C" if kind == "creator" else crit_seq[k]))
        assert kinds == want
    assert seen_rec == set(range(R))
