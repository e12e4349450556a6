"""Files on disk -> finished .par2 files through the GPU backend, compared byte
for byte with the files the oracle's restatement of the reference's writers
builds from the same input bytes (oracle/par2_packets.py: lib/par2.js packet
formats, lib/par2gen.js layout and names, IFSC / file MD5 / recovery data from
the oracle), and parsed with par-compare's packet checks."""
import numpy as np
import pytest

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
    from parpar_gb300.create import create
    from oracle import par2_packets as OP
    paths = _files(tmp_path / "in", sizes, names, seed=S + R)
    creator = "par2cuda test creator"
    base = str(tmp_path / "set")
    out = create(paths, S, R, base, creator=creator)
    data = [open(p, "rb").read() for p in paths]
    # the oracle's restatement of lib/par2.js + lib/par2gen.js, built from the
    # files' bytes alone: every output file byte for byte
    names_ = OP.display_names(paths)
    assert names_ == names
    want, set_id = OP.expected_files(data, names_, S, R, creator)
    assert sorted(out) == sorted(base + sfx for sfx in want)
    for sfx, wbytes in want.items():
        got = open(base + sfx, "rb").read()
        pkts = OP.parse(got)               # par-compare's checks: signature, length, set ID, packet MD5
        assert pkts and len(got) == len(wbytes)
        assert got == wbytes, sfx
