"""CPU checks of the oracle's restatement of the .par2 writers
(oracle/par2_packets.py): layout, names, packet framing and the parser."""
import hashlib
import struct

import numpy as np

from oracle import par2_packets as OP


def test_volume_names_follow_par2ext():
    assert OP.volume_suffix(0, 0, 10) == ".par2"
    assert OP.volume_suffix(2, 1, 3) == ".vol01+02.par2"
    assert OP.volume_suffix(4096, 5903, 10000) == ".vol05903+04096.par2"


def test_file_plan_pow2_and_critical_repetition():
    # index only
    plan = OP.file_plan(3, 0)
    assert plan == [[".par2", [("crit", 0), ("crit", 1), ("crit", 2), ("creator", None)]]]
    plan = OP.file_plan(2, 7)
    assert [p[0] for p in plan] == [".par2", ".vol00+01.par2", ".vol01+02.par2", ".vol03+04.par2"]
    # 4 slices: round(log2 4) = 2 copies of 2 critical packets spread one per slice
    assert plan[3][1] == [("recovery", 3), ("crit", 0), ("recovery", 4), ("crit", 1), ("recovery", 5), ("crit", 0),
                          ("recovery", 6), ("crit", 1), ("creator", None)]
    # 1 slice: max(round(log2 1), 1) = 1 copy
    assert plan[1][1] == [("recovery", 0), ("crit", 0), ("crit", 1), ("creator", None)]


def test_set_order_compares_reversed_ids():
    a = bytes(range(16))
    b = bytes([255] + [0] * 15)          # bigger first byte, smaller last byte
    assert OP.set_order([a, b]) == [1, 0]


def test_expected_files_parse_and_framing():
    rng = np.random.default_rng(1)
    datas = [rng.integers(0, 256, size=n, dtype=np.uint8).tobytes() for n in (5000, 0, 1234)]
    names = ["x.bin", "empty", "ünï"]
    files, set_id = OP.expected_files(datas, names, 1024, 3, "creator")
    assert sorted(files) == [".par2", ".vol00+01.par2", ".vol01+02.par2"]
    pk = OP.parse(files[".par2"])
    types = [t for t, _, _ in pk]
    # three FileDesc (one with its UniFileN), two IFSC (the empty file has none), Main, Creator
    assert types.count(b"PAR 2.0\0FileDesc") == 3 and types.count(b"PAR 2.0\0UniFileN") == 1
    assert types.count(b"PAR 2.0\0IFSC\0\0\0\0") == 2 and types[-2:] == [b"PAR 2.0\0Main\0\0\0\0", b"PAR 2.0\0Creator\0"]
    main = [b for t, _, b in pk if t == b"PAR 2.0\0Main\0\0\0\0"][0]
    assert hashlib.md5(main).digest() == set_id
    assert struct.unpack_from("<QI", main) == (1024, 3)
    rec = [b for t, _, b in OP.parse(files[".vol01+02.par2"]) if t == b"PAR 2.0\0RecvSlic"]
    assert [struct.unpack_from("<I", b)[0] for b in rec] == [1, 2] and all(len(b) == 4 + 1024 for b in rec)
