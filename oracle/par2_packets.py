"""ORACLE — test infrastructure, not product code: the finished .par2 files of a
create, restated from the reference's JavaScript independently of the
product's packet module (parpar_gb300/par2packets.py, parpar_gb300/create.py).

Everything data-dependent comes from the oracle (oracle/par2_oracle.c: IFSC
entries, file MD5s, recovery slices, all pinned to the compiled reference) or
from hashlib (packet MD5s, file IDs, MD5 of the first 16 KiB); the layout rules
are restated from lib/par2gen.js, the packet bytes from lib/par2.js, and the
parser from test/par-compare.js.  Only tests/ import it.

  packet header / MD5 ............. lib/par2.js:475-495 (_writePktHeader)
  file ID ......................... lib/par2.js:694-709 (_setId)
  set order of files .............. lib/par2.js:61-66, 412-427 (BufferCompareReverse)
  Main packet / set ID ............ lib/par2.js:429-445
  FileDesc (+ UniFileN) ........... lib/par2.js:760-825
  IFSC ............................ lib/par2.js:755-764
  Creator ......................... lib/par2.js:539-556
  RecvSlic ........................ lib/par2.js:506-520
  display names ('common') ........ lib/par2gen.js:727-756
  critical packet list ............ lib/par2gen.js:769-781
  pow2 volumes .................... lib/par2gen.js:790-827
  packets of one file (_rfPush) ... lib/par2gen.js:920-977
  volume names (par2Ext) .......... lib/par2gen.js:1501-1519
  parser .......................... test/par-compare.js:48-133
"""
from __future__ import annotations

import hashlib
import math
import os
import struct

import numpy as np

from . import oracle as O

MAGIC = b"PAR2\0PKT"


def _u64(v: int) -> bytes:
    return struct.pack("<Q", v)


def _ceil4(n: int) -> int:
    return (n + 3) // 4 * 4


def _js_round(x: float) -> int:
    # JavaScript Math.round: halves go up
    return int(math.floor(x + 0.5))


def make_packet(set_id: bytes, ptype: bytes, body: bytes) -> bytes:
    """64-byte header + body: magic, u64 length, MD5 over bytes 32.., set ID, type."""
    assert len(ptype) == 16 and len(body) % 4 == 0
    rest = set_id + ptype + body
    return MAGIC + _u64(64 + len(body)) + hashlib.md5(rest).digest() + rest


def file_id(md5_16k: bytes, size: int, display_name: str) -> bytes:
    return hashlib.md5(md5_16k + _u64(size) + display_name.encode("utf-8")).digest()


def set_order(ids):
    """Indices of `ids` in set order: Buffer.compare of the byte-reversed IDs."""
    return sorted(range(len(ids)), key=lambda i: bytes(reversed(ids[i])))


def display_names(paths):
    """'common' display names: paths relative to the deepest directory that
    holds every file, '/' separated."""
    full = [os.path.abspath(p) for p in paths]
    root = None
    for f in full:
        d = os.path.dirname(os.path.normpath(f)).split(os.sep)
        if root is None:
            root = d
        else:
            i = 0
            while i < len(root) and i < len(d) and root[i] == d[i]:
                i += 1
            root = root[:i]
    if not root:
        return [os.path.basename(f) for f in full]
    if root[-1] == "":
        root = root[:-1]
    strip = len(os.sep.join(root)) + 1
    return [f[strip:].replace(os.sep, "/") for f in full]


class FileFacts:
    """One input file as the reference sees it."""

    def __init__(self, data: bytes, display_name: str, slice_size: int):
        self.data = data
        self.size = len(data)
        self.name = display_name
        self.md5_16k = hashlib.md5(data[:16384]).digest()
        self.id = file_id(self.md5_16k, self.size, display_name)
        self.num_slices = (self.size + slice_size - 1) // slice_size
        if self.size:
            ifsc, md5 = O.hash_file(np.frombuffer(data, dtype=np.uint8), slice_size)
            self.ifsc, self.md5 = ifsc, md5
        else:
            self.ifsc, self.md5 = b"", hashlib.md5(b"").digest()


def _unicode(name: str) -> bool:
    return any(ord(c) >= 0x80 for c in name)


def filedesc_packets(set_id: bytes, f: FileFacts) -> bytes:
    """FileDesc, followed by UniFileN when the name is not ASCII (the
    addon's automatic unicode choice)."""
    raw = f.name.encode("utf-8")
    body = f.id + f.md5 + f.md5_16k + _u64(f.size) + raw + bytes(_ceil4(len(raw)) - len(raw))
    out = make_packet(set_id, b"PAR 2.0\0FileDesc", body)
    if _unicode(f.name):
        u = f.name.encode("utf-16-le")
        out += make_packet(set_id, b"PAR 2.0\0UniFileN", f.id + u + bytes(_ceil4(len(u)) - len(u)))
    return out


def ifsc_packet(set_id: bytes, f: FileFacts) -> bytes:
    return make_packet(set_id, b"PAR 2.0\0IFSC\0\0\0\0", f.id + f.ifsc)


def creator_packet(set_id: bytes, creator: str) -> bytes:
    raw = creator.encode("utf-8")
    return make_packet(set_id, b"PAR 2.0\0Creator\0", raw + bytes(_ceil4(len(raw)) - len(raw)))


def recovery_packet(set_id: bytes, exponent: int, data: bytes) -> bytes:
    return make_packet(set_id, b"PAR 2.0\0RecvSlic", struct.pack("<I", exponent) + data)


def volume_suffix(num_slices: int, offset: int, total: int) -> str:
    if not num_slices:
        return ".par2"
    digits = max(2, len(str(total)))
    return ".vol%s+%s.par2" % (str(offset).zfill(digits), str(num_slices).zfill(digits))


def file_plan(n_crit: int, recovery: int, min_crit: int = 1):
    """[(suffix, [("crit", k) | ("recovery", exponent) | ("creator", None)])]
    for the default options: an index file, pow2 volumes (1, 2, 4, ...
    slices), critical packets repeated max(round(log2 n), 1) times spread
    evenly among a volume's n recovery packets, the creator packet last."""
    plan = []

    def push(n, off):
        if n:
            copies = max(_js_round(math.log(n) / math.log(2)), min_crit)
            crit_num = copies * n_crit
            ratio = crit_num / n
            pk, written = [], 0
            for i in range(n):
                pk.append(("recovery", i + off))
                while written < _js_round(ratio * (i + 1)):
                    pk.append(("crit", written % n_crit))
                    written += 1
        else:
            pk = [("crit", j) for _ in range(min_crit) for j in range(n_crit)]
        pk.append(("creator", None))
        plan.append([volume_suffix(n, off, recovery), pk])

    push(0, 0)
    i, n = 0, 1
    while i < recovery:
        push(min(n, recovery - i), i)
        i += n
        n = min(n * 2, 65535)
    if len(plan) == 1:
        plan[0][0] = ".par2"
    return plan


def expected_files(datas, names, slice_size: int, recovery: int, creator: str, threads: int = 8):
    """{suffix: bytes} of every .par2 file the reference writes for these
    files with default options, `recovery` slices (exponents 0..recovery-1)."""
    files = [FileFacts(d, n, slice_size) for d, n in zip(datas, names)]
    ids = [f.id for f in files]
    order = set_order(ids)
    main_body = _u64(slice_size) + struct.pack("<I", len(files)) + b"".join(ids[i] for i in order)
    set_id = hashlib.md5(main_body).digest()
    main = make_packet(set_id, b"PAR 2.0\0Main\0\0\0\0", main_body)
    crit = []
    for i in order:
        crit.append(filedesc_packets(set_id, files[i]))
        if files[i].size:
            crit.append(ifsc_packet(set_id, files[i]))
    crit.append(main)
    rec = None
    if recovery:
        rows, lens = [], []
        for i in order:
            f = files[i]
            for k in range(f.num_slices):
                chunk = f.data[k * slice_size:(k + 1) * slice_size]
                rows.append(np.frombuffer(chunk + bytes(slice_size - len(chunk)), dtype=np.uint8))
                lens.append(len(chunk))
        rec = O.recover(np.stack(rows), np.array(lens), np.arange(len(rows)), list(range(recovery)), threads=threads)
    cre = creator_packet(set_id, creator)
    out = {}
    for suffix, pk in file_plan(len(crit), recovery):
        parts = []
        for kind, k in pk:
            if kind == "crit":
                parts.append(crit[k])
            elif kind == "recovery":
                parts.append(recovery_packet(set_id, k, rec[k].tobytes()))
            else:
                parts.append(cre)
        out[suffix] = b"".join(parts)
    return out, set_id


def parse(buf: bytes):
    """[(type, id-or-None, body)] of a .par2 file; raises on a bad signature,
    length, set ID mismatch or packet MD5, and requires the packets to cover
    the file exactly."""
    pos, rs_id, out = 0, None, []
    while pos != len(buf):
        if buf[pos:pos + 8] != MAGIC:
            raise ValueError("invalid packet signature @%d" % pos)
        (ln,) = struct.unpack_from("<Q", buf, pos + 8)
        if ln % 4 or ln < 64 or pos + ln > len(buf):
            raise ValueError("invalid packet length @%d" % pos)
        sid = buf[pos + 32:pos + 48]
        if rs_id is None:
            rs_id = sid
        elif sid != rs_id:
            raise ValueError("mismatching recovery set ID @%d" % pos)
        if hashlib.md5(buf[pos + 32:pos + ln]).digest() != buf[pos + 16:pos + 32]:
            raise ValueError("invalid packet MD5 @%d" % pos)
        ptype = buf[pos + 48:pos + 64]
        id_len = 16 if ptype in (b"PAR 2.0\0FileDesc", b"PAR 2.0\0IFSC\0\0\0\0", b"PAR 2.0\0UniFileN") else \
            4 if ptype == b"PAR 2.0\0RecvSlic" else 0
        out.append((ptype, buf[pos + 64:pos + 64 + id_len] if id_len else None, buf[pos + 64:pos + ln]))
        pos += ln
    return out
