"""PAR2 packet assembly for a create job (the packets ParPar's lib/par2.js writes).

Packet layout (PAR2 2.0): 64-byte header
    magic "PAR2\\0PKT" | u64 length | MD5 of bytes 32..end | recovery set ID | 16-byte type
followed by the body (length a multiple of 4).  Bodies, as lib/par2.js builds them:
    Main      u64 slice size, u32 file count, file IDs sorted as little-endian
              128-bit integers (lib/par2.js:403-447); set ID = MD5(main body)
    FileDesc  file ID, file MD5, MD5 of the first 16 KiB, u64 size, name padded
              to 4 bytes (lib/par2.js:754-793)
    IFSC      file ID, then MD5(16) + CRC32(4 LE) per slice (lib/par2.js:737-753)
    RecvSlic  u32 exponent + the recovery slice (lib/par2.js:486-520)
    Creator   ASCII text padded to 4 bytes (lib/par2.js:539-556)
    UniFileN  file ID + UTF-16LE name (written when the name is not ASCII)
    file ID = MD5(MD5-16k || u64 size || name bytes) (lib/par2.js:696-709)

The data-dependent hashes come from the GPU (IFSC entries and file MD5s from
the resident job; recovery-packet MD5s from par2cuda_rows_md5 over the
recovery rows with each packet's 36-byte header prefix); this module only
assembles bytes.
"""
from __future__ import annotations

import hashlib
import struct

import numpy as np

MAGIC = b"PAR2\0PKT"
T_MAIN = b"PAR 2.0\0Main\0\0\0\0"
T_DESC = b"PAR 2.0\0FileDesc"
T_IFSC = b"PAR 2.0\0IFSC\0\0\0\0"
T_RECV = b"PAR 2.0\0RecvSlic"
T_CREATOR = b"PAR 2.0\0Creator\0"
T_UNI = b"PAR 2.0\0UniFileN"


def _pad4(b: bytes) -> bytes:
    return b + bytes((-len(b)) % 4)


def packet(set_id: bytes, ptype: bytes, body: bytes) -> bytes:
    if len(body) % 4:
        raise ValueError("packet body length must be a multiple of 4")
    tail = set_id + ptype + body
    return MAGIC + struct.pack("<Q", 64 + len(body)) + hashlib.md5(tail).digest() + tail


def file_id(md5_16k: bytes, size: int, name: str) -> bytes:
    return hashlib.md5(md5_16k + struct.pack("<Q", size) + name.encode("utf-8")).digest()


def sort_file_ids(ids):
    """Ascending as little-endian 128-bit integers (lib/par2.js:417-419)."""
    return sorted(ids, key=lambda x: int.from_bytes(x, "little"))


def main_packet(slice_size: int, file_ids):
    ids = sort_file_ids(file_ids)
    body = struct.pack("<QI", slice_size, len(ids)) + b"".join(ids)
    set_id = hashlib.md5(body).digest()
    return packet(set_id, T_MAIN, body), set_id


def filedesc_packets(set_id: bytes, fid: bytes, md5: bytes, md5_16k: bytes, size: int, name: str) -> bytes:
    raw = name.encode("utf-8")
    out = packet(set_id, T_DESC, fid + md5 + md5_16k + struct.pack("<Q", size) + _pad4(raw))
    if any(ord(c) > 127 for c in name):
        out += packet(set_id, T_UNI, fid + _pad4(name.encode("utf-16-le")))
    return out


def ifsc_packet(set_id: bytes, fid: bytes, entries: bytes) -> bytes:
    if len(entries) % 20:
        raise ValueError("IFSC entries are 20 bytes each")
    return packet(set_id, T_IFSC, fid + entries)


def creator_packet(set_id: bytes, text: str) -> bytes:
    return packet(set_id, T_CREATOR, _pad4(text.encode("ascii")))


def recovery_prefixes(set_id: bytes, exps) -> np.ndarray:
    """The 36 bytes of each recovery packet that precede its data in the packet
    MD5 (set ID, type, exponent): input for par2cuda_rows_md5."""
    head = set_id + T_RECV
    return np.frombuffer(b"".join(head + struct.pack("<I", int(e)) for e in exps), dtype=np.uint8).reshape(len(exps), 36).copy()


def recovery_header(set_id: bytes, exponent: int, data_len: int, md5: bytes) -> bytes:
    """The 68 bytes of a RecvSlic packet before its data (`md5` from the GPU)."""
    return MAGIC + struct.pack("<Q", 64 + 4 + data_len) + md5 + set_id + T_RECV + struct.pack("<I", exponent)


def recovery_packet(set_id: bytes, exponent: int, data: bytes, md5: bytes | None = None) -> bytes:
    """RecvSlic packet; `md5` (from the GPU) must equal MD5(prefix || data)."""
    tail = set_id + T_RECV + struct.pack("<I", exponent) + data
    if md5 is None:
        md5 = hashlib.md5(tail).digest()
    return MAGIC + struct.pack("<Q", 64 + 4 + len(data)) + md5 + tail


def parse(buf: bytes):
    """Yields (type, set_id, body) for every packet; raises on a bad magic,
    length or packet MD5."""
    pos = 0
    while pos < len(buf):
        if buf[pos:pos + 8] != MAGIC:
            raise ValueError("bad magic at %d" % pos)
        (ln,) = struct.unpack_from("<Q", buf, pos + 8)
        if ln < 64 or ln % 4 or pos + ln > len(buf):
            raise ValueError("bad length at %d" % pos)
        if hashlib.md5(buf[pos + 32:pos + ln]).digest() != buf[pos + 16:pos + 32]:
            raise ValueError("bad packet MD5 at %d" % pos)
        yield buf[pos + 48:pos + 64], buf[pos + 32:pos + 48], buf[pos + 64:pos + ln]
        pos += ln


def index_file(slice_size: int, files, creator: str = "par2cuda (GB300 PAR2 recovery backend)"):
    """files: list of dicts {name, size, md5, md5_16k, ifsc}.  Returns
    (index .par2 bytes, set ID, file IDs in set order)."""
    ids = [file_id(f["md5_16k"], f["size"], f["name"]) for f in files]
    main, set_id = main_packet(slice_size, ids)
    order = sort_file_ids(ids)
    by_id = dict(zip(ids, files))
    out = [main]
    for fid in order:
        f = by_id[fid]
        out.append(filedesc_packets(set_id, fid, f["md5"], f["md5_16k"], f["size"], f["name"]))
        if f["size"]:
            out.append(ifsc_packet(set_id, fid, f["ifsc"]))
    out.append(creator_packet(set_id, creator))
    return b"".join(out), set_id, order
