"""PAR2 create from files on disk through the GPU backend: ParPar's PAR2Gen
flow with its default output options, files in, finished .par2 files out.

    create(["a.bin", "b.bin"], slice_size=1 << 20, recovery_slices=100, out_base="set")
      -> ["set.par2", "set.vol00+01.par2", "set.vol01+02.par2", ...]

Stages:
  1. ingest: a reader thread reads the files (largest first), slice by slice,
     into a ring of pinned host buffers; each filled buffer is copied to its
     rows of the resident job (2-D host-to-device copies), overlapping the next
     reads (the role of lib/fileseqreader.js feeding PAR2Gen), and each file's
     MD5 starts on a high-priority stream as soon as its last row is copied;
  2. on the device: MD5 of each file's first 16 KiB (file IDs), then, with the
     input slices numbered in file-ID order, zero padding + checksum, the
     recovery contraction, verification, IFSC entries and file MD5s
     (ResidentJob.run) and the recovery-packet MD5s;
  3. packets (parpar_gb300/par2packets.py) laid out into files as PAR2Gen does
     by default.

Restated from the reference (lib/par2gen.js, lib/par2.js):
  display names, 'common' format .......... par2gen.js:727-756
  input slice numbering by sorted file ID . par2.js:403-425
  critical packet list and order .......... par2gen.js:770-781, 1026-1041
  index file + pow2 recovery volumes ...... par2gen.js:783-803, 918-979
  critical packet repetition (log 2) ...... par2gen.js:924-946, 104-128
  volume names (alternative scheme) ....... par2gen.js:1501-1519
The creator text is this backend's own unless one is passed.  The whole input
must fit the device memory budget (no multi-pass chunking here).
"""
from __future__ import annotations

import math
import os
import queue
import threading
from dataclasses import dataclass

import numpy as np
import torch

from . import par2packets as P
from .job import ResidentJob

DEFAULT_CREATOR = "par2cuda (GB300 PAR2 recovery backend)"

# Pinned host buffers (the ingest ring and the recovery download) are kept
# for later calls: pinning hundreds of MB per call costs more than the work it
# carries.  create() calls run one at a time (the buffers are shared);
# release_pinned() frees them.
_PINNED: dict = {}
_CREATE_LOCK = threading.Lock()


def release_pinned() -> None:
    """Frees the pinned host buffers kept from earlier create() calls."""
    with _CREATE_LOCK:
        _PINNED.clear()


def _pinned(key, rows: int, cols: int) -> torch.Tensor:
    """A pinned host buffer of rows x cols bytes, kept for later calls."""
    n = rows * cols
    t = _PINNED.get(key)
    if t is None or t.numel() < n:
        t = torch.empty(n, dtype=torch.uint8, pin_memory=True)
        _PINNED[key] = t
    return t[:n].view(rows, cols)


def js_round(x: float) -> int:
    """JavaScript Math.round for non-negative values (halves round up)."""
    return int(math.floor(x + 0.5))


def display_names(paths):
    """ParPar's default 'common' display names: each path relative to the
    deepest directory containing all files, '/' separated (par2gen.js:727-756)."""
    full = [os.path.abspath(p) for p in paths]
    common = None
    for f in full:
        d = os.path.dirname(os.path.normpath(f)).split(os.sep)
        if common is None:
            common = d
        else:
            i = 0
            while i < len(common) and i < len(d) and d[i] == common[i]:
                i += 1
            common = common[:i]
    if not common:
        return [os.path.basename(p) for p in paths]
    if common[-1] == "":
        common = common[:-1]
    strip = len(os.sep.join(common)) + 1
    return [f[strip:].replace(os.sep, "/") for f in full]


def volume_name(num_slices: int, slice_offset: int, total_slices: int) -> str:
    """'.volOFFSET+COUNT.par2' (par2gen.js:1501-1519, alternative scheme)."""
    if not num_slices:
        return ".par2"
    digits = max(2, len(str(total_slices)))
    return ".vol%s+%s.par2" % (str(slice_offset).zfill(digits), str(num_slices).zfill(digits))


def pow2_volumes(recovery_slices: int, first_slices: int = 1, max_slices: int = 65535):
    """(slices, first exponent) of every recovery volume: sizes 1, 2, 4, ... up
    to max_slices, the last one holding the rest (par2gen.js:786-799)."""
    out, i, n = [], 0, first_slices or 1
    while i < recovery_slices:
        f = min(n, recovery_slices - i)
        out.append((f, i))
        i += n
        n = min(n * 2, max_slices)
    return out


@dataclass
class OutFile:
    name: str
    packets: list          # ("crit", k) | ("recovery", exponent) | ("creator", None)


def plan_files(out_base: str, n_crit: int, recovery_slices: int, index: bool = True, min_crit: int = 1,
               max_crit: int = 0, first_slices: int = 1, max_slices: int = 65535):
    """Output files and their packet order for ParPar's default options: an
    index file, then pow2 recovery volumes; in a volume of n recovery slices
    the critical packets are repeated max(round(log2 n), min_crit) times,
    spread evenly after the recovery packets, creator last (par2gen.js:918-979)."""
    files = []

    def push(num_slices, offset):
        if num_slices:
            copies = max(js_round(math.log(num_slices) / math.log(2)), min_crit)
            if max_crit:
                copies = min(copies, max_crit)
            crit_num = copies * n_crit
            ratio = crit_num / num_slices
            pk, written = [], 0
            for i in range(num_slices):
                pk.append(("recovery", i + offset))
                while written < js_round(ratio * (i + 1)):
                    pk.append(("crit", written % n_crit))
                    written += 1
        else:
            pk = [("crit", j) for _ in range(min_crit) for j in range(n_crit)]
        pk.append(("creator", None))
        files.append(OutFile(out_base + volume_name(num_slices, offset, recovery_slices), pk))

    if index:
        push(0, 0)
    for n, off in pow2_volumes(recovery_slices, first_slices, max_slices):
        push(n, off)
    if not files:
        raise ValueError("nothing to generate: need an index or at least one recovery slice")
    if len(files) == 1:
        files[0].name = out_base + ".par2"
    return files


def _ingest(paths, sizes, job: ResidentJob, order, on_file=None, buf_rows: int = 32, nbuf: int = 3):
    """Reads the files (in `order`) into their rows of the job through a ring
    of pinned buffers (reader thread), one host-to-device copy per filled
    buffer; on_file(f) runs on the calling thread once the copy holding file
    f's last row has been issued."""
    S = job.S
    bufs = [_pinned(("ring", k), buf_rows, S) for k in range(nbuf)]
    free = [torch.cuda.Event() for _ in range(nbuf)]
    for e in free:
        e.record()
    filled: queue.Queue = queue.Queue(maxsize=nbuf)
    err = []

    def reader():
        try:
            slot, k = 0, 0
            rows, done = [], []          # destination row of each buffered slice, files completed
            for f in order:
                path, size = paths[f], sizes[f]
                n = (size + S - 1) // S
                first = int(job.first_row[f])
                with open(path, "rb", buffering=0) as fh:
                    for j in range(max(n, 1)):
                        if k == 0:
                            free[slot].synchronize()
                            mv = memoryview(bufs[slot].numpy()).cast("B")
                        want = min(S, size - j * S) if size else 0
                        got = 0
                        while got < want:
                            m = fh.readinto(mv[k * S + got: k * S + want])
                            if not m:
                                raise IOError("%s: file shorter than its size" % path)
                            got += m
                        rows.append(first + j)
                        k += 1
                        if j == max(n, 1) - 1:
                            done.append(f)
                        if k == buf_rows:
                            filled.put((slot, rows, done))
                            slot, k, rows, done = (slot + 1) % nbuf, 0, [], []
            if k:
                filled.put((slot, rows, done))
        except Exception as e:   # reported on the main thread
            err.append(e)
        filled.put(None)

    th = threading.Thread(target=reader, daemon=True)
    th.start()
    dst = job.d_in.view(torch.uint8)
    while True:
        item = filled.get()
        if item is None:
            break
        slot, rows, done = item
        # runs of consecutive destination rows -> one 2-D copy each
        a = 0
        while a < len(rows):
            b = a + 1
            while b < len(rows) and rows[b] == rows[b - 1] + 1:
                b += 1
            dst[rows[a]:rows[a] + (b - a), :S].copy_(bufs[slot][a:b], non_blocking=True)
            a = b
        free[slot].record()
        if on_file and done:
            on_file(done)
    th.join()
    if err:
        raise err[0]


def create(paths, slice_size: int, recovery_slices: int, out_base: str, creator: str = DEFAULT_CREATOR,
           names=None, device: int = 0, index: bool = True, stats: dict | None = None):
    """Creates the PAR2 set for `paths`; returns the written file names.
    `stats`, if given, receives the wall-clock time (s) at which each stage
    ended, measured from the call (stages are synchronised to measure them).
    Concurrent calls run one after the other.  Output files are written under
    temporary names and renamed once complete; on an error none is left."""
    with _CREATE_LOCK:
        return _create(paths, slice_size, recovery_slices, out_base, creator, names, device, index, stats)


def _create(paths, slice_size, recovery_slices, out_base, creator, names, device, index, stats):
    import time
    t0 = time.perf_counter()

    def mark(name, sync=None):
        if stats is not None:
            if sync is not None:
                sync.synchronize()
            stats[name] = time.perf_counter() - t0
    if slice_size <= 0 or slice_size % 4:
        raise ValueError("slice size must be a positive multiple of 4")
    if not (0 <= recovery_slices <= 65535):
        raise ValueError("recovery slice count must be 0..65535")
    paths = list(paths)
    sizes = [os.path.getsize(p) for p in paths]
    names = list(names) if names is not None else display_names(paths)
    S = int(slice_size)
    n_in = sum((s + S - 1) // S for s in sizes)
    if n_in > 32768:
        raise ValueError("PAR2 allows at most 32768 input slices (%d needed)" % n_in)
    torch.cuda.set_device(device)   # the job's streams and buffers live on this device
    R = max(recovery_slices, 1)
    job = ResidentJob(S, sizes, list(range(R)), device=device)
    # largest file first: its MD5 chain (the longest serial work) starts as
    # soon as its rows are on the device, while the other files are read
    read_order = sorted(range(len(paths)), key=lambda f: -sizes[f])
    job.file_md5_prepare(read_order)
    launched = [0, 0]                   # [files launched, files complete]

    def on_file(done):                  # file MD5s in launches of >= 5 files
        launched[1] += len(done)
        if launched[1] - launched[0] >= 5:
            job.file_md5_launch(launched[0], launched[1])
            launched[0] = launched[1]
    _ingest(paths, sizes, job, read_order, on_file=on_file)
    job.file_md5_launch(launched[0], len(paths))
    mark("ingest", torch.cuda.current_stream())

    # file IDs from the first 16 KiB, files sorted by ID, slices numbered in that order
    m16 = job.md5_16k()
    mark("md5_16k")
    ids = [P.file_id(m16[f], sizes[f], names[f]) for f in range(len(paths))]
    order = sorted(range(len(paths)), key=lambda f: int.from_bytes(ids[f], "little"))
    nums = np.zeros(job.N, dtype=np.int64)
    off = 0
    for f in order:
        n = (sizes[f] + S - 1) // S
        first = int(job.first_row[f])
        nums[first:first + n] = np.arange(off, off + n)
        off += n
    job.set_input_nums(nums)
    job.run(hashes=True, file_md5=False)   # the current stream waits for the contraction, not the file MD5s
    mark("contraction+ifsc", job.sa)
    if not bool(job.d_flags.all()):
        raise RuntimeError("recovery checksum verification failed")

    # The recovery packets are written while the file MD5 chains still run:
    # every packet's length is known now (the critical packets' contents wait
    # for the file MD5s, their sizes do not), so each file is laid out at
    # once and the recovery packets go to their offsets; the critical packets
    # fill their places when the MD5s are in.
    ifsc = job.d_ifsc.cpu().numpy().reshape(job.N, 20)
    main, set_id = P.main_packet(S, ids)
    zero16 = bytes(16)

    def critical(fmd5_of):
        out = []
        for f in order:
            out.append(P.filedesc_packets(set_id, ids[f], fmd5_of(f), m16[f], sizes[f], names[f]))
            if sizes[f]:
                first = int(job.first_row[f])
                n = (sizes[f] + S - 1) // S
                out.append(P.ifsc_packet(set_id, ids[f], ifsc[first:first + n].tobytes()))
        out.append(main)
        return out

    crit_len = [len(c) for c in critical(lambda f: zero16)]
    creator_pkt = P.creator_packet(set_id, creator)
    plan = plan_files(out_base, len(crit_len), recovery_slices, index=index)
    rec_len = 68 + S
    layouts = []                      # per file: [(offset, kind, k)]
    for of in plan:
        pos, lay = 0, []
        for kind, k in of.packets:
            lay.append((pos, kind, k))
            pos += crit_len[k] if kind == "crit" else (len(creator_pkt) if kind == "creator" else rec_len)
        layouts.append((of.name, pos, lay))
    rec_md5 = job.recovery_packet_md5s(set_id) if recovery_slices else []
    rec_host = _pinned("rec", R, S)
    rec_host.copy_(job.d_rec.view(torch.uint8)[:, :S])
    rec_np = rec_host.numpy()

    def tmp_name(name):
        return name + ".part"

    def write_recovery(item):
        name, total, lay = item
        fd = os.open(tmp_name(name), os.O_WRONLY | os.O_CREAT | os.O_TRUNC, 0o644)
        try:
            os.ftruncate(fd, total)
            for pos, kind, k in lay:
                if kind == "recovery":
                    os.pwrite(fd, P.recovery_header(set_id, k, S, rec_md5[k]), pos)
                    os.pwrite(fd, memoryview(rec_np[k]), pos + 68)
        finally:
            os.close(fd)
        return name

    from concurrent.futures import ThreadPoolExecutor
    try:
        with ThreadPoolExecutor(max_workers=min(8, len(layouts))) as ex:
            written = list(ex.map(write_recovery, layouts))
        mark("recovery written")

        job.file_md5_finish()
        torch.cuda.synchronize()
        mark("file_md5")
        fmd5 = job.d_fmd5.cpu().numpy().reshape(len(paths), 16)
        crit = critical(lambda f: fmd5[f].tobytes())
        if [len(c) for c in crit] != crit_len:
            raise RuntimeError("critical packet sizes changed")
        for name, total, lay in layouts:
            fd = os.open(tmp_name(name), os.O_WRONLY)
            try:
                for pos, kind, k in lay:
                    if kind == "crit":
                        os.pwrite(fd, crit[k], pos)
                    elif kind == "creator":
                        os.pwrite(fd, creator_pkt, pos)
            finally:
                os.close(fd)
        for name in written:
            os.replace(tmp_name(name), name)
    except BaseException:
        for name, _, _ in layouts:
            try:
                os.remove(tmp_name(name))
            except OSError:
                pass
        raise
    mark("written")
    return written
