"""Device-resident PAR2 create job: one read pass over slices held in HBM.

A job is the unit of work of PAR2Gen's single-pass create (lib/par2gen.js:
1198-1330): N input slices of S bytes (the last slice of each file shorter,
zero-padded), R recovery exponents, and the per-slice / per-file hashes.  The
slices are staged once into HBM rows (par2cuda_row_pitch_bytes apart); then,
on two streams that read the same rows:

  stream A: zero padding + internal checksum of every input row,
            multiply-accumulate into the R recovery rows (comb kernel),
            checksum verification of every recovery row, IFSC entries
            (MD5+CRC32 per slice, one thread per slice);
  stream B: the file MD5s (one thread per file).

All device work goes through libpar2cuda.so's C ABI; torch is used only for
device memory, streams and events.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .layout import file_layout  # noqa: F401  (re-exported)


def par2_coefficients(input_nums, exps) -> np.ndarray:
    """[R][N] uint16 PAR2 coefficients (gfmat_coeff), from the library."""
    L = _lib.load()
    nums = np.asarray(input_nums)
    out = np.empty((len(exps), len(nums)), dtype=np.uint16)
    # 2^(log_i * e) via the library's per-pair helper would be N*R calls; use
    # the log/exp form with tables built from one call per input and exponent
    logs = np.array([_input_log(L, int(i)) for i in nums], dtype=np.int64)
    expt = _exp_table()
    e = np.asarray(exps, dtype=np.int64)
    out[:] = expt[(e[:, None] * logs[None, :]) % 65535]
    return out


_EXP = None


def _exp_table():
    global _EXP
    if _EXP is None:
        t = np.empty(65535, dtype=np.uint16)
        n = 1
        for i in range(65535):
            t[i] = n
            n <<= 1
            if n & 0x10000:
                n ^= 0x1100B
        _EXP = t
    return _EXP


_LOGS = None


def _input_log(L, i):
    # log_i: coefficient of input i for exponent 1 is 2^log_i
    global _LOGS
    if _LOGS is None:
        exp = _exp_table()
        log = np.zeros(65536, dtype=np.int64)
        log[exp] = np.arange(65535)
        _LOGS = np.array([log[L.par2cuda_coeff(k, 1)] for k in range(32768)], dtype=np.int64)
    return int(_LOGS[i])


class ResidentJob:
    """One PAR2 create job with its input rows resident on the current device."""

    def __init__(self, slice_size: int, file_lens, exps, input_nums=None, method: int = _lib.METHOD_COMB,
                 device: int = 0, stream_a=None, stream_b=None):
        self.L = _lib.load()
        self.S = int(slice_size)
        self.file_lens = [int(x) for x in file_lens]
        self.first_row, self.row_lens = file_layout(self.file_lens, self.S)
        self.N = len(self.row_lens)
        self.exps = list(exps)
        self.R = len(self.exps)
        self.input_nums = np.arange(self.N) if input_nums is None else np.asarray(input_nums)
        self.method = method
        self.pitch = self.L.par2cuda_row_pitch_bytes(self.S)
        self.pw = self.pitch // 2
        self.n_words = self.pitch // 2  # full rows: data + checksum block (+ pitch padding)
        self.row_words = ((self.S + 7) // 8 * 8 + 8) // 2
        dev = torch.device("cuda", device)
        self.dev = dev
        self.d_in = torch.empty((self.N, self.pw), dtype=torch.int16, device=dev)
        self.d_rec = torch.empty((self.R, self.pw), dtype=torch.int16, device=dev)
        coeff = par2_coefficients(self.input_nums, self.exps)
        self.d_coeff = torch.from_numpy(coeff.view(np.int16)).to(dev)
        self.d_lens = torch.from_numpy(self.row_lens.view(np.int32)).to(dev)
        self.d_flen = torch.tensor(self.file_lens, dtype=torch.int64, device=dev)
        self.d_first = torch.from_numpy(self.first_row.view(np.int32)).to(dev)
        self.scratch_bytes = self.L.par2cuda_muladd_scratch_bytes(self.R, self.N)
        if method == _lib.METHOD_TENSOR_FP4:
            self.scratch_bytes = self.L.par2cuda_tensor_fp4_scratch_bytes(self.R, self.N, self.row_words)
        self.d_scratch = torch.empty(max(self.scratch_bytes, 256), dtype=torch.uint8, device=dev)
        self.d_ck = torch.empty(max(self.N, self.R) * 8, dtype=torch.uint8, device=dev)
        self.d_flags = torch.empty(self.R, dtype=torch.uint8, device=dev)
        self.d_ifsc = torch.empty(self.N * 20, dtype=torch.uint8, device=dev)
        self.d_fmd5 = torch.empty(len(self.file_lens) * 16, dtype=torch.uint8, device=dev)
        self.sa = stream_a or torch.cuda.Stream(device=dev)
        # the per-file MD5 chains run for the whole job on a few threads: their
        # stream gets the highest priority so that their CTAs are dispatched as
        # soon as an SM frees, ahead of pending multiply-accumulate CTAs of
        # other jobs in flight
        self.sb = stream_b or torch.cuda.Stream(device=dev, priority=-10)
        # checksum (2), the multiply-accumulate, verification (2), IFSC, file MD5
        self.launches_per_run = 6 + self.L.par2cuda_muladd_launches(self.R, self.N, self.row_words, method,
                                                                    self.scratch_bytes)

    def set_input_nums(self, input_nums):
        """PAR2 input number of every row (e.g. once the file order by file ID
        is known); the coefficients follow from them and the exponents."""
        self.input_nums = np.asarray(input_nums)
        coeff = par2_coefficients(self.input_nums, self.exps)
        self.d_coeff = torch.from_numpy(coeff.view(np.int16)).to(self.dev)

    # -------------------------------------------------------------- inputs
    def fill_synthetic(self, seed: int):
        """Seeded rows (parpar_gb300.synth layout); bytes past each row's length are
        left for the zero-padding step of run()."""
        _lib.check(self.L.par2cuda_synth_fill(self.d_in.data_ptr(), self.pitch, self.N, self.S, seed, 0,
                                             torch.cuda.current_stream(self.dev).cuda_stream), "synth")

    def upload(self, host_rows: torch.Tensor, stream=None):
        """H2D of host rows [N, S] (pinned for an asynchronous copy) into the resident rows."""
        st = stream or torch.cuda.current_stream(self.dev)
        with torch.cuda.stream(st):
            self.d_in.view(torch.uint8)[:, : self.S].copy_(host_rows, non_blocking=True)
        return self.N * self.S

    # -------------------------------------------------------------- compute
    def file_md5_prepare(self, order, max_launches: int = 64):
        """Sets up file MD5 launches issued while the rows arrive: files are
        taken in `order` (the read order), so each launch covers a contiguous
        range of it.  Device arrays and streams are made here, before the
        rows are copied, so that a launch is a bare C-ABI call."""
        order = [int(f) for f in order]
        if getattr(self, "_ro", None) == order:
            self._md5_used = 0
            return
        self._ro = order
        self._ro_flen = torch.tensor([self.file_lens[f] for f in order], dtype=torch.int64, device=self.dev)
        self._ro_first = torch.tensor([int(self.first_row[f]) for f in order], dtype=torch.int32, device=self.dev)
        self._ro_out = torch.empty(16 * max(len(order), 1), dtype=torch.uint8, device=self.dev)
        self._ro_idx = torch.tensor(order, dtype=torch.int64, device=self.dev)
        self._md5_streams = [torch.cuda.Stream(device=self.dev, priority=-10) for _ in range(max_launches)]
        self._md5_used = 0
        torch.cuda.current_stream(self.dev).synchronize()

    def file_md5_launch(self, a: int, b: int):
        """MD5 of the files at read-order positions [a, b) as one launch on
        its own high-priority stream, ordered after the work already issued on
        the current stream (the copies of their rows).  Several files per
        launch: measured on GB300, one launch per file ran each chain at half
        speed (40 single-file launches 3.0 s vs 1.59 s), while launches of 5 or
        more files ran at full speed."""
        if b <= a:
            return
        st = self._md5_streams[self._md5_used % len(self._md5_streams)]
        self._md5_used += 1
        st.wait_stream(torch.cuda.current_stream(self.dev))
        _lib.check(self.L.par2cuda_file_md5(self.d_in.data_ptr(), self.pitch, b - a, self._ro_flen.data_ptr() + 8 * a,
                                           self._ro_first.data_ptr() + 4 * a, self.S,
                                           self._ro_out.data_ptr() + 16 * a, st.cuda_stream), "file_md5")

    def file_md5_finish(self):
        """Joins the launches of file_md5_launch and stores the digests in
        file order (the current stream waits for them)."""
        cur = torch.cuda.current_stream(self.dev)
        for st in self._md5_streams:
            cur.wait_stream(st)
        self.d_fmd5.view(-1, 16).index_copy_(0, self._ro_idx, self._ro_out.view(-1, 16)[: len(self._ro)])

    def run_from_host(self, host_rows: torch.Tensor, hashes: bool = True, group: int = 5):
        """upload() + run() with the copies and the file MD5s overlapped: files
        are copied largest first, one 2-D copy per file, and the MD5 chains of
        every `group` completed files start at once on their own streams
        (the longest chain starts after the first file's copy instead of after
        the whole upload).  host_rows: pinned [N, S] rows in row order."""
        order = sorted(range(len(self.file_lens)), key=lambda f: -self.file_lens[f])
        if hashes:
            self.file_md5_prepare(order)
        dst = self.d_in.view(torch.uint8)
        done = launched = 0
        for f in order:
            a = int(self.first_row[f])
            n = max(1, (self.file_lens[f] + self.S - 1) // self.S)
            dst[a:a + n, : self.S].copy_(host_rows[a:a + n], non_blocking=True)
            done += 1
            if hashes and done - launched >= group:
                self.file_md5_launch(launched, done)
                launched = done
        if hashes:
            self.file_md5_launch(launched, done)
        self.run(hashes=hashes, file_md5=False)
        if hashes:
            self.file_md5_finish()

    def run(self, hashes: bool = True, file_md5: bool = True, packed_md5: bool = False):
        """Issues the whole job on streams A and B (asynchronous); file_md5 =
        False when the file MD5s were already launched (file_md5_launch);
        packed_md5 packs the file MD5 chains 32 per warp (several jobs in
        flight: the chains then leave the other SMs to the other jobs)."""
        L = self.L
        cur = torch.cuda.current_stream(self.dev)
        self.sa.wait_stream(cur)
        self.sb.wait_stream(cur)
        a = self.sa.cuda_stream
        b = self.sb.cuda_stream
        # A: zero padding + checksum of the inputs, then the mul-add, then verification
        _lib.check(L.par2cuda_rows_checksum(self.d_in.data_ptr(), self.pw, self.N, self.d_lens.data_ptr(), self.S, 0,
                                           None, self.d_ck.data_ptr(), a), "rows_checksum")
        if hashes and file_md5:
            # the file MD5s (long serial chains) start at once on B: they read
            # only each file's own bytes, not the padding A writes
            md5 = L.par2cuda_file_md5_packed if packed_md5 else L.par2cuda_file_md5
            _lib.check(md5(self.d_in.data_ptr(), self.pitch, len(self.file_lens), self.d_flen.data_ptr(),
                           self.d_first.data_ptr(), self.S, self.d_fmd5.data_ptr(), b), "file_md5")
        _lib.check(L.par2cuda_muladd(self.d_in.data_ptr(), self.pw, self.N, self.d_coeff.data_ptr(), self.d_rec.data_ptr(),
                                    self.pw, self.R, self.row_words, 0, self.method, self.d_scratch.data_ptr(),
                                    self.scratch_bytes, a), "muladd")
        _lib.check(L.par2cuda_rows_checksum(self.d_rec.data_ptr(), self.pw, self.R, None, self.S, 1,
                                           self.d_flags.data_ptr(), self.d_ck.data_ptr(), a), "verify")
        if hashes:
            _lib.check(L.par2cuda_slice_hash(self.d_in.data_ptr(), self.pitch, self.N, self.d_lens.data_ptr(), self.S,
                                            self.d_ifsc.data_ptr(), a), "slice_hash")
        cur.wait_stream(self.sa)
        cur.wait_stream(self.sb)

    # -------------------------------------------------------------- results
    def download(self, rec_host: torch.Tensor | None = None, stream=None):
        """D2H of recovery slices, IFSC entries, file MD5s and checksum verdicts
        (asynchronous on `stream`).  IFSC, MD5s and verdicts land in pinned
        buffers owned by the job and reused by the next call: synchronise
        `stream` before reading them, and copy them (e.g. .clone()) before
        calling download() again if they are to be kept."""
        st = stream or torch.cuda.current_stream(self.dev)
        if not hasattr(self, "_h_small"):
            # pinned host buffers made once: allocating pinned memory per call
            # can synchronise the device and stall the next job's launches
            self._h_small = (torch.empty_like(self.d_ifsc, device="cpu", pin_memory=True),
                             torch.empty_like(self.d_fmd5, device="cpu", pin_memory=True),
                             torch.empty_like(self.d_flags, device="cpu", pin_memory=True))
        ifsc, fmd5, flags = self._h_small
        with torch.cuda.stream(st):
            if rec_host is None:
                rec_host = torch.empty((self.R, self.S), dtype=torch.uint8, pin_memory=True)
            rec_host.copy_(self.d_rec.view(torch.uint8)[:, : self.S], non_blocking=True)
            ifsc.copy_(self.d_ifsc, non_blocking=True)
            fmd5.copy_(self.d_fmd5, non_blocking=True)
            flags.copy_(self.d_flags, non_blocking=True)
        return rec_host, ifsc, fmd5, flags

    # -------------------------------------------------------------- PAR2 packets
    def md5_16k(self) -> list:
        """MD5 of the first 16 KiB of every file (the FileDesc / file ID hash),
        on the device: one thread per file over its first row(s)."""
        L = self.L
        out = [None] * len(self.file_lens)
        st = torch.cuda.current_stream(self.dev).cuda_stream
        groups = {}
        for f, ln in enumerate(self.file_lens):
            groups.setdefault(min(16384, ln), []).append(f)
        for n, files in groups.items():
            if n > self.S:
                # the first 16 KiB span several rows: hash them as one stream
                flen = torch.tensor([n] * len(files), dtype=torch.int64, device=self.dev)
                first = torch.tensor([int(self.first_row[f]) for f in files], dtype=torch.int32, device=self.dev)
                d = torch.empty(16 * len(files), dtype=torch.uint8, device=self.dev)
                _lib.check(L.par2cuda_file_md5(self.d_in.data_ptr(), self.pitch, len(files), flen.data_ptr(),
                                              first.data_ptr(), self.S, d.data_ptr(), st), "md5_16k")
            else:
                rows = self.d_in[torch.tensor([int(self.first_row[f]) for f in files], device=self.dev)].contiguous()
                d = torch.empty(16 * len(files), dtype=torch.uint8, device=self.dev)
                _lib.check(L.par2cuda_rows_md5(rows.data_ptr(), self.pitch, len(files), n, None, 0, d.data_ptr(), st),
                           "md5_16k")
            h = d.cpu().numpy().reshape(len(files), 16)
            for k, f in enumerate(files):
                out[f] = h[k].tobytes()
        return out

    def recovery_packet_md5s(self, set_id: bytes):
        """Packet MD5 of every recovery slice packet (MD5 over set ID, type,
        exponent and the slice), one GPU thread per recovery row."""
        from .par2packets import recovery_prefixes
        pre = torch.from_numpy(np.ascontiguousarray(recovery_prefixes(set_id, self.exps))).to(self.dev)
        d = torch.empty(16 * self.R, dtype=torch.uint8, device=self.dev)
        _lib.check(self.L.par2cuda_rows_md5(self.d_rec.data_ptr(), self.pitch, self.R, self.S, pre.data_ptr(), 36,
                                           d.data_ptr(), torch.cuda.current_stream(self.dev).cuda_stream), "rows_md5")
        return [bytes(x) for x in d.cpu().numpy().reshape(self.R, 16)]

    def d2h_bytes(self):
        return self.R * self.S + self.N * 20 + len(self.file_lens) * 16 + self.R
