"""A stream of PAR2 create jobs of one shape on one GPU.

A single create job is bound by the MD5 of its largest file: that hash is one
serial dependency chain (RFC 1321), and one GPU thread runs it at ~108 MB/s,
so a 162 MB file takes 1.5 s while the job's whole GF(2^16) contraction takes
~70-90 ms.  A service that creates recovery for many file sets keeps the GPU
busy by having several jobs in flight.  JobStream does that for jobs of one
shape (slice size, file lengths, recovery exponents):

  * `slots` jobs are resident at once, each in its own rows of one device
    buffer (inputs, recovery rows, IFSC entries, file MD5s, verdicts);
  * each job's zero padding + input checksum, multiply-accumulate and
    checksum verification run back to back on one compute stream (the
    contraction fills the GPU on its own), its IFSC hashes (one thread per
    slice) on a side stream, so that they overlap the next contraction;
  * the file MD5 chains of each group of `group` consecutive jobs run as one
    launch of `group x files` threads, `md5_block` of them per block
    (par2cuda_file_md5_pooled), on a high-priority stream of the group: a
    few SMs hold all of them while later jobs' contractions use the others.

With host buffers (run(..., host_in=..., host_out=...)) every job's inputs are
copied to its slot on a copy stream and its results (recovery slices, IFSC
entries, file MD5s, verdicts) copied back on a download stream; a slot is
refilled only after every read of its previous job is done.  The copies of a
window of jobs go largest files first: the files are split into size classes
(`size_classes`, fractions of the largest file's length), and the rows of
class 0 of the window's jobs land before those of class 1, and so on, in a
staircase (upload_order) that also lands the first jobs whole early.
Each class of a group has its own file MD5 launch (par2cuda_file_md5_staged_
indexed, digests in their files' places), started as soon as that class's
rows of the group have landed, so the longest chains start within the first
few percent of the copies instead of after the whole window; a job's
contraction starts once its last class has landed.

Every job's work is exactly the single-job path's (parpar_gb300.job), through
the same C-ABI entry points; the PAR2 semantics follow lib/par2gen.js's
single-pass create (lib/par2gen.js:1198-1330).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .job import par2_coefficients
from .layout import file_layout


class JobStream:
    def __init__(self, slice_size: int, file_lens, exps, slots: int = 24, group: int = 8, device: int = 0,
                 method: int = _lib.METHOD_COMB, md5_block: int = 64, md5_staged: bool = True,
                 size_classes=(0.9, 0.75)):
        if slots % group:
            raise ValueError("slots must be a multiple of group")
        L = self.L = _lib.load()
        self.S = S = int(slice_size)
        self.file_lens = [int(x) for x in file_lens]
        self.first_row, self.row_lens = file_layout(self.file_lens, S)
        self.N = N = len(self.row_lens)
        self.F = F = len(self.file_lens)
        self.exps = list(exps)
        self.R = R = len(self.exps)
        self.slots, self.group = slots, group
        # file MD5 chains per block: a chain issues about one instruction per
        # two cycles of its ~4-cycle dependency steps, so 4 warps (one per
        # scheduler) run at full speed on one SM while more start to slow
        # each other
        self.md5_block = md5_block
        # staged: each chain's bytes arrive in shared memory by bulk copies
        # (par2cuda_file_md5_staged, 32 or 64 chains per block), so chains do
        # not stall on L2 misses while contractions stream through L2
        self.md5_staged = md5_staged and md5_block in (32, 64) and S % 64 == 0
        if group * F > 512:
            raise ValueError("group x files must be at most 512 (one block of file MD5 chains)")
        self.method = method
        self.pitch = L.par2cuda_row_pitch_bytes(S)
        self.pw = self.pitch // 2
        self.row_words = ((S + 7) // 8 * 8 + 8) // 2
        self.dev = dev = torch.device("cuda", device)
        self.d_in = torch.empty((slots * N, self.pw), dtype=torch.int16, device=dev)
        self.d_rec = torch.empty((slots * R, self.pw), dtype=torch.int16, device=dev)
        self.d_ifsc = torch.empty((slots, N * 20), dtype=torch.uint8, device=dev)
        self.d_fmd5 = torch.empty((slots, F * 16), dtype=torch.uint8, device=dev)
        self.d_flags = torch.empty((slots, R), dtype=torch.uint8, device=dev)
        self.d_lens = torch.from_numpy(self.row_lens.view(np.int32)).to(dev)
        self.d_coeff = torch.from_numpy(par2_coefficients(np.arange(N), self.exps).view(np.int16)).to(dev)
        self.scratch_bytes = L.par2cuda_muladd_scratch_bytes(R, N)
        if method == _lib.METHOD_TENSOR_FP4:
            self.scratch_bytes = L.par2cuda_tensor_fp4_scratch_bytes(R, N, self.row_words)
        self.d_scratch = torch.empty(max(self.scratch_bytes, 256), dtype=torch.uint8, device=dev)
        self.muladd_launches = L.par2cuda_muladd_launches(R, N, self.row_words, method, self.scratch_bytes)
        self.d_ck = torch.empty(max(N, R) * 8, dtype=torch.uint8, device=dev)
        # file MD5 tables of one group: the files of its `group` slots in
        # slot order, rows counted from the group's first row
        self.d_gflen = torch.tensor(self.file_lens * group, dtype=torch.int64, device=dev)
        gfirst = np.concatenate([self.first_row.astype(np.int64) + j * N for j in range(group)]).astype(np.uint32)
        self.d_gfirst = torch.from_numpy(gfirst.view(np.int32)).to(dev)
        ng = slots // group
        # size classes of the files for copies from host buffers: class c
        # holds the files of length >= size_classes[c] x the largest (and
        # below the previous bound); empty classes are dropped
        bounds = sorted((float(t) for t in size_classes), reverse=True) if self.md5_staged else []
        mx = max(self.file_lens) if F else 0
        cls = [sum(1 for t in bounds if n < t * mx) for n in self.file_lens]
        self.classes = [c for c in ([f for f in range(F) if cls[f] == k] for k in range(len(bounds) + 1)) if c]
        nrows = np.diff(np.append(self.first_row.astype(np.int64), N))
        self.class_runs, self.class_tables = [], []
        for files in self.classes:
            # row runs to copy: consecutive files of the class merged
            runs = []
            for f in files:
                r0, nr = int(self.first_row[f]), int(nrows[f])
                if runs and runs[-1][0] + runs[-1][1] == r0:
                    runs[-1][1] += nr
                else:
                    runs.append([r0, nr])
            self.class_runs.append(runs)
            # file MD5 table of the class for a whole group: lengths, first
            # rows and digest places counted from the group's first slot
            lens = np.array([self.file_lens[f] for _ in range(group) for f in files], dtype=np.int64)
            first = np.array([int(self.first_row[f]) + j * N for j in range(group) for f in files], dtype=np.uint32)
            out = np.array([j * F + f for j in range(group) for f in files], dtype=np.uint32)
            self.class_tables.append(tuple(torch.from_numpy(a.view(np.int64 if a.dtype == np.int64 else np.int32)).to(dev)
                                           for a in (lens, first, out)))
        self.s_comp = torch.cuda.Stream(device=dev)
        self.s_ifsc = [torch.cuda.Stream(device=dev) for _ in range(ng)]
        self.s_md5 = [torch.cuda.Stream(device=dev, priority=-10) for _ in range(ng)]
        # one more MD5 stream per group for each further size class, so that
        # the classes' chains run side by side
        self.s_md5c = [[self.s_md5[g]] + [torch.cuda.Stream(device=dev, priority=-10)
                                          for _ in range(len(self.classes) - 1)] for g in range(ng)]
        self.s_up = torch.cuda.Stream(device=dev)
        self.s_down = torch.cuda.Stream(device=dev)
        # reads of a slot's rows that must finish before the slot is refilled,
        # and the download of its results before they are overwritten
        self.ev_gf = [None] * slots
        self.ev_ifsc = [None] * slots
        # per group, the last file MD5 launch on each of its MD5 streams (each
        # stream runs in order, so these cover every launch still reading
        # the group's slots)
        self.ev_md5 = [[None] * len(self.classes or [0]) for _ in range(ng)]
        self.ev_down = [None] * slots
        self.launches = 0
        self.jobs_done = []
        self._up_span = None

    # ---------------------------------------------------------------- setup
    def fill_synthetic(self, seed0: int):
        """Seeded rows (parpar_gb300.synth) for every slot: slot s gets seed0 + s."""
        st = torch.cuda.current_stream(self.dev).cuda_stream
        for s in range(self.slots):
            _lib.check(self.L.par2cuda_synth_fill(self.d_in[s * self.N].data_ptr(), self.pitch, self.N, self.S,
                                                 seed0 + s, 0, st), "synth")

    def _wait(self, stream, ev):
        if ev is not None:
            stream.wait_event(ev)

    def _event(self, stream, timing=False):
        e = torch.cuda.Event(enable_timing=timing)
        e.record(stream)
        return e

    # ---------------------------------------------------------------- jobs
    def run(self, count: int, first_job: int = 0, host_in=None, host_out=None, timing: bool = False):
        """Issues jobs first_job .. first_job+count-1 (asynchronous; the current
        stream waits for all of them).  host_in: a list of pinned [N, S] uint8
        tensors, job k reading host_in[k % len]; host_out: a list of tuples
        (rec [R, S], ifsc [N*20], fmd5 [F*16], flags [R]) of pinned uint8
        tensors, job k writing host_out[k % len].  timing=True records events
        for per-job latencies (latencies())."""
        cur = torch.cuda.current_stream(self.dev)
        streams = [self.s_comp, self.s_up, self.s_down] + self.s_ifsc + [st for c in self.s_md5c for st in c]
        for st in streams:
            st.wait_stream(cur)
        self._up_span = None
        if timing and host_in is not None:
            self._up_span = [self._event(self.s_up, True), None]
        k = first_job
        end = first_job + count
        if host_in is not None and len(self.classes) > 1:
            # windows of at most `slots` jobs: no slot holds two jobs of a window
            while k < end:
                n = min(self.slots, end - k)
                self._run_window(list(range(k, k + n)), host_in, host_out, timing)
                k += n
        else:
            for g, jobs in self._chunks(k, end):
                landed = {}
                for j in jobs:
                    landed[j] = self._upload_whole(j, host_in)
                    self._issue_gf(j, timing, landed[j])
                self._issue_md5(g, jobs, timing, landed)
                if host_out is not None:
                    for j in jobs:
                        self._issue_download(j, host_out)
        if self._up_span is not None:
            self._up_span[1] = self._event(self.s_up, True)
        for st in streams:
            cur.wait_stream(st)

    def _chunks(self, k, end):
        """(group, consecutive jobs of that group) for jobs k .. end-1."""
        out = []
        while k < end:
            g = (k % self.slots) // self.group
            n = min(self.group - (k % self.slots) % self.group, end - k)
            out.append((g, list(range(k, k + n))))
            k += n
        return out

    def _slot_free(self, stream, k):
        """`stream` waits until every read of slot k % slots by its previous job
        is done and that job's results have been copied out."""
        s = k % self.slots
        for ev in [self.ev_gf[s], self.ev_ifsc[s], self.ev_down[s]] + self.ev_md5[s // self.group]:
            self._wait(stream, ev)

    def _upload_whole(self, k, host_in):
        """All rows of job k in one 2-D copy (no size classes); returns the
        event of their landing (None for resident rows)."""
        if host_in is None:
            return None
        s = k % self.slots
        up = self.s_up
        self._slot_free(up, k)
        src = host_in[k % len(host_in)]
        _lib.check(self.L.par2cuda_copy_rows(self.d_in[s * self.N].data_ptr(), self.pitch, src.data_ptr(), self.S,
                                             self.S, self.N, up.cuda_stream), "h2d")
        return self._event(up)

    @staticmethod
    def upload_order(n, classes):
        """(job index in the window, size class) in copy order: a staircase
        that lands job 0 whole, then class 0 of every other job, then the rest
        of job 1, class 1 of jobs 2.., the rest of job 2, and so on; the
        largest files' MD5 chains start within the first copies while the
        contraction of the first jobs need not wait for the whole window."""
        order, done = [], set()

        def add(i, c):
            if (i, c) not in done:
                done.add((i, c))
                order.append((i, c))
        for c in range(classes):
            add(0, c)
        for c in range(classes):
            for i in range(c + 1, n):
                add(i, c)
            if c + 1 < n:
                for cc in range(c + 1, classes):
                    add(c + 1, cc)
        return order

    def _run_window(self, jobs, host_in, host_out, timing):
        """Copies by size class in upload_order(), each class's file MD5 launch
        per group as soon as that class of the group's jobs has landed, each
        job's kernels once its last class has landed."""
        up, S, N = self.s_up, self.S, self.N
        C = len(self.classes)
        chunks = self._chunks(jobs[0], jobs[-1] + 1)
        chunk_of = {k: ci for ci, (_, cj) in enumerate(chunks) for k in cj}
        waiting = {(c, ci): len(cj) for c in range(C) for ci, (_, cj) in enumerate(chunks)}
        left = {k: C for k in jobs}
        for k in jobs:
            self._slot_free(up, k)
        md5_evs = {k: [] for k in jobs}
        md5_t0 = {}
        for i, c in self.upload_order(len(jobs), C):
            k = jobs[i]
            s = k % self.slots
            src = host_in[k % len(host_in)].data_ptr()
            base = self.d_in[s * N].data_ptr()
            for r0, nr in self.class_runs[c]:
                _lib.check(self.L.par2cuda_copy_rows(base + r0 * self.pitch, self.pitch, src + r0 * S, S, S, nr,
                                                     up.cuda_stream), "h2d")
            left[k] -= 1
            if not left[k]:
                self._issue_gf(k, timing, self._event(up))
            ci = chunk_of[k]
            waiting[c, ci] -= 1
            if not waiting[c, ci]:
                g, cj = chunks[ci]
                t0, ev = self._issue_md5_class(g, cj, c, self._event(up), timing)
                for kk in cj:
                    md5_evs[kk].append(ev)
                    md5_t0.setdefault(kk, t0)
        for rec in self.jobs_done[-len(jobs):]:
            rec["md5"] = md5_evs[rec["job"]]
            if timing:
                rec["md5_start"] = md5_t0[rec["job"]]
        if host_out is not None:
            for k in jobs:
                self._issue_download(k, host_out)

    def _issue_md5_class(self, g, jobs, c, ev_landed, timing):
        """The file MD5 launch of size class c for `jobs` (consecutive slots of group g)."""
        st = self.s_md5c[g][c]
        st.wait_event(ev_landed)
        s0 = jobs[0] % self.slots
        lens, first, out = self.class_tables[c]
        nf = len(jobs) * len(self.classes[c])
        t0 = self._event(st, True) if timing else None
        _lib.check(self.L.par2cuda_file_md5_staged_indexed(self.d_in[s0 * self.N].data_ptr(), self.pitch, nf,
                                                           lens.data_ptr(), first.data_ptr(), out.data_ptr(), self.S,
                                                           self.d_fmd5[s0].data_ptr(), self.md5_block, st.cuda_stream),
                   "file_md5")
        ev = self._event(st, timing)
        self.ev_md5[g][c] = ev
        self.launches += 1
        return t0, ev

    def _issue_gf(self, k, timing, landed=None):
        """Job k's kernels: checksum, contraction and verification on the
        compute stream, IFSC on its group's side stream; with host buffers
        they wait for the job's rows to have landed (event `landed`)."""
        L, N, R = self.L, self.N, self.R
        s = k % self.slots
        g = s // self.group
        comp, side = self.s_comp, self.s_ifsc[g]
        d_in = self.d_in[s * N].data_ptr()
        d_rec = self.d_rec[s * R].data_ptr()
        rec = {"job": k}
        # the slot's previous results have been copied out (their copy came
        # before this job's rows were copied in, when there is one)
        self._wait(comp, self.ev_down[s])
        if landed is not None:
            comp.wait_event(landed)
            side.wait_event(landed)
        if timing:
            rec["start"] = self._event(comp, True)
        a = comp.cuda_stream
        _lib.check(L.par2cuda_rows_checksum(d_in, self.pw, N, self.d_lens.data_ptr(), self.S, 0, None,
                                           self.d_ck.data_ptr(), a), "rows_checksum")
        if timing:
            rec["mul0"] = self._event(comp, True)
        _lib.check(L.par2cuda_muladd(d_in, self.pw, N, self.d_coeff.data_ptr(), d_rec, self.pw, R, self.row_words, 0,
                                    self.method, self.d_scratch.data_ptr(), self.scratch_bytes, a), "muladd")
        if timing:
            rec["mul1"] = self._event(comp, True)
        _lib.check(L.par2cuda_rows_checksum(d_rec, self.pw, R, None, self.S, 1, self.d_flags[s].data_ptr(),
                                           self.d_ck.data_ptr(), a), "verify")
        self.ev_gf[s] = self._event(comp, timing)
        self._wait(side, self.ev_down[s])
        _lib.check(L.par2cuda_slice_hash(d_in, self.pitch, N, self.d_lens.data_ptr(), self.S,
                                        self.d_ifsc[s].data_ptr(), side.cuda_stream), "slice_hash")
        self.ev_ifsc[s] = self._event(side, timing)
        # checksum (2 kernels), the multiply-accumulate's own launches,
        # verification (2), IFSC
        self.launches += 5 + self.muladd_launches
        rec["gf"], rec["ifsc"] = self.ev_gf[s], self.ev_ifsc[s]
        self.jobs_done.append(rec)

    def _issue_md5(self, g, jobs, timing, landed):
        """One pooled launch for the file MD5s of `jobs` (consecutive slots of group g)."""
        s0 = jobs[0] % self.slots
        st = self.s_md5[g]
        # the group's inputs are in place (copies), and the digests of the
        # slots' previous jobs have been copied out
        for j in jobs:
            s = j % self.slots
            self._wait(st, landed.get(j))
            self._wait(st, self.ev_down[s])
        j0 = s0 - g * self.group
        nf = len(jobs) * self.F
        if timing:
            t0 = self._event(st, True)
        md5 = self.L.par2cuda_file_md5_staged if self.md5_staged else self.L.par2cuda_file_md5_pooled
        _lib.check(md5(self.d_in[s0 * self.N].data_ptr(), self.pitch, nf, self.d_gflen.data_ptr() + 8 * j0 * self.F,
                       self.d_gfirst.data_ptr(), self.S, self.d_fmd5[s0].data_ptr(), self.md5_block, st.cuda_stream),
                   "file_md5")
        ev = self._event(st, timing)
        self.ev_md5[g][0] = ev
        self.launches += 1
        for rec in self.jobs_done[-len(jobs):]:
            rec["md5"] = [ev]
            if timing:
                rec["md5_start"] = t0

    def _issue_download(self, k, host_out):
        s = k % self.slots
        g = s // self.group
        d = self.s_down
        for ev in [self.ev_gf[s], self.ev_ifsc[s]] + self.ev_md5[g]:
            self._wait(d, ev)
        rec_h, ifsc_h, fmd5_h, flags_h = host_out[k % len(host_out)]
        L, ds = self.L, d.cuda_stream
        _lib.check(L.par2cuda_copy_rows(rec_h.data_ptr(), self.S, self.d_rec[s * self.R].data_ptr(), self.pitch, self.S,
                                       self.R, ds), "d2h")
        for h, dv in ((ifsc_h, self.d_ifsc[s]), (fmd5_h, self.d_fmd5[s]), (flags_h, self.d_flags[s])):
            _lib.check(L.par2cuda_copy_rows(h.data_ptr(), h.numel(), dv.data_ptr(), dv.numel(), dv.numel(), 1, ds), "d2h")
        self.ev_down[s] = self._event(d)

    # ---------------------------------------------------------------- results
    def latencies(self):
        """Seconds from each timed job's first kernel (contraction side or its
        group's file MD5 launch, whichever started first) to its last."""
        out = []
        for rec in self.jobs_done:
            if "start" not in rec:
                continue
            start = rec["start"]
            t_end = max([start.elapsed_time(rec["gf"]), start.elapsed_time(rec["ifsc"])] +
                        [start.elapsed_time(e) for e in rec["md5"]])
            t_beg = min(0.0, start.elapsed_time(rec["md5_start"]))
            out.append((t_end - t_beg) / 1e3)
        return out

    def muladd_ms(self):
        """Mean device time of the timed jobs' multiply-accumulate launches (ms)."""
        t = [r["mul0"].elapsed_time(r["mul1"]) for r in self.jobs_done if "mul0" in r]
        return float(np.mean(t)) if t else 0.0

    def upload_span_ms(self):
        """Milliseconds from the copy stream's start to its last copy of the
        last timed run with host buffers (0 when it read resident rows)."""
        if not self._up_span or self._up_span[1] is None:
            return 0.0
        return self._up_span[0].elapsed_time(self._up_span[1])

    def timeline(self, t0):
        """Per timed job, milliseconds from event t0 to each recorded event
        (upload, contraction, IFSC, file MD5 start and end)."""
        out = []
        for r in self.jobs_done:
            if "start" not in r:
                continue
            d = {"job": r["job"]}
            for k in ("start", "mul0", "mul1", "gf", "ifsc", "md5_start"):
                if k in r:
                    d[k] = t0.elapsed_time(r[k])
            d["md5"] = [t0.elapsed_time(e) for e in r["md5"]]
            out.append(d)
        return out

    def clear_records(self):
        self.jobs_done = []

    def h2d_bytes(self):
        return self.N * self.S

    def d2h_bytes(self):
        return self.R * self.S + self.N * 20 + self.F * 16 + self.R

    def host_out_buffers(self, count: int):
        return [(torch.empty((self.R, self.S), dtype=torch.uint8, pin_memory=True),
                 torch.empty(self.N * 20, dtype=torch.uint8, pin_memory=True),
                 torch.empty(self.F * 16, dtype=torch.uint8, pin_memory=True),
                 torch.empty(self.R, dtype=torch.uint8, pin_memory=True)) for _ in range(count)]

    def slot_results(self, s: int):
        """(recovery rows [R, S], IFSC bytes, file MD5 bytes, verdicts) of slot s, on the host."""
        rec = self.d_rec.view(torch.uint8)[s * self.R:(s + 1) * self.R, : self.S].cpu().numpy()
        return rec, self.d_ifsc[s].cpu().numpy(), self.d_fmd5[s].cpu().numpy(), self.d_flags[s].cpu().numpy()
