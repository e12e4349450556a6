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
refilled only after every read of its previous job is done.

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
                 method: int = _lib.METHOD_COMB, md5_block: int = 64, md5_staged: bool = True):
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
        self.d_ck = torch.empty(max(N, R) * 8, dtype=torch.uint8, device=dev)
        # file MD5 tables of one group: the files of its `group` slots in
        # slot order, rows counted from the group's first row
        self.d_gflen = torch.tensor(self.file_lens * group, dtype=torch.int64, device=dev)
        gfirst = np.concatenate([self.first_row.astype(np.int64) + j * N for j in range(group)]).astype(np.uint32)
        self.d_gfirst = torch.from_numpy(gfirst.view(np.int32)).to(dev)
        ng = slots // group
        self.s_comp = torch.cuda.Stream(device=dev)
        self.s_ifsc = [torch.cuda.Stream(device=dev) for _ in range(ng)]
        self.s_md5 = [torch.cuda.Stream(device=dev, priority=-10) for _ in range(ng)]
        self.s_up = torch.cuda.Stream(device=dev)
        self.s_down = torch.cuda.Stream(device=dev)
        # reads of a slot's rows that must finish before the slot is refilled,
        # and the download of its results before they are overwritten
        self.ev_gf = [None] * slots
        self.ev_ifsc = [None] * slots
        self.ev_md5 = [None] * ng
        self.ev_down = [None] * slots
        self.ev_up = [None] * slots
        self.launches = 0
        self.jobs_done = []

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
        L, N, R, G = self.L, self.N, self.R, self.group
        cur = torch.cuda.current_stream(self.dev)
        for st in [self.s_comp, self.s_up, self.s_down] + self.s_ifsc + self.s_md5:
            st.wait_stream(cur)
        k = first_job
        end = first_job + count
        while k < end:
            g = (k % self.slots) // G
            n_in_group = min(G - (k % self.slots) % G, end - k)
            jobs = list(range(k, k + n_in_group))
            for j in jobs:
                self._issue_gf(j, host_in, timing)
            self._issue_md5(g, jobs, timing)
            if host_out is not None:
                for j in jobs:
                    self._issue_download(j, host_out)
            k += n_in_group
        for st in [self.s_comp, self.s_up, self.s_down] + self.s_ifsc + self.s_md5:
            cur.wait_stream(st)

    def _issue_gf(self, k, host_in, timing):
        L, N, R = self.L, self.N, self.R
        s = k % self.slots
        g = s // self.group
        comp, side = self.s_comp, self.s_ifsc[g]
        d_in = self.d_in[s * N].data_ptr()
        d_rec = self.d_rec[s * R].data_ptr()
        rec = {"job": k}
        if host_in is not None:
            up = self.s_up
            # the slot's previous job has read its rows and its results have
            # been copied out before new rows land
            for ev in (self.ev_gf[s], self.ev_ifsc[s], self.ev_md5[g], self.ev_down[s]):
                self._wait(up, ev)
            src = host_in[k % len(host_in)]
            _lib.check(L.par2cuda_copy_rows(d_in, self.pitch, src.data_ptr(), self.S, self.S, N, up.cuda_stream), "h2d")
            ev_up = self._event(up)
            self.ev_up[s] = ev_up
            comp.wait_event(ev_up)
            side.wait_event(ev_up)
        else:
            self._wait(comp, self.ev_down[s])
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
        self.launches += 7   # checksum (2 kernels), coefficient index, contraction, verification (2), IFSC
        rec["gf"], rec["ifsc"] = self.ev_gf[s], self.ev_ifsc[s]
        self.jobs_done.append(rec)

    def _issue_md5(self, g, jobs, timing):
        """One pooled launch for the file MD5s of `jobs` (consecutive slots of group g)."""
        s0 = jobs[0] % self.slots
        st = self.s_md5[g]
        # the group's inputs are in place (copies), and the digests of the
        # slots' previous jobs have been copied out
        for j in jobs:
            s = j % self.slots
            self._wait(st, self.ev_up[s])
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
        self.ev_md5[g] = ev
        self.launches += 1
        for rec in self.jobs_done[-len(jobs):]:
            rec["md5"] = ev
            if timing:
                rec["md5_start"] = t0

    def _issue_download(self, k, host_out):
        s = k % self.slots
        g = s // self.group
        d = self.s_down
        for ev in (self.ev_gf[s], self.ev_ifsc[s], self.ev_md5[g]):
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
            t_end = max(start.elapsed_time(rec["gf"]), start.elapsed_time(rec["ifsc"]), start.elapsed_time(rec["md5"]))
            t_beg = min(0.0, start.elapsed_time(rec["md5_start"]))
            out.append((t_end - t_beg) / 1e3)
        return out

    def muladd_ms(self):
        """Mean device time of the timed jobs' multiply-accumulate launches (ms)."""
        t = [r["mul0"].elapsed_time(r["mul1"]) for r in self.jobs_done if "mul0" in r]
        return float(np.mean(t)) if t else 0.0

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
