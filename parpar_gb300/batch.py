"""Batched PAR2 jobs: many independent create jobs through one persistent,
graph-captured multiply-accumulate launch per pass.

Workload model (the uneven job mix): each job has N input slices of S bytes
(seeded synthetic data), R recovery slices (exponents 0..R-1), PAR2
coefficients for inputs 0..N-1.  The mix is larger than device memory, so it
is processed in byte-window passes, the way PAR2Chunked processes a slice in
chunks (lib/par2.js:837-879, lib/par2gen.js:1043-1063, 1287-1330): pass p
holds the window [p*W_j, (p+1)*W_j) of every slice of every job j, and each
recovery window is complete after its pass (no accumulation across passes).

Two ways to run a mix:
  * per-job launches (`run_per_job`): for each job, for each pass, the
    device-level C-ABI calls (synthetic window, zero pad + checksum, comb
    multiply-accumulate, verification), then wait for the job;
  * batched (`capture` + `run_batched`): per pass the window kernels of all
    jobs, then the multiply-accumulate of all jobs, then their verification,
    captured once into a CUDA graph and replayed.  The multiply-accumulate
    runs in one of two modes, chosen by timing one pass of each
    (`tune_mode`):
      - "persistent": one persistent comb launch per CTA-shape group (jobs
        grouped by the autotuner's shape for their recovery count), CTAs
        taking (job, tile, recovery block) units from an atomic ticket;
      - "grid": each job's own grid launch of its automatic shape, the jobs
        spread over four side streams so that small jobs overlap.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib, autotune
from .job import par2_coefficients
from .layout import JobSpec, make_job_mix  # noqa: F401  (re-exported)



def plan_passes(jobs, budget_bytes: int):
    """Number of byte-window passes P so that one pass's rows fit the budget,
    and each job's window size (a multiple of 64 bytes)."""
    total = sum((j.N + j.R) * j.S for j in jobs)
    P = max(1, math.ceil(total / budget_bytes))
    while True:
        wins = [max(64, -(-math.ceil(j.S / P) // 64) * 64) for j in jobs]
        need = sum((j.N + j.R) * _lib.load().par2cuda_row_pitch_bytes(w) for j, w in zip(jobs, wins))
        if need <= budget_bytes or P > 4096:
            return P, wins
        P += 1


class _JobBufs:
    def __init__(self, L, spec: JobSpec, window: int, dev):
        self.spec = spec
        self.W = window
        self.pitch = L.par2cuda_row_pitch_bytes(window)
        self.pw = self.pitch // 2
        self.d_in = torch.empty((spec.N, self.pw), dtype=torch.int16, device=dev)
        self.d_rec = torch.empty((spec.R, self.pw), dtype=torch.int16, device=dev)
        coeff = par2_coefficients(np.arange(spec.N), spec.exps)
        self.d_coeff = torch.from_numpy(coeff.view(np.int16)).to(dev)
        # index bytes (also the per-job path's scratch, which is rounded up to 256 bytes)
        self.idx_bytes = max(L.par2cuda_coeff_index_bytes(spec.R, spec.N), L.par2cuda_muladd_scratch_bytes(spec.R, spec.N))
        self.d_idx = torch.empty(max(self.idx_bytes, 256), dtype=torch.uint8, device=dev)
        self.d_ck = torch.empty(max(spec.N, spec.R) * 8, dtype=torch.uint8, device=dev)
        self.d_flags = torch.zeros(spec.R, dtype=torch.uint8, device=dev)
        self.ok_passes = torch.zeros(1, dtype=torch.int32, device=dev)

    def window(self, p: int):
        """(byte offset, bytes) of pass p's window of every slice (bytes may be 0)."""
        off = p * self.W
        return off, max(0, min(self.W, self.spec.S - off))


class BatchRunner:
    MODES = ("persistent", "grid")

    def __init__(self, jobs, budget_bytes: int = 64 << 30, device: int = 0, shape_of=None, mode: str = "persistent",
                 method_of=None):
        if mode not in self.MODES:
            raise ValueError("mode must be one of %s" % (self.MODES,))
        self.mode = mode
        self.L = _lib.load()
        self.dev = torch.device("cuda", device)
        # largest jobs first: their units are handed out first, the tail is small units
        self.jobs = sorted(jobs, key=lambda j: -j.mul_adds)
        self.P, wins = plan_passes(self.jobs, budget_bytes)
        self.bufs = [_JobBufs(self.L, j, w, self.dev) for j, w in zip(self.jobs, wins)]
        self.shape_of = shape_of or (lambda R: autotune.best_shape(R))
        # multiply method of each job's grid launch (the persistent launch is
        # the comb kernel's)
        self.method_of = method_of or (lambda R: autotune.best_method(R))
        self.shapes = [self.shape_of(j.R) for j in self.jobs]
        st = torch.cuda.current_stream(self.dev).cuda_stream
        for b in self.bufs:  # coefficients -> index bytes, once per job (same for every pass)
            _lib.check(self.L.par2cuda_coeff_index(b.d_coeff.data_ptr(), b.spec.R, b.spec.N, b.d_idx.data_ptr(), st), "index")
        self.graph = None
        self._side = [torch.cuda.Stream(device=self.dev) for _ in range(4)]
        self._descs = {}

    @property
    def mul_adds(self) -> int:
        return sum(j.mul_adds for j in self.jobs)

    # ------------------------------------------------------------ kernels
    def _window_prep(self, b: _JobBufs, p: int, st):
        off, n = b.window(p)
        if n == 0:
            return False
        L = self.L
        _lib.check(L.par2cuda_synth_fill_at(b.d_in.data_ptr(), b.pitch, b.spec.N, n, b.spec.seed, 0, off, st), "synth")
        _lib.check(L.par2cuda_rows_checksum(b.d_in.data_ptr(), b.pw, b.spec.N, None, n, 0, None, b.d_ck.data_ptr(), st), "cksum")
        return True

    def _verify(self, b: _JobBufs, p: int, st):
        off, n = b.window(p)
        _lib.check(self.L.par2cuda_rows_checksum(b.d_rec.data_ptr(), b.pw, b.spec.R, None, n, 1, b.d_flags.data_ptr(),
                                                b.d_ck.data_ptr(), st), "verify")

    @staticmethod
    def _n_words(n_bytes: int) -> int:
        return ((n_bytes + 7) // 8 * 8 + 8) // 2

    def _muladd_grid(self, b: _JobBufs, p: int, st):
        """One job's window through the single-job C-ABI call (grid launch;
        converts the coefficients to index bytes in its scratch each call)."""
        off, n = b.window(p)
        _lib.check(self.L.par2cuda_muladd(b.d_in.data_ptr(), b.pw, b.spec.N, b.d_coeff.data_ptr(), b.d_rec.data_ptr(),
                                          b.pw, b.spec.R, self._n_words(n), 0, _lib.METHOD_COMB, b.d_idx.data_ptr(),
                                          b.d_idx.numel(), st), "muladd")

    def _muladd_index(self, b: _JobBufs, p: int, st):
        """One job's window as a grid launch: the comb kernel from its resident
        index bytes, or, where the autotuner found another method faster for
        its recovery count, that method from the coefficients."""
        off, n = b.window(p)
        method = self.method_of(b.spec.R)
        if method == "comb":
            _lib.check(self.L.par2cuda_muladd_index(b.d_in.data_ptr(), b.pw, b.spec.N, b.d_idx.data_ptr(),
                                                    b.d_rec.data_ptr(), b.pw, b.spec.R, self._n_words(n), 0, st),
                       "muladd_index")
        else:
            self._muladd_method(b, p, st, method)

    def _muladd_method(self, b: _JobBufs, p: int, st, method: str):
        """One job's window with a non-comb method, from its coefficients, in
        scratch of its own (made on the first, eager, call; the resident index
        bytes stay untouched for the persistent launch)."""
        off, n = b.window(p)
        if getattr(b, "d_mscratch", None) is None:
            sb = autotune.scratch_bytes(method, b.spec.R, b.spec.N, self._n_words(b.W))
            b.d_mscratch = torch.empty(max(sb, 256), dtype=torch.uint8, device=self.dev)
        _lib.check(self.L.par2cuda_muladd(b.d_in.data_ptr(), b.pw, b.spec.N, b.d_coeff.data_ptr(), b.d_rec.data_ptr(),
                                          b.pw, b.spec.R, self._n_words(n), 0, autotune.METHODS[method],
                                          b.d_mscratch.data_ptr(), b.d_mscratch.numel(), st), "muladd")

    # ------------------------------------------------------------ per-job path
    def run_per_job(self, verify_cb=None, tuned_methods: bool = False):
        """Each job on its own: its launches for every pass, then wait for it.
        tuned_methods: each job's multiply method is the one the batched path
        uses for its recovery count (method_of), else the single-job default
        (comb).  Returns per-job wall latencies (s)."""
        L = self.L
        cur = torch.cuda.current_stream(self.dev)
        st = cur.cuda_stream
        lat = []
        for b in self.bufs:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(cur)
            for p in range(self.P):
                if not self._window_prep(b, p, st):
                    continue
                method = self.method_of(b.spec.R) if tuned_methods else "comb"
                if method == "comb":
                    self._muladd_grid(b, p, st)
                else:
                    self._muladd_method(b, p, st, method)
                self._verify(b, p, st)
                if verify_cb:
                    verify_cb(b, p)
            e1.record(cur)
            e1.synchronize()
            lat.append(e0.elapsed_time(e1) / 1e3)
        return lat

    # ------------------------------------------------------------ batched path
    def _pass_descs(self, p: int, group):
        """Device descriptor array for pass p's jobs of one shape group."""
        key = (p, tuple(group))
        if key in self._descs:
            return self._descs[key]
        L = self.L
        arr = (_lib.BatchJob * len(group))()
        base = 0
        shape = self.shapes[group[0]]
        for k, ji in enumerate(group):
            b = self.bufs[ji]
            off, n = b.window(p)
            arr[k].d_in = b.d_in.data_ptr()
            arr[k].in_pitch_words = b.pw
            arr[k].num_in = b.spec.N
            arr[k].d_index = b.d_idx.data_ptr()
            arr[k].d_rec = b.d_rec.data_ptr()
            arr[k].rec_pitch_words = b.pw
            arr[k].num_rec = b.spec.R
            arr[k].accumulate = 0
            arr[k].unit_base = base
            base += L.par2cuda_batch_units(b.spec.R, self._n_words(n), shape)
        host = torch.frombuffer(bytearray(arr), dtype=torch.uint8)
        d = host.to(self.dev)
        counter = torch.zeros(1, dtype=torch.int64, device=self.dev)
        self._descs[key] = (d, base, counter, shape)
        return self._descs[key]

    def _issue_batched(self, verify_cb=None):
        cur = torch.cuda.current_stream(self.dev)
        st = cur.cuda_stream
        groups = {}
        for ji, s in enumerate(self.shapes):
            groups.setdefault(s, []).append(ji)
        for p in range(self.P):
            live = [ji for ji, b in enumerate(self.bufs) if b.window(p)[1] > 0]
            for ji in live:
                self._window_prep(self.bufs[ji], p, st)
            for side in self._side:
                side.wait_stream(cur)
            if self.mode == "persistent":
                # one persistent launch per shape group, groups concurrently on side streams
                for gi, (shape, members) in enumerate(sorted(groups.items())):
                    members = [ji for ji in members if ji in live]
                    if not members:
                        continue
                    d, total, counter, shp = self._pass_descs(p, members)
                    side = self._side[gi % len(self._side)]
                    _lib.check(self.L.par2cuda_batch_muladd(d.data_ptr(), len(members), total, counter.data_ptr(), shp,
                                                            side.cuda_stream), "batch_muladd")
            else:
                # each job's grid launch (largest first), round-robin over the side streams
                for k, ji in enumerate(live):
                    self._muladd_index(self.bufs[ji], p, self._side[k % len(self._side)].cuda_stream)
            for side in self._side:
                cur.wait_stream(side)
            for ji in live:
                self._verify(self.bufs[ji], p, st)
                if verify_cb:
                    verify_cb(self.bufs[ji], p)

    def tune_mode(self):
        """Times the multiply-accumulate of pass 0 in each mode (eagerly, after
        one untimed run of each) and keeps the faster; returns the times (ms)."""
        cur = torch.cuda.current_stream(self.dev)
        st = cur.cuda_stream
        live = [ji for ji, b in enumerate(self.bufs) if b.window(0)[1] > 0]
        for ji in live:
            self._window_prep(self.bufs[ji], 0, st)
        times = {}
        for mode in self.MODES:
            for rep in range(2):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(cur)
                for side in self._side:
                    side.wait_stream(cur)
                if mode == "persistent":
                    groups = {}
                    for ji in live:
                        groups.setdefault(self.shapes[ji], []).append(ji)
                    for gi, (shape, members) in enumerate(sorted(groups.items())):
                        d, total, counter, shp = self._pass_descs(0, members)
                        _lib.check(self.L.par2cuda_batch_muladd(d.data_ptr(), len(members), total, counter.data_ptr(),
                                                                shp, self._side[gi % len(self._side)].cuda_stream), "batch")
                else:
                    for k, ji in enumerate(live):
                        self._muladd_index(self.bufs[ji], 0, self._side[k % len(self._side)].cuda_stream)
                for side in self._side:
                    cur.wait_stream(side)
                e1.record(cur)
                e1.synchronize()
                times[mode] = e0.elapsed_time(e1)
        self.mode = min(times, key=times.get)
        self.graph = None
        return times

    def capture(self):
        """Runs the batched sequence once eagerly (one-time set-up), then
        captures it into a CUDA graph."""
        self._issue_batched()
        torch.cuda.synchronize(self.dev)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(device=self.dev)
        s.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self._issue_batched()
        torch.cuda.current_stream(self.dev).wait_stream(s)
        self.graph = g
        return g

    def run_batched(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def all_valid(self) -> bool:
        """Verdicts of the last pass of every job (each pass re-verifies)."""
        return all(bool(b.d_flags.all()) for b in self.bufs)

    def launches_per_run(self):
        """Kernel launches of one run_batched() in the current mode."""
        n = 0
        for p in range(self.P):
            live = [b for b in self.bufs if b.window(p)[1] > 0]
            n += len(live) * 5  # synth, cksum partial + finish, verify partial + finish
            if self.mode == "persistent":
                n += len({self.shapes[i] for i, b in enumerate(self.bufs) if b.window(p)[1] > 0})
                continue
            for b in live:
                method = self.method_of(b.spec.R)
                if method == "comb":
                    n += 1   # the comb kernel from the resident index bytes
                else:
                    nw = self._n_words(b.window(p)[1])
                    sb = autotune.scratch_bytes(method, b.spec.R, b.spec.N, self._n_words(b.W))
                    n += self.L.par2cuda_muladd_launches(b.spec.R, b.spec.N, nw, autotune.METHODS[method], sb)
        return n
