"""Serving loop: recovery-generation requests admitted continuously by free HBM.

Requests arrive as a Poisson process; each is a PAR2 create job (sizes as the
uneven job mix).  A host scheduler keeps a FIFO queue and admits the head
request as soon as a slot is free and its resident footprint fits the HBM
budget (<= 150 GB by default); admitted jobs run on their own CUDA streams, so
work of different requests overlaps on the device and new requests enter
while others are running (continuous batching, not a drain-and-refill queue).
A request whose rows exceed its share of the budget is processed in
byte-window passes (PAR2Chunked's chunking, lib/par2.js:837-879) with its
coefficient index table resident across the passes.  Latency = completion -
arrival; the loop reports jobs/s and p50/p99 latency.

Per job and window: synthetic slice window, zero pad + checksum, the
multiply-accumulate, checksum verification.  The multiply method is the
autotuner's choice for the job's recovery count (autotune.best_method): the
comb kernel from the job's resident index table (a grid launch, or one
persistent launch over the job's units), or another method (on GB300 the
block-scaled 4-bit tensor form) from the job's coefficient matrix, computed
once on the device, with scratch of its own.  All device work goes through
libpar2cuda.so's C ABI.
"""
from __future__ import annotations

import hashlib
import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib, autotune
from .batch import JobSpec, make_job_mix


@dataclass
class Request:
    rid: int
    spec: JobSpec
    arrival: float
    admitted: float = 0.0
    done: float = 0.0
    digest: str = ""
    valid: bool = False
    bytes: int = 0
    state: dict = field(default_factory=dict)


def poisson_arrivals(n: int, rate: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


class Server:
    def __init__(self, budget_bytes: int = 150 * 10**9, slots: int = 8, device: int = 0, digests: bool = False,
                 chunk_share: float = 0.5, persistent: bool = False):
        self.L = _lib.load()
        self.persistent = persistent     # persistent batch launch per chunk instead of a grid launch
        self.dev = torch.device("cuda", device)
        self.budget = budget_bytes
        self.slots = slots
        self.digests = digests
        self.chunk_share = chunk_share   # largest share of the budget one request may hold
        self.streams = [torch.cuda.Stream(device=self.dev) for _ in range(slots)]
        self.free_streams = deque(range(slots))
        self.in_use = 0
        self.launches = 0

    # ---------------------------------------------------------------- sizing
    def _method(self, spec: JobSpec) -> str:
        return "comb" if self.persistent else autotune.best_method(spec.R)

    @staticmethod
    def _n_words(W: int) -> int:
        return ((W + 7) // 8 * 8 + 8) // 2

    def _scratch_bytes(self, spec: JobSpec, method: str, W: int) -> int:
        """Scratch of a non-comb method for a window of W bytes (0 for comb):
        the 4-bit tensor method's expanded operands for the whole window, or
        the index scratch of the others."""
        if method == "comb":
            return 0
        if method == "tensor_fp4":
            return self.L.par2cuda_tensor_fp4_scratch_bytes(spec.R, spec.N, self._n_words(W))
        return autotune.scratch_bytes(method, spec.R, spec.N, self._n_words(W))

    def _window_bytes(self, spec: JobSpec, W: int, method: str) -> int:
        """Device bytes of a window: input and recovery rows, and for a
        non-comb method its coefficient matrix and scratch."""
        b = (spec.N + spec.R) * self.L.par2cuda_row_pitch_bytes(W)
        if method != "comb":
            b += 2 * spec.R * spec.N + self._scratch_bytes(spec, method, W)
        return b

    def _window(self, spec: JobSpec):
        """Window bytes so the job's window fits its share of the budget."""
        share = int(self.budget * self.chunk_share)
        method = self._method(spec)
        W = spec.S
        while self._window_bytes(spec, W, method) > share and W > 64:
            W = max(64, -(-(W // 2) // 64) * 64)
        return W

    def footprint(self, spec: JobSpec) -> int:
        W = self._window(spec)
        return (self._window_bytes(spec, W, self._method(spec)) + self.L.par2cuda_coeff_index_bytes(spec.R, spec.N) +
                4 * (spec.N + spec.R) + 4096)

    # ---------------------------------------------------------------- issue
    def _issue(self, req: Request, si: int):
        L = self.L
        spec = req.spec
        st_obj = self.streams[si]
        st = st_obj.cuda_stream
        W = self._window(spec)
        pitch = L.par2cuda_row_pitch_bytes(W)
        pw = pitch // 2
        with torch.cuda.stream(st_obj):
            d_in = torch.empty((spec.N, pw), dtype=torch.int16, device=self.dev)
            d_rec = torch.empty((spec.R, pw), dtype=torch.int16, device=self.dev)
            d_nums = torch.arange(spec.N, dtype=torch.int16, device=self.dev)
            d_exps = torch.tensor(np.asarray(spec.exps, dtype=np.uint16).view(np.int16), device=self.dev)
            idx_bytes = L.par2cuda_coeff_index_bytes(spec.R, spec.N)
            d_idx = torch.empty(max(idx_bytes, 256), dtype=torch.uint8, device=self.dev)
            d_ck = torch.empty(max(spec.N, spec.R) * 8, dtype=torch.uint8, device=self.dev)
            d_flags = torch.zeros(spec.R, dtype=torch.uint8, device=self.dev)
            d_ok = torch.ones(1, dtype=torch.uint8, device=self.dev)
            counter = torch.zeros(1, dtype=torch.int64, device=self.dev)
        shape = autotune.best_shape(spec.R) if self.persistent else 0
        method = self._method(spec)
        if method == "comb":
            _lib.check(L.par2cuda_par2_index(d_nums.data_ptr(), spec.N, d_exps.data_ptr(), spec.R, d_idx.data_ptr(), st),
                       "index")
            d_coeff = d_scr = None
        else:
            with torch.cuda.stream(st_obj):
                d_coeff = torch.empty((spec.R, spec.N), dtype=torch.int16, device=self.dev)
                d_scr = torch.empty(max(self._scratch_bytes(spec, method, W), 256), dtype=torch.uint8, device=self.dev)
            _lib.check(L.par2cuda_par2_coeffs(d_nums.data_ptr(), spec.N, d_exps.data_ptr(), spec.R, d_coeff.data_ptr(), st),
                       "coeffs")
        n_pass = math.ceil(spec.S / W)
        descs = []
        host_out = []
        for p in range(n_pass):
            off = p * W
            n = min(W, spec.S - off)
            nw = ((n + 7) // 8 * 8 + 8) // 2
            _lib.check(L.par2cuda_synth_fill_at(d_in.data_ptr(), pitch, spec.N, n, spec.seed, 0, off, st), "synth")
            _lib.check(L.par2cuda_rows_checksum(d_in.data_ptr(), pw, spec.N, None, n, 0, None, d_ck.data_ptr(), st), "cksum")
            if self.persistent:
                jd = _lib.BatchJob(d_in.data_ptr(), pw, spec.N, d_idx.data_ptr(), d_rec.data_ptr(), pw, spec.R, 0, 0)
                units = L.par2cuda_batch_units(spec.R, nw, shape)
                dd = torch.frombuffer(bytearray(jd), dtype=torch.uint8).to(self.dev)
                descs.append(dd)
                _lib.check(L.par2cuda_batch_muladd(dd.data_ptr(), 1, units, counter.data_ptr(), shape, st), "muladd")
            elif method == "comb":
                # grid launch from the resident index bytes (measured faster than
                # the persistent launch on GB300)
                _lib.check(L.par2cuda_muladd_index(d_in.data_ptr(), pw, spec.N, d_idx.data_ptr(), d_rec.data_ptr(), pw,
                                                   spec.R, nw, 0, st), "muladd")
            else:
                _lib.check(L.par2cuda_muladd(d_in.data_ptr(), pw, spec.N, d_coeff.data_ptr(), d_rec.data_ptr(), pw,
                                             spec.R, nw, 0, autotune.METHODS[method], d_scr.data_ptr(), d_scr.numel(), st),
                           "muladd")
            _lib.check(L.par2cuda_rows_checksum(d_rec.data_ptr(), pw, spec.R, None, n, 1, d_flags.data_ptr(),
                                               d_ck.data_ptr(), st), "verify")
            with torch.cuda.stream(st_obj):
                torch.minimum(d_ok, d_flags.min().reshape(1), out=d_ok)
                if self.digests:
                    host_out.append(d_rec.view(torch.uint8)[:, :n].to("cpu", non_blocking=True))
            # synth, checksum (2), the multiply-accumulate, verification (2)
            if self.persistent or method == "comb":
                self.launches += 6
            else:
                self.launches += 5 + L.par2cuda_muladd_launches(spec.R, spec.N, nw, autotune.METHODS[method],
                                                                 d_scr.numel())
        ev = torch.cuda.Event()
        ev.record(st_obj)
        req.state = dict(tensors=(d_in, d_rec, d_nums, d_exps, d_idx, d_ck, d_flags, counter, descs, d_coeff, d_scr),
                         ok=d_ok, ev=ev, method=method,
                         host_out=host_out, stream=si)

    def _finish(self, req: Request):
        s = req.state
        req.valid = bool(s["ok"].item())
        if self.digests:
            h = hashlib.md5()
            for t in s["host_out"]:
                h.update(t.numpy().tobytes())
            req.digest = h.hexdigest()
        self.free_streams.append(s["stream"])
        self.in_use -= req.bytes
        req.state = {}

    # ---------------------------------------------------------------- loop
    def run(self, requests):
        """Serves the requests (arrival times relative to the start)."""
        autotune.warm()
        for r in requests:
            r.bytes = self.footprint(r.spec)
        queue = deque(sorted(requests, key=lambda r: r.arrival))
        running = []
        done = []
        t0 = time.perf_counter()
        while queue or running:
            now = time.perf_counter() - t0
            for r in list(running):
                if r.state["ev"].query():
                    r.done = time.perf_counter() - t0
                    self._finish(r)
                    running.remove(r)
                    done.append(r)
            while queue and queue[0].arrival <= now and self.free_streams and \
                    (self.in_use + queue[0].bytes <= self.budget or not running):
                r = queue.popleft()
                r.admitted = time.perf_counter() - t0
                self.in_use += r.bytes
                self._issue(r, self.free_streams.popleft())
                running.append(r)
            if running or queue:
                nxt = queue[0].arrival - (time.perf_counter() - t0) if queue and not running else 0.0005
                time.sleep(max(0.0, min(nxt, 0.002)))
        return done


def serve_stats(done, wall=None):
    lat = np.array([r.done - r.arrival for r in done])
    first = min(r.arrival for r in done)
    last = max(r.done for r in done)
    span = wall or (last - first)
    return {"jobs": len(done), "jobs_per_s": len(done) / span, "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "mean_latency_s": float(lat.mean()),
            "mul_adds_per_s": sum(r.spec.mul_adds for r in done) / span, "all_valid": all(r.valid for r in done),
            "span_s": span}


def make_requests(n: int, rate: float, seed: int = 5, **mix_kw):
    specs = make_job_mix(n, seed=seed, **mix_kw)
    arr = poisson_arrivals(n, rate, seed + 1)
    return [Request(i, s, float(a)) for i, (s, a) in enumerate(zip(specs, arr))]
