"""Benchmark: PAR2 recovery generation on one GB300 vs the reference's CPU path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload bandwidth|dense|plain|batched|serving|create] [--slots S] [--group G]
                    [--no-e2e] [--no-cpu-baseline] [--no-dense]

Workload (default "bandwidth", the configuration the metric is quoted on):
2000 input slices x 2 MiB (40 files of seeded uneven lengths; the last slice of
each file zero-padded), 200 recovery slices (exponents 0..199), with the
per-slice MD5+CRC32 (IFSC) and per-file MD5 hashes, single read pass.  Inputs
are seeded synthetic data (parpar_gb300.synth).

One step = one whole job.  The GPU arm streams K jobs through S resident slots
(parpar_gb300.stream.JobStream: each job's contraction, checksums and IFSC, and
the file MD5 chains of G jobs pooled into one launch), so that the serial MD5
chain of one job's largest file overlaps other jobs' contractions; the timed
region holds every kernel of all K jobs, and each job's latency is reported
(p50/p99).  `single_job` gives one job at a time.  value: GF16 mul-adds/s with
the inputs resident in HBM (CUDA events).  e2e: the same stream with every
job's slices copied from pinned host memory and its results copied back.
`dense`: the 4096 x 4096 x 256 KiB contraction.  --impl reference runs the
reference's own CPU implementation (ParPar's PAR2ProcCPU with GF16_AUTO and its
HasherInput per file, compiled on this host from staged sources) one whole job
per step, on the same config.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

# enough hardware queues for the job stream's concurrent streams; must be set
# before the CUDA context exists (parpar_gb300/__init__.py explains why)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from parpar_gb300.layout import file_lengths  # noqa: E402  (pure host code, no device library)

METRIC = "GF16 mul-adds/s"
UNIT = "mul-adds/s"

# one ncu capture per contraction kernel on a 512-input x 512 KiB case:
# dram__bytes_read.sum + dram__bytes_write.sum, and the algorithmic (N + R) x S
# one ncu capture of k_file_md5 (4 files, 266.6 MB in all): DRAM bytes per byte hashed
MD5_TRAFFIC = (272723456 + 4043776, 266590293)
# k_tc4_gemm, one launch (one word chunk) captured by ncu: DRAM read + write,
# the chunk's expanded input-plane bytes; keyed by (inputs, recovery)
TC4_TRAFFIC = {
    (2000, 200): (3963986944 + 29081600, 67072 * 16000,
                  "k_tc4_gemm on 2000x200x512KiB (first 1 GiB word chunk: the bandwidth workload's chunk shape)"),
    (4096, 4096): (71958856192 + 272894976, 32768 * 32768, "k_tc4_gemm on the dense workload (first 1 GiB word chunk)"),
}
KERNEL_TRAFFIC = {
    "k_comb_pair": (270406912 + 87077120, (512 + 200) * 524288, "k_comb_pair<6,12,2> on 512x200x512KiB"),
    "k_comb_pair_rr": (268913408 + 81736448, (512 + 192) * 524288, "k_comb_pair_rr<8,12,2,152,56> on 512x192x512KiB"),
}

WORKLOADS = {
    # name: (slice bytes, input slices, files, recovery slices, hashing)
    "bandwidth": dict(S=2 * 1048576, N=2000, files=40, R=200, hashes=True,
                      desc="2000 input slices x 2 MiB over 40 uneven files, 200 recovery (exp 0..199), IFSC + file MD5, single read pass"),
    "dense": dict(S=262144, N=4096, files=1, R=4096, hashes=False,
                  desc="4096 input slices x 256 KiB, 4096 recovery (exp 0..4095), GF contraction only"),
    "plain": dict(S=1048576, N=100, files=1, R=10, hashes=True,
                  desc="100 input slices x 1 MiB (one 100 MiB file), 10 recovery (exp 0..9), IFSC + file MD5"),
    # small case for ncu captures of the contraction kernel (inputs 256 MiB > L2)
    "profile": dict(S=524288, N=512, files=1, R=192, hashes=False,
                    desc="512 input slices x 512 KiB, 192 recovery, GF contraction only (ncu capture size)"),
    "profile_ws": dict(S=524288, N=512, files=1, R=200, hashes=False,
                       desc="512 input slices x 512 KiB, 200 recovery, GF contraction only (ncu capture size, 72-row CTAs)"),
    "profile_bw": dict(S=524288, N=2000, files=1, R=200, hashes=False,
                       desc="2000 input slices x 512 KiB, 200 recovery, GF contraction only (ncu capture size: the "
                            "bandwidth workload's inputs and recovery count, so each 1 GiB word chunk of the 4-bit "
                            "tensor method has the full-size launch's shape)"),
    "profile_hash": dict(S=1048576, N=256, files=4, R=8, hashes=True,
                         desc="256 input slices x 1 MiB over 4 files, 8 recovery, with hashing (ncu capture size)"),
    # the bandwidth workload as files on the host's disk: files in, finished .par2 files out
    "create": dict(S=2 * 1048576, N=2000, files=40, R=200, hashes=True,
                   desc="the bandwidth workload's 40 files (3.9 GiB) written to the host's disk, then PAR2 create "
                        "end to end: read, GPU hashing + recovery, .par2 index + pow2 volumes written"),
    # ncu capture cases of the remaining kernels (no bench line): the
    # recovery-packet MD5 over 256 x 1 MiB rows, and the persistent batched
    # multiply-accumulate over a small mix
    "profile_rows_md5": dict(S=1048576, N=8, files=1, R=256, hashes=False,
                             desc="recovery-packet MD5 of 256 recovery rows x 1 MiB (ncu capture size)"),
    "profile_batched": dict(S=0, N=0, files=0, R=0, hashes=False, jobs=12,
                            desc="12 jobs, N 64..600, S 256 KiB..2 MiB: pass 0 persistent + grid (ncu capture size)"),
    # serving: Poisson requests, admitted by free HBM, continuous batching
    "serving": dict(S=0, N=0, files=0, R=0, hashes=False, jobs=48,
                    desc="Poisson requests (sizes as the 64-job mix) at 200/s and at a sub-saturation rate; admission by "
                         "free HBM (<=150 GB), chunked when over budget; jobs/s and p50/p99 latency"),
    # batched: 64 uneven jobs, one graph-captured sequence of launches per pass
    "batched": dict(S=0, N=0, files=0, R=0, hashes=False, jobs=64,
                    desc="64 PAR2 jobs: N log-uniform [10,5000], S uniform 64 KiB..8 MiB (4-byte steps), R 1-30% of N; "
                         "byte-window passes under a 64 GiB HBM budget; persistent graph-captured comb launches vs per-job launches"),
}


def sample_clocks(stop, out):
    cmd = ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
           "--format=csv,noheader,nounits", "-lms", "200"]
    try:
        p = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except Exception:
        return
    try:
        while not stop.is_set():
            line = p.stdout.readline()
            if not line:
                break
            out.append(line.strip())
    finally:
        p.terminate()
        try:
            p.wait(timeout=2)
        except Exception:
            p.kill()


def summarize_clocks(lines, device):
    sm, mx, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for ln in lines:
        f = [x.strip() for x in ln.split(",")]
        if len(f) < 9 or f[0] != str(device):
            continue
        try:
            sm.append(float(f[1]))
            mx = float(f[2])
        except ValueError:
            continue
        for n, v in zip(names, f[5:9]):
            if v.lower() == "active":
                reasons.add(n)
    if not sm:
        return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


# ---------------------------------------------------------------------------- ranks
def reduce_max(v: float, world: int, device=None) -> float:
    """Max of a per-rank value over all ranks (the slowest rank's time); the
    process group's backend decides the device of the exchange tensor."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(units_per_rank: float, ms: float, world: int) -> float:
    """Units all ranks processed (replicas: the same work on each rank, weak
    scaling) per second of the slowest rank's time."""
    return units_per_rank * world / (ms / 1e3)


# ---------------------------------------------------------------------------- CPU
class CpuJob:
    """One job of the workload in host memory for the CPU legs: the same seeded
    bytes as the GPU arm's rows (parpar_gb300.synth, generated by the oracle's
    C filler), the slice layout of the files, and the output buffers.  Nothing
    here loads a library of this repository's product."""

    def __init__(self, cfg, file_lens, seed=1):
        from oracle import oracle as O
        from parpar_gb300.layout import file_layout
        self.S, self.N, self.R = cfg["S"], cfg["N"], cfg["R"]
        self.hashes = cfg["hashes"]
        self.file_lens = np.array(file_lens, dtype=np.uint64)
        self.first_row, row_lens = file_layout(file_lens, self.S)
        self.lens = row_lens.astype(np.uint64)
        self.x = O.synth_rows(seed, 0, self.N, self.S)
        self.nums = np.arange(self.N, dtype=np.uint16)
        self.exps = np.arange(self.R, dtype=np.uint16)
        self.out = np.zeros((self.R, self.S), dtype=np.uint8)
        self.valid = np.zeros(self.R, dtype=np.int32)
        self.ifsc = np.zeros(self.N * 20, dtype=np.uint8)
        self.fmd5 = np.zeros(max(1, len(file_lens)) * 16, dtype=np.uint8)
        self.mul_adds = self.N * self.R * (self.S // 2)


def reference_core():
    """True when the reference's own CPU core is compiled on this host
    (oracle/_ref), else False and the reason it is not there."""
    from oracle import refsrc
    if not os.path.exists(refsrc.REF_LIB):
        err = os.path.join(refsrc.REF_OUT, "build_error.txt")
        why = open(err).read().strip().splitlines()[0] if os.path.exists(err) else \
            "reference sources not staged on this host (oracle/_ref/src)"
        return False, why
    return True, None


def _reference_step(job, threads):
    """One whole job through ParPar's PAR2Proc + PAR2ProcCPU (GF16_AUTO) with
    its HasherInput per file concurrently (oracle/ref_shim.cpp ref_job);
    returns (wall, gf, hash) seconds."""
    from oracle import oracle as O
    nf = len(job.file_lens) if job.hashes else 0
    out, valid, _, _, t = O.ref_job(job.x, job.lens, job.nums, job.exps, job.file_lens[:nf] if nf else None,
                                    job.first_row[:nf] if nf else None, threads)
    if not valid.all():
        raise RuntimeError("reference checksum verdict false")
    return t


def _port_step(job, threads):
    """The oracle's restatement of the reference's automatic SIMD method on
    this host (used only where the reference core did not build): the GF
    multiply-accumulate over `threads` threads and, concurrently, each file's
    IFSC + file MD5 on a thread of its own, as the reference runs them."""
    import concurrent.futures as cf
    from oracle import oracle as O
    if not hasattr(job, "coeffs"):
        job.coeffs = O.par2_coeff_matrix(job.nums, job.exps)
        for i in range(job.N):   # the restatement takes zero-padded rows
            job.x[i, int(job.lens[i]):] = 0
        job.port_fn, job.port_name = ((O.recover_clmul, O.lib().or_clmul_method().decode())
                                      if O.recover_clmul(job.x[:2, :64], job.coeffs[:1, :2]) is not None
                                      else (O.recover_fast, O.lib().or_fast_method().decode()))
    t0 = time.perf_counter()
    hash_t = [0.0]

    def hash_all():
        def one(f):
            a = int(job.first_row[f])
            n = max(1, (int(job.file_lens[f]) + job.S - 1) // job.S)
            O.hash_file(job.x[a:a + n].reshape(-1)[: int(job.file_lens[f])], job.S)
        with cf.ThreadPoolExecutor(max_workers=len(job.file_lens)) as ex:
            list(ex.map(one, range(len(job.file_lens))))
        hash_t[0] = time.perf_counter() - t0
    th = threading.Thread(target=hash_all) if job.hashes else None
    if th:
        th.start()
    job.out[:] = job.port_fn(job.x, job.coeffs, threads=threads)
    t_gf = time.perf_counter() - t0
    if th:
        th.join()
    return time.perf_counter() - t0, t_gf, hash_t[0]


def cpu_step_fn(threads):
    """(step function(job) -> (wall, gf, hash) seconds, description dict) of the
    best available CPU path: the reference's own core where it built on this
    host, else the oracle's port of its automatic method."""
    have, why = reference_core()
    if have:
        import ctypes
        from oracle import oracle as O
        buf = ctypes.create_string_buffer(512)
        O.ref().ref_host_info(buf, 512)
        info = dict(kv.split("=", 1) for kv in buf.value.decode().split(";") if "=" in kv)
        host = buf.value.decode().split(";")[-1]
        desc = {"kind": "reference", "cores": threads,
                "method": "ParPar PAR2ProcCPU, GF16_AUTO -> %s, %d threads; HasherInput per file (%s)"
                          % (info.get("method", "?"), threads, host)}
        return (lambda job: _reference_step(job, threads)), desc
    desc = {"kind": "port", "cores": threads, "reference_unavailable": why}

    def step(job):
        r = _port_step(job, threads)
        desc["method"] = "%s, %d threads (oracle restatement of the reference's automatic method)" % (job.port_name, threads)
        return r
    return step, desc


def cpu_baseline_run(cfg, file_lens, threads, steps=1):
    """cpu_baseline of the GPU arm's line: whole jobs of the workload through
    the best available CPU path (cpu_step_fn), `steps` of them after one
    untimed warm-up job."""
    job = CpuJob(cfg, file_lens)
    step, desc = cpu_step_fn(threads)
    step(job)
    walls = [step(job)[0] for _ in range(steps)]
    t = float(np.mean(walls))
    out = dict(desc)
    out.update({"value": job.mul_adds / t, "unit": UNIT,
                "sample": "%d whole job(s) of the workload (%d inputs x %d recovery x %d bytes%s), %.2f s each"
                          % (steps, job.N, job.R, job.S, " + IFSC + file MD5 per file" if job.hashes else "", t)})
    return out


def run_reference(args, cfg, file_lens):
    """--impl reference: the reference's CPU implementation of the path on this
    host's cores, one whole job per step, on the GPU arm's config, metric and
    unit.  Under torchrun only rank 0 measures."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    job = CpuJob(cfg, file_lens)
    step, desc = cpu_step_fn(threads)
    for _ in range(args.warmup):
        step(job)
    walls, gfs, hashes = [], [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        w, g, h = step(job)
        walls.append(w)
        gfs.append(g)
        hashes.append(h)
    wall = time.perf_counter() - t0
    ms = wall / args.steps * 1e3
    value = job.mul_adds / (ms / 1e3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16 GF(2^16)",
        "data": "synthetic (seeded splitmix64 slices)",
        "config": bench_config(args, cfg, file_lens, world),
        "src_GBps_x_recovery": job.N * job.S * job.R / (ms / 1e3) / 1e9,
        "p50_latency_s": float(np.percentile(walls, 50)), "p99_latency_s": float(np.percentile(walls, 99)),
        "cpu_parts_s": {"gf_mean": float(np.mean(gfs)), "hash_mean": float(np.mean(hashes))},
        "cpu_baseline": dict(desc, value=value, unit=UNIT,
                             sample="every step is one whole job of the workload (%d inputs x %d recovery x %d bytes%s); "
                                    "jobs run back to back" % (job.N, job.R, job.S,
                                                               " + IFSC + file MD5 per file" if job.hashes else "")),
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(line))
    return 0


def run_reference_mix(args, cfg):
    """--impl reference for the batched and serving workloads: the jobs of the
    same seeded mix through the reference's own CPU core one after another
    (the reference has no batching; PAR2ProcCPU with GF16_AUTO on all host
    cores, no hashing, as the GPU mix has none).  The whole mix would take the
    CPU minutes, so the sample is the mix's jobs in order whose estimated time
    fits a budget of --cpu-budget seconds; jobs/s for the whole mix follows
    from the sample's mul-adds/s, and p50/p99 are the sampled service times."""
    from oracle import oracle as O
    from parpar_gb300.layout import make_job_mix
    have, why = reference_core()
    if not have:
        print(json.dumps({"impl": "reference", "unavailable": why}))
        return 0
    threads = os.cpu_count() or 1
    jobs = make_job_mix(cfg["jobs"], seed=4 if args.workload == "batched" else 5)
    est_rate = 90e9   # first guess of the CPU's mul-adds/s, refined by the sample
    spent, done = 0.0, []
    for spec in jobs:
        if spent + spec.mul_adds / est_rate > args.cpu_budget or (spec.N + spec.R) * spec.S > 48 << 30:
            continue
        x = O.synth_rows(spec.seed, 0, spec.N, spec.S)
        t0 = time.perf_counter()
        out, valid, _, _, t = O.ref_job(x, np.full(spec.N, spec.S), np.arange(spec.N), spec.exps, threads=threads)
        wall = time.perf_counter() - t0
        if not valid.all():
            raise RuntimeError("reference checksum verdict false")
        done.append((spec, t[0]))
        spent += wall
        est_rate = sum(s.mul_adds for s, _ in done) / sum(w for _, w in done)
        del x, out
    if not done:
        print(json.dumps({"impl": "reference", "unavailable": "no job of the mix fits the CPU budget"}))
        return 0
    rate = sum(s.mul_adds for s, _ in done) / sum(w for _, w in done)
    mix = sum(s.mul_adds for s in jobs)
    walls = [w for _, w in done]
    info = ctypes.create_string_buffer(512)
    O.ref().ref_host_info(info, 512)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": 1,
        "warmup": 0, "ms_per_step": mix / rate * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u16 GF(2^16)", "data": "synthetic (seeded per-job slices)",
        "config": {"workload": args.workload, "desc": cfg["desc"], "jobs": len(jobs)},
        "jobs_per_s": len(jobs) / (mix / rate),
        "p50_latency_s": float(np.percentile(walls, 50)), "p99_latency_s": float(np.percentile(walls, 99)),
        "latency_def": "service time of each sampled job (jobs run back to back on all cores)",
        "cpu_baseline": {"kind": "reference", "cores": threads, "value": rate, "unit": UNIT,
                         "method": "ParPar PAR2ProcCPU, GF16_AUTO (%s), jobs back to back" % info.value.decode(),
                         "sample": "%d of the %d jobs of the mix (in mix order, those whose estimated time fits %.0f s), "
                                   "%.3g of %.3g mul-adds" % (len(done), len(jobs), args.cpu_budget,
                                                               sum(s.mul_adds for s, _ in done), mix)},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def bench_config(args, cfg, file_lens, world):
    """The `config` object of both arms' lines (identical for the same run)."""
    S, N = cfg["S"], cfg["N"]
    return {"workload": args.workload, "desc": cfg["desc"], "slice_bytes": S, "inputs": N, "recovery": cfg["R"],
            "files": len(file_lens),
            "l2": "inputs (%.1f GiB per job) larger than L2 (129 MB); no flush" % (N * S / 2**30),
            "parallelism": "replicas" if world > 1 else "single GPU"}


# ---------------------------------------------------------------------------- GPU
def single_job_measure(args, cfg, file_lens, job, steps, warmup, e2e=True):
    """One job at a time on the resident job's rows (ResidentJob): `steps`
    whole jobs back to back, each waiting for the previous one, timed with
    CUDA events; returns ms per job, the contraction's and file MD5's device
    times, and (e2e) the same job from pinned host buffers."""
    import torch
    from parpar_gb300 import _lib
    L = _lib.load()
    S, N, R = cfg["S"], cfg["N"], cfg["R"]
    ev = []

    def step(record=False):
        cur = torch.cuda.current_stream(job.dev)
        job.sa.wait_stream(cur)
        job.sb.wait_stream(cur)
        a, b = job.sa.cuda_stream, job.sb.cuda_stream
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)] if record else None
        _lib.check(L.par2cuda_rows_checksum(job.d_in.data_ptr(), job.pw, N, job.d_lens.data_ptr(), S, 0, None,
                                           job.d_ck.data_ptr(), a), "cksum")
        if cfg["hashes"]:
            if record:
                e[2].record(job.sb)
            _lib.check(L.par2cuda_file_md5(job.d_in.data_ptr(), job.pitch, len(file_lens), job.d_flen.data_ptr(),
                                          job.d_first.data_ptr(), S, job.d_fmd5.data_ptr(), b), "file_md5")
            if record:
                e[3].record(job.sb)
        if record:
            e[0].record(job.sa)
        _lib.check(L.par2cuda_muladd(job.d_in.data_ptr(), job.pw, N, job.d_coeff.data_ptr(), job.d_rec.data_ptr(),
                                    job.pw, R, job.row_words, 0, job.method, job.d_scratch.data_ptr(),
                                    job.scratch_bytes, a), "muladd")
        if record:
            e[1].record(job.sa)
        _lib.check(L.par2cuda_rows_checksum(job.d_rec.data_ptr(), job.pw, R, None, S, 1, job.d_flags.data_ptr(),
                                           job.d_ck.data_ptr(), a), "verify")
        if cfg["hashes"]:
            _lib.check(L.par2cuda_slice_hash(job.d_in.data_ptr(), job.pitch, N, job.d_lens.data_ptr(), S,
                                            job.d_ifsc.data_ptr(), a), "slice_hash")
        cur.wait_stream(job.sa)
        cur.wait_stream(job.sb)
        if record:
            ev.append(e)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(steps):
        step(record=True)
    t1.record()
    torch.cuda.synchronize()
    if int(job.d_flags.sum()) != R:
        raise RuntimeError("recovery checksum verification failed")
    out = {"ms_per_job": t0.elapsed_time(t1) / steps, "jobs": steps,
           "muladd_ms": float(np.mean([e[0].elapsed_time(e[1]) for e in ev])),
           "file_md5_ms": float(np.mean([e[2].elapsed_time(e[3]) for e in ev])) if cfg["hashes"] else 0.0,
           "launches_per_job": 4 + L.par2cuda_muladd_launches(R, N, job.row_words, job.method, job.scratch_bytes) +
                               (2 if cfg["hashes"] else 0)}
    out["value"] = N * R * (S // 2) / (out["ms_per_job"] / 1e3)
    if e2e:
        host_in = torch.empty((N, S), dtype=torch.uint8, pin_memory=True)
        host_in.copy_(job.d_in.view(torch.uint8)[:, :S])
        rec_host = torch.empty((R, S), dtype=torch.uint8, pin_memory=True)
        torch.cuda.synchronize()
        job.run_from_host(host_in, hashes=cfg["hashes"])
        job.download(rec_host)
        torch.cuda.synchronize()
        t0.record()
        for _ in range(steps):
            job.run_from_host(host_in, hashes=cfg["hashes"])
            _, _, _, flags = job.download(rec_host)
        t1.record()
        torch.cuda.synchronize()
        if int(flags.sum()) != R:
            raise RuntimeError("recovery checksum verification failed (e2e)")
        ems = t0.elapsed_time(t1) / steps
        out["e2e"] = {"value": N * R * (S // 2) / (ems / 1e3), "unit": UNIT, "h2d_bytes_per_step": N * S,
                      "d2h_bytes_per_step": job.d2h_bytes(), "ms_per_step": ems,
                      "path": "par2cuda C ABI: pinned host slices -> H2D (per file, largest first, file MD5s starting "
                              "as files land) -> job -> D2H recovery + IFSC + file MD5 + verdicts"}
        del host_in, rec_host
    return out


def stream_measure(args, cfg, file_lens, local, rank, barrier, max_over_ranks):
    """The job stream (parpar_gb300.stream.JobStream): args.steps jobs of the
    workload, args.slots resident at once, file MD5s pooled per args.group
    jobs; device-resident (value) and from pinned host buffers (e2e)."""
    import torch
    from parpar_gb300 import _lib
    from parpar_gb300.stream import JobStream
    S, N, R = cfg["S"], cfg["N"], cfg["R"]
    js = JobStream(S, file_lens, list(range(R)), slots=args.slots, group=args.group, device=local,
                   method=_lib.METHOD_NAMES[args.method], md5_block=args.md5_block, md5_staged=not args.md5_unstaged)
    js.fill_synthetic(seed0=1 + 1000 * rank)
    torch.cuda.synchronize()
    warm = max(args.warmup, args.group)
    js.run(warm, first_job=0)
    torch.cuda.synchronize()
    js.clear_records()
    launches0 = js.launches
    barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    js.run(args.steps, first_job=warm, timing=True)
    t1.record()
    torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(t0.elapsed_time(t1) / args.steps)
    used = min(js.slots, warm + args.steps)
    if int(js.d_flags[:used].sum()) != used * R:
        raise RuntimeError("recovery checksum verification failed in the job stream")
    lat = js.latencies()
    out = {"ms": ms, "launches": js.launches - launches0, "muladd_ms": js.muladd_ms(),
           "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
           "slots": js.slots, "group": js.group}
    if not args.no_e2e:
        host_in = [torch.empty((N, S), dtype=torch.uint8, pin_memory=True) for _ in range(2)]
        for k, h in enumerate(host_in):
            h.copy_(js.d_in.view(torch.uint8)[k * N:(k + 1) * N, :S])
        host_out = js.host_out_buffers(3)
        torch.cuda.synchronize()
        # the host->device copy rate of one job's inputs on its own
        c0 = torch.cuda.Event(enable_timing=True)
        c1 = torch.cuda.Event(enable_timing=True)
        L = _lib.load()
        cur = torch.cuda.current_stream()
        c0.record()
        _lib.check(L.par2cuda_copy_rows(js.d_in.data_ptr(), js.pitch, host_in[0].data_ptr(), S, S, N, cur.cuda_stream), "h2d")
        c1.record()
        torch.cuda.synchronize()
        h2d_gbps = N * S / (c0.elapsed_time(c1) / 1e3) / 1e9
        first = warm + args.steps
        js.run(warm, first_job=first, host_in=host_in, host_out=host_out)
        torch.cuda.synchronize()
        js.clear_records()
        barrier()
        t0.record()
        js.run(args.steps, first_job=first + warm, host_in=host_in, host_out=host_out, timing=True)
        t1.record()
        torch.cuda.synchronize()
        barrier()
        ems = max_over_ranks(t0.elapsed_time(t1) / args.steps)
        if not all(int(o[3].sum()) == R for o in host_out):
            raise RuntimeError("recovery checksum verification failed in the job stream (e2e)")
        lat = js.latencies()
        out["e2e"] = {"value": N * R * (S // 2) / (ems / 1e3), "unit": UNIT, "h2d_bytes_per_step": N * S,
                      "d2h_bytes_per_step": js.d2h_bytes(), "ms_per_step": ems,
                      "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                      "h2d_GBps_one_job": h2d_gbps,
                      "h2d_GBps_in_stream": (args.steps * N * S / (js.upload_span_ms() / 1e3) / 1e9
                                             if js.upload_span_ms() else None),
                      "size_classes": [len(c) for c in js.classes],
                      "path": "par2cuda C ABI, job stream: each job's slices copied from pinned host memory into "
                              "its slot by 2-D H2D copies (files in size classes, largest first across the jobs in flight; each "
                              "class's file MD5 launch per group starts when its rows have landed), the job's kernels, "
                              "one D2H of recovery + IFSC + file MD5 + verdicts into pinned host buffers; %d slots, "
                              "file MD5s pooled per %d jobs" % (js.slots, js.group)}
        del host_in, host_out
    del js
    torch.cuda.empty_cache()
    return out


def dense_measure(args, local, steps):
    """The 4096 x 4096 x 256 KiB contraction (configs' dense workload) inside
    the default run: device-resident value with its integer-ALU roofline, and
    e2e from pinned host buffers."""
    import torch
    from parpar_gb300 import _lib
    from parpar_gb300.job import ResidentJob
    cfg = WORKLOADS["dense"]
    S, N, R = cfg["S"], cfg["N"], cfg["R"]
    fl = [N * S]
    job = ResidentJob(S, fl, list(range(R)), device=local, method=_lib.METHOD_NAMES[args.dense_method])
    job.fill_synthetic(seed=7)
    torch.cuda.synchronize()
    r = single_job_measure(args, cfg, fl, job, steps, warmup=3, e2e=not args.no_e2e)
    del job
    torch.cuda.empty_cache()
    return r


def plugin_measure(args, cfg, file_lens, local, steps):
    """e2e through the reference-facing plugin boundary: the PAR2ProcCUDA
    engine driven the way GfProc drives a backend (src/gf.cc AddSlice /
    EndInput / GetOutputSlice) with pinned host slices; GF + internal checksum
    only (the reference's plugin does not hash; hashing is HasherInput's job)."""
    import torch
    from parpar_gb300 import _lib
    from parpar_gb300.gfproc import GfProc
    from parpar_gb300.layout import file_layout
    S, N, R = cfg["S"], cfg["N"], cfg["R"]
    _, row_lens = file_layout(file_lens, S)
    host_in = torch.empty((N, S), dtype=torch.uint8, pin_memory=True)
    tmp = torch.empty((N, S), dtype=torch.uint8, device=torch.device("cuda", local))
    _lib.check(_lib.load().par2cuda_synth_fill(tmp.data_ptr(), S, N, S, 1, 0,
                                              torch.cuda.current_stream().cuda_stream), "synth")
    host_in.copy_(tmp)
    del tmp
    rec_host = torch.empty((R, S), dtype=torch.uint8, pin_memory=True)
    g = GfProc(S, method=args.plugin_method, device=local, input_batchsize=args.plugin_batch)
    g.set_recovery_slices(list(range(R)))
    L = _lib.load()
    ctx = g._ctx
    ptrs = [host_in[i].data_ptr() for i in range(N)]
    lens_ = [int(x) for x in row_lens]
    null_cb = _lib.DONE_FN()  # NULL: no completion callback

    def plugin_pass():
        # the calls a native adapter makes: discardOutput, waitForAdd +
        # addInput per slice, endInput, getOutput per recovery slice
        L.par2cuda_discard_output(ctx)
        for i in range(N):
            L.par2cuda_wait_for_add(ctx)
            _lib.check(L.par2cuda_add_input(ctx, ptrs[i], lens_[i], i, 0, null_cb, None), "add")
        _lib.check(L.par2cuda_end_input(ctx, null_cb, None), "end")
        _lib.check(L.par2cuda_sync(ctx), "sync")
        # outputs without a per-slice callback (a ctypes callback into Python
        # costs ~57 us per slice, which is this harness's cost, not the
        # library's); verdicts read once all copies are done
        for r in range(R):
            _lib.check(L.par2cuda_get_output(ctx, r, rec_host[r].data_ptr(), null_cb, None), "get")
        _lib.check(L.par2cuda_sync(ctx), "sync")
        return all(L.par2cuda_output_valid(ctx, r) == 1 for r in range(R))
    for _ in range(3):
        plugin_pass()
    times = []
    okp = True
    for _ in range(steps):
        t0 = time.perf_counter()
        okp = plugin_pass() and okp
        times.append(time.perf_counter() - t0)
    if not okp:
        raise RuntimeError("plugin path checksum verdict failed")
    inf = g.info()
    g.close()
    tp = float(np.median(times))
    mul_adds = N * R * (S // 2)
    return {"value": mul_adds / tp, "unit": UNIT, "h2d_bytes_per_step": int(row_lens.sum()),
            "d2h_bytes_per_step": R * S, "ms_per_step": tp * 1e3, "steps": steps,
            "ms_min_max": [min(times) * 1e3, max(times) * 1e3],
            "ms_each": [round(t * 1e3, 2) for t in times],
            "spread": (max(times) - min(times)) / tp,
            "spread_p10_p90": float(np.percentile(times, 90) - np.percentile(times, 10)) / tp,
            "spread_iqr": float(np.percentile(times, 75) - np.percentile(times, 25)) / tp,
            "batch": inf["staging_size"], "staging_areas": inf["staging_count"], "method_desc": inf["method_desc"],
            "path": "C ABI plugin calls from the host: wait_for_add + add_input x N (pinned host slices), "
                    "end_input, get_output x R, verdicts by output_valid; GF multiply-accumulate + internal "
                    "checksum, no hashing (the reference plugin does not hash); host wall clock, median of steps"}


def roofline_gf(mul_adds, muladd_ms, lop3_ops, n_sm, sm_mhz, kname, alg_bytes):
    """Integer-ALU roofline of the contraction: 2 three-input LOP3 per word
    mul-add (16x16 GF(2) matrix, ~128 set bits, 32-way bit slicing) against the
    LOP3 rate measured on this device (par2cuda_lop3_rate)."""
    rate = mul_adds / (muladd_ms / 1e3)
    out = {"bound": "int-alu", "kernel": kname, "achieved": 2 * rate / 1e12, "peak": lop3_ops / 1e12,
           "unit": "Tops/s", "frac": 2 * rate / lop3_ops, "traffic": None, "alg_bytes": alg_bytes,
           "peak_source": "measured: LOP3 calibration kernel k_lop3_rate on this GPU (%.1f lanes/SM/clk at %.0f MHz); "
                          "nominal 128 lanes would be %.1f Tops/s"
                          % (lop3_ops / n_sm / (sm_mhz * 1e6), sm_mhz, n_sm * 128 * sm_mhz * 1e6 / 1e12),
           "mul_adds_per_s": rate, "muladd_ms": muladd_ms}
    if kname in KERNEL_TRAFFIC:
        # DRAM bytes per launch scaled from the ncu capture of the same kernel
        # (profiles/): inputs are read once and recovery rows written once, so
        # traffic grows with (N + R) x S
        tb, ab, what = KERNEL_TRAFFIC[kname]
        out["traffic"] = tb / ab * alg_bytes
        out["traffic_source"] = "ncu dram__bytes_read+write of %s (%.1f MB for %.1f MB algorithmic), scaled by " \
                                "(N+R)*S" % (what, tb / 1e6, ab / 1e6)
    return out


def tc4_gemm_traffic(N, R, n_words):
    """DRAM bytes of the GEMM launches of one tensor_fp4 call: the ncu capture
    of one launch of the same (inputs, recovery) shape, scaled by the call's
    expanded input-plane bytes (every launch but the last takes a 1 GiB word
    chunk); None for shapes without a capture."""
    cap = TC4_TRAFFIC.get((N, R))
    if cap is None:
        return None
    a_call = (N + 15) // 16 * 16 * 8 * ((n_words + 127) // 128 * 128)
    return cap[0] / cap[1] * a_call


def tc4_traffic_source(N, R):
    cap = TC4_TRAFFIC.get((N, R))
    return None if cap is None else ("ncu dram__bytes_read+write of %s: %.2f GB for %.2f GB of expanded input "
                                     "planes, scaled by this call's expanded input bytes" %
                                     (cap[2], cap[0] / 1e9, cap[1] / 1e9))


def roofline_tensor(mul_adds, muladd_ms, mma_macs, kname, traffic=None, traffic_source=None):
    """Tensor roofline of the block-scaled 4-bit form: 256 binary
    multiply-accumulates (512 flops) per word mul-add against the MMA rate of
    the same instruction measured on this device (par2cuda_tensor_fp4_rate);
    the call's time includes its two operand-preparation kernels."""
    flops = mul_adds * 512 / (muladd_ms / 1e3)
    return {"bound": "tensor", "kernel": kname, "achieved": flops / 1e12, "peak": 2 * mma_macs / 1e12,
            "unit": "TFLOP/s", "frac": flops / (2 * mma_macs), "traffic": traffic,
            "traffic_source": traffic_source if traffic else None,
            "peak_source": "measured: k_tc4_mma_rate, tcgen05.mma kind::mxf4 M=128 N=256 K=64 back to back on "
                           "shared-memory operands, one CTA per SM (nominal dense fp4 of the part: 13.5 PFLOP/s)",
            "mul_adds_per_s": mul_adds / (muladd_ms / 1e3), "muladd_ms": muladd_ms}


def run_ours(args, cfg, file_lens):
    import torch
    import torch.distributed as dist
    from parpar_gb300 import _lib
    from parpar_gb300.job import ResidentJob

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        if world > 1:
            dist.barrier()

    def max_over_ranks(v):
        return reduce_max(v, world, dev)

    S, N, R = cfg["S"], cfg["N"], cfg["R"]
    mul_adds = N * R * (S // 2)
    L = _lib.load()
    if args.comb_shape:
        _lib.check(L.par2cuda_set_comb_shape(args.comb_shape), "set_comb_shape")
    # roofline denominators measured on this device: the LOP3 rate (integer-ALU
    # bound of the contraction) and one MD5 chain's rate on one thread (the
    # latency bound of the one-stream-per-thread hash kernels)
    lop3 = ctypes.c_double(0)
    _lib.check(L.par2cuda_lop3_rate(ctypes.byref(lop3), None), "lop3_rate")
    md5_chain = ctypes.c_double(0)
    if cfg["hashes"]:
        _lib.check(L.par2cuda_md5_chain_rate(ctypes.byref(md5_chain), None), "md5_chain_rate")
    fp4_rate = ctypes.c_double(0)
    if "tensor_fp4" in (args.method, args.dense_method):
        _lib.check(L.par2cuda_tensor_fp4_rate(ctypes.byref(fp4_rate), None), "tensor_fp4_rate")
    torch.cuda.synchronize()

    clock_lines, stop = [], threading.Event()
    th = None
    if rank == 0 and not args.no_clocks:
        th = threading.Thread(target=sample_clocks, args=(stop, clock_lines), daemon=True)
        th.start()
        time.sleep(0.5)

    use_stream = cfg["hashes"] and args.slots > 1
    single = None
    if use_stream:
        st = stream_measure(args, cfg, file_lens, local, rank, barrier, max_over_ranks)
        ms, muladd_ms, e2e = st["ms"], st["muladd_ms"], st.get("e2e")
        launches = st["launches"]
        job = ResidentJob(S, file_lens, list(range(R)), device=local, method=_lib.METHOD_NAMES[args.method])
        job.fill_synthetic(seed=1 + rank)
        single = single_job_measure(args, cfg, file_lens, job, min(args.steps, 3), warmup=1, e2e=not args.no_e2e)
        del job
        torch.cuda.empty_cache()
    else:
        job = ResidentJob(S, file_lens, list(range(R)), device=local, method=_lib.METHOD_NAMES[args.method])
        job.fill_synthetic(seed=1 + rank)
        barrier()
        r = single_job_measure(args, cfg, file_lens, job, args.steps, warmup=args.warmup, e2e=not args.no_e2e)
        barrier()
        ms = max_over_ranks(r["ms_per_job"])
        muladd_ms, e2e = r["muladd_ms"], r.get("e2e")
        launches = r["launches_per_job"] * args.steps
        st = None
        del job
        torch.cuda.empty_cache()
    value = whole_job_value(mul_adds, ms, world)
    if e2e is not None:
        e2e["value"] = e2e["value"] * world

    dense = None
    if args.workload == "bandwidth" and not args.no_dense:
        dense = dense_measure(args, local, min(args.steps, 10))
    e2e_plugin = None
    if not args.no_e2e and not args.no_plugin:
        e2e_plugin = plugin_measure(args, cfg, file_lens, local, args.plugin_steps)

    stop.set()
    if th:
        th.join(timeout=3)
    clocks = summarize_clocks(clock_lines, local) if rank == 0 else None

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return 0

    peaks = measured_peaks()
    sm_mhz = (clocks or {}).get("sm_mhz") or (peaks or {}).get("sm_max_mhz") or 2070.0
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    kname = _lib.comb_kernel_name(L.par2cuda_comb_shape_for(R)) if args.method in ("comb", "auto") else \
        {"xor": "k_xor_planes", "nibble": "k_nibble_muladd", "tensor": "k_tc_muladd",
         "tensor_fp4": "k_tc4_gemm"}[args.method]
    alg_bytes = (N + R) * S  # read every input once, write every recovery once
    hbm_peak = (peaks or {}).get("hbm_gbs", 6800.0)
    rgf = roofline_gf(mul_adds, muladd_ms, lop3.value, n_sm, sm_mhz, kname, alg_bytes)
    if args.traffic_bytes:
        rgf["traffic"] = args.traffic_bytes
    rtc = roofline_tensor(mul_adds, muladd_ms, fp4_rate.value, kname, tc4_gemm_traffic(N, R, ((S + 7) // 8 * 8 + 8) // 2),
                          tc4_traffic_source(N, R)) if args.method == "tensor_fp4" else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u16 GF(2^16)", "data": "synthetic (seeded splitmix64 slices), inputs resident in HBM",
        "config": bench_config(args, cfg, file_lens, world),
        "step": ("one whole job of the workload; jobs stream through %d resident slots (file MD5 chains of %d jobs "
                 "pooled in one launch, %d per block, %s), the timed region holding every kernel of all %d jobs" %
                 (args.slots, args.group, args.md5_block,
                  "global loads" if args.md5_unstaged else "bytes staged in shared memory by bulk copies",
                  args.steps)) if use_stream else "one whole job, jobs back to back",
        "src_GBps_x_recovery": N * S * R * world / (ms / 1e3) / 1e9,
        "method": args.method,
        "roofline_gf": rgf,
        "roofline_hbm": {"bound": "hbm", "kernel": kname, "achieved": alg_bytes / (muladd_ms / 1e3) / 1e9,
                         "peak": hbm_peak, "unit": "GB/s", "frac": alg_bytes / (muladd_ms / 1e3) / 1e9 / hbm_peak,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6800 GB/s"},
        "gpu_launches": launches,
        "clocks": clocks,
        "e2e": e2e,
        "e2e_plugin": e2e_plugin,
    }
    if st is not None:
        line["p50_latency_s"] = st["p50_latency_s"]
        line["p99_latency_s"] = st["p99_latency_s"]
        line["latency_def"] = "per job: first kernel (its contraction side or its group's file MD5 launch) to last"
        line["kernels_ms"] = {"muladd_in_stream": muladd_ms, "step": ms}
    if single is not None:
        line["single_job"] = {"value": single["value"], "ms_per_job": single["ms_per_job"],
                              "muladd_ms": single["muladd_ms"], "file_md5_ms": single["file_md5_ms"],
                              "e2e": single.get("e2e"),
                              "desc": "one job in flight at a time: bound by the MD5 chain of its largest file "
                                      "(%.0f MB) on one GPU thread" % (max(file_lens) / 1e6)}
    if cfg["hashes"]:
        fm = single["file_md5_ms"] if single else None
        if fm:
            big = max(file_lens)
            line["roofline_md5"] = {
                "bound": "latency", "kernel": "k_file_md5", "achieved": big / (fm / 1e3) / 1e6,
                "peak": md5_chain.value / 1e6, "unit": "MB/s per GPU thread (largest file's chain)",
                "frac": big / (fm / 1e3) / md5_chain.value,
                "traffic": MD5_TRAFFIC[0] / MD5_TRAFFIC[1] * sum(file_lens),
                "traffic_source": "ncu dram__bytes_read+write of k_file_md5 on 4 files (%.1f MB for %.1f MB hashed), "
                                  "scaled by the bytes hashed" % (MD5_TRAFFIC[0] / 1e6, MD5_TRAFFIC[1] / 1e6),
                "peak_source": "measured: k_md5_chain, one MD5 stream on one thread with its data in registers"}
    # `roofline`: the kernel that takes most of the timed region's device time
    # (the contraction in the job stream and the dense workload)
    if rtc is not None:
        line["roofline_tensor"] = rtc
    line["roofline"] = dict(rtc if rtc is not None else rgf)
    if dense is not None:
        dm = WORKLOADS["dense"]
        d_mul = dm["N"] * dm["R"] * (dm["S"] // 2)
        dkn = {"xor": "k_xor_planes", "nibble": "k_nibble_muladd", "tensor": "k_tc_muladd", "tensor_fp4": "k_tc4_gemm"}
        dk = _lib.comb_kernel_name(L.par2cuda_comb_shape_for(dm["R"])) if args.dense_method in ("comb", "auto") else \
            dkn[args.dense_method]
        line["dense"] = {"desc": dm["desc"], "method": args.dense_method, "value": dense["value"], "unit": UNIT,
                         "ms_per_step": dense["ms_per_job"], "steps": dense["jobs"], "e2e": dense.get("e2e"),
                         "roofline_gf": roofline_gf(d_mul, dense["muladd_ms"], lop3.value, n_sm, sm_mhz, dk,
                                                    (dm["N"] + dm["R"]) * dm["S"])}
        if args.dense_method == "tensor_fp4":
            line["dense"]["roofline_tensor"] = roofline_tensor(
                d_mul, dense["muladd_ms"], fp4_rate.value, dk,
                tc4_gemm_traffic(dm["N"], dm["R"], ((dm["S"] + 7) // 8 * 8 + 8) // 2), tc4_traffic_source(dm["N"], dm["R"]))
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline_run(cfg, file_lens, os.cpu_count() or 1)
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_serving_workload(args, cfg):
    """Serving: Poisson arrivals at 200/s (offered load above the GPU's
    capacity) and at a sub-saturation rate; latency = completion - arrival."""
    import torch
    from parpar_gb300 import autotune
    from parpar_gb300.serve import Server, make_requests, serve_stats
    torch.cuda.set_device(0)
    autotune.warm()
    # untimed warm-up passes of the loop: kernel modules load on first use and
    # the caching allocator grows to the working set (tens of GB) on the first pass
    for _ in range(max(1, args.warmup // 3)):
        Server(budget_bytes=150 * 10**9, slots=8).run(make_requests(cfg["jobs"], 200.0, seed=5))
    out = {}
    for label, rate, n in (("offered_200_per_s", 200.0, cfg["jobs"]), ("sub_saturation_4_per_s", 4.0, cfg["jobs"] // 2)):
        reqs = make_requests(n, rate, seed=5)
        srv = Server(budget_bytes=150 * 10**9, slots=8)
        t0 = time.perf_counter()
        done = srv.run(reqs)
        wall = time.perf_counter() - t0
        st = serve_stats(done)
        st["rate_per_s"] = rate
        st["wall_s"] = wall
        st["gpu_launches"] = srv.launches
        out[label] = st
    sat = out["offered_200_per_s"]
    line = {
        "metric": METRIC, "value": sat["mul_adds_per_s"], "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 0,
        "ms_per_step": sat["span_s"] * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u16 GF(2^16)", "data": "synthetic (seeded per-request slices generated on the device)",
        "config": {"workload": "serving", "desc": cfg["desc"], "jobs": cfg["jobs"], "budget_GB": 150, "slots": 8},
        "jobs_per_s": sat["jobs_per_s"], "p50_latency_s": sat["p50_latency_s"], "p99_latency_s": sat["p99_latency_s"],
        "rates": out, "autotune": {str(k): v[0] for k, v in autotune.table().items()},
        "autotune_methods": {str(k): v for k, v in autotune.method_table().items()},
        "gpu_launches": sat["gpu_launches"],
    }
    print(json.dumps(line))
    return 0


def small_mix_run(args):
    """Supplement to the 64-job mix: 512 small jobs (N log-uniform [10, 200],
    S 64 KiB..1 MiB, R 1-30 % of N), where per-job launches leave the GPU
    partly idle; per-job launches (each with its tuned multiply method) vs the
    tuned batched graph."""
    import torch
    from parpar_gb300.batch import BatchRunner, make_job_mix
    jobs = make_job_mix(512, seed=6, n_range=(10, 200), s_range=(64 * 1024, 1 << 20))
    runner = BatchRunner(jobs, budget_bytes=args.budget_gib << 30)
    runner.run_per_job(tuned_methods=True)
    t0 = time.perf_counter()
    runner.run_per_job(tuned_methods=True)
    t_job = time.perf_counter() - t0
    modes = runner.tune_mode()
    runner.capture()
    for _ in range(max(args.warmup, 1)):
        runner.run_batched()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        runner.run_batched()
    e1.record()
    torch.cuda.synchronize()
    assert runner.all_valid()
    ms = e0.elapsed_time(e1) / args.steps
    return {"jobs": len(jobs), "mul_adds": runner.mul_adds, "passes": runner.P,
            "batched_jobs_per_s": len(jobs) / (ms / 1e3), "per_job_jobs_per_s": len(jobs) / t_job,
            "speedup_vs_per_job_launch": t_job / (ms / 1e3), "batched_mode": runner.mode, "mode_pass0_ms": modes}


def run_create_workload(args, cfg):
    """Files on disk -> .par2 files through parpar_gb300.create (wall clock;
    the input files are written once before timing and are in the page cache)."""
    import tempfile
    import torch
    from parpar_gb300 import synth
    from parpar_gb300.create import create
    S, N, R = cfg["S"], cfg["N"], cfg["R"]
    file_lens = file_lengths(N, cfg["files"], S, seed=2000)
    work = tempfile.mkdtemp(prefix="par2cuda_create_")
    paths = []
    row = 0
    for f, ln in enumerate(file_lens):
        n = (ln + S - 1) // S
        data = synth.slices(1, row, n, S).reshape(-1)[:ln]
        p = os.path.join(work, "file%02d.bin" % f)
        data.tofile(p)
        paths.append(p)
        row += n
    out_base = os.path.join(work, "set")
    torch.cuda.set_device(0)
    for _ in range(max(1, args.warmup)):
        create(paths, S, R, out_base)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        outs = create(paths, S, R, out_base)
        times.append(time.perf_counter() - t0)
    out_bytes = sum(os.path.getsize(o) for o in outs)
    for p in paths + outs:
        os.remove(p)
    os.rmdir(work)
    t = float(np.median(times))
    mul_adds = N * R * (S // 2)
    line = {
        "metric": METRIC, "value": mul_adds / t, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u16 GF(2^16)", "data": "synthetic seeded files on the host's disk (page cache)",
        "config": {"workload": "create", "desc": cfg["desc"], "slice_bytes": S, "inputs": N, "recovery": R,
                   "files": len(file_lens), "input_bytes": int(sum(file_lens)), "output_bytes": out_bytes,
                   "output_files": len(outs)},
        "input_GBps": sum(file_lens) / t / 1e9,
        "e2e": {"value": mul_adds / t, "unit": UNIT, "h2d_bytes_per_step": int(sum(file_lens)),
                "d2h_bytes_per_step": R * S, "path": "parpar_gb300.create: files -> pinned ring -> HBM -> "
                                                     "hashes + recovery -> .par2 files (host wall clock)"},
        "gpu_launches": None,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_run(cfg, file_lens, os.cpu_count() or 1)
    print(json.dumps(line))
    return 0


def run_profile_case(args, cfg):
    """The profile_* capture cases that are not multiply-accumulate workloads:
    runs the kernel(s) once after a warm-up and prints a short JSON line."""
    import torch
    from parpar_gb300 import _lib
    torch.cuda.set_device(0)
    if args.workload == "profile_rows_md5":
        from parpar_gb300.job import ResidentJob
        S, N, R = cfg["S"], cfg["N"], cfg["R"]
        job = ResidentJob(S, [N * S], list(range(R)))
        job.fill_synthetic(seed=3)
        job.run(hashes=False)
        for _ in range(2):
            md5s = job.recovery_packet_md5s(bytes(16))
        ok = bool(job.d_flags.all()) and len(md5s) == R
    else:
        from parpar_gb300.batch import BatchRunner
        from parpar_gb300.layout import make_job_mix
        jobs = make_job_mix(cfg["jobs"], seed=9, n_range=(64, 600), s_range=(256 * 1024, 2 << 20))
        runner = BatchRunner(jobs, budget_bytes=args.budget_gib << 30)
        times = runner.tune_mode()
        ok = True
        md5s = times
    torch.cuda.synchronize()
    print(json.dumps({"workload": args.workload, "ok": ok, "desc": cfg["desc"],
                      "detail": md5s if isinstance(md5s, dict) else None}))
    return 0 if ok else 1


def run_batched_workload(args, cfg):
    """The uneven 64-job mix, batched (graph replay) vs per-job launches."""
    import torch
    from parpar_gb300 import autotune
    from parpar_gb300.batch import BatchRunner, make_job_mix
    torch.cuda.set_device(0)
    jobs = make_job_mix(cfg["jobs"], seed=4)
    runner = BatchRunner(jobs, budget_bytes=args.budget_gib << 30)
    mul_adds = runner.mul_adds
    # per-job launches: each job's passes, then wait for the job
    for _ in range(max(1, args.warmup // 3)):
        runner.run_per_job()
    t0 = time.perf_counter()
    lat = runner.run_per_job()
    t_job = time.perf_counter() - t0
    assert runner.all_valid()
    # per-job launches with the multiply method the batched path uses for each
    # job (the autotuner's choice per recovery count): the batching gain alone
    runner.run_per_job(tuned_methods=True)
    t0 = time.perf_counter()
    lat_tuned = runner.run_per_job(tuned_methods=True)
    t_job_tuned = time.perf_counter() - t0
    assert runner.all_valid()
    mode_ms = runner.tune_mode()   # persistent launch vs per-job grid launches, pass 0 timed on the device
    runner.capture()
    for _ in range(args.warmup):
        runner.run_batched()
    torch.cuda.synchronize()
    clock_lines, stop = [], threading.Event()
    th = None
    if not args.no_clocks:
        th = threading.Thread(target=sample_clocks, args=(stop, clock_lines), daemon=True)
        th.start()
        time.sleep(0.5)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        runner.run_batched()
    e1.record()
    torch.cuda.synchronize()
    stop.set()
    if th:
        th.join(timeout=3)
    assert runner.all_valid()
    ms = e0.elapsed_time(e1) / args.steps
    line = {
        "metric": METRIC, "value": mul_adds / (ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u16 GF(2^16)", "data": "synthetic (seeded per-job slices generated on the device per pass)",
        "config": {"workload": "batched", "desc": cfg["desc"], "jobs": len(jobs), "passes": runner.P,
                   "input_GB": sum(j.input_bytes for j in jobs) / 1e9, "mul_adds": mul_adds,
                   "l2": "per-pass working set tens of GB, far above L2"},
        "jobs_per_s": len(jobs) / (ms / 1e3),
        "per_job_launch": {"jobs_per_s": len(jobs) / t_job, "s": t_job,
                           "p50_job_s": float(np.percentile(lat, 50)), "p99_job_s": float(np.percentile(lat, 99))},
        "per_job_launch_tuned_methods": {"jobs_per_s": len(jobs) / t_job_tuned, "s": t_job_tuned,
                                         "p50_job_s": float(np.percentile(lat_tuned, 50)),
                                         "p99_job_s": float(np.percentile(lat_tuned, 99))},
        "speedup_vs_per_job_launch": (len(jobs) / (ms / 1e3)) / (len(jobs) / t_job_tuned),
        "speedup_vs_per_job_launch_comb": (len(jobs) / (ms / 1e3)) / (len(jobs) / t_job),
        "speedup_def": "speedup_vs_per_job_launch: batched vs each job launched on its own with the same per-job "
                       "multiply method (the batching gain); _comb: vs each job on its own with the single-job "
                       "default method (comb)",
        "batched_mode": runner.mode, "mode_pass0_ms": mode_ms,
        "small_jobs_mix": small_mix_run(args),
        "autotune": {str(k): v[0] for k, v in autotune.table().items()},
        "autotune_methods": {str(k): v for k, v in autotune.method_table().items()},
        "gpu_launches": runner.launches_per_run() * args.steps,
        "clocks": summarize_clocks(clock_lines, 0),
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # a step is one whole job; the job stream's timed region cannot be shorter
    # than one job's longest file MD5 chain (~1.3 s), so K = 20 jobs by default
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="bandwidth")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-clocks", action="store_true")
    ap.add_argument("--no-plugin", action="store_true", help="skip the plugin-boundary e2e measurement")
    ap.add_argument("--plugin-steps", type=int, default=9)
    ap.add_argument("--plugin-method", choices=["auto", "comb", "xor", "nibble", "tensor", "tensor_fp4"],
                    default="tensor_fp4", help="backend method of the plugin-boundary measurement")
    ap.add_argument("--plugin-batch", type=int, default=0,
                    help="inputs per staging area of the plugin-boundary measurement (0 = the backend's default)")
    ap.add_argument("--method", choices=["auto", "comb", "xor", "nibble", "tensor", "tensor_fp4"], default="tensor_fp4",
                    help="multiply-accumulate kernel of the resident-job workloads and the job stream")
    ap.add_argument("--budget-gib", type=int, default=64, help="HBM budget of one pass of the batched workload")
    ap.add_argument("--comb-shape", type=int, default=0,
                    help="pin the comb kernel's CTA shape (par2cuda_set_comb_shape; 0 = automatic)")
    ap.add_argument("--slots", type=int, default=24,
                    help="jobs resident at once in the job stream of hashing workloads (1 = one job at a time)")
    ap.add_argument("--group", type=int, default=8, help="jobs whose file MD5 chains share one launch in the job stream")
    ap.add_argument("--md5-block", type=int, default=64, help="file MD5 chains per block in the job stream (32..512)")
    ap.add_argument("--md5-unstaged", action="store_true",
                    help="file MD5 chains load from global memory (par2cuda_file_md5_pooled) instead of bulk-copy staging")
    ap.add_argument("--cpu-budget", type=float, default=40.0,
                    help="seconds of CPU work in the reference arm's sample of the batched / serving mix")
    ap.add_argument("--no-dense", action="store_true", help="skip the dense-contraction figure of the default run")
    ap.add_argument("--dense-method", choices=["comb", "xor", "nibble", "tensor", "tensor_fp4"], default="tensor_fp4",
                    help="multiply-accumulate kernel of the default run's dense figure")
    ap.add_argument("--traffic-bytes", type=float, default=None,
                    help="DRAM bytes per comb launch from an ncu capture (profiles/), reported as roofline_gf.traffic")
    args = ap.parse_args()
    cfg = WORKLOADS[args.workload]
    if args.workload in ("batched", "serving", "create") and int(os.environ.get("RANK", "0")) != 0:
        return 0   # single-GPU workloads: under torchrun only rank 0 measures
    if args.workload in ("batched", "serving"):
        if args.impl == "reference":
            return run_reference_mix(args, cfg)
        return run_batched_workload(args, cfg) if args.workload == "batched" else run_serving_workload(args, cfg)
    if args.workload in ("profile_rows_md5", "profile_batched"):
        return run_profile_case(args, cfg)
    if args.workload == "create" and args.impl != "reference":
        return run_create_workload(args, cfg)
    file_lens = file_lengths(cfg["N"], cfg["files"], cfg["S"], seed=2000)
    if args.impl == "reference":
        return run_reference(args, cfg, file_lens)
    return run_ours(args, cfg, file_lens)


if __name__ == "__main__":
    sys.exit(main())
