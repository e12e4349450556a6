"""Benchmark: PAR2 recovery generation on one GB300 vs the reference's CPU path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload bandwidth|dense|plain|batched|serving] [--no-e2e] [--no-cpu-baseline]

Workload (default "bandwidth", the configuration the metric is quoted on):
2000 input slices x 2 MiB (40 files of seeded uneven lengths; the last slice of
each file zero-padded), 200 recovery slices (exponents 0..199), with the
per-slice MD5+CRC32 (IFSC) and per-file MD5 hashes, single read pass.  One
step = one whole job.  Inputs are seeded synthetic data (parpar_gb300.synth).

value: GF16 mul-adds/s with the inputs resident in HBM (device-timed with CUDA
events).  e2e: the same job through the C ABI with pinned host buffers, the
input H2D and result D2H inside the timed region.  --impl reference times the
reference algorithm's CPU implementation on this host's cores.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GF16 mul-adds/s"
UNIT = "mul-adds/s"

# one ncu capture per contraction kernel on a 512-input x 512 KiB case:
# dram__bytes_read.sum + dram__bytes_write.sum, and the algorithmic (N + R) x S
# one ncu capture of k_file_md5 (4 files, 266.6 MB in all): DRAM bytes per byte hashed
MD5_TRAFFIC = (272723456 + 4043776, 266590293)
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
    "profile_hash": dict(S=1048576, N=256, files=4, R=8, hashes=True,
                         desc="256 input slices x 1 MiB over 4 files, 8 recovery, with hashing (ncu capture size)"),
    # the bandwidth workload as files on the host's disk: files in, finished .par2 files out
    "create": dict(S=2 * 1048576, N=2000, files=40, R=200, hashes=True,
                   desc="the bandwidth workload's 40 files (3.9 GiB) written to the host's disk, then PAR2 create "
                        "end to end: read, GPU hashing + recovery, .par2 index + pow2 volumes written"),
    # serving: Poisson requests, admitted by free HBM, continuous batching
    "serving": dict(S=0, N=0, files=0, R=0, hashes=False, jobs=48,
                    desc="Poisson requests (sizes as the 64-job mix) at 200/s and at a sub-saturation rate; admission by "
                         "free HBM (<=150 GB), chunked when over budget; jobs/s and p50/p99 latency"),
    # batched: 64 uneven jobs, one graph-captured sequence of launches per pass
    "batched": dict(S=0, N=0, files=0, R=0, hashes=False, jobs=64,
                    desc="64 PAR2 jobs: N log-uniform [10,5000], S uniform 64 KiB..8 MiB (4-byte steps), R 1-30% of N; "
                         "byte-window passes under a 64 GiB HBM budget; persistent graph-captured comb launches vs per-job launches"),
}


def file_lengths(N, files, S, seed):
    """Seeded uneven file lengths with sum(ceil(len/S)) == N, last slice partial."""
    rng = np.random.default_rng(seed)
    if files == 1:
        return [N * S]
    w = rng.uniform(0.5, 1.5, size=files)
    counts = np.maximum(1, np.floor(w / w.sum() * N)).astype(int)
    while counts.sum() < N:
        counts[rng.integers(files)] += 1
    while counts.sum() > N:
        k = int(np.argmax(counts))
        counts[k] -= 1
    tails = rng.integers(1, S + 1, size=files)
    return [int((c - 1) * S + t) for c, t in zip(counts, tails)]


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
    """The reference's own CPU core compiled on this host (oracle/_ref), or
    None and the reason it is not there."""
    import ctypes
    from oracle import refsrc
    if not os.path.exists(refsrc.REF_LIB):
        err = os.path.join(refsrc.REF_OUT, "build_error.txt")
        why = open(err).read().strip().splitlines()[0] if os.path.exists(err) else \
            "reference sources not staged on this host (oracle/_ref/src)"
        return None, why
    L = ctypes.CDLL(refsrc.REF_LIB)
    vp, sz, u = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint
    L.ref_job.restype = ctypes.c_int
    L.ref_job.argtypes = [vp, sz, vp, vp, u, sz, vp, u, vp, vp, vp, vp, u, vp, vp, ctypes.c_int,
                          ctypes.POINTER(ctypes.c_double)]
    L.ref_host_info.restype = ctypes.c_int
    L.ref_host_info.argtypes = [ctypes.c_char_p, sz]
    L.ref_last_method_name.restype = ctypes.c_char_p
    return L, None


def _reference_step(L, job, threads):
    """One whole job through ParPar's PAR2Proc + PAR2ProcCPU (GF16_AUTO) with
    its HasherInput per file concurrently (oracle/ref_shim.cpp ref_job);
    returns (wall, gf, hash) seconds."""
    import ctypes
    from oracle.oracle import _p
    t = (ctypes.c_double * 3)()
    nf = len(job.file_lens) if job.hashes else 0
    rc = L.ref_job(_p(job.x), job.S, _p(job.lens), _p(job.nums), job.N, job.S, _p(job.exps), job.R, _p(job.out),
                   _p(job.valid), _p(job.file_lens), _p(job.first_row), nf, _p(job.ifsc), _p(job.fmd5), threads, t)
    if rc != 0:
        raise RuntimeError("reference job failed: %d" % rc)
    if not job.valid.all():
        raise RuntimeError("reference checksum verdict false")
    return t[0], t[1], t[2]


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
    L, why = reference_core()
    if L is not None:
        import ctypes
        buf = ctypes.create_string_buffer(512)
        L.ref_host_info(buf, 512)
        info = dict(kv.split("=", 1) for kv in buf.value.decode().split(";") if "=" in kv)
        host = buf.value.decode().split(";")[-1]
        desc = {"kind": "reference", "cores": threads,
                "method": "ParPar PAR2ProcCPU, GF16_AUTO -> %s, %d threads; HasherInput per file (%s)"
                          % (info.get("method", "?"), threads, host)}
        return (lambda job: _reference_step(L, job, threads)), desc
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


def bench_config(args, cfg, file_lens, world):
    """The `config` object of both arms' lines (identical for the same run)."""
    S, N = cfg["S"], cfg["N"]
    return {"workload": args.workload, "desc": cfg["desc"], "slice_bytes": S, "inputs": N, "recovery": cfg["R"],
            "files": len(file_lens),
            "l2": "inputs (%.1f GiB per job) larger than L2 (129 MB); no flush" % (N * S / 2**30),
            "parallelism": "replicas" if world > 1 else "single GPU"}


# ---------------------------------------------------------------------------- GPU
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
    if args.comb_shape:
        _lib.check(_lib.load().par2cuda_set_comb_shape(args.comb_shape), "set_comb_shape")
    job = ResidentJob(S, file_lens, list(range(R)), device=local, method=_lib.METHOD_NAMES[args.method])
    job.fill_synthetic(seed=1 + rank)
    torch.cuda.synchronize()

    # per-kernel events on the launching streams (comb kernel on A, file MD5 on B)
    L = _lib.load()
    ev = []

    def step(record=False):
        h0 = h1 = None
        cur = torch.cuda.current_stream(dev)
        job.sa.wait_stream(cur)
        job.sb.wait_stream(cur)
        a, b = job.sa.cuda_stream, job.sb.cuda_stream
        _lib.check(L.par2cuda_rows_checksum(job.d_in.data_ptr(), job.pw, N, job.d_lens.data_ptr(), S, 0, None,
                                           job.d_ck.data_ptr(), a), "cksum")
        if cfg["hashes"]:
            # the file MD5s (long serial chains) start at once on B; they read
            # only each file's own bytes
            h0 = torch.cuda.Event(enable_timing=True) if record else None
            h1 = torch.cuda.Event(enable_timing=True) if record else None
            if record:
                h0.record(job.sb)
            _lib.check(L.par2cuda_file_md5(job.d_in.data_ptr(), job.pitch, len(file_lens), job.d_flen.data_ptr(),
                                          job.d_first.data_ptr(), S, job.d_fmd5.data_ptr(), b), "file_md5")
            if record:
                h1.record(job.sb)
        k0 = torch.cuda.Event(enable_timing=True) if record else None
        k1 = torch.cuda.Event(enable_timing=True) if record else None
        if record:
            k0.record(job.sa)
        _lib.check(L.par2cuda_muladd(job.d_in.data_ptr(), job.pw, N, job.d_coeff.data_ptr(), job.d_rec.data_ptr(),
                                    job.pw, R, job.row_words, 0, job.method, job.d_scratch.data_ptr(),
                                    job.scratch_bytes, a), "muladd")
        if record:
            k1.record(job.sa)
        _lib.check(L.par2cuda_rows_checksum(job.d_rec.data_ptr(), job.pw, R, None, S, 1, job.d_flags.data_ptr(),
                                           job.d_ck.data_ptr(), a), "verify")
        if cfg["hashes"]:
            _lib.check(L.par2cuda_slice_hash(job.d_in.data_ptr(), job.pitch, N, job.d_lens.data_ptr(), S,
                                            job.d_ifsc.data_ptr(), a), "slice_hash")
        cur.wait_stream(job.sa)
        cur.wait_stream(job.sb)
        if record:
            ev.append((k0, k1, h0, h1))

    launches_per_step = 6 + (2 if cfg["hashes"] else 0)  # cksum x2, coeff->idx, comb, verify x2 (+ slice hash, file md5)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    assert int(job.d_flags.sum()) == R, "recovery checksum verification failed"
    # roofline denominators measured on this device: the LOP3 rate (integer-ALU
    # bound of the contraction) and one MD5 chain's rate on one thread (the
    # latency bound of the one-stream-per-thread hash kernels)
    lop3 = ctypes.c_double(0)
    _lib.check(L.par2cuda_lop3_rate(ctypes.byref(lop3), None), "lop3_rate")
    md5_chain = ctypes.c_double(0)
    if cfg["hashes"]:
        _lib.check(L.par2cuda_md5_chain_rate(ctypes.byref(md5_chain), None), "md5_chain_rate")
    torch.cuda.synchronize()

    clock_lines, stop = [], threading.Event()
    th = None
    if rank == 0 and not args.no_clocks:
        th = threading.Thread(target=sample_clocks, args=(stop, clock_lines), daemon=True)
        th.start()
        time.sleep(0.5)
    barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(args.steps):
        step(record=True)
    t1.record()
    torch.cuda.synchronize()
    barrier()
    ms = t0.elapsed_time(t1) / args.steps
    ms = max_over_ranks(ms)
    comb_ms = float(np.mean([k0.elapsed_time(k1) for k0, k1, _, _ in ev]))
    hash_ms = float(np.mean([h0.elapsed_time(h1) for _, _, h0, h1 in ev])) if cfg["hashes"] else 0.0
    value = whole_job_value(mul_adds, ms, world)

    # e2e: pinned host inputs -> H2D -> job -> D2H of every result, via the C ABI
    e2e = None
    if not args.no_e2e:
        host_in = torch.empty((N, S), dtype=torch.uint8, pin_memory=True)
        host_in.copy_(job.d_in.view(torch.uint8)[:, :S])
        rec_host = torch.empty((R, S), dtype=torch.uint8, pin_memory=True)
        torch.cuda.synchronize()
        for _ in range(max(1, args.warmup // 2)):
            job.run_from_host(host_in, hashes=cfg["hashes"])
            job.download(rec_host)
        torch.cuda.synchronize()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            job.run_from_host(host_in, hashes=cfg["hashes"])
            _, _, _, flags = job.download(rec_host)
        e1.record()
        torch.cuda.synchronize()
        barrier()
        ems = max_over_ranks(e0.elapsed_time(e1) / args.steps)
        assert int(flags.sum()) == R
        e2e = {"value": mul_adds * world / (ems / 1e3), "unit": UNIT, "h2d_bytes_per_step": N * S,
               "d2h_bytes_per_step": job.d2h_bytes(), "ms_per_step": ems,
               "path": "par2cuda C ABI: pinned host slices -> H2D (per file, largest first, file MD5s starting as "
                       "files land) -> job -> D2H recovery + IFSC + file MD5 + verdicts"}
    # e2e through the reference-facing plugin boundary: the PAR2ProcCUDA engine
    # driven like GfProc (src/gf.cc AddSlice / EndInput / GetOutputSlice) with
    # pinned host slices; GF + internal checksum only (the reference's plugin
    # does not hash; hashing is HasherInput's job)
    e2e_plugin = None
    if not args.no_e2e and not args.no_plugin:
        from parpar_gb300.gfproc import GfProc
        from parpar_gb300.job import file_layout
        _, row_lens = file_layout(file_lens, S)
        g = GfProc(S, method=args.method, device=local)
        g.set_recovery_slices(list(range(R)))
        views = [host_in[i, : int(row_lens[i])] for i in range(N)]

        L2 = _lib.load()
        ctx = g._ctx
        ptrs = [v.data_ptr() for v in views]
        lens_ = [int(x) for x in row_lens]
        null_cb = _lib.DONE_FN()  # NULL: no completion callback

        def plugin_pass():
            # the calls a native adapter makes: discardOutput, waitForAdd +
            # addInput per slice, endInput, getOutput per recovery slice
            L2.par2cuda_discard_output(ctx)
            for i in range(N):
                L2.par2cuda_wait_for_add(ctx)
                _lib.check(L2.par2cuda_add_input(ctx, ptrs[i], lens_[i], i, 0, null_cb, None), "add")
            _lib.check(L2.par2cuda_end_input(ctx, null_cb, None), "end")
            _lib.check(L2.par2cuda_sync(ctx), "sync")
            # outputs without a per-slice callback (a ctypes callback into Python
            # costs ~57 us per slice, which is this harness's cost, not the
            # library's); verdicts read once all copies are done
            for r in range(R):
                _lib.check(L2.par2cuda_get_output(ctx, r, rec_host[r].data_ptr(), null_cb, None), "get")
            _lib.check(L2.par2cuda_sync(ctx), "sync")
            return all(L2.par2cuda_output_valid(ctx, r) == 1 for r in range(R))
        plugin_pass()
        t0p = time.perf_counter()
        okp = True
        for _ in range(args.plugin_steps):
            okp = plugin_pass() and okp
        tp = (time.perf_counter() - t0p) / args.plugin_steps
        assert okp, "plugin path checksum verdict failed"
        inf = g.info()
        g.close()
        e2e_plugin = {"value": mul_adds * world / tp, "unit": UNIT, "h2d_bytes_per_step": int(row_lens.sum()),
                      "d2h_bytes_per_step": R * S, "ms_per_step": tp * 1e3, "steps": args.plugin_steps,
                      "batch": inf["staging_size"], "staging_areas": inf["staging_count"], "method_desc": inf["method_desc"],
                      "path": "C ABI plugin calls from the host: wait_for_add + add_input x N (pinned host slices), "
                              "end_input, get_output x R, verdicts by output_valid; GF multiply-accumulate + internal "
                              "checksum, no hashing (the reference plugin does not hash); host wall clock"}
    # several independent jobs in flight: job k runs its whole pass on its own
    # context stream with its own seeded inputs, so one job's per-file MD5
    # chains (serial, ~100 MB/s per GPU thread) overlap the others' work;
    # each job's steps stay in order on its stream
    inflight = None
    if args.inflight > 1 and cfg["hashes"]:
        jobs_k = [job] + [ResidentJob(S, file_lens, list(range(R)), device=local, method=_lib.METHOD_NAMES[args.method])
                          for _ in range(args.inflight - 1)]
        for k, jk in enumerate(jobs_k[1:], 1):
            jk.fill_synthetic(seed=1 + rank + 1000 * k)
        ctx = [torch.cuda.Stream(device=dev) for _ in jobs_k]
        cur = torch.cuda.current_stream(dev)

        def round_(upload=None, down=None):
            for k, jk in enumerate(jobs_k):
                ctx[k].wait_stream(cur)
                with torch.cuda.stream(ctx[k]):
                    if upload is not None:
                        jk.upload(upload)
                    jk.run(hashes=True, packed_md5=True)
                    if down is not None:
                        jk.download(down[k])
            for c in ctx:
                cur.wait_stream(c)
        round_()
        torch.cuda.synchronize()
        i0 = torch.cuda.Event(enable_timing=True)
        i1 = torch.cuda.Event(enable_timing=True)
        i0.record()
        for _ in range(args.steps):
            round_()
        i1.record()
        torch.cuda.synchronize()
        ims = max_over_ranks(i0.elapsed_time(i1) / args.steps)
        assert all(int(jk.d_flags.sum()) == R for jk in jobs_k)
        inflight = {"jobs_in_flight": len(jobs_k), "value": mul_adds * len(jobs_k) * world / (ims / 1e3), "unit": UNIT,
                    "ms_per_round": ims, "jobs_per_s": len(jobs_k) * world / (ims / 1e3),
                    "desc": "%d independent jobs of this workload (distinct seeded inputs, each resident) per round, "
                            "each on its own stream; whole pass per job incl. IFSC + file MD5 (chains packed 32 per "
                            "warp so that they leave the other SMs to the other jobs)" % len(jobs_k)}
        if e2e is not None:
            downs = [torch.empty((R, S), dtype=torch.uint8, pin_memory=True) for _ in jobs_k]
            round_(host_in, downs)
            torch.cuda.synchronize()
            i0.record()
            for _ in range(args.steps):
                round_(host_in, downs)
            i1.record()
            torch.cuda.synchronize()
            ems_k = max_over_ranks(i0.elapsed_time(i1) / args.steps)
            inflight["e2e"] = {"value": mul_adds * len(jobs_k) * world / (ems_k / 1e3), "unit": UNIT,
                               "ms_per_round": ems_k, "h2d_bytes_per_round": N * S * len(jobs_k),
                               "d2h_bytes_per_round": job.d2h_bytes() * len(jobs_k)}
            del downs
        del jobs_k
        torch.cuda.empty_cache()

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
    # int-ALU roofline of the contraction: 2 three-input LOP3 per word mul-add
    # (16x16 GF(2) matrix, ~128 set bits, 32-way bit slicing) against the
    # LOP3 rate measured on this device (par2cuda_lop3_rate)
    alu_peak = lop3.value / 1e12
    alu_nominal = n_sm * 128 * sm_mhz * 1e6 / 1e12
    kname = _lib.comb_kernel_name(L.par2cuda_comb_shape_for(R)) if args.method in ("comb", "auto") else \
        {"xor": "k_xor_muladd", "nibble": "k_nibble_muladd", "tensor": "k_tc_muladd"}[args.method]
    comb_rate = mul_adds / (comb_ms / 1e3)
    alg_bytes = (N + R) * S  # read every input once, write every recovery once
    hbm_peak = (peaks or {}).get("hbm_gbs", 6800.0)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u16 GF(2^16)", "data": "synthetic (seeded splitmix64 slices), inputs resident in HBM",
        "config": bench_config(args, cfg, file_lens, world),
        "src_GBps_x_recovery": N * S * R * world / (ms / 1e3) / 1e9,
        "kernels_ms": {"muladd": comb_ms, "file_md5": hash_ms, "step": ms},
        "method": args.method,
        "roofline_gf": {"bound": "int-alu", "kernel": kname, "achieved": 2 * comb_rate / 1e12,
                     "peak": alu_peak, "unit": "Tops/s", "frac": 2 * comb_rate / 1e12 / alu_peak,
                     "traffic": None, "alg_bytes": alg_bytes,
                     "peak_source": "measured: LOP3 calibration kernel k_lop3_rate on this GPU (%.1f lanes/SM/clk at "
                                    "%.0f MHz); nominal 128 lanes would be %.1f Tops/s" %
                                    (lop3.value / n_sm / (sm_mhz * 1e6), sm_mhz, alu_nominal),
                     "mul_adds_per_s": comb_rate},
        "roofline_hbm": {"bound": "hbm", "kernel": kname, "achieved": alg_bytes / (comb_ms / 1e3) / 1e9,
                         "peak": hbm_peak, "unit": "GB/s", "frac": alg_bytes / (comb_ms / 1e3) / 1e9 / hbm_peak,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6800 GB/s"},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
        "e2e": e2e,
        "e2e_plugin": e2e_plugin,
        "inflight": inflight,
    }
    if args.traffic_bytes:
        line["roofline_gf"]["traffic"] = args.traffic_bytes
    elif kname in KERNEL_TRAFFIC:
        # DRAM bytes per launch scaled from the ncu capture of the same kernel
        # (profiles/): inputs are read once and recovery rows written once, so
        # traffic grows with (N + R) x S
        tb, ab, what = KERNEL_TRAFFIC[kname]
        line["roofline_gf"]["traffic"] = tb / ab * alg_bytes
        line["roofline_gf"]["traffic_source"] = "ncu dram__bytes_read+write of %s (%.1f MB for %.1f MB algorithmic), " \
            "scaled by (N+R)*S" % (what, tb / 1e6, ab / 1e6)
    if cfg["hashes"]:
        big = max(file_lens)
        line["roofline_md5"] = {
            "bound": "latency", "kernel": "k_file_md5", "achieved": big / (hash_ms / 1e3) / 1e6,
            "peak": md5_chain.value / 1e6, "unit": "MB/s per GPU thread (largest file's chain)",
            "frac": big / (hash_ms / 1e3) / md5_chain.value,
            "traffic": MD5_TRAFFIC[0] / MD5_TRAFFIC[1] * sum(file_lens),
            "traffic_source": "ncu dram__bytes_read+write of k_file_md5 on 4 files (%.1f MB for %.1f MB hashed), "
                              "scaled by the bytes hashed" % (MD5_TRAFFIC[0] / 1e6, MD5_TRAFFIC[1] / 1e6),
            "peak_source": "measured: k_md5_chain, one MD5 stream on one thread with its data in registers"}
    # `roofline` is the kernel that bounds the step (the longest live kernel time)
    line["roofline"] = dict(line["roofline_md5"] if cfg["hashes"] and hash_ms > comb_ms else line["roofline_gf"])
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
        "gpu_launches": sat["gpu_launches"],
    }
    print(json.dumps(line))
    return 0


def small_mix_run(args):
    """Supplement to the 64-job mix: 512 small jobs (N log-uniform [10, 200],
    S 64 KiB..1 MiB, R 1-30 % of N), where per-job launches leave the GPU
    partly idle; per-job launches vs the tuned batched graph."""
    import torch
    from parpar_gb300.batch import BatchRunner, make_job_mix
    jobs = make_job_mix(512, seed=6, n_range=(10, 200), s_range=(64 * 1024, 1 << 20))
    runner = BatchRunner(jobs, budget_bytes=args.budget_gib << 30)
    runner.run_per_job()
    t0 = time.perf_counter()
    runner.run_per_job()
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
        "speedup_vs_per_job_launch": (len(jobs) / (ms / 1e3)) / (len(jobs) / t_job),
        "batched_mode": runner.mode, "mode_pass0_ms": mode_ms,
        "small_jobs_mix": small_mix_run(args),
        "autotune": {str(k): v[0] for k, v in autotune.table().items()},
        "gpu_launches": runner.launches_per_run() * args.steps,
        "clocks": summarize_clocks(clock_lines, 0),
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="bandwidth")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-clocks", action="store_true")
    ap.add_argument("--no-plugin", action="store_true", help="skip the plugin-boundary e2e measurement")
    ap.add_argument("--plugin-steps", type=int, default=2)
    ap.add_argument("--method", choices=["auto", "comb", "xor", "nibble", "tensor"], default="comb",
                    help="multiply-accumulate kernel of the resident-job workloads")
    ap.add_argument("--budget-gib", type=int, default=64, help="HBM budget of one pass of the batched workload")
    ap.add_argument("--comb-shape", type=int, default=0,
                    help="pin the comb kernel's CTA shape (par2cuda_set_comb_shape; 0 = automatic)")
    ap.add_argument("--inflight", type=int, default=8,
                    help="independent jobs in flight for the multi-job figure of hashing workloads (0/1 = skip)")
    ap.add_argument("--traffic-bytes", type=float, default=None,
                    help="DRAM bytes per comb launch from an ncu capture (profiles/), reported as roofline_gf.traffic")
    args = ap.parse_args()
    cfg = WORKLOADS[args.workload]
    if args.workload in ("batched", "serving", "create") and int(os.environ.get("RANK", "0")) != 0:
        return 0   # single-GPU workloads: under torchrun only rank 0 measures
    if args.workload in ("batched", "serving"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the %s workload is reported against this backend's per-job path" % args.workload}))
            return 0
        return run_batched_workload(args, cfg) if args.workload == "batched" else run_serving_workload(args, cfg)
    if args.workload == "create" and args.impl != "reference":
        return run_create_workload(args, cfg)
    file_lens = file_lengths(cfg["N"], cfg["files"], cfg["S"], seed=2000)
    if args.impl == "reference":
        return run_reference(args, cfg, file_lens)
    return run_ours(args, cfg, file_lens)


if __name__ == "__main__":
    sys.exit(main())
