"""Slice layout of files (pure host code, no device library).

PAR2 cuts every file into slices of the set's slice size, the last one
shorter and zero-padded (lib/par2.js PAR2File, lib/par2gen.js:1198-1285);
input slices are numbered in file order.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

KIB, MIB = 1024, 1024 * 1024


def file_layout(file_lens, S):
    """(first_row[f], per-row byte lengths) for files laid out as slices of S bytes;
    an empty file still takes one (empty) row."""
    first, lens = [], []
    r = 0
    for ln in file_lens:
        first.append(r)
        n = max(1, (int(ln) + S - 1) // S)
        for k in range(n):
            lens.append(int(min(S, ln - k * S)) if ln else 0)
        r += n
    return np.array(first, dtype=np.uint32), np.array(lens, dtype=np.uint32)


def file_lengths(N, files, S, seed):
    """Seeded uneven file lengths with sum(ceil(len/S)) == N, the last slice
    of each file partial: the file sets of the benchmark workloads."""
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


@dataclass
class JobSpec:
    N: int
    S: int
    R: int
    seed: int
    exps: list = field(default_factory=list)

    @property
    def mul_adds(self) -> int:
        return self.N * self.R * (self.S // 2)

    @property
    def input_bytes(self) -> int:
        return self.N * self.S


def make_job_mix(n_jobs: int = 64, seed: int = 4, n_range=(10, 5000), s_range=(64 * KIB, 8 * MIB), r_frac=(0.01, 0.30)):
    """Seeded uneven jobs: N log-uniform in n_range, S uniform over the 4-byte
    multiples in s_range, R = round(U(r_frac) * N) (at least 1)."""
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(n_jobs):
        N = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        S = int(rng.integers(s_range[0] // 4, s_range[1] // 4 + 1)) * 4
        R = max(1, int(round(rng.uniform(*r_frac) * N)))
        jobs.append(JobSpec(N, S, R, seed * 1000 + j, list(range(R))))
    return jobs
