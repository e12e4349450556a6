"""A model of the barrier protocol of the persistent 4-bit tensor GEMM
(parpar_gb300/csrc/k_tc4.cu: k_tc4_gemm), run on the CPU with random
interleavings: mbarriers with arrival counts and parity waits, a TMA thread
that fills stage g % 4 once "empty" has completed phase g / 4 - 1, an MMA
thread that waits "full" and, per tile after the first, "tmemEmpty" (4
arrivals), and four epilogue warps that wait "tmemFull".  Copies and MMA
commits complete later, in order.  Every stage the MMA thread reads must hold
its own (tile, k-block), every accumulator an epilogue reads must be its
tile's, and nothing may deadlock."""
import random

NST = 4


class Bar:
    def __init__(self, count):
        self.count, self.pending, self.phase = count, count, 0

    def arrive(self):
        self.pending -= 1
        if self.pending == 0:
            self.phase += 1
            self.pending = self.count

    def try_wait(self, parity):
        return (self.phase & 1) != parity


def run_cta(tiles, k_blocks, rng):
    full = [Bar(1) for _ in range(NST)]
    empty = [Bar(1) for _ in range(NST)]
    tmem_full, tmem_empty = Bar(1), Bar(4)
    stage = [None] * NST
    acc = [None]
    out = []
    copies, commits = [], []

    def producer():
        g = 0
        for t in tiles:
            for kb in range(k_blocks):
                s = g % NST
                if g >= NST:
                    while not empty[s].try_wait(((g // NST) - 1) & 1):
                        yield
                copies.append((s, (t, kb)))
                g += 1

    def mma():
        g = 0
        for i, t in enumerate(tiles):
            if i > 0:
                while not tmem_empty.try_wait((i - 1) & 1):
                    yield
            for kb in range(k_blocks):
                s = g % NST
                while not full[s].try_wait((g // NST) & 1):
                    yield
                assert stage[s] == (t, kb)
                acc[0] = (t, kb)
                commits.append(empty[s])
                g += 1
            commits.append(tmem_full)

    def epilogue(q):
        for i, t in enumerate(tiles):
            while not tmem_full.try_wait(i & 1):
                yield
            assert acc[0] == (t, k_blocks - 1)
            if q == 0:
                out.append(t)
            yield
            tmem_empty.arrive()

    alive = [producer(), mma()] + [epilogue(q) for q in range(4)]
    steps = 0
    while alive or copies or commits:
        steps += 1
        assert steps < 10 ** 6, "deadlock"
        x = rng.random()
        if copies and x < 0.2:
            s, d = copies.pop(0)
            stage[s] = d
            full[s].arrive()
        elif commits and x < 0.4:
            commits.pop(0).arrive()
        elif alive:
            r = rng.choice(alive)
            try:
                next(r)
            except StopIteration:
                alive.remove(r)
    assert out == list(tiles)


def test_tc4_persistent_protocol():
    for seed in range(200):
        rng = random.Random(seed)
        n_all = rng.randint(1, 40)
        grid = rng.randint(1, min(n_all, 6))
        k_blocks = rng.randint(1, 9)
        for b in range(grid):
            run_cta(list(range(b, n_all, grid)), k_blocks, rng)
