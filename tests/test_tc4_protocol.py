"""A model of the barrier protocol of the persistent 4-bit tensor GEMM
(parpar_gb300/csrc/k_tc4.cu: k_tc4_gemm), run on the CPU with random
interleavings of several CTAs: mbarriers with arrival counts and parity waits;
per CTA a producer that takes tiles from a shared counter, publishes each tile
number in a ring of TR slots ("idFull", reused once "idEmpty" has its 5
arrivals: the MMA thread and the four epilogue warps) and fills stage g % NST
once "empty" has completed phase g / NST - 1; an MMA thread that reads the
tile numbers, waits "full" and, for tile j >= NACC, "tmemEmpty[j % NACC]" (4
arrivals), and accumulates tile j in accumulator j % NACC; four epilogue warps
that read the tile numbers and wait "tmemFull[j % NACC]".  Both tile shapes
are modelled: two accumulators and 5 stages, one accumulator and 4 stages.  Copies and MMA
commits complete later, in order.  Every stage the MMA thread reads must hold
its own (tile, k-block), every accumulator an epilogue reads must be its
tile's, every tile is written exactly once, the counter advances by tiles +
CTAs, and nothing may deadlock."""
import random

TR = 8
NO_TILE = -1


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


def cta(n_all, k_blocks, counter, out, pending, nacc, nst):
    """The roles of one CTA as generators; `pending` receives its async
    completions (copies, commits) in issue order."""
    NST = nst
    full = [Bar(1) for _ in range(NST)]
    empty = [Bar(1) for _ in range(NST)]
    tmem_full = [Bar(1), Bar(1)]
    tmem_empty = [Bar(4), Bar(4)]
    id_full = [Bar(1) for _ in range(TR)]
    id_empty = [Bar(5) for _ in range(TR)]
    ids = [None] * TR
    stage = [None] * NST
    acc = [None, None]
    copies, commits = pending

    def producer():
        g = 0
        j = 0
        while True:
            slot = j % TR
            if j >= TR:
                while not id_empty[slot].try_wait(((j // TR) - 1) & 1):
                    yield
            t = counter[0]
            counter[0] += 1
            more = t < n_all
            ids[slot] = t if more else NO_TILE
            id_full[slot].arrive()
            j += 1
            if not more:
                return
            for kb in range(k_blocks):
                s = g % NST
                if g >= NST:
                    while not empty[s].try_wait(((g // NST) - 1) & 1):
                        yield
                copies.append((stage, full, s, (t, kb)))
                g += 1
                yield

    def mma():
        g = 0
        j = 0
        while True:
            slot = j % TR
            while not id_full[slot].try_wait((j // TR) & 1):
                yield
            t = ids[slot]
            id_empty[slot].arrive()
            if t == NO_TILE:
                return
            buf, use = j % nacc, j // nacc
            if use >= 1:
                while not tmem_empty[buf].try_wait((use - 1) & 1):
                    yield
            for kb in range(k_blocks):
                s = g % NST
                while not full[s].try_wait((g // NST) & 1):
                    yield
                assert stage[s] == (t, kb), (stage[s], t, kb)
                acc[buf] = (t, kb)
                commits.append(empty[s])
                g += 1
                yield
            commits.append(tmem_full[buf])
            j += 1

    def epilogue(q):
        j = 0
        while True:
            slot = j % TR
            while not id_full[slot].try_wait((j // TR) & 1):
                yield
            t = ids[slot]
            yield
            id_empty[slot].arrive()
            if t == NO_TILE:
                return
            buf, use = j % nacc, j // nacc
            while not tmem_full[buf].try_wait(use & 1):
                yield
            assert acc[buf] == (t, k_blocks - 1), (acc[buf], t)
            if q == 0:
                out.append(t)
            yield
            tmem_empty[buf].arrive()
            j += 1

    return [producer(), mma()] + [epilogue(q) for q in range(4)]


def run(n_all, grid, k_blocks, rng, nacc, nst):
    counter = [0]
    out = []
    copies, commits = [], []
    alive = []
    for _ in range(grid):
        alive += cta(n_all, k_blocks, counter, out, (copies, commits), nacc, nst)
    steps = 0
    while alive or copies or commits:
        steps += 1
        assert steps < 10 ** 6, "deadlock"
        x = rng.random()
        if copies and x < 0.2:
            stage, full, s, d = copies.pop(0)
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
    assert sorted(out) == list(range(n_all))
    assert counter[0] == n_all + grid


def test_tc4_persistent_protocol():
    # both tile shapes: 192 rows with two accumulators and 5 stages, 256 rows
    # with one accumulator and 4 stages
    for nacc, nst in ((2, 5), (1, 4)):
        for seed in range(150):
            rng = random.Random(seed)
            n_all = rng.randint(1, 40)
            grid = rng.randint(1, min(n_all, 6))
            k_blocks = rng.randint(1, 9)
            run(n_all, grid, k_blocks, rng, nacc, nst)
