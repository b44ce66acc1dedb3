"""Model of the mbarrier protocol of the tensor-core contraction kernel
(dftcxx_gb300/csrc/k_contract_tc.cu), checked on the CPU under random
schedules: ring slots with a loader (A slices), producer warps (B slices;
eight in the kernel), one MMA issuer and the epilogue over one or two
accumulator buffers (two in the kernel: the drain of a chunk overlaps the
MMAs of the next).  A wait passes when the phase of the
given parity has completed, as mbarrier.try_wait.parity does (a fresh barrier
counts its preceding phase as complete).  In the kernel every producer warp
fills its rows of every stage and the stage-full barrier expects one
arrival per producer warp; each waiter then sees each slot's phases strictly in order, which
keeps every stage's data consistent for every ring depth.  Splitting stages
between warps round-robin instead ("stage % 4") breaks rings shorter than the
number of warps: a warp then waits on a parity whose preceding phase counts as
complete and reads a stage that has not landed."""
import random

import pytest


class _Bar:
    def __init__(self, count=1):
        self.ph = 0
        self.count = count
        self.pending = count

    def arrive(self):
        self.pending -= 1
        if self.pending == 0:
            self.ph += 1
            self.pending = self.count

    def ok(self, parity):
        return (self.ph & 1) != parity


def _run(nst, chunks, owner, seed, per_stage=1, nwarps=4, nbuf=1):
    """owner(it, s) -> the producing warp of stage it, or None when all
    per_stage warps produce every stage (full barrier count per_stage).
    nbuf accumulator buffers: chunk c uses buffer c % nbuf for the
    (c // nbuf + 1)-th time."""
    rng = random.Random(seed)
    a_full = [_Bar() for _ in range(nst)]
    full = [_Bar(per_stage) for _ in range(nst)]
    empty = [_Bar() for _ in range(nst)]
    tmem_full, tmem_empty = [_Bar() for _ in range(nbuf)], [_Bar() for _ in range(nbuf)]
    acc = [None] * nbuf            # chunk whose sums the buffer holds
    a_in = [None] * nst
    b_in = [[None] * nwarps for _ in range(nst)]
    ns = sum(chunks)

    def loader():
        for it in range(ns):
            s, n = it % nst, it // nst
            while not empty[s].ok((n & 1) ^ 1):
                yield
            a_in[s] = it
            yield
            a_full[s].arrive()

    def producer(w):
        for it in range(ns):
            s, n = it % nst, it // nst
            if owner is not None and owner(it, s) != w:
                continue
            while not a_full[s].ok(n & 1):
                yield
            if a_in[s] != it:
                raise AssertionError("producer %d read stage %s for %d" % (w, a_in[s], it))
            for part in range(nwarps):
                if owner is None and part != w:
                    continue
                b_in[s][part] = it
            yield
            full[s].arrive()

    def mma():
        it = 0
        for c, kb in enumerate(chunks):
            b, use = c % nbuf, c // nbuf
            while not tmem_empty[b].ok((use & 1) ^ 1):
                yield
            if acc[b] is not None:
                raise AssertionError("MMA overwrote buffer %d holding chunk %d" % (b, acc[b]))
            acc[b] = c
            for _ in range(kb):
                s, n = it % nst, it // nst
                while not full[s].ok(n & 1):
                    yield
                if a_in[s] != it or any(b != it for b in b_in[s]):
                    raise AssertionError("MMA saw (%s, %s) for %d" % (a_in[s], b_in[s], it))
                yield
                empty[s].arrive()
                it += 1
            tmem_full[b].arrive()

    def epilogue():
        for c in range(len(chunks)):
            b, use = c % nbuf, c // nbuf
            while not tmem_full[b].ok(use & 1):
                yield
            if acc[b] != c:
                raise AssertionError("epilogue read chunk %s for %d" % (acc[b], c))
            yield
            acc[b] = None
            tmem_empty[b].arrive()

    alive = [loader(), mma(), epilogue()] + [producer(w) for w in range(nwarps)]
    steps = 0
    while alive:
        a = rng.choice(alive)
        try:
            next(a)
        except StopIteration:
            alive.remove(a)
        steps += 1
        if steps > 500000:
            raise AssertionError("no progress")


@pytest.mark.parametrize("nbuf", [1, 2])
@pytest.mark.parametrize("nwarps", [4, 8])
@pytest.mark.parametrize("nst", [2, 3, 4, 5, 6, 8])
@pytest.mark.parametrize("chunks", [[8] * 7, [8] * 6 + [3], [1, 1, 2], [5], [14] * 4])
def test_all_warps_per_stage_keep_stages_consistent(nst, chunks, nwarps, nbuf):
    for seed in range(12):
        _run(nst, chunks, None, seed, per_stage=nwarps, nwarps=nwarps, nbuf=nbuf)


@pytest.mark.parametrize("nst", [2, 3, 4, 8])
def test_slot_owned_producers_keep_stages_consistent(nst):
    for seed in range(20):
        _run(nst, [8] * 7, lambda it, s: s & 3, seed)


def test_stage_round_robin_breaks_short_rings():
    with pytest.raises(AssertionError):
        for seed in range(20):
            _run(3, [8] * 7, lambda it, s: it & 3, seed)


@pytest.mark.parametrize("nst", [2, 4, 6, 8])
@pytest.mark.parametrize("chunks", [[14] * 4, [7, 9, 1], [16] * 3])
def test_two_producer_groups_two_buffers(nst, chunks):
    """The kernel's schedule: producer groups owning the even and the odd ring
    slots (even ring depth) and two accumulator buffers."""
    for seed in range(20):
        _run(nst, chunks, lambda it, s: s & 1, seed, nbuf=2)
