"""Model of the mbarrier protocol of the tensor-core contraction kernel
(dftcxx_gb300/csrc/k_contract_tc.cu), checked on the CPU under random
schedules: ring slots with a loader (A slices), producer warps (B slices),
one MMA issuer and the epilogue.  A wait passes when the phase of the given
parity has completed, as mbarrier.try_wait.parity does (a fresh barrier
counts its preceding phase as complete).  The kernel's rule -- each ring slot
is produced by exactly one warp (slot % 4) -- must keep every stage's data
consistent for every ring depth; the rule "stage % 4" fails for rings shorter
than the number of producer warps."""
import random

import pytest


class _Bar:
    def __init__(self):
        self.ph = 0

    def arrive(self):
        self.ph += 1

    def ok(self, parity):
        return (self.ph & 1) != parity


def _run(nst, chunks, owner, seed):
    rng = random.Random(seed)
    a_full = [_Bar() for _ in range(nst)]
    full = [_Bar() for _ in range(nst)]
    empty = [_Bar() for _ in range(nst)]
    tmem_full, tmem_empty = _Bar(), _Bar()
    a_in, b_in = [None] * nst, [None] * nst
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
            if owner(it, s) != w:
                continue
            while not a_full[s].ok(n & 1):
                yield
            if a_in[s] != it:
                raise AssertionError("producer %d read stage %s for %d" % (w, a_in[s], it))
            b_in[s] = it
            yield
            full[s].arrive()

    def mma():
        it = 0
        for c, kb in enumerate(chunks):
            while not tmem_empty.ok((c & 1) ^ 1):
                yield
            for _ in range(kb):
                s, n = it % nst, it // nst
                while not full[s].ok(n & 1):
                    yield
                if a_in[s] != it or b_in[s] != it:
                    raise AssertionError("MMA saw (%s, %s) for %d" % (a_in[s], b_in[s], it))
                yield
                empty[s].arrive()
                it += 1
            tmem_full.arrive()

    def epilogue():
        for c in range(len(chunks)):
            while not tmem_full.ok(c & 1):
                yield
            yield
            tmem_empty.arrive()

    alive = [loader(), mma(), epilogue()] + [producer(w) for w in range(4)]
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


@pytest.mark.parametrize("nst", [2, 3, 4, 5, 6, 8])
@pytest.mark.parametrize("chunks", [[8] * 7, [8] * 6 + [3], [1, 1, 2], [5]])
def test_slot_owned_producers_keep_stages_consistent(nst, chunks):
    for seed in range(20):
        _run(nst, chunks, lambda it, s: s & 3, seed)


def test_stage_round_robin_breaks_short_rings():
    with pytest.raises(AssertionError):
        for seed in range(20):
            _run(3, [8] * 7, lambda it, s: it & 3, seed)
