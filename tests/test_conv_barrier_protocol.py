"""The mbarrier protocols of the tensor-core convolution (geye_gb300/csrc/conv_tc.cu),
restated as coroutines and run under random schedules on the CPU.

Each role of a kernel (the copying thread, the MMA-issuing threads, the epilogue
warps) waits on barrier phases by parity and arrives on barriers exactly as the
kernel does; copies land and MMA commits arrive asynchronously, in random order
(commits of one issuing thread in the order it made them, as tcgen05.commit
tracks every earlier MMA of that thread).  A wait by parity cannot tell phase n
from phase n+2, so every wait must find its barrier at most one phase past the
phase it means; the simulation asserts that, and that no schedule deadlocks.
A copy of each protocol with one wait removed must fail, so the check is known
to catch the mistakes it is for."""
import random

import pytest


class Bar:
    """An mbarrier: `count` arrivals plus the expected transaction bytes complete a phase."""

    def __init__(self, count):
        self.count, self.pending, self.tx, self.done = count, count, 0, 0

    def arrive(self):
        self.pending -= 1
        self._check()

    def expect(self, tx):
        self.tx += tx
        self.arrive()

    def land(self, tx):
        self.tx -= tx
        self._check()

    def _check(self):
        if self.pending == 0 and self.tx == 0:
            self.done += 1
            self.pending = self.count


class Sim:
    def __init__(self, seed):
        self.rnd = random.Random(seed)
        self.copies = []     # async copies: land in any order
        self.commits = {}    # issuer -> FIFO of commit arrivals

    def copy(self, bar):
        bar.expect(1)
        self.copies.append(bar)

    def commit(self, who, bar):
        self.commits.setdefault(who, []).append(bar)

    def run(self, roles):
        state = [next(r, None) for r in roles]
        while True:
            ready = []
            for i, st in enumerate(state):
                if st is None:
                    continue
                bar, n = st
                assert bar.done <= n + 1, "a parity wait could see a phase two ahead"
                if bar.done >= n + 1:
                    ready.append(i)
            events = len(self.copies) + sum(1 for q in self.commits.values() if q)
            if not ready and not events:
                if all(s is None for s in state):
                    return
                raise RuntimeError("deadlock")
            if ready and (not events or self.rnd.random() < 0.5):
                i = self.rnd.choice(ready)
                state[i] = next(roles[i], None)
            elif self.copies and (not any(self.commits.values()) or self.rnd.random() < 0.5):
                self.copies.pop(self.rnd.randrange(len(self.copies))).land(1)
            else:
                who = self.rnd.choice([w for w, q in self.commits.items() if q])
                self.commits[who].pop(0).arrive()


def ring_kernel(sim, phases, stages_per_phase, NS, nis, drop_free_wait=False):
    """k_conv_tc: one slab per phase, the bank through a ring of NS stages, nis issuers."""
    slab_full, slab_free, done = Bar(1), Bar(nis), Bar(nis)
    stage_full = [Bar(1) for _ in range(NS)]
    stage_free = [Bar(nis) for _ in range(NS)]

    def producer():
        issued = 0
        for ph in range(phases):
            if ph > 0:
                yield slab_free, ph - 1
            sim.copy(slab_full)
            for _ in range(stages_per_phase):
                s = issued % NS
                if issued >= NS and not drop_free_wait:
                    yield stage_free[s], issued // NS - 1
                sim.copy(stage_full[s])
                issued += 1

    def issuer(w):
        used = 0
        for ph in range(phases):
            yield slab_full, ph
            for _ in range(stages_per_phase):
                s = used % NS
                yield stage_full[s], used // NS
                sim.commit(w, stage_free[s])
                used += 1
            sim.commit(w, slab_free)
        sim.commit(w, done)

    def epilogue():
        yield done, 0

    return [producer()] + [issuer(w) for w in range(nis)] + [epilogue() for _ in range(4)]


def persistent_kernel(sim, units, issuers=2, drop_unit_wait=False):
    """k_conv_tcp: units (bank, big) walked with two slab buffers and two accumulator sets."""
    slab_full = [Bar(1), Bar(1)]
    mma_done = [Bar(issuers), Bar(issuers)]
    acc_full = [Bar(issuers), Bar(issuers)]
    acc_free = [Bar(8), Bar(8)]
    bank_full, end = Bar(1), Bar(issuers)
    nu = len(units)

    def producer():
        cur = None
        for k, (bank, big) in enumerate(units):
            prev_big = k > 0 and units[k - 1][1]
            new_bank = bank != cur
            if k >= 2 and not drop_unit_wait:
                yield mma_done[(k - 2) & 1], (k - 2) >> 1
            if k >= 1 and (big or prev_big or new_bank):
                yield mma_done[(k - 1) & 1], (k - 1) >> 1
            if new_bank:
                sim.copy(bank_full)
                cur = bank
            sim.copy(slab_full[k & 1])

    def issuer(w):
        cur, banks = None, 0
        for k, (bank, big) in enumerate(units):
            if bank != cur:
                yield bank_full, banks
                cur, banks = bank, banks + 1
            yield slab_full[k & 1], k >> 1
            if k >= 2:
                yield acc_free[k & 1], (k - 2) >> 1
            sim.commit(w, mma_done[k & 1])
            sim.commit(w, acc_full[k & 1])
        if nu:
            sim.commit(w, end)

    def epilogue():
        for k in range(nu):
            yield acc_full[k & 1], k >> 1
            acc_free[k & 1].arrive()

    return [producer()] + [issuer(w) for w in range(issuers)] + [epilogue() for _ in range(8)]


def _random_units(rnd):
    units, bank = [], 0
    for _ in range(rnd.randint(0, 10)):
        if rnd.random() < 0.15:
            bank += 1
        units.append((bank, rnd.random() < 0.3))
    return units


def test_ring_kernel_protocol_holds():
    rnd = random.Random(5)
    for trial in range(400):
        NS = rnd.randint(1, 8)
        nis = rnd.randint(1, 7)
        sim = Sim(trial)
        sim.run(ring_kernel(sim, rnd.randint(1, 3), rnd.randint(1, 12), NS, nis))


def test_persistent_kernel_protocol_holds():
    rnd = random.Random(7)
    for trial in range(400):
        sim = Sim(trial)
        sim.run(persistent_kernel(sim, _random_units(rnd)))


@pytest.mark.parametrize("which", ["ring", "persistent"])
def test_a_missing_wait_is_caught(which):
    """The protocol with one wait removed must fail under some schedule."""
    rnd = random.Random(11)
    caught = 0
    for trial in range(300):
        sim = Sim(trial)
        if which == "ring":
            roles = ring_kernel(sim, 2, 8, 2, rnd.randint(1, 4), drop_free_wait=True)
        else:
            roles = persistent_kernel(sim, [(0, False)] * rnd.randint(3, 10), drop_unit_wait=True)
        try:
            sim.run(roles)
        except (AssertionError, RuntimeError):
            caught += 1
    assert caught > 0
