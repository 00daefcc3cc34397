"""The barrier protocols of the tensor-core kernel sums (ksum_um_kernel and
ksum_grid_kernel in fmca_gb300/csrc/h2_umma_kernels.cuh), modelled on the
CPU.

Roles and barriers follow the kernel: a producer fills stages (full /
empty), two threads issue the products of each 16-source chunk (afull /
aempty per A slot; one target half each, or alternate chunks with a single
half) and commit a tile's accumulators (accf), and NSETS sets
of 4 evaluation warps write A slots, release stages and add finished
accumulators, tile after tile (tdone), into the shared total (acce).  mbarrier waits are parity waits:
they pass when the barrier's current phase has the other parity, which is
the intended phase only while the waiter is at most one phase ahead.  Random
schedules (with asynchronous product completions) must finish without a
deadlock and without a wait that passes before its phase completed."""
from __future__ import annotations

import random

import pytest


class Bar:
    def __init__(self, count):
        self.count = count
        self.pending = count
        self.phase = 0          # index of the phase in progress

    def arrive(self):
        self.pending -= 1
        if self.pending == 0:
            self.phase += 1
            self.pending = self.count

    def parity_passes(self, parity):
        return (self.phase & 1) != parity


def nslot(H, NSETS, cols=512):
    # accumulators [buffer][product thread] x 64 columns, one total of
    # H x 32, A slots of H x 16 columns, at most one tile (8 chunks) of them
    a0 = 2 * 2 * 64 + H * 32
    fit = (cols - a0) // (H * 16)
    assert fit >= 4
    return min(8, fit)              # as in the kernel


def simulate(ntiles, NSETS, H, seed, NST=6, slots=None, nbars=4, pairs=False):
    """'ok', 'deadlock' or 'early' for one random schedule.  pairs: set s
    evaluates the consecutive chunks 2 s and 2 s + 1 (the tensor-grid far
    field) instead of s, s + NSETS, ..."""
    rnd = random.Random(seed)
    NSLOT = slots or nslot(H, NSETS)
    NEVAL = 4 * NSETS
    full = [Bar(1) for _ in range(NST)]
    empty = [Bar(NEVAL + 2) for _ in range(NST)]
    afull = [Bar(4) for _ in range(16)]
    # two product threads: with two target halves both read every A slot,
    # with one half thread j takes the chunks kk = j mod 2
    aempty = [Bar(2 if H == 2 else 1) for _ in range(16)]
    # tile accumulators complete on accf[k % 4] (two buffers, four barriers):
    # with one product thread up to a tile behind the other, a flush of tile
    # k may start before tile k - 2 completes, but not before tile k - 4
    accf = [Bar(2) for _ in range(nbars)]
    acce = [Bar(4) for _ in range(2)]
    tdone = Bar(4)      # one phase per finished flush (the shared total)

    def producer():
        for k in range(ntiles):
            st = k % NST
            if k >= NST:
                yield ("wait", empty[st], k // NST - 1)
            yield ("arrive", full[st])

    def products(j):
        for k in range(ntiles):
            st, b = k % NST, k & 1
            yield ("wait", full[st], k // NST)
            if k >= 2:
                yield ("wait", acce[b], (k >> 1) - 1)
            for kk in range(8):
                if H == 1 and kk % 2 != j:
                    continue
                c = k * 8 + kk
                yield ("wait", afull[c % NSLOT], c // NSLOT)
                yield ("commit", aempty[c % NSLOT])
            yield ("commit", empty[st])
            yield ("commit", accf[k % nbars])

    def evaluation(s):
        def flush(k):
            yield ("wait", accf[k % nbars], k // nbars)
            if k >= 1:
                yield ("wait", tdone, k - 1)
            yield ("arrive", acce[k & 1])
            yield ("arrive", tdone)
        for k in range(ntiles):
            st = k % NST
            yield ("wait", full[st], k // NST)
            for kk in ([2 * s, 2 * s + 1] if pairs else range(s, 8, NSETS)):
                c = k * 8 + kk
                if c >= NSLOT:
                    yield ("wait", aempty[c % NSLOT], c // NSLOT - 1)
                yield ("arrive", afull[c % NSLOT])
            yield ("arrive", empty[st])
            if k >= 1 and (k - 1) % NSETS == s:
                yield from flush(k - 1)
        if ntiles >= 1 and (ntiles - 1) % NSETS == s:
            yield from flush(ntiles - 1)

    roles = ([producer(), products(0), products(1)] +
             [evaluation(s) for s in range(NSETS) for _ in range(4)])
    cur = [None] * len(roles)
    alive = [True] * len(roles)
    inflight = []       # committed products complete later, in order
    while True:
        runnable = []
        for i, r in enumerate(roles):
            if not alive[i]:
                continue
            if cur[i] is None:
                try:
                    cur[i] = next(r)
                except StopIteration:
                    alive[i] = False
                    continue
            op = cur[i]
            if op[0] == "wait" and not op[1].parity_passes(op[2] & 1):
                continue
            runnable.append(i)
        if not any(alive) and not inflight:
            return "ok"
        choices = runnable + (["done"] if inflight else [])
        if not choices:
            return "deadlock"
        ch = rnd.choice(choices)
        if ch == "done":
            inflight.pop(0).arrive()
            continue
        op = cur[ch]
        cur[ch] = None
        if op[0] == "wait":
            if op[1].phase <= op[2]:
                return "early"
        elif op[0] == "arrive":
            op[1].arrive()
        else:
            inflight.append(op[1])


@pytest.mark.parametrize("NSETS,H", [(2, 2), (2, 1), (4, 2), (4, 1)])
def test_protocol_has_no_deadlock_or_early_pass(NSETS, H):
    for seed in range(60):
        for ntiles in (1, 2, 3, 5, 9, 17):
            assert simulate(ntiles, NSETS, H, seed) == "ok", (ntiles, seed)


def test_model_detects_aliased_accumulator_waits():
    # with one target half the two product threads drift up to a tile apart;
    # two accumulator barriers (one per buffer) then let a flush pass the
    # parity of tile k - 2 while waiting for tile k
    bad = [simulate(n, 4, 1, s, nbars=2) for s in range(40) for n in (9, 17)]
    assert "early" in bad


def test_protocol_with_chunk_pairs_per_set():
    for seed in range(60):
        for ntiles in (1, 2, 3, 5, 9, 17):
            assert simulate(ntiles, 4, 1, seed, pairs=True) == "ok", (ntiles, seed)


def simulate_grid(ntiles, seed, NST=6, NPS=8, nbars=4):
    """ksum_grid_kernel: set s writes A pair slot (4 k + s) mod NPS of tile k;
    product thread j issues the pairs of sets j and j + 2 (one commit per
    pair, aempty) and commits the tile on accf[k % nbars]; the set of tile
    k - 1 flushes it after writing its pair of tile k, and that flush also
    frees the stage (one arrival).  Each product thread's commits complete
    in order, independently of the other thread's."""
    rnd = random.Random(seed)
    full = [Bar(1) for _ in range(NST)]
    empty = [Bar(1) for _ in range(NST)]
    afull = [Bar(4) for _ in range(NPS)]
    aempty = [Bar(1) for _ in range(NPS)]
    accf = [Bar(2) for _ in range(nbars)]
    acce = [Bar(4) for _ in range(2)]

    def producer():
        for k in range(ntiles):
            st = k % NST
            if k >= NST:
                yield ("wait", empty[st], k // NST - 1)
            yield ("arrive", full[st])

    def products(j):
        for k in range(ntiles):
            st, b = k % NST, k & 1
            yield ("wait", full[st], k // NST)
            if k >= 2:
                yield ("wait", acce[b], (k >> 1) - 1)
            for s in (j, j + 2):
                p = 4 * k + s
                yield ("wait", afull[p % NPS], p // NPS)
                yield ("commit", aempty[p % NPS])
            yield ("commit", accf[k % nbars])

    def evaluation(s, w):
        def flush(k):
            yield ("wait", accf[k % nbars], k // nbars)
            yield ("arrive", acce[k & 1])
            if w == 0:
                yield ("arrive", empty[k % NST])
        for k in range(ntiles):
            yield ("wait", full[k % NST], k // NST)
            p = 4 * k + s
            if p >= NPS:
                yield ("wait", aempty[p % NPS], p // NPS - 1)
            yield ("arrive", afull[p % NPS])
            if k >= 1 and (k - 1) % 4 == s:
                yield from flush(k - 1)
        if ntiles >= 1 and (ntiles - 1) % 4 == s:
            yield from flush(ntiles - 1)

    roles = ([producer(), products(0), products(1)] +
             [evaluation(s, w) for s in range(4) for w in range(4)])
    cur = [None] * len(roles)
    alive = [True] * len(roles)
    inflight = [[], []]     # per product thread, completing in order
    while True:
        runnable = []
        for i, r in enumerate(roles):
            if not alive[i]:
                continue
            if cur[i] is None:
                try:
                    cur[i] = next(r)
                except StopIteration:
                    alive[i] = False
                    continue
            op = cur[i]
            if op[0] == "wait" and not op[1].parity_passes(op[2] & 1):
                continue
            runnable.append(i)
        if not any(alive) and not inflight[0] and not inflight[1]:
            return "ok"
        choices = runnable + [("done", t) for t in (0, 1) if inflight[t]]
        if not choices:
            return "deadlock"
        ch = rnd.choice(choices)
        if isinstance(ch, tuple):
            inflight[ch[1]].pop(0).arrive()
            continue
        op = cur[ch]
        cur[ch] = None
        if op[0] == "wait":
            if op[1].phase <= op[2]:
                return "early"
        elif op[0] == "arrive":
            op[1].arrive()
        else:
            inflight[ch - 1].append(op[1])


def test_grid_protocol_has_no_deadlock_or_early_pass():
    for seed in range(80):
        for ntiles in (1, 2, 3, 4, 5, 9, 17, 33):
            assert simulate_grid(ntiles, seed) == "ok", (ntiles, seed)


def test_grid_model_detects_aliased_accumulator_waits():
    # two accumulator barriers alias the parity of tile k - 2
    bad = [simulate_grid(n, s, nbars=2) for s in range(40) for n in (9, 17)]
    assert "early" in bad
