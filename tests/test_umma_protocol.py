"""The barrier protocol of the tensor-core kernel sum (ksum_um_kernel in
fmca_gb300/csrc/h2_umma_kernels.cuh), modelled on the CPU.

Roles and barriers follow the kernel:
- A producer fills stages (full); a stage is freed (empty) by the flush of
  the accumulation unit holding its tile.
- Four sets of 4 evaluation warps write the A pair slot (4 k + s) mod NPS of
  tile k (afull), after the products of that slot's previous use completed
  (aempty).
- Two product threads issue the pairs. With two target halves each thread
  issues every pair (aempty counts both); with one half, thread j issues the
  pairs of sets j and j + 2. Each thread commits every pair (aempty) and the
  last tile of every accumulation unit of F tiles (accf[u % 4]), and waits
  for the flush of unit u - 2 (acce[u & 1]) before the first tile of unit u.
- Four flush warps (one per tensor-memory lane quarter) take the units in
  order: each waits for unit u (accf[u % 4]) and releases its accumulator
  buffer (acce[u & 1]); the first also frees the unit's stages.
- A persistent CTA runs the tiles of several groups through the same ring,
  pair slots and accumulator buffers: the counters run on, and the last
  unit of every group closes early (units never span two groups).

mbarrier waits are parity waits: they pass when the barrier's current phase
has the other parity, which is the intended phase only while the waiter is
at most one phase ahead. Random schedules, with product completions in
order per thread, must finish without a deadlock and without a wait that
passes before its phase completed."""
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


def nstages(H):
    return 5 if H == 2 else 6          # um_stages in the kernel


def npair_slots(H, cols=512):
    # accumulators [buffer][product thread] x 64 columns, then pair slots
    # of H x 32 columns
    return (cols - 256) // (H * 32)


def units_of(items, F):
    """(first tile, tile count) of every accumulation unit: units of F tiles
    that never span two items (a CTA of the persistent kernel sum runs its
    items' tiles through one ring, closing the last unit of every item)."""
    out, k = [], 0
    for n in items:
        for t in range(0, n, F):
            out.append((k + t, min(F, n - t)))
        k += n
    return out


def simulate(ntiles, H, seed, F=1, NST=None, NPS=None, nbars=4, rnd=None):
    """'ok', 'deadlock' or 'early' for one random schedule.  ntiles: the
    tile count of one group, or a list of the tile counts of the items one
    persistent CTA processes in turn."""
    rnd = rnd or random.Random(seed)
    NST = NST or nstages(H)
    NPS = NPS or npair_slots(H)
    items = list(ntiles) if isinstance(ntiles, (list, tuple)) else [ntiles]
    units = units_of(items, F)
    total = sum(items)
    unit_of = {}
    for u, (t0, c) in enumerate(units):
        for t in range(t0, t0 + c):
            unit_of[t] = u
    full = [Bar(1) for _ in range(NST)]
    empty = [Bar(1) for _ in range(NST)]
    afull = [Bar(4) for _ in range(NPS)]
    aempty = [Bar(2 if H == 2 else 1) for _ in range(NPS)]
    accf = [Bar(2) for _ in range(nbars)]
    acce = [Bar(4) for _ in range(2)]

    def producer():
        for k in range(total):
            st = k % NST
            if k >= NST:
                yield ("wait", empty[st], k // NST - 1)
            yield ("arrive", full[st])

    def products(j):
        for k in range(total):
            st, u = k % NST, unit_of[k]
            t0, c = units[u]
            yield ("wait", full[st], k // NST)
            if k == t0 and u >= 2:
                yield ("wait", acce[u & 1], (u >> 1) - 1)
            for s in (range(4) if H == 2 else (j, j + 2)):
                p = 4 * k + s
                yield ("wait", afull[p % NPS], p // NPS)
                yield ("commit", aempty[p % NPS])
            if k == t0 + c - 1:
                yield ("commit", accf[u % nbars])

    def evaluation(s, w):
        for k in range(total):
            yield ("wait", full[k % NST], k // NST)
            p = 4 * k + s
            if p >= NPS:
                yield ("wait", aempty[p % NPS], p // NPS - 1)
            yield ("arrive", afull[p % NPS])

    def flusher(w):
        for u, (t0, c) in enumerate(units):
            yield ("wait", accf[u % nbars], u // nbars)
            yield ("arrive", acce[u & 1])
            if w == 0:
                for t in range(t0, t0 + c):
                    yield ("arrive", empty[t % NST])

    roles = ([producer(), products(0), products(1)] +
             [evaluation(s, w) for s in range(4) for w in range(4)] +
             [flusher(w) for w in range(4)])
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


def role_class(i):
    """0 producer, 1 / 2 product threads, 3 evaluation warps, 4 flush warps."""
    return i if i < 3 else (3 if i < 19 else 4)


class BiasedRandom(random.Random):
    """Picks roles with fixed weights, so that one role can run far ahead."""

    def __init__(self, seed, weights):
        super().__init__(seed)
        self.weights = weights

    def choice(self, seq):
        w = [self.weights.get(c[0] if isinstance(c, tuple) else role_class(c), 1.0)
             for c in seq]
        t = self.random() * sum(w)
        for c, x in zip(seq, w):
            t -= x
            if t <= 0:
                return c
        return seq[-1]


# (H, F): two target halves (near field, points), one half (far field on
# interpolation nodes), one half with units of two tiles (tensor grids)
CASES = [(2, 1), (1, 1), (1, 2), (2, 2)]


@pytest.mark.parametrize("H,F", CASES)
def test_protocol_has_no_deadlock_or_early_pass(H, F):
    for seed in range(60):
        for ntiles in (1, 2, 3, 4, 5, 7, 9, 17, 33):
            assert simulate(ntiles, H, seed, F=F) == "ok", (ntiles, seed)


@pytest.mark.parametrize("H,F", CASES)
def test_protocol_under_biased_schedules(H, F):
    # role classes (role_class) and "done" for product completions
    biases = [{"done": 0.05}, {"done": 20.0}, {1: 20.0}, {2: 0.05},
              {3: 20.0, "done": 0.2}, {0: 50.0, "done": 0.1},
              {4: 0.05}, {4: 20.0, 3: 0.2}]
    for b in biases:
        for seed in range(25):
            for ntiles in (5, 9, 17):
                rnd = BiasedRandom(seed, b)
                assert simulate(ntiles, H, seed, F=F, rnd=rnd) == "ok", (b, ntiles, seed)


def test_model_detects_a_shared_accumulator_barrier():
    # with one target half the two product threads drift up to a tile
    # apart; one accumulator barrier for all units then mixes the commits of
    # consecutive units
    bad = [simulate(n, 1, s, nbars=1) for s in range(40) for n in (9, 17)]
    assert any(r != "ok" for r in bad)


def test_model_detects_a_ring_of_partial_tiles():
    # three pair slots with two halves: pair 4 k + s and pair 4 k + s + 3
    # share a slot while the sets run a tile apart
    bad = [simulate(n, 2, s, NPS=3) for s in range(40) for n in (5, 9)]
    assert "early" in bad


# the launch shapes the autotuner may choose: 2..7 stages, units of 1..3
# tiles (at most the stage count), one or two target halves
SHAPES = [(H, NST, F) for H in (1, 2) for NST in range(2, 8) for F in (1, 2, 3) if F <= NST]


@pytest.mark.parametrize("H,NST,F", SHAPES)
def test_protocol_over_tuned_launch_shapes(H, NST, F):
    for seed in range(12):
        for ntiles in (1, 2, 3, 5, 8, 13, 21):
            assert simulate(ntiles, H, seed, F=F, NST=NST) == "ok", (ntiles, seed)
    for b in ({"done": 0.05}, {0: 50.0, "done": 0.1}, {4: 0.05}, {3: 20.0, "done": 0.2}):
        for seed in range(6):
            rnd = BiasedRandom(seed, b)
            assert simulate(13, H, seed, F=F, NST=NST, rnd=rnd) == "ok", (b, seed)


# items of a persistent CTA: tile counts of consecutive groups (empty groups
# included), the units closing at every group's end
ITEMS = [[3, 1, 4], [1, 1, 1, 1, 1], [0, 5, 0, 2], [7, 0, 0, 6, 1], [2, 9, 3, 3]]


@pytest.mark.parametrize("H,NST,F", [(1, 6, 1), (2, 5, 2), (2, 4, 3), (1, 5, 2), (2, 7, 3),
                                     (2, 2, 2), (1, 3, 3)])
def test_protocol_over_items_of_a_persistent_cta(H, NST, F):
    for seed in range(25):
        for items in ITEMS:
            assert simulate(items, H, seed, F=F, NST=NST) == "ok", (items, seed)
    for b in ({"done": 0.05}, {0: 50.0, "done": 0.1}, {4: 0.05}, {3: 20.0, "done": 0.2}):
        for seed in range(8):
            for items in ITEMS:
                rnd = BiasedRandom(seed, b)
                assert simulate(items, H, seed, F=F, NST=NST, rnd=rnd) == "ok", (b, items, seed)
