"""The tensor-core contraction's role protocol, simulated on the CPU.

k_tab_s12_tc (geosmie_gb300/csrc/gbmie_table_tc.cu) runs a producer thread,
two MMA-issuing threads, eight epilogue warps and a weights warp that hand
off through mbarriers: ring stages (full/empty), TMEM accumulator sets
(full/empty) and weight slots (full/empty).  A wait on an mbarrier passes when
the phase of the given parity has completed, so a wait two phases ahead would
also pass on the older phase; the kernel guards the ring with a per-stage
chunk tag.  This test runs a parity-exact model of the protocol (the item and
window rules of the kernel, its ring, set and slot counts read from the
source) over random mixes of whole-tile and half-tile items and windows 1 to
4, with MMA commits that land in order after random delays and roles
scheduled at random, and checks that every wait that passes on parity meant
the phase it was waiting for, that an MMA reads the chunk it expects, that the
epilogue reads the window and slot of its own item, and that every role
finishes.  A model with a planted mistake (one accumulator set for a
whole-tile window) must be caught.
"""
import os
import random
import re

import pytest

SRC = os.path.join(os.path.dirname(__file__), "..", "geosmie_gb300", "csrc", "gbmie_table_tc.cu")


def kernel_constants():
    s = open(SRC).read()
    nsets = int(re.search(r"#define TC_NSETS (\d+)", s).group(1))
    nw = int(re.search(r"#define TC_NW (\d+)", s).group(1))
    winmax = int(re.search(r"#define TC_WIN_MAX (\d+)", s).group(1))
    m = re.search(r"#define TC_NS\(NB\) \(\(NB\) <= (\d+) \? (\d+) : (\d+)\)", s)
    ns = sorted({int(m.group(2)), int(m.group(3))}) if m else [int(re.search(r"#define TC_NS\(NB\) (\d+)", s).group(1))]
    return ns, nsets, nw, winmax


class Barrier:
    """An mbarrier: arrivals complete phases; a parity wait passes once the
    phase of that parity has completed (completed phases' parity differs)."""

    def __init__(self, count):
        self.count, self.pending, self.done = count, 0, 0

    def arrive(self):
        self.pending += 1
        if self.pending == self.count:
            self.pending = 0
            self.done += 1

    def passes(self, parity):
        return (self.done & 1) != parity


class Fail(Exception):
    pass


def items_of(tiles, win):
    """The kernel's items: a tile whose chunks fit one window is one item
    (both of an issuer's sets), else one item per half tile with sizes."""
    out = []
    for t, (nc, ntile) in enumerate(tiles):
        whole = nc <= win
        for h in range(1 if whole else (2 if ntile > 32 else 1)):
            out.append((t, whole, h, nc))
    return out


def simulate(tiles, win, ns, nsets, nw, seed, whole_sets=2):
    rng = random.Random(seed)
    items = items_of(tiles, win)
    full = [Barrier(1) for _ in range(ns)]
    empty = [Barrier(1) for _ in range(ns)]
    accf = [Barrier(1) for _ in range(nsets)]
    acce = [Barrier(1) for _ in range(nsets)]
    wfull = [Barrier(1) for _ in range(nw)]
    wempty = [Barrier(1) for _ in range(nw)]
    s_chunk = [-1] * ns
    stage = [None] * ns            # (position, landed)
    set_window = {}                # (set, use) -> (item, window start, part)
    slot_item = {}                 # (slot, use) -> (tile, whole, half)
    pending = []                   # (due, issuer, barrier kind, index)

    def check(cond, msg):
        if not cond:
            raise Fail(msg)

    def producer():
        it = 0
        for (t, whole, h, nc) in items:
            for j in range(nc):
                c, st = it, it % ns
                it += 1
                if c >= ns:
                    while not empty[st].passes((c // ns - 1) & 1):
                        yield
                    check(empty[st].done >= c // ns, "producer: stage %d reused early" % st)
                s_chunk[st] = c
                stage[st] = (c, False)
                yield
                stage[st] = (c, True)
                full[st].arrive()

    def issuer(p):
        it = wc = 0
        for ii, (t, whole, h, nc) in enumerate(items):
            if (ii & 1) != p:
                it += nc
                continue
            for w0 in range(0, nc, win):
                nj = min(win, nc - w0)
                nset = whole_sets if whole else 1
                sets = []
                for q in range(nset):
                    x = wc + q
                    s_, use = 2 * p + (x & 1), x >> 1
                    if use > 0:
                        while not acce[s_].passes((use - 1) & 1):
                            yield
                        check(acce[s_].done >= use, "issuer: set %d reused early" % s_)
                    sets.append((s_, use))
                for j in range(nj):
                    c = it + j
                    st = c % ns
                    while not (s_chunk[st] == c and full[st].passes((c // ns) & 1)):
                        yield
                    check(full[st].done >= c // ns + 1, "issuer: stale stage for chunk %d" % c)
                for j in range(nj):
                    c = it + j
                    check(stage[c % ns] == (c, True), "MMA on stage %d without chunk %d" % (c % ns, c))
                    pending.append((rng.randint(1, 20), p, "empty", c % ns))
                it += nj
                for q, (s_, use) in enumerate(sets):
                    set_window[(s_, use)] = (ii, w0, q)
                    pending.append((rng.randint(1, 20), p, "accf", s_))
                wc += nset
                yield

    def epilogue():
        wce = [0, 0]
        for ie, (t, whole, h, nc) in enumerate(items):
            slot = ie % nw
            while not wfull[slot].passes((ie // nw) & 1):
                yield
            check(wfull[slot].done >= ie // nw + 1, "epilogue: stale weight slot")
            check(slot_item.get((slot, ie // nw)) == (t, whole, h), "epilogue: slot of another item")
            ip = ie & 1
            if whole:
                wi = wce[ip]
                for q in range(2):
                    x = wi + q
                    s_ = 2 * ip + (x & 1)
                    while not accf[s_].passes((x >> 1) & 1):
                        yield
                    check(accf[s_].done >= (x >> 1) + 1, "epilogue: stale set")
                    check(set_window.get((s_, x >> 1)) == (ie, 0, q), "epilogue: set of another window")
                yield
                for q in range(2):
                    acce[2 * ip + ((wi + q) & 1)].arrive()
                wce[ip] += 2
            else:
                for w in range((nc + win - 1) // win):
                    wi = wce[ip]
                    s_, use = 2 * ip + (wi & 1), wi >> 1
                    while not accf[s_].passes(use & 1):
                        yield
                    check(accf[s_].done >= use + 1, "epilogue: stale set")
                    check(set_window.get((s_, use)) == (ie, w * win, 0), "epilogue: set of another window")
                    acce[s_].arrive()
                    wce[ip] += 1
                    yield
            wempty[slot].arrive()

    def weights():
        iw = 0
        for t, (nc, ntile) in enumerate(tiles):
            whole = nc <= win
            yield   # the tile's loads
            for h in range(1 if whole else (2 if ntile > 32 else 1)):
                slot = iw % nw
                if iw >= nw:
                    while not wempty[slot].passes((iw // nw - 1) & 1):
                        yield
                    check(wempty[slot].done >= iw // nw, "weights: slot reused early")
                slot_item[(slot, iw // nw)] = (t, whole, h)
                wfull[slot].arrive()
                iw += 1

    roles = {"producer": producer(), "issuer0": issuer(0), "issuer1": issuer(1), "epilogue": epilogue(),
             "weights": weights()}
    for step in range(2_000_000):
        # each issuer's commits land in order
        for p in (0, 1):
            mine = [x for x in pending if x[1] == p]
            if mine and rng.random() < 0.3:
                due, _, kind, idx = mine[0]
                if due <= 0:
                    pending.remove(mine[0])
                    (empty if kind == "empty" else accf)[idx].arrive()
                else:
                    pending[pending.index(mine[0])] = (due - 1, p, kind, idx)
        if not roles:
            if not pending:
                return
            continue
        name = rng.choice(sorted(roles))
        try:
            next(roles[name])
        except StopIteration:
            del roles[name]
    raise Fail("no progress: a role waits forever")


def random_case(seed, winmax):
    rng = random.Random(seed)
    win = rng.randint(1, winmax)
    tiles = [(rng.choice([1, 1, 1, 1, 2, 3, 4, 5, 7, 9]), rng.choice([64, 64, 64, 40, 20]))
             for _ in range(rng.randint(1, 30))]
    return tiles, win


@pytest.mark.parametrize("ns_index", [0, 1])
def test_contraction_protocol_cpu(ns_index):
    ns_all, nsets, nw, winmax = kernel_constants()
    ns = ns_all[min(ns_index, len(ns_all) - 1)]
    assert winmax <= ns, "a window's chunks must fit the ring"
    for seed in range(150):
        tiles, win = random_case(seed, winmax)
        simulate(tiles, win, ns, nsets, nw, seed)


def test_protocol_model_catches_a_planted_mistake_cpu():
    ns_all, nsets, nw, winmax = kernel_constants()
    caught = 0
    for seed in range(40):
        tiles, win = random_case(seed, winmax)
        try:
            simulate(tiles, win, ns_all[0], nsets, nw, seed, whole_sets=1)
        except Fail:
            caught += 1
    assert caught >= 30, caught
