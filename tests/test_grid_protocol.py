"""The gridded kernel's handoff protocol, modelled on the CPU.

``rotate_average_gridded`` (icrar-leap-accelerate_gb300/csrc/kernels_grid.cuh) runs four
roles per block: a bulk-copy producer, an MMA issuer, 4 fold warps and 8 epilogue warps.
They hand operand stages and TMEM regions (RS[0], RS[1], IS, AC) to one another through
mbarriers, and every wait is by phase parity: a wait for phase k passes once the barrier
has completed k + 1 phases, but parity cannot tell k + 1 from k - 1 or k + 3.  A role
that waits for a phase two ahead of the barrier would pass at once, and one that lags
two phases behind would block.

This model replays each role's loops, counters, waits and arrivals as the kernel writes
them (producer, MMA issuer, fold and epilogue sections of the kernel), with the bulk
copies landing in any order and the MMA commits completing in issue order, under seeded
random interleavings of 14 actors and many unit shapes (chunks per tile, tiles per
unit, passes per tile).  It checks that
  - every wait is for phase c or c - 1 of a barrier that has completed c phases (and
    that the parity the kernel passes is that phase's);
  - no stage is refilled while MMAs that read it are in flight, and no TMEM region is
    overwritten, or read, before its previous readers and writers are done;
  - every actor finishes (no deadlock).
The ring and segment sizes are read from the kernel header.
"""
import os
import random
import re

import pytest

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "icrar-leap-accelerate_gb300",
                      "csrc", "kernels_grid.cuh")


def _constants():
    text = open(HEADER).read()

    def get(name):
        m = re.search(r"constexpr int %s = (\d+);" % name, text)
        assert m, name
        return int(m.group(1))

    stages, macro, seg = get("kGrStages"), get("kGrMacro"), get("kGrSegChunks")
    assert macro == seg and stages % macro == 0
    return stages // macro, macro, seg


MS, MACRO, SEG = _constants()
FOLD_WARPS, EPI_WARPS = 4, 8


class Bar:
    def __init__(self, name, count):
        self.name, self.count, self.pending, self.phases = name, count, 0, 0

    def arrive(self):
        self.pending += 1
        assert self.pending <= self.count, self.name
        if self.pending == self.count:
            self.pending = 0
            self.phases += 1


class Wait:
    def __init__(self, bar, parity, k):
        self.bar, self.parity, self.k = bar, parity, k


class Model:
    def __init__(self, units, rng):
        self.units, self.rng = units, rng
        self.vfull = [Bar("vfull%d" % i, 1) for i in range(MS)]
        self.sdone = [Bar("sdone%d" % i, 1) for i in range(MS)]
        self.is_empty = Bar("is_empty", FOLD_WARPS)
        self.ac_free = Bar("ac_free", FOLD_WARPS)
        self.rs_full = [Bar("rs_full%d" % i, FOLD_WARPS) for i in range(2)]
        self.rs_free = [Bar("rs_free%d" % i, EPI_WARPS) for i in range(2)]
        self.landing = []        # rounds whose copies are in flight (land in any order)
        self.commits = []        # rounds whose MMA commits are in flight (complete in order)
        self.rounds_done = 0     # rounds whose MMAs have all completed
        self.mid_folds = {}      # (tile, segment) -> fold warps done with it
        self.final_folds = {}    # tile -> fold warps done with its final fold
        self.epi_done = {}       # tile -> epilogue warps done reading its running sum
        self.is_owner = None     # (tile, segment) whose hi*hi products IS holds
        self.rs_owner = [None, None]

    # ---- helpers -------------------------------------------------------------------------
    def tiles(self):
        for nchunk, ntb, npass in self.units:
            for _ in range(ntb):
                for _ in range(npass):
                    yield nchunk

    def _count(self, d, key):
        return d.get(key, 0)

    # ---- roles (the kernel's loops) -------------------------------------------------------
    def producer(self):
        ctr = 0
        for nchunk in self.tiles():
            for _ in range(0, nchunk, MACRO):
                m = ctr % MS
                if ctr >= MS:
                    yield Wait(self.sdone[m], ((ctr // MS) - 1) & 1, (ctr // MS) - 1)
                    # The stage's previous round: every MMA that read it has completed.
                    assert self.rounds_done >= ctr - MS + 1, "stage refilled under in-flight MMAs"
                self.landing.append((m, ctr))
                ctr += 1

    def issuer(self):
        ctr = blk = mids = 0
        for nchunk in self.tiles():
            b = blk & 1
            if blk >= 2:
                yield Wait(self.rs_free[b], ((blk >> 1) - 1) & 1, (blk >> 1) - 1)
            if blk >= 1:
                yield Wait(self.ac_free, (blk - 1) & 1, blk - 1)
            for q0 in range(0, nchunk, MACRO):
                m, nq, seg = ctr % MS, min(MACRO, nchunk - q0), q0 // SEG
                yield Wait(self.vfull[m], (ctr // MS) & 1, ctr // MS)
                # Corrections into AC; the tile's first round overwrites it.
                if q0 == 0 and blk >= 1:
                    assert self._count(self.final_folds, blk - 1) == FOLD_WARPS, "AC overwritten before its fold"
                if seg >= 2:
                    yield Wait(self.is_empty, (mids - 1) & 1, mids - 1)
                if seg == 0:
                    if blk >= 2:
                        assert self._count(self.epi_done, blk - 2) == EPI_WARPS, "RS overwritten while read"
                    self.rs_owner[b] = blk
                else:
                    prev = self.is_owner
                    if prev is not None:
                        pt, ps = prev
                        if pt == blk:
                            assert self._count(self.mid_folds, prev) == FOLD_WARPS, "IS restarted before its fold"
                        else:
                            assert self._count(self.final_folds, pt) == FOLD_WARPS, "IS restarted before its fold"
                    self.is_owner = (blk, seg)
                if seg >= 1 and q0 + nq < nchunk:
                    mids += 1
                self.commits.append(ctr)
                ctr += 1
            blk += 1

    def fold(self, w):
        blk = rnd = 0
        for nchunk in self.tiles():
            nseg = (nchunk + SEG - 1) // SEG
            b = blk & 1
            for sg in range(1, nseg - 1):
                r = rnd + sg
                yield Wait(self.sdone[r % MS], (r // MS) & 1, r // MS)
                assert self.rounds_done >= r + 1, "segment folded before its MMAs completed"
                assert self.is_owner == (blk, sg), "IS holds another segment"
                assert self.rs_owner[b] == blk and (blk < 2 or self._count(self.epi_done, blk - 2) == EPI_WARPS)
                self.mid_folds[(blk, sg)] = self._count(self.mid_folds, (blk, sg)) + 1
                self.is_empty.arrive()
            rl = rnd + nseg - 1
            if blk >= 2:
                yield Wait(self.rs_free[b], ((blk >> 1) - 1) & 1, (blk >> 1) - 1)
            yield Wait(self.sdone[rl % MS], (rl // MS) & 1, rl // MS)
            assert self.rounds_done >= rl + 1, "final fold before the tile's MMAs completed"
            assert nseg < 2 or self.is_owner == (blk, nseg - 1), "IS holds another segment"
            assert self.rs_owner[b] == blk
            self.final_folds[blk] = self._count(self.final_folds, blk) + 1
            self.ac_free.arrive()
            self.rs_full[b].arrive()
            blk += 1
            rnd += nseg

    def epilogue(self, e):
        blk = 0
        for nchunk in self.tiles():
            rb = blk & 1
            yield Wait(self.rs_full[rb], (blk >> 1) & 1, blk >> 1)
            assert self._count(self.final_folds, blk) == FOLD_WARPS, "running sum read before its final fold"
            assert self.rs_owner[rb] == blk, "running sum overwritten while read"
            yield None  # reads and interpolation: other roles may run meanwhile
            assert self.rs_owner[rb] == blk, "running sum overwritten while read"
            self.epi_done[blk] = self._count(self.epi_done, blk) + 1
            self.rs_free[rb].arrive()
            blk += 1

    # ---- scheduler ----------------------------------------------------------------------
    def run(self):
        actors = [self.producer(), self.issuer()] + [self.fold(w) for w in range(FOLD_WARPS)] + \
            [self.epilogue(e) for e in range(EPI_WARPS)]
        state = [None] * len(actors)  # the request each actor is blocked on (None: runnable)
        done = [False] * len(actors)

        def step(i):
            try:
                state[i] = next(actors[i])
            except StopIteration:
                done[i] = True
                state[i] = None

        for i in range(len(actors)):
            step(i)
        while True:
            choices = []
            for i, req in enumerate(state):
                if done[i]:
                    continue
                if req is None:
                    choices.append(("actor", i))
                    continue
                c, k = req.bar.phases, req.k
                assert k <= c <= k + 1, "%s: wait for phase %d with %d completed" % (req.bar.name, k, c)
                assert req.parity == (k & 1), req.bar.name
                if (c & 1) != req.parity:  # the parity test the hardware does
                    choices.append(("actor", i))
            choices += [("land", j) for j in range(len(self.landing))]
            if self.commits:
                choices.append(("commit", 0))
            if not choices:
                assert all(done), "deadlock: blocked on %s" % [r.bar.name for r in state if r is not None]
                assert not self.landing and not self.commits
                return
            kind, j = self.rng.choice(choices)
            if kind == "actor":
                step(j)
            elif kind == "land":
                m, _ = self.landing.pop(j)
                self.vfull[m].arrive()
            else:
                r = self.commits.pop(0)
                assert r == self.rounds_done
                self.rounds_done += 1
                self.sdone[r % MS].arrive()


def _shapes(rng, n):
    for _ in range(n):
        units = []
        for _ in range(rng.randint(1, 4)):
            units.append((rng.randint(1, 26), rng.randint(1, 4), rng.choice([0, 1, 1, 1, 2, 3])))
        yield units


@pytest.mark.parametrize("seed", range(12))
def test_gridded_handoff_protocol(seed):
    rng = random.Random(seed)
    for units in _shapes(rng, 25):
        Model(units, rng).run()


def test_gridded_handoff_protocol_fixed_shapes():
    rng = random.Random(99)
    # 384 channels (24 chunks, 6 segments), 4 tiles per unit; one-chunk tiles; a partial last segment.
    for units in ([(24, 4, 1)] * 3, [(1, 1, 1)] * 5, [(13, 2, 3), (5, 1, 1)], [(24, 1, 2), (2, 3, 0), (9, 4, 1)]):
        for _ in range(20):
            Model(units, rng).run()


def test_model_catches_a_wrong_phase():
    # Plant a mistake in the model (not the kernel): the epilogue waits one phase ahead.
    class Bad(Model):
        def epilogue(self, e):
            for req in Model.epilogue(self, e):
                if isinstance(req, Wait):
                    req = Wait(req.bar, (req.k + 1) & 1, req.k + 1)
                yield req

    with pytest.raises(AssertionError):
        for seed in range(5):
            Bad([(24, 4, 1)] * 2, random.Random(seed)).run()
