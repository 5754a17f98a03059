"""A CPU model of the tensor-core kernel's barrier protocol, explored under
random schedules: the race and deadlock check the GPU pool cannot run
(compute-sanitizer is closed there).

The model follows bf_form_beams_tc role by role: the E producer (raw E
slots), the W producer (digit rows and W slots; in the two-group layout it
reuses a W slot once the tensor core's commit for that slot's last stage
arrives), the W forwarder, the unpack groups (raw slot -> TMEM stage), the
MMA issuer (offset MMA, stage MMAs, commits, and the exit drain) and the
epilogue.  Barriers have the hardware's semantics: an expected arrival count
and transaction bytes per phase, and parity waits that see only the parity
of the phase in progress.  TMA copies and tcgen05 commits complete
asynchronously, in any order the scheduler picks (MMAs in issue order).  A
checker tracks every shared-memory and TMEM slot: what it holds, who is
writing or reading it, and flags a read of the wrong content, a write over
content still in use, a parity wait that could alias a phase, and deadlock.
"""
from __future__ import annotations

import random

import pytest


class Barrier:
    def __init__(self, name, count):
        self.name, self.count = name, count
        self.pending, self.tx, self.completed = count, 0, 0

    def _maybe_complete(self):
        if self.pending == 0 and self.tx == 0:
            self.completed += 1
            self.pending = self.count

    def arrive(self, expect_tx=0):
        assert self.pending > 0, f"{self.name}: arrival beyond the expected count"
        self.tx += expect_tx
        self.pending -= 1
        self._maybe_complete()

    def complete_tx(self, nbytes):
        self.tx -= nbytes
        self._maybe_complete()

    def parity_done(self, parity):
        """try_wait.parity: true when the phase in progress has the other parity."""
        return (self.completed & 1) != parity


class Hazard(AssertionError):
    pass


class Model:
    """One CTA of the kernel over `ntiles` tiles of `nk` K stages."""

    def __init__(self, S, SW, R, groups, nk, ntiles, rng):
        self.S, self.SW, self.R, self.G, self.nk, self.nt = S, SW, R, groups, nk, ntiles
        self.total = ntiles * nk
        self.rng = rng
        fwd = groups > 1
        self.fwd = fwd
        B = Barrier
        self.raw_full = [B(f"raw_full{i}", 1) for i in range(R)]
        self.raw_empty = [B(f"raw_empty{i}", 1) for i in range(R)]  # one arrival per unpack group-stage
        self.w_full = [B(f"w_full{i}", 1) for i in range(SW)]
        self.w_empty = [B(f"w_empty{i}", 1) for i in range(SW)]
        self.a_full = [B(f"a_full{i}", 1 + (1 if fwd else 0)) for i in range(S)]
        self.empty = [B(f"empty{i}", 1) for i in range(S)]
        self.accfull = [B(f"accfull{i}", 1) for i in range(2)]
        self.accempty = [B(f"accempty{i}", 1) for i in range(2)]
        self.d_full = [B(f"d_full{i}", 1) for i in range(2)]
        self.d_empty = [B(f"d_empty{i}", 1) for i in range(2)]
        # slot contents: (what, id, complete?) and in-flight readers
        self.raw = [None] * R
        self.wslot = [None] * SW
        self.dslot = [None] * 2
        self.stage = [None] * S
        self.acc = [None] * 2
        self.readers = {}  # (kind, index) -> set of in-flight reader ids
        self.events = []   # asynchronous completions: callables
        self.mma_queue = []  # in-flight MMAs in issue order: (reads, write, id)
        self.commits = []  # (barrier, mma count at commit)
        self.mma_issued = 0
        self.mma_done = 0
        self.acc_tile_done = {}

    # --------------------------------------------------------------- helpers
    def wait(self, bar, phase):
        """A role waits for phase `phase` of `bar` (the phase index it means)."""
        return ("wait", bar, phase)

    def check_wait(self, bar, phase):
        # the parity wait returns when the phase in progress has the other parity;
        # it means "phase `phase` is complete" only while the barrier is at most
        # one phase past it
        if bar.completed > phase + 1:
            raise Hazard(f"{bar.name}: waiting for phase {phase} after {bar.completed} completed (parity alias)")
        done = bar.parity_done(phase & 1)
        if done and bar.completed != phase + 1:
            # the phase before is still in progress: the same parity as "done"
            raise Hazard(f"{bar.name}: the wait for phase {phase} returns while phase {bar.completed} is in progress")
        return done

    def busy(self, kind, i):
        return bool(self.readers.get((kind, i)))

    # ------------------------------------------------------ asynchronous work
    def tma(self, bar, nbytes, on_land):
        def land():
            on_land()
            bar.complete_tx(nbytes)
        self.events.append(land)

    def mma(self, reads, write):
        """Issue one MMA: reads [(kind, index, expected content)], writes (kind, index, tile)."""
        for kind, i, want in reads:
            slot = getattr(self, kind)[i]
            if slot != (want, True):
                raise Hazard(f"MMA reads {kind}[{i}] holding {slot}, wants {want}")
        mid = self.mma_issued
        self.mma_issued += 1
        for kind, i, _ in reads:
            self.readers.setdefault((kind, i), set()).add(mid)
        self.mma_queue.append((reads, write, mid))

    def commit(self, bar):
        self.commits.append((bar, self.mma_issued))

    def complete_next_mma(self):
        reads, write, mid = self.mma_queue.pop(0)
        for kind, i, _ in reads:
            self.readers[(kind, i)].discard(mid)
        self.mma_done += 1
        if write is not None:
            t = write
            self.acc_tile_done[t] = self.acc_tile_done.get(t, 0) + 1

    def deliverable_commits(self):
        return [c for c in self.commits if c[1] <= self.mma_done]

    # ------------------------------------------------------------------ roles
    def e_producer(self):
        for k in range(self.total):
            r = k % self.R
            yield self.wait(self.raw_empty[r], k // self.R - 1) if k >= self.R else ("go",)
            prev = self.raw[r]
            if prev is not None and prev != (("consumed", k - self.R), True):
                raise Hazard(f"E producer overwrites raw[{r}] holding {prev} for sequence {k}")
            self.raw[r] = (k, False)

            def land(r=r, k=k):
                self.raw[r] = (k, True)
            self.raw_full[r].arrive(expect_tx=1)
            self.tma(self.raw_full[r], 1, land)

    def w_producer(self):
        k = 0
        for t in range(self.nt):
            d = t % 2
            if t >= 2:
                yield self.wait(self.d_empty[d], t // 2 - 1)
            if self.busy("dslot", d):
                raise Hazard(f"digits for tile {t} overwrite a slot the tensor core reads")
            self.dslot[d] = (t, False)

            def dland(d=d, t=t):
                self.dslot[d] = (t, True)
            self.d_full[d].arrive(expect_tx=1)
            self.tma(self.d_full[d], 1, dland)
            for _ in range(self.nk):
                s = k % self.SW
                if self.fwd:
                    if k >= self.SW:
                        j = k - self.SW
                        yield self.wait(self.empty[j % self.S], j // self.S)
                elif k >= self.SW:
                    yield self.wait(self.w_empty[s], k // self.SW - 1)
                if self.busy("wslot", s):
                    raise Hazard(f"W producer overwrites W slot {s} for sequence {k} while the tensor core reads it")
                self.wslot[s] = (k, False)

                def wland(s=s, k=k):
                    self.wslot[s] = (k, True)
                self.w_full[s].arrive(expect_tx=1)
                self.tma(self.w_full[s], 1, wland)
                k += 1

    def forwarder(self):
        for k in range(self.total):
            yield self.wait(self.w_full[k % self.SW], k // self.SW)
            if k >= self.S:
                yield self.wait(self.a_full[(k - self.S) % self.S], (k - self.S) // self.S)
            self.a_full[k % self.S].arrive()

    def unpack(self, g):
        for k in range(g, self.total, self.G):
            r, s = k % self.R, k % self.S
            yield self.wait(self.raw_full[r], k // self.R)
            if self.raw[r] != (k, True):
                raise Hazard(f"unpack of sequence {k} reads raw[{r}] holding {self.raw[r]}")
            self.raw[r] = (("consumed", k), True)
            self.raw_empty[r].arrive()
            if k >= self.S:
                yield self.wait(self.empty[s], k // self.S - 1)
            if self.busy("stage", s):
                raise Hazard(f"unpack of sequence {k} writes TMEM stage {s} while the tensor core reads it")
            self.stage[s] = (k, True)
            if not self.fwd:
                # one group: hand back the W slot of sequence k - S, wait for this one's
                if k >= self.S:
                    self.w_empty[(k - self.S) % self.SW].arrive()
                yield self.wait(self.w_full[k % self.SW], k // self.SW)
            self.a_full[s].arrive()

    def mma_thread(self):
        k = 0
        nstage = ndig = nacc = 0
        for t in range(self.nt):
            ab = t % 2
            if t >= 2:
                yield self.wait(self.accempty[ab], t // 2 - 1)
            yield self.wait(self.d_full[ab], t // 2)
            if self.acc[ab] is not None and self.acc[ab][0] != t - 2:
                raise Hazard(f"tile {t} starts accumulator {ab} holding {self.acc[ab]}")
            self.acc[ab] = (t, True)
            self.mma([("dslot", ab, t)], t)
            self.commit(self.d_empty[ab])
            ndig += 1
            for _ in range(self.nk):
                s, sw = k % self.S, k % self.SW
                yield self.wait(self.a_full[s], k // self.S)
                self.mma([("stage", s, k), ("wslot", sw, k)], t)
                self.commit(self.empty[s])
                nstage += 1
                k += 1
            self.commit(self.accfull[ab])
            nacc += 1
        # exit drain: the last phase committed on every barrier
        for q in range(max(0, nstage - self.S), nstage):
            yield self.wait(self.empty[q % self.S], q // self.S)
        for q in range(max(0, ndig - 2), ndig):
            yield self.wait(self.d_empty[q % 2], q // 2)
        for q in range(max(0, nacc - 2), nacc):
            yield self.wait(self.accfull[q % 2], q // 2)

    def epilogue(self):
        for t in range(self.nt):
            ab = t % 2
            yield self.wait(self.accfull[ab], t // 2)
            if self.acc_tile_done.get(t, 0) != 1 + self.nk:
                raise Hazard(f"epilogue reads tile {t} with {self.acc_tile_done.get(t, 0)} of {1 + self.nk} MMAs done")
            self.accempty[ab].arrive()

    # -------------------------------------------------------------- scheduler
    def run(self, inorder_commits=True):
        roles = {"E": self.e_producer(), "W": self.w_producer(), "MMA": self.mma_thread(), "epi": self.epilogue()}
        for g in range(self.G):
            roles[f"unpack{g}"] = self.unpack(g)
        if self.fwd:
            roles["fwd"] = self.forwarder()
        blocked = {name: None for name in roles}
        done = set()

        def step(name):
            gen = roles[name]
            while True:
                op = blocked[name]
                if op is None:
                    try:
                        op = next(gen)
                    except StopIteration:
                        done.add(name)
                        return
                if op[0] == "go":
                    blocked[name] = None
                    continue
                _, bar, phase = op
                if self.check_wait(bar, phase):
                    blocked[name] = None
                    continue
                blocked[name] = op
                return

        for name in list(roles):
            step(name)
        while len(done) < len(roles):
            runnable = [n for n in roles if n not in done and (blocked[n] is None or
                                                               self.check_wait(blocked[n][1], blocked[n][2]))]
            choices = [("role", n) for n in runnable]
            choices += [("event", i) for i in range(len(self.events))]
            if self.mma_queue:
                choices.append(("mma", 0))
            dc = self.deliverable_commits()
            if dc:
                choices += [("commit", i) for i in range(1 if inorder_commits else len(dc))]
            if not choices:
                raise Hazard(f"deadlock: blocked {[(n, blocked[n][1].name, blocked[n][2]) for n in roles if n not in done]}")
            kind, i = self.rng.choice(choices)
            if kind == "role":
                step(i)
            elif kind == "event":
                self.events.pop(i)()
            elif kind == "mma":
                self.complete_next_mma()
            else:
                bar, _ = dc[i]
                self.commits.remove(dc[i])
                bar.arrive()
        assert not self.events and not self.mma_queue
        # every commit's arrival landed before the CTA's exit
        assert not self.commits, f"commits still to land at exit: {[c[0].name for c in self.commits]}"


# The layouts the planner produces: S stages, SW W slots, R raw slots, unpack groups.
LAYOUTS = {
    "b96 one group": dict(S=2, SW=3, R=4, groups=1, nk=4),
    "b96 one group, odd raw ring": dict(S=2, SW=3, R=5, groups=1, nk=4),
    "b64 two groups": dict(S=4, SW=4, R=4, groups=2, nk=4),
    "b32 two groups": dict(S=6, SW=6, R=6, groups=2, nk=4),
    "b16 half-SM": dict(S=2, SW=5, R=4, groups=1, nk=4),
    "d1024 one group": dict(S=2, SW=3, R=6, groups=1, nk=8),
    "b64 two groups, ring plan 2": dict(S=4, SW=2, R=8, groups=2, nk=4),
}


@pytest.mark.parametrize("name", sorted(LAYOUTS))
@pytest.mark.parametrize("inorder", [True, False])
def test_protocol_random_schedules(name, inorder):
    """No deadlock, no hazard and no phase alias over many random schedules."""
    cfg = LAYOUTS[name]
    for seed in range(150):
        rng = random.Random(hash((name, inorder, seed)) & 0xFFFFFFFF)
        Model(ntiles=7, rng=rng, **cfg).run(inorder_commits=inorder)


def test_protocol_model_finds_odd_raw_rings_with_two_groups():
    """The planted mistake, on the CPU: two unpack groups over an odd number of
    raw E slots (5 and 7, which the planner gave b=64 and b=32 passes before it
    kept the ring even) let a group's raw_full parity wait return a phase
    early; the model must catch it under some schedule."""
    for R, S in ((5, 4), (7, 6)):
        found = False
        for seed in range(400):
            try:
                Model(S=S, SW=S, R=R, groups=2, nk=4, ntiles=8, rng=random.Random(seed)).run()
            except Hazard:
                found = True
                break
        assert found, (R, S)


def test_protocol_model_finds_the_old_w_slot_rule():
    """The planted mistake, on the CPU: two unpack groups with more W slots than
    TMEM stages (6 against 4, which the planner allowed before it clamped W
    slots to stages) let the W producer's parity wait on `empty` alias a phase;
    the model must catch it under some schedule."""
    found = False
    for seed in range(400):
        try:
            Model(S=4, SW=6, R=7, groups=2, nk=4, ntiles=8, rng=random.Random(seed)).run()
        except Hazard:
            found = True
            break
    assert found
