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
import zlib

import pytest


def _seed(*parts):
    """A reproducible seed (str hashes change from process to process)."""
    return zlib.crc32("|".join(map(str, parts)).encode())


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

    def __init__(self, S, SW, R, groups, nk, ntiles, rng, drain_always=True, naccs=2):
        self.S, self.SW, self.R, self.G, self.nk, self.nt = S, SW, R, groups, nk, ntiles
        # the producers drain their copies on every exit (False: only after an
        # error of their own, which leaves copies landing after the exit)
        self.drain_always = drain_always
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
        # accumulators in TMEM: the kernel double-buffers them (2); 1 is the
        # candidate layout whose epilogue releases its accumulator right after
        # reading it
        self.A = naccs
        self.accfull = [B(f"accfull{i}", 1) for i in range(naccs)]
        self.accempty = [B(f"accempty{i}", 1) for i in range(naccs)]
        self.d_full = [B(f"d_full{i}", 1) for i in range(2)]
        self.d_empty = [B(f"d_empty{i}", 1) for i in range(2)]
        # slot contents: (what, id, complete?) and in-flight readers
        self.raw = [None] * R
        self.wslot = [None] * SW
        self.dslot = [None] * 2
        self.stage = [None] * S
        self.acc = [None] * naccs
        self.readers = {}  # (kind, index) -> set of in-flight reader ids
        self.events = []   # asynchronous completions: callables
        self.mma_queue = []  # in-flight MMAs in issue order: (reads, write, id)
        self.commits = []  # (barrier, mma count at commit)
        self.mma_issued = 0
        self.mma_done = 0
        self.acc_tile_done = {}
        self.acc_reading = [None] * naccs  # tile whose accumulator the epilogue is reading
        self.acc_read = set()            # tiles the epilogue has read
        self.mma_skips_accempty = False  # planted mistake: start a tile without waiting for accempty
        self.unpack_signals_early = False  # planted mistake: a_full before the TMEM stores are waited on

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
        land.barrier = bar.name
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
    # A role yields ("wait", barrier, phase) and receives True when the phase
    # completed, or False when the wait gave up (the kernel's bounded wait:
    # its own time limit, or another role's error seen in the error word);
    # ("drain", barrier, phase) ignores the error word, as the kernel's
    # mbar_wait_drain does.
    def e_producer(self):
        issued = 0
        ok = True
        for k in range(self.total):
            r = k % self.R
            if k >= self.R:
                ok = yield self.wait(self.raw_empty[r], k // self.R - 1)
                if not ok:
                    break
            prev = self.raw[r]
            if prev is not None and prev != (("consumed", k - self.R), True):
                raise Hazard(f"E producer overwrites raw[{r}] holding {prev} for sequence {k}")
            self.raw[r] = (k, False)

            def land(r=r, k=k):
                self.raw[r] = (k, True)
            self.raw_full[r].arrive(expect_tx=1)
            self.tma(self.raw_full[r], 1, land)
            issued += 1
        # let the copies already issued land before the CTA exits, also when
        # this role saw no error (another role's error can end the consumers)
        if self.drain_always or not ok:
            for q in range(max(0, issued - self.R), issued):
                yield ("drain", self.raw_full[q % self.R], q // self.R)

    def w_producer(self):
        k = dit = 0
        ok = True
        for t in range(self.nt):
            d = t % 2
            if t >= 2:
                ok = yield self.wait(self.d_empty[d], t // 2 - 1)
                if not ok:
                    break
            if self.busy("dslot", d):
                raise Hazard(f"digits for tile {t} overwrite a slot the tensor core reads")
            self.dslot[d] = (t, False)

            def dland(d=d, t=t):
                self.dslot[d] = (t, True)
            self.d_full[d].arrive(expect_tx=1)
            self.tma(self.d_full[d], 1, dland)
            dit += 1
            for _ in range(self.nk):
                s = k % self.SW
                if self.fwd:
                    if k >= self.SW:
                        j = k - self.SW
                        ok = yield self.wait(self.empty[j % self.S], j // self.S)
                elif k >= self.SW:
                    ok = yield self.wait(self.w_empty[s], k // self.SW - 1)
                if not ok:
                    break
                if self.busy("wslot", s):
                    raise Hazard(f"W producer overwrites W slot {s} for sequence {k} while the tensor core reads it")
                self.wslot[s] = (k, False)

                def wland(s=s, k=k):
                    self.wslot[s] = (k, True)
                self.w_full[s].arrive(expect_tx=1)
                self.tma(self.w_full[s], 1, wland)
                k += 1
            if not ok:
                break
        if self.drain_always or not ok:
            for q in range(max(0, k - self.SW), k):
                yield ("drain", self.w_full[q % self.SW], q // self.SW)
            for q in range(max(0, dit - 2), dit):
                yield ("drain", self.d_full[q % 2], q // 2)

    def forwarder(self):
        for k in range(self.total):
            if not (yield self.wait(self.w_full[k % self.SW], k // self.SW)):
                return
            if k >= self.S and not (yield self.wait(self.a_full[(k - self.S) % self.S], (k - self.S) // self.S)):
                return
            self.a_full[k % self.S].arrive()

    def unpack(self, g):
        for k in range(g, self.total, self.G):
            r, s = k % self.R, k % self.S
            if not (yield self.wait(self.raw_full[r], k // self.R)):
                return
            if self.raw[r] != (k, True):
                raise Hazard(f"unpack of sequence {k} reads raw[{r}] holding {self.raw[r]}")
            self.raw[r] = (("consumed", k), True)
            self.raw_empty[r].arrive()
            if k >= self.S and not (yield self.wait(self.empty[s], k // self.S - 1)):
                return
            if self.busy("stage", s):
                raise Hazard(f"unpack of sequence {k} writes TMEM stage {s} while the tensor core reads it")
            # the TMEM stores take time: other roles may run before they are waited on
            self.stage[s] = (k, False)
            if self.unpack_signals_early:
                self.a_full[s].arrive()
            yield ("step", None, None)
            if self.busy("stage", s):
                raise Hazard(f"the tensor core reads TMEM stage {s} while the unpack of sequence {k} writes it")
            self.stage[s] = (k, True)
            if not self.fwd:
                # one group: hand back the W slot of sequence k - S, wait for this one's
                if k >= self.S:
                    self.w_empty[(k - self.S) % self.SW].arrive()
                if not (yield self.wait(self.w_full[k % self.SW], k // self.SW)):
                    return
            if not self.unpack_signals_early:
                self.a_full[s].arrive()

    def mma_thread(self):
        k = 0
        nstage = ndig = nacc = 0
        A = self.A
        for t in range(self.nt):
            ab, dd = t % A, t % 2  # accumulator, digit-row slot
            if t >= A and not self.mma_skips_accempty and not (yield self.wait(self.accempty[ab], t // A - 1)):
                break
            if not (yield self.wait(self.d_full[dd], t // 2)):
                break
            if self.acc[ab] is not None and self.acc[ab][0] != t - A:
                raise Hazard(f"tile {t} starts accumulator {ab} holding {self.acc[ab]}")
            if t >= A and (self.acc_reading[ab] is not None or t - A not in self.acc_read):
                raise Hazard(f"tile {t} overwrites accumulator {ab} before the epilogue has read tile {t - A}")
            self.acc[ab] = (t, True)
            self.mma([("dslot", dd, t)], t)
            self.commit(self.d_empty[dd])
            ndig += 1
            ok = True
            for _ in range(self.nk):
                s, sw = k % self.S, k % self.SW
                ok = yield self.wait(self.a_full[s], k // self.S)
                if not ok:
                    break
                self.mma([("stage", s, k), ("wslot", sw, k)], t)
                self.commit(self.empty[s])
                nstage += 1
                k += 1
            if not ok:
                break
            self.commit(self.accfull[ab])
            nacc += 1
        # exit drain: the last phase committed on every barrier
        for q in range(max(0, nstage - self.S), nstage):
            yield ("drain", self.empty[q % self.S], q // self.S)
        for q in range(max(0, ndig - 2), ndig):
            yield ("drain", self.d_empty[q % 2], q // 2)
        for q in range(max(0, nacc - A), nacc):
            yield ("drain", self.accfull[q % A], q // A)

    def epilogue(self):
        for t in range(self.nt):
            ab = t % self.A
            if not (yield self.wait(self.accfull[ab], t // self.A)):
                return
            if self.acc_tile_done.get(t, 0) != 1 + self.nk:
                raise Hazard(f"epilogue reads tile {t} with {self.acc_tile_done.get(t, 0)} of {1 + self.nk} MMAs done")
            # the TMEM loads take time: other roles may run before they are waited on
            self.acc_reading[ab] = t
            yield ("step", None, None)
            self.acc_reading[ab] = None
            self.acc_read.add(t)
            self.accempty[ab].arrive()

    # -------------------------------------------------------------- scheduler
    def run(self, inorder_commits=True, fail=None):
        """Runs every role to its end.  `fail` = (role, n): that role's n-th wait
        gives up (its time limit), setting the error word; the other roles then
        give up at any later poll of a wait, as the kernel's do."""
        roles = {"E": self.e_producer(), "W": self.w_producer(), "MMA": self.mma_thread(), "epi": self.epilogue()}
        for g in range(self.G):
            roles[f"unpack{g}"] = self.unpack(g)
        if self.fwd:
            roles["fwd"] = self.forwarder()
        blocked = {name: None for name in roles}
        nwaits = {name: 0 for name in roles}
        done = set()
        err = [False]

        def resume(name, value):
            gen = roles[name]
            try:
                op = gen.send(value) if value is not None else next(gen)
            except StopIteration:
                done.add(name)
                blocked[name] = None
                return
            blocked[name] = op
            settle(name)

        def settle(name):
            # run a role on while its waits are already decided
            while name not in done:
                op = blocked[name]
                kind, bar, phase = op
                if kind == "step":  # a scheduling point: the scheduler resumes it
                    return
                if kind == "wait":
                    nwaits[name] += 1
                    if fail == (name, nwaits[name]):
                        err[0] = True
                        resume(name, False)
                        return
                if self.check_wait(bar, phase):
                    resume(name, True)
                    return
                return

        for name in list(roles):
            resume(name, None)
        while len(done) < len(roles):
            choices = []
            for n in roles:
                if n in done:
                    continue
                kind, bar, phase = blocked[n]
                if kind == "step" or self.check_wait(bar, phase):
                    choices.append(("role", n, True))
                elif kind == "wait" and err[0]:
                    choices.append(("role", n, False))  # gives up at a poll of the error word
            choices += [("event", i, None) for i in range(len(self.events))]
            if self.mma_queue:
                choices.append(("mma", 0, None))
            dc = self.deliverable_commits()
            if dc:
                choices += [("commit", i, None) for i in range(1 if inorder_commits else len(dc))]
            if not choices:
                raise Hazard(f"deadlock: blocked {[(n, getattr(blocked[n][1], 'name', None), blocked[n][2]) for n in roles if n not in done]}")
            kind, i, val = self.rng.choice(choices)
            if kind == "role":
                resume(i, val)
            elif kind == "event":
                self.events.pop(i)()
            elif kind == "mma":
                self.complete_next_mma()
            else:
                bar, _ = dc[i]
                self.commits.remove(dc[i])
                bar.arrive()
        # nothing asynchronous may land after the CTA exits: every copy landed,
        # every MMA finished, every commit's arrival delivered
        assert not self.events, f"copies still to land at exit: {[e.barrier for e in self.events]}"
        assert not self.mma_queue, f"{len(self.mma_queue)} MMAs still running at exit"
        assert not self.commits, f"commits still to land at exit: {[c[0].name for c in self.commits]}"
        return err[0]


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
        rng = random.Random(_seed(name, inorder, seed))
        Model(ntiles=7, rng=rng, **cfg).run(inorder_commits=inorder)


@pytest.mark.parametrize("name", sorted(LAYOUTS))
def test_protocol_error_paths(name):
    """One role's wait gives up at a random point (its time limit); the others
    give up at later polls and drain: no deadlock, no hazard, and nothing
    asynchronous left to land after the CTA exits."""
    cfg = LAYOUTS[name]
    roles = ["E", "W", "MMA", "epi", "unpack0"] + (["unpack1", "fwd"] if cfg["groups"] > 1 else [])
    failed = 0
    for seed in range(150):
        rng = random.Random(_seed(name, "fail", seed))
        fail = (rng.choice(roles), rng.randint(1, 12))
        failed += Model(ntiles=5, rng=rng, **cfg).run(inorder_commits=bool(seed % 2), fail=fail)
    assert failed > 50  # most injections hit a wait that happened


def _planned_layouts(bflib):
    """Every ring layout the kernel's planner (bf_plan_rings) gives over the
    dish counts and pass widths it takes and the batch autotuner's three ring
    plans, with the dish counts that give each."""
    layouts = {}
    for D in (8, 64, 128, 192, 512, 1024, 2048):
        for nb in range(8, 97, 8):
            for wslots, raw in ((0, 0), (4, 8), (2, 12)):
                pl = bflib.plan_rings(D, nb, wslots, raw)
                assert pl is not None, (D, nb, wslots, raw)
                key = (pl["stages"], pl["wslots"], pl["raw"], pl["groups"])
                layouts.setdefault(key, set()).add(pl["nk"])
    return layouts


def test_every_planned_layout_passes_the_model(bflib):
    """The model over every layout the planner produces (not only the ones
    listed above), with 1, 2, 3 and 8 K stages per tile as well as the
    planner's own: random schedules with commits in and out of order, and
    injected failures."""
    layouts = _planned_layouts(bflib)
    assert len(layouts) >= 10
    for (S, SW, R, groups), nks in sorted(layouts.items()):
        assert groups == 1 or (R % 2 == 0 and S % 2 == 0 and SW <= S), (S, SW, R, groups)  # two-group rules
        roles = ["E", "W", "MMA", "epi", "unpack0"] + (["unpack1", "fwd"] if groups > 1 else [])
        for nk in sorted(set(nks) | {1, 2, 3, 8}):
            cfg = dict(S=S, SW=SW, R=R, groups=groups, nk=min(nk, 8))
            for seed in range(12):
                rng = random.Random(_seed(S, SW, R, groups, nk, seed))
                Model(ntiles=5, rng=rng, **cfg).run(inorder_commits=bool(seed % 2))
                fail = (rng.choice(roles), rng.randint(1, 12))
                Model(ntiles=5, rng=rng, **cfg).run(inorder_commits=bool(seed % 2), fail=fail)


SMEM_PER_SM = 233472  # 228 KiB of shared memory per SM
SMEM_PER_CTA = 232448  # 227 KiB opt-in per block
SMEM_RESERVED_PER_CTA = 1024
TMEM_COLS_PER_SM = 512


def test_every_planned_layout_fits_the_hardware(bflib):
    """Every layout the planner gives stays inside the SM: shared memory per
    CTA and per SM (two CTAs in the half-SM layout), a tensor-memory
    allocation of a power of two >= 32 columns whose CTAs fit the SM's 512,
    and unpacked stages whose columns overlap neither accumulator nor each
    other."""
    for D in (8, 64, 128, 192, 512, 1024, 2048):
        for nb in range(8, 97, 8):
            for wslots, raw in ((0, 0), (4, 8), (2, 12), (6, 16), (2, 2)):
                pl = bflib.plan_rings(D, nb, wslots, raw)
                if pl is None:
                    continue
                what = (D, nb, wslots, raw, pl)
                n = pl["ctas_per_sm"]
                assert pl["smem_bytes"] <= SMEM_PER_CTA, what
                assert n * (pl["smem_bytes"] + SMEM_RESERVED_PER_CTA) <= SMEM_PER_SM, what
                cols = pl["tmem_cols"]
                assert cols >= 32 and cols & (cols - 1) == 0 and n * cols <= TMEM_COLS_PER_SM, what
                acc, acc2, per = pl["acc_cols"], pl["acc2_col"], pl["stages_per_acc"]
                assert acc == 2 * nb and acc <= acc2 and acc2 + acc <= cols, what
                used = [(0, acc), (acc2, acc2 + acc)]
                for i in range(pl["stages"]):
                    c0 = acc + 64 * i if i < per else acc2 + acc + 64 * (i - per)
                    used.append((c0, c0 + 64))
                used.sort()
                assert all(a[1] <= b[0] for a, b in zip(used, used[1:])), what  # no overlap
                assert used[-1][1] <= cols and used[-1][1] >= pl["stage_end_col"], what
                assert pl["stages"] >= 2 and pl["wslots"] >= 2 and pl["raw"] >= 2, what


def test_planner_refuses_passes_it_cannot_hold(bflib):
    assert bflib.plan_rings(512, 104) is None  # wider than 96 beams: no TMEM room for two stages
    assert bflib.plan_rings(4096, 96) is None  # beyond the kernel's 2048 dishes
    assert bflib.plan_rings(512, 16)["ctas_per_sm"] == 2
    assert bflib.plan_rings(512, 96)["groups"] == 1
    assert bflib.plan_rings(512, 64)["groups"] == 2


@pytest.mark.parametrize("S,SW,R", [(4, 4, 4), (4, 2, 8), (4, 4, 8), (6, 4, 6)])
def test_one_accumulator_candidate_layout(S, SW, R):
    """The candidate b=96 layout (one accumulator released right after the
    epilogue reads it, four stages, two unpack groups and the W forwarder):
    no hazard, deadlock or alias under random schedules and injected
    failures, before any of it is built."""
    roles = ["E", "W", "MMA", "epi", "unpack0", "unpack1", "fwd"]
    for seed in range(60):
        rng = random.Random(_seed("one acc", S, SW, R, seed))
        cfg = dict(S=S, SW=SW, R=R, groups=2, nk=4, naccs=1)
        Model(ntiles=6, rng=rng, **cfg).run(inorder_commits=bool(seed % 2))
        Model(ntiles=6, rng=rng, **cfg).run(fail=(rng.choice(roles), rng.randint(1, 12)))


def test_protocol_model_finds_odd_stage_rings_with_two_groups():
    """Stage slot k % S serves sequences k and k + S; with an odd S they
    belong to different unpack groups, and the group with k + S can pass its
    `empty` parity wait one phase early, as with an odd raw ring.  The
    planner's stage counts are even (two per accumulator times the stages
    beside each); the one-accumulator candidate must keep S even too (four
    stages at b=96, not the five its TMEM would hold)."""
    for seed in range(300):  # found only when commit arrivals may land out of order (undocumented either way)
        try:
            Model(ntiles=6, rng=random.Random(seed), S=5, SW=4, R=6, groups=2, nk=4, naccs=1).run(
                inorder_commits=False)
        except Hazard as e:
            assert "empty" in str(e)
            return
    raise AssertionError("the odd stage ring was not found")


def test_protocol_model_finds_an_accumulator_overwritten_before_it_is_read():
    """With the MMA thread not waiting for accempty, some schedule starts a
    tile on an accumulator the epilogue is still reading."""
    for seed in range(200):
        m = Model(ntiles=6, rng=random.Random(seed), **LAYOUTS["b64 two groups"])
        m.mma_skips_accempty = True
        try:
            m.run()
        except Hazard as e:
            assert "before the epilogue has read" in str(e)
            return
    raise AssertionError("the planted mistake was not found")


def test_protocol_model_finds_a_stage_signalled_before_its_stores_land():
    for seed in range(200):
        m = Model(ntiles=4, rng=random.Random(seed), **LAYOUTS["b64 two groups"])
        m.unpack_signals_early = True
        try:
            m.run()
        except Hazard as e:
            assert "stage" in str(e)
            return
    raise AssertionError("the planted mistake was not found")


def test_protocol_model_finds_producers_that_drain_only_on_own_errors():
    """With the producers draining only after an error of their own, some
    injected failure leaves a copy landing after the CTA exits."""
    found = False
    for seed in range(300):
        rng = random.Random(seed)
        fail = (rng.choice(["MMA", "unpack0", "unpack1", "fwd", "epi"]), rng.randint(1, 12))
        try:
            Model(ntiles=5, rng=rng, drain_always=False, **LAYOUTS["b32 two groups"]).run(fail=fail)
        except AssertionError as e:
            assert "still to land" in str(e)
            found = True
            break
    assert found


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
