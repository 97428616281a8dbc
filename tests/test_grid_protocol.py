"""CPU models of the grid kernel's step protocols (tv_grid.cuh): the head
CTA (grid_head), the worker pipeline (grid_worker) and the tagged message
rings between them (further down this file).

The head CTA runs five roles that meet at named non-aligned barriers:
  * critical lanes: the matvec of slot t-1, then the dense phase of delta[t];
  * upper-half matvec warps: hand their half over at a pair barrier;
  * two state-helper groups: group g prepares step t+1 for the steps t of
    parity g (short candidates after slot t-2, partials after PW, d = 1
    after slot t-1), then stores step t-1's results;
  * intake: worker partials, the emission prefix, window-sum copies three
    steps ahead, the coarse base.

The model runs each role as two actors (warp subsets) under random
interleavings.  A barrier counts arrivals and completes a generation when the
count is reached; a sync blocks until its generation completes.  Every shared
buffer carries the step whose value it holds; every read checks that it sees
the step it needs and that no asynchronous copy into it is in flight.  The
checks: no deadlock, no barrier over-arrival or count mismatch, no stale or
torn read, every barrier left empty, and after an injected intake failure
all roles leave the step loops at the same step (the kernel's exit protocol
through the two flag words s_fb).

The model is test infrastructure: it restates the kernel's ordering argument
so that a change to the protocol can be checked here before it runs on a GPU.
"""
from __future__ import annotations

import random

import pytest

L = 8

# barrier ids as in tv_grid.cuh
STEP, SLOT0, PW0, SLOT1, PW1, PRE0, PRE1, END, PAIR0 = 1, 2, 4, 5, 6, 7, 8, 9, 10


def SLOT(g):
    return SLOT1 if g else SLOT0


def PW(g):
    return PW1 if g else PW0


def PRE(g):
    return PRE1 if g else PRE0


class _Deadlock(Exception):
    pass


class _Bar:
    def __init__(self):
        self.count, self.expect, self.gen = 0, None, 0


def run_protocol(T, D, fail_at, seed, mutate=None):
    """Run one interleaving; return the list of violations found."""
    rnd = random.Random(seed)
    cs = st = inn = 4          # threads per role (two actors of 2)
    nthr = 2 * cs + 2 * st + inn
    bars, mem, inflight, errs, exits = {}, {}, set(), [], {}
    s_fb = [0, 0]

    def bar(i):
        return bars.setdefault(i, _Bar())

    def W(key, ver):
        mem[key] = ver

    def R(who, key, ver):
        if key in inflight:
            errs.append(f"{who}: read {key} while a copy into it is in flight")
        elif mem.get(key) != ver:
            errs.append(f"{who}: read {key} holds step {mem.get(key)}, needs {ver}")

    def arrive(i, n, cnt):
        b = bar(i)
        if b.expect is None:
            b.expect = cnt
        elif b.expect != cnt:
            errs.append(f"barrier {i}: count {cnt} against {b.expect}")
        b.count += n
        if b.count > b.expect:
            errs.append(f"barrier {i}: over-arrival")
        if b.count >= b.expect:
            b.count, b.expect, b.gen = 0, None, b.gen + 1
        return ("go",)

    def sync(i, n, cnt):
        g0 = bar(i).gen
        arrive(i, n, cnt)
        return ("wait", i, g0)

    # set-up (all threads, before the first CTA-wide barrier)
    W(("ptil", 0), 0)
    if T > 1:
        W(("ptil", 1), 1)
    for r in range(4):
        if r < T:
            W(("hwr", r), r)
    W(("dstar", 0), 0)
    W(("dq", 0), 0)
    W(("dqcp", 0), 0)
    W(("base", 0), 0)
    W(("base", 1), 1)
    if T > 1:
        W(("pw", 1), 1)
    W(("pre", 1), 1)

    def critical(name, n, k):
        for t in range(1, T):
            cur, prv = t & 1, (t & 1) ^ 1
            R(name, ("dqcp", prv), t - 1)
            R(name, ("ptil", (t - 1) & 3), t - 1)
            if mutate != "no_pair":
                yield sync(PAIR0 + k, n, 2 * n)
            R(name, ("xch", k), t)
            W(("slot", (t - 1) & 7), t - 1)
            yield arrive(SLOT(cur), n, cs + 2 * st if t + 1 < T else cs + st)
            if t >= 2 and mutate != "no_pre":
                yield sync(PRE(prv), n, cs + st)
            R(name, ("pre", cur), t)
            R(name, ("hwr", t & 3), t)
            R(name, ("dstar", (t - 1) % (L + 1)), t - 1)
            R(name, ("base", cur), t)
            W(("dstar", t % (L + 1)), t)
            W(("dq", cur), t)
            W(("dqcp", cur), t)
            W(("psirec", t & 3), t)
            yield sync(STEP, n, 2 * cs + inn)
            if s_fb[cur]:
                exits[name] = t
                break
        yield sync(END, n, nthr)
        yield ("done",)

    def upper_half(name, n, k):
        for t in range(1, T):
            cur, prv = t & 1, (t & 1) ^ 1
            R(name, ("dqcp", prv), t - 1)
            W(("xch", k), t)
            yield arrive(PAIR0 + k, n, 2 * n)
            yield sync(STEP, n, 2 * cs + inn)
            if s_fb[cur]:
                exits[name] = t
                break
        yield sync(END, n, nthr)
        yield ("done",)

    def helper(name, n, g):
        t = 1 if g else 2
        while t < T:
            t1 = t + 1
            nxt = t1 < T
            hl1 = min(t1, D, L)
            own = cs + 2 * st if nxt else cs + st
            if t >= 2 and mutate != "no_early_slot":
                yield sync(SLOT((t - 1) & 1), n, cs + 2 * st)
            if nxt:
                for d in range(2, hl1):
                    R(name, ("slot", (t - d) & 7), t - d)
            yield sync(PW(g), n, st + inn)
            fb = s_fb[g]
            if fb == 2:
                exits[name] = t
                break
            if fb == 1:
                yield sync(SLOT(g), n, own)
                exits[name] = t
                break
            if nxt:
                R(name, ("ptil", t1 & 3), t1)
                R(name, ("pw", t1 & 1), t1)
                R(name, ("hwr", t1 & 3), t1)
                for d in range(2, hl1):
                    R(name, ("dstar", (t - d) % (L + 1)), t - d)
            yield sync(SLOT(g), n, own)
            if nxt:
                if hl1 > 1:
                    R(name, ("slot", (t - 1) & 7), t - 1)
                    R(name, ("dstar", (t - 1) % (L + 1)), t - 1)
                    R(name, ("hwr", t1 & 3), t1)
                W(("pre", t1 & 1), t1)
                yield arrive(PRE(g), n, cs + st)
            R(name, ("slot", (t - 1) & 7), t - 1)
            R(name, ("dstar", (t - 1) % (L + 1)), t - 1)
            if t >= 2:
                R(name, ("psirec", (t - 1) & 3), t - 1)
            t += 2
        yield sync(END, n, nthr)
        yield ("done",)

    def intake(name, n, fails):
        pending = []  # the window-sum copy in flight
        for t in range(1, T):
            t1 = t + 1
            nxt = t1 < T
            cur, prv = t & 1, (t & 1) ^ 1
            if nxt:
                if fails and t == fail_at:
                    s_fb[cur] = 1
                W(("pw", t1 & 1), t1)
                R(name, ("ptil", t & 3), t)
                W(("ptil", t1 & 3), t1)
            if mutate != "no_copy_wait":
                while pending:  # the copy issued at the previous step is complete before PW
                    key, v = pending.pop()
                    inflight.discard(key)
                    W(key, v)
            yield arrive(PW(cur), n, st + inn)
            if t + 3 < T:
                key = ("hwr", (t + 3) & 3)
                inflight.add(key)
                pending.append((key, t + 3))
            R(name, ("dq", prv), t - 1)
            W(("base", cur ^ 1), t1)
            yield sync(STEP, n, 2 * cs + inn)
            if s_fb[cur]:
                s_fb[prv] = 2
                yield arrive(PW(prv), n, st + inn)
                exits[name] = t
                break
        for key, v in pending:
            inflight.discard(key)
            W(key, v)
        yield sync(END, n, nthr)
        yield ("done",)

    actors = {
        "crit0": critical("crit0", cs // 2, 0), "crit1": critical("crit1", cs // 2, 1),
        "upper0": upper_half("upper0", cs // 2, 0), "upper1": upper_half("upper1", cs // 2, 1),
        "g0a": helper("g0a", st // 2, 0), "g0b": helper("g0b", st // 2, 0),
        "g1a": helper("g1a", st // 2, 1), "g1b": helper("g1b", st // 2, 1),
        "in_a": intake("in_a", inn // 2, True), "in_b": intake("in_b", inn // 2, False),
    }
    waiting = {k: None for k in actors}
    done = set()
    for _ in range(10 ** 6):
        if len(done) == len(actors):
            break
        ready = [k for k in actors if k not in done and
                 (waiting[k] is None or bars[waiting[k][1]].gen > waiting[k][2])]
        if not ready:
            raise _Deadlock(", ".join(f"{k} at barrier {waiting[k][1]}" for k in actors if k not in done))
        k = rnd.choice(ready)
        waiting[k] = None
        op = next(actors[k])
        if op[0] == "wait":
            waiting[k] = op
        elif op[0] == "done":
            done.add(k)
    else:
        raise _Deadlock("no progress")
    loop_roles = ("crit0", "crit1", "upper0", "upper1", "in_a", "in_b")
    if fail_at is not None and fail_at + 1 < T:
        for k in loop_roles:
            if exits.get(k) != fail_at:
                errs.append(f"{k} left the loops at step {exits.get(k)}, not at the failed step {fail_at}")
    elif exits:
        errs.append(f"unexpected early exits {exits}")
    for i, b in bars.items():
        if b.count:
            errs.append(f"barrier {i} left with {b.count} arrivals")
    return errs


def _violations(T, D, fail_at, seeds, mutate=None):
    out = []
    for seed in seeds:
        try:
            out += run_protocol(T, D, fail_at, seed, mutate)
        except _Deadlock as e:
            out.append(f"deadlock: {e}")
    return out


@pytest.mark.parametrize("T", [1, 2, 3, 4, 5, 7, 10, 13, 40])
@pytest.mark.parametrize("D", [1, 2, 3, 9, 20])
def test_head_protocol_runs_clean(T, D):
    """Every interleaving completes with fresh reads and empty barriers."""
    assert _violations(T, D, None, range(12)) == []


@pytest.mark.parametrize("T", [3, 6, 13])
def test_head_protocol_intake_failure_exits_every_role_at_the_same_step(T):
    for fail_at in range(1, T):
        assert _violations(T, 9, fail_at, range(8)) == [], fail_at


@pytest.mark.parametrize("mutate", ["no_pair", "no_pre", "no_early_slot", "no_copy_wait"])
def test_head_protocol_model_detects_a_missing_wait(mutate):
    """The model has teeth: dropping any one wait of the protocol is caught."""
    found = _violations(13, 20, None, range(12), mutate) + _violations(5, 3, None, range(12), mutate)
    assert found


# ---------------------------------------------------------------------------
# Worker CTA (tv_grid.cuh, grid_worker): scan threads, a certify warp and an
# intake warp meet at one CTA barrier per step (worker_sync_all) and a last
# one after the loops.  During the scan of step t+1 the certify warp serves
# step t (scan results by step parity, window sums E_t of three buffers) and
# the intake warp loads the slot that enters the scan at step t+2.
# ---------------------------------------------------------------------------

def run_worker_protocol(T, D, fail_at, seed, mutate=None):
    rnd = random.Random(seed)
    bars, mem, errs, exits = {}, {}, [], {}
    s_bad = [0, 0]
    n_scan, n_serv = 4, 2
    total = n_scan + n_serv

    def bar(i):
        return bars.setdefault(i, _Bar())

    def W(key, ver):
        mem[key] = ver

    def R(who, key, ver):
        if mem.get(key) != ver:
            errs.append(f"{who}: read {key} holds step {mem.get(key)}, needs {ver}")

    def sync(i, n, cnt):
        b = bar(i)
        g0 = b.gen
        if b.expect is None:
            b.expect = cnt
        elif b.expect != cnt:
            errs.append(f"barrier {i}: count {cnt} against {b.expect}")
        b.count += n
        if b.count >= b.expect:
            b.count, b.expect, b.gen = 0, None, b.gen + 1
        return ("wait", i, g0)

    ALL = 2
    # set-up: window sums of step 1 in buffer 1 (t % 3), slots below L loaded
    # as they enter (none before step L+1 is scanned)
    W(("acc", 1), 1)

    def slot_ver(s):
        return ("slot", s % D)

    def scan(name, n):
        for t in range(1, T):
            tau = min(t, D)
            # cells of d in [L, tau): slots t-1-d
            for d in range(L, tau):
                R(name, slot_ver(t - 1 - d), t - 1 - d)
            R(name, ("acc", t % 3), t)
            if t + 1 < T:
                W(("acc", (t + 1) % 3), t + 1)
            W(("red", t & 1), t)
            yield sync(ALL, n, total)
            if s_bad[(t - 1) & 1]:
                exits[name] = t
                break
        yield sync(ALL, n, total)
        yield ("done",)

    def certify(name, n):
        for t in range(1, T):
            yield sync(ALL, n, total)
            if s_bad[(t - 1) & 1]:
                exits[name] = t
                break
            R(name, ("red", t & 1), t)
            R(name, ("acc", t % 3), t)
            tau = min(t, D)
            for d in range(L, tau):
                R(name, slot_ver(t - 1 - d), t - 1 - d)
            if fail_at == t:
                s_bad[t & 1] = 1
        yield sync(ALL, n, total)
        yield ("done",)

    def intake(name, n):
        for t in range(1, T):
            yield sync(ALL, n, total)
            if s_bad[(t - 1) & 1]:
                exits[name] = t
                break
            # the slot that enters the scan at step t+2 (one step ahead of
            # its first use, so the scan of step t+1 may run meanwhile)
            sp = t + 1 - L if mutate != "late_slot" else t - L
            if t + 2 < T and sp >= 0:
                W(slot_ver(sp), sp)
        yield sync(ALL, n, total)
        yield ("done",)

    actors = {"scan_a": scan("scan_a", n_scan // 2), "scan_b": scan("scan_b", n_scan // 2),
              "certify": certify("certify", 1), "intake": intake("intake", 1)}
    waiting = {k: None for k in actors}
    done = set()
    for _ in range(10 ** 6):
        if len(done) == len(actors):
            break
        ready = [k for k in actors if k not in done and
                 (waiting[k] is None or bars[waiting[k][1]].gen > waiting[k][2])]
        if not ready:
            raise _Deadlock(", ".join(k for k in actors if k not in done))
        k = rnd.choice(ready)
        waiting[k] = None
        op = next(actors[k])
        if op[0] == "wait":
            waiting[k] = op
        elif op[0] == "done":
            done.add(k)
    if fail_at is not None and fail_at + 1 < T:
        left = {exits.get(k) for k in actors}
        if len(left) != 1 or left.pop() != fail_at + 1:
            errs.append(f"roles left at different steps: {exits}")
    for i, b in bars.items():
        if b.count:
            errs.append(f"barrier {i} left with {b.count} arrivals")
    return errs


def _worker_violations(T, D, fail_at, seeds, mutate=None):
    out = []
    for seed in seeds:
        try:
            out += run_worker_protocol(T, D, fail_at, seed, mutate)
        except _Deadlock as e:
            out.append(f"deadlock: {e}")
    return out


@pytest.mark.parametrize("T", [1, 2, 9, 12, 30])
@pytest.mark.parametrize("D", [9, 10, 16, 25])
def test_worker_pipeline_runs_clean(T, D):
    """Scan, certify and intake overlap without a stale read of the window
    sums, the scan results or a slot, for any interleaving."""
    assert _worker_violations(T, D, None, range(10)) == []


@pytest.mark.parametrize("T", [6, 20])
def test_worker_pipeline_failure_exits_every_role_at_the_same_step(T):
    for fail_at in range(1, T - 1):
        assert _worker_violations(T, 10, fail_at, range(6)) == [], fail_at


def test_worker_pipeline_model_detects_a_slot_loaded_too_late():
    """The model has teeth: an intake that loads, during the scan of step
    t+1, the slot that scan already needs is caught as a stale read."""
    assert _worker_violations(30, 12, None, range(10), mutate="late_slot")


# ---------------------------------------------------------------------------
# Messages between the head and the workers (tv_grid.cuh): three tagged rings
# in global memory, read by polling for the expected tag.
#   partials   worker -> head, PART_RING rows: the worker's winners of step t
#              (tag t), taken in by the head during its step t-1;
#   slots      head -> workers, SLOT_RING rows: slot s (tag s+1), sent once the
#              head has finished step s+1, taken in by a worker at iteration
#              s+L-1 for its scan of step s+L+1;
#   exact delta head -> workers, D + 2L + 8 rows: delta[s] (tag s+1), read by a
#              worker's certification at step t for s in [t-D, t-1-L].
# A poll that finds a newer tag than it waits for would wait until its time
# limit: the model reports that as an overrun, and a writer that replaces a
# partial the head has not taken in yet as lost.
# ---------------------------------------------------------------------------

PART_RING, SLOT_RING = 32, 64


def run_message_protocol(T, D, n_workers, seed, part_ring=PART_RING, slot_ring=SLOT_RING, rd_extra=2 * L + 8):
    rnd = random.Random(seed)
    PART, SLOTS = part_ring, slot_ring
    Rd = D + rd_extra
    part = [[None] * PART for _ in range(n_workers)]   # tag per row, per worker
    slot = [None] * SLOTS
    dstar = [None] * Rd
    errs = []
    # set-up: delta[0] (tag 1)
    dstar[0] = 1

    def poll(ring, row, tag, who):
        have = ring[row]
        if have is not None and have > tag:
            errs.append(f"{who}: row {row} already holds tag {have}, waited for {tag}")
            return True   # do not block: the error is recorded
        return have == tag

    def head():
        # set-up: the workers' partials of step 1 (no candidate d >= L yet)
        if T > 1:
            for w in range(n_workers):
                while not poll(part[w], 1, 1, "head set-up"):
                    yield
                part[w][1] = -1
        h = 1
        while h < T:
            # step h takes in every worker's partial of step h+1
            if h + 1 < T:
                for w in range(n_workers):
                    while not poll(part[w], (h + 1) % PART, h + 1, "head"):
                        yield
                    part[w][(h + 1) % PART] = -(h + 1)   # taken in
            # results of step h-1 (the helpers' stores after step h): slot h-1 and delta[h-1]
            if h >= 2:
                dstar[(h - 1) % Rd] = h
            slot[(h - 1) % SLOTS] = h
            h += 1
            yield
        # delta[T-2] is stored at the last step; the tail takes in step T's partials
        for w in range(n_workers):
            while not poll(part[w], T % PART, T, "head tail"):
                yield

    def worker(w):
        for t in range(1, T):
            tau = min(t, D)
            # certification of step t (after the scan of step t): exact deltas
            # of the candidates it may re-score
            for d in range(L, tau):
                s = t - 1 - d
                while not poll(dstar, s % Rd, s + 1, f"worker {w} re-score"):
                    yield
            # send the partial of step t, if its row was taken in
            row = t % PART
            old = part[w][row]
            if old is not None and old > 0:
                errs.append(f"worker {w}: partial tag {old} lost to tag {t}")
            part[w][row] = t
            # intake: slot t+1-L for the scan of step t+2
            sp = t + 1 - L
            if t + 2 < T and sp >= 0:
                while not poll(slot, sp % SLOTS, sp + 1, f"worker {w} slot"):
                    yield
            yield
        # tail (t = T-1): exact deltas of every candidate, then the tail partial
        t = T - 1
        for d in range(L, min(t, D)):
            s = t - 1 - d
            while not poll(dstar, s % Rd, s + 1, f"worker {w} tail"):
                yield
        part[w][T % PART] = T

    actors = {"head": head(), **{f"w{w}": worker(w) for w in range(n_workers)}}
    live = dict(actors)
    idle = 0
    while live:
        k = rnd.choice(list(live))
        try:
            next(live[k])
        except StopIteration:
            del live[k]
        idle += 1
        if idle > 200 * T * (n_workers + 1) * (D + 4):
            errs.append("no progress: " + ", ".join(live))
            break
    return errs


@pytest.mark.parametrize("T", [2, 9, 12, 40, 120])
@pytest.mark.parametrize("D", [9, 12, 30])
def test_message_rings_never_overrun(T, D):
    """With the rings' sizes, no poll finds a newer tag than it waits for, no
    partial is replaced before the head takes it in, and nobody waits for
    ever, whatever the relative speeds of the head and the workers."""
    for seed in range(6):
        assert run_message_protocol(T, D, 3, seed) == [], seed


@pytest.mark.parametrize("rings", [dict(part_ring=4), dict(slot_ring=4), dict(rd_extra=-2)])
def test_message_model_detects_rings_that_are_too_small(rings):
    """The model has teeth: a partial ring shorter than the workers' lead, a
    slot ring shorter than the head's, or an exact-delta ring shorter than D
    rows (the kernel keeps D + 2L + 8) is caught."""
    found = []
    for seed in range(12):
        found += run_message_protocol(60, 12, 3, seed, **rings)
    assert found
