"""A model of the tcgen05 apply kernel's barrier protocol (mrchem_gb300/csrc/mw_apply_tc05.cu),
checked under random interleavings on the CPU.

An mbarrier tells its phases apart by parity only: a thread waiting for the phase of parity p
succeeds while the barrier's current phase has the other parity.  A waiter that sleeps through
two completions therefore sees "not complete" and waits for a phase that may never come.  The
kernel's items of one row do not sync, so the issuing thread can run through several x passes
while the epilogue warps poll.  The model below runs the issuing thread and one epilogue warp of
one CTA over a node's items, with MMA completions that land after random delays and a scheduler
that may leave either thread unscheduled for many steps, and checks that

- with the epilogue warps waiting on their own barrier, committed once per row (the kernel's
  protocol), no schedule deadlocks;
- with the epilogue warps waiting on the per-item x barrier (the protocol it replaced), some
  schedules deadlock -- the model can see the race it guards against.
"""
import random


class Barrier:
    """Phase counter: completed phases 0..phase-1; a commit completes the current phase later."""

    def __init__(self):
        self.phase = 0
        self.pending = 0  # commits whose MMAs have not completed yet

    def complete_one(self):
        self.pending -= 1
        self.phase += 1

    def done(self, parity):
        return (self.phase & 1) != parity


def run(rows, per_row_barrier, rng, max_steps=20000):
    """rows: items per row of one node.  Returns True when both threads finish, False on deadlock."""
    bars = {b: Barrier() for b in (1, 2, 5)}
    items = []
    for n in rows:
        items += [j == n - 1 for j in range(n)]  # is the item the last of its row

    # each thread is a generator of actions: ("wait", b) or ("commit", b) or ("sync",)
    def producer():
        for last in items:
            yield ("commit", 1)              # x MMAs of the item
            if last and per_row_barrier:
                yield ("commit", 5)          # the row's x MMAs, for the epilogue warps
            yield ("wait", 1)                # S and the other B set are free again
            if last:
                yield ("sync",)              # x epilogue written
                yield ("commit", 2)          # y MMAs
                yield ("sync",)              # y epilogue written; z MMAs follow

    def epilogue():
        for last in items:
            if per_row_barrier:
                if last:
                    yield ("wait", 5)
            else:
                yield ("wait", 1)
            if last:
                yield ("sync",)
                yield ("wait", 2)
                yield ("sync",)

    threads = {"P": producer(), "E": epilogue()}
    parity = {("P", b): 0 for b in bars} | {("E", b): 0 for b in bars}
    current = {t: next(g) for t, g in threads.items()}
    for _ in range(max_steps):
        if all(a is None for a in current.values()):
            return True
        choices = []
        for b in bars.values():
            if b.pending:
                choices.append(("mma", b))
        for t, a in current.items():
            if a is None:
                continue
            if a[0] == "commit":
                choices.append(("run", t))
            elif a[0] == "wait":
                if bars[a[1]].done(parity[(t, a[1])]):
                    choices.append(("run", t))
            elif a[0] == "sync":
                others = [u for u in current if u != t and current[u] is not None]
                if all(current[u] == ("sync",) for u in others):
                    choices.append(("run", t))
        if not choices:
            return False
        # one move chosen uniformly among the threads and MMA completions able to move, so either
        # thread can be left unscheduled for many steps
        kind, x = rng.choice(choices)
        if kind == "mma":
            x.complete_one()
            continue
        t, a = x, current[x]
        if a[0] == "commit":
            bars[a[1]].pending += 1
        elif a[0] == "wait":
            parity[(t, a[1])] ^= 1
        elif a[0] == "sync":
            # every live thread passes the sync together
            for u in list(current):
                if current[u] == ("sync",):
                    current[u] = next(threads[u], None)
            continue
        current[t] = next(threads[t], None)
    return False


def schedules(n):
    rng = random.Random(20261204)
    for _ in range(n):
        rows = [rng.randint(1, 4) for _ in range(rng.randint(1, 6))]
        yield rows, random.Random(rng.getrandbits(32))


def test_per_row_barrier_never_deadlocks():
    for rows, rng in schedules(3000):
        assert run(rows, True, rng), rows


def test_per_item_barrier_can_deadlock():
    # the protocol that was replaced: the epilogue warps wait on the per-item barrier
    assert any(not run(rows, False, rng) for rows, rng in schedules(3000))
