"""The mbarrier protocol of the tensor-core residual update (k_update_tc in
sodabayes_gb300/csrc/update_tc.cuh), as a model run on the CPU.

The kernel's roles hand buffers to one another through mbarriers waited on by
phase parity: a wait for phase i returns as soon as the barrier's completed
phase count k has the other parity than i.  It is therefore sound only if it
is never asked while k <= i - 1: it would return at once, a phase early.
The model runs the producer (TMA issue), the converters, the MMA issuer and
the asynchronous completions (TMA arrival, MMA commit) under random
interleavings, with the slot counts read from the kernel's source, and checks
that

  * every wait that returns has its phase really completed, and
  * no buffer is written while a reader of its previous contents is pending
    (A slots, code slots and the two B operands),

for random mixes of row units (codes converted into B) and ra units (B
loaded by TMA).  A variant with more A slots than 2 x NOB and without the
producer's extra wait (the mistake planted in the model) must be caught."""
import os
import random
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "sodabayes_gb300", "csrc", "update_tc.cuh")


def _consts():
    txt = open(SRC).read()
    out = {}
    for name in ("TV_NA", "TV_NC", "TV_NOB"):
        m = re.search(r"constexpr int %s = (\d+);" % name, txt)
        assert m, name
        out[name] = int(m.group(1))
    # the producer's extra wait before an ra unit's B operand is part of the protocol
    out["guard"] = "TV_NA > 2 * TV_NOB && s >= 2 * TV_NOB" in txt
    return out


class Unsound(AssertionError):
    pass


class Bar:
    def __init__(self):
        self.k = 0   # completed phases

    def ready(self, i):
        """try_wait.parity for phase i: true when k has the other parity than i."""
        ok = (self.k & 1) != (i & 1)
        if ok and self.k < i + 1:
            raise Unsound("parity wait for phase %d returned with %d phases complete" % (i, self.k))
        return ok


def run(kinds, NA, NC, NOB, guard, seed):
    rnd = random.Random(seed)
    nu = len(kinds)
    fulla = [Bar() for _ in range(NA)]
    emptya = [Bar() for _ in range(NA)]
    fullc = [Bar() for _ in range(NC)]
    emptyc = [Bar() for _ in range(NC)]
    conv = [Bar() for _ in range(NOB)]
    opfree = [Bar() for _ in range(NOB)]
    # buffer occupancy: which unit's data a slot holds and whether its reader finished
    a_owner = [None] * NA        # unit whose A tile is in the slot, until its MMAs complete
    c_owner = [None] * NC        # unit whose codes are in the slot, until converted
    b_owner = [None] * NOB       # unit whose B operand is in the buffer, until its MMAs complete
    mma_done = set()
    conv_done = set()

    def write_a(s):
        a = s % NA
        if a_owner[a] is not None and a_owner[a] not in mma_done:
            raise Unsound("A slot %d overwritten by unit %d while unit %d's MMAs read it" % (a, s, a_owner[a]))
        a_owner[a] = s

    def write_c(s):
        c = s % NC
        if c_owner[c] is not None and c_owner[c] not in conv_done:
            raise Unsound("code slot %d overwritten by unit %d before unit %d was converted" % (c, s, c_owner[c]))
        c_owner[c] = s

    def write_b(s):
        ob = s % NOB
        if b_owner[ob] is not None and b_owner[ob] not in mma_done:
            raise Unsound("B operand %d overwritten by unit %d while unit %d's MMAs read it" % (ob, s, b_owner[ob]))
        b_owner[ob] = s

    # each role is a generator that yields the (barrier, phase) it waits for next and acts in between
    pending = []   # asynchronous completions: callables

    def producer():
        for s in range(nu):
            a, cb, ob = s % NA, s % NC, s % NOB
            if s >= NA:
                yield emptya[a], s // NA - 1
            if s >= NC:
                yield emptyc[cb], s // NC - 1
            if kinds[s] == 1 and s >= NOB:
                if guard and NA > 2 * NOB and s >= 2 * NOB:
                    yield emptya[(s - 2 * NOB) % NA], (s - 2 * NOB) // NA
                yield opfree[ob], (s - NOB) // NOB
            write_a(s)
            pending.append(lambda a=a: setattr(fulla[a], "k", fulla[a].k + 1))
            if kinds[s] == 0:
                write_c(s)
            else:
                write_b(s)   # TMA writes the B operand of an ra unit
            pending.append(lambda cb=cb: setattr(fullc[cb], "k", fullc[cb].k + 1))

    def converter():
        for s in range(nu):
            cb, ob = s % NC, s % NOB
            yield fullc[cb], s // NC
            if kinds[s] == 0:
                if s >= NOB:
                    yield opfree[ob], (s - NOB) // NOB
                write_b(s)   # widened codes into the B operand
            conv_done.add(s)
            emptyc[cb].k += 1
            conv[ob].k += 1

    def mma():
        for s in range(nu):
            a, ob = s % NA, s % NOB
            yield conv[ob], s // NOB
            yield fulla[a], s // NA

            def commit(s=s, a=a, ob=ob):
                mma_done.add(s)
                opfree[ob].k += 1
                emptya[a].k += 1
            pending.append(commit)

    roles = [producer(), converter(), mma()]
    waits = [None, None, None]
    alive = [True, True, True]
    for i in range(3):
        waits[i] = next(roles[i], None)
        alive[i] = waits[i] is not None
    steps = 0
    while any(alive) or pending:
        steps += 1
        assert steps < 100000
        choices = [("async", j) for j in range(len(pending))]
        for i in range(3):
            if alive[i]:
                bar, ph = waits[i]
                if bar.ready(ph):
                    choices.append(("role", i))
        if not choices:
            raise AssertionError("deadlock")
        kind, j = rnd.choice(choices)
        if kind == "async":
            pending.pop(j)()
        else:
            w = next(roles[j], None)
            waits[j] = w
            alive[j] = w is not None


def _mixes(rnd, n):
    for _ in range(n):
        nu = rnd.randint(1, 40)
        split = rnd.randint(0, nu)
        # row units first, then ra units (the kernel's unit order), or a random mix
        if rnd.random() < 0.5:
            yield [0] * split + [1] * (nu - split)
        else:
            yield [rnd.randint(0, 1) for _ in range(nu)]


def test_update_protocol_is_sound():
    c = _consts()
    rnd = random.Random(7)
    for t, kinds in enumerate(_mixes(rnd, 300)):
        run(kinds, c["TV_NA"], c["TV_NC"], c["TV_NOB"], c["guard"], seed=t)


def test_update_protocol_more_a_slots_needs_the_guard():
    """Six A and code slots: sound with the producer's extra wait, caught without it."""
    c = _consts()
    assert c["guard"], "the producer's extra wait is missing from update_tc.cuh"
    rnd = random.Random(11)
    mixes = list(_mixes(rnd, 300))
    for t, kinds in enumerate(mixes):
        run(kinds, 6, 6, c["TV_NOB"], True, seed=t)
    caught = 0
    for t, kinds in enumerate(mixes):
        try:
            run(kinds, 6, 6, c["TV_NOB"], False, seed=t)
        except Unsound:
            caught += 1
    assert caught > 0
