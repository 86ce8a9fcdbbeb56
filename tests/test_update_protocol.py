"""The mbarrier protocol of the tensor-core residual update (k_update_tc in
sodabayes_gb300/csrc/update_tc.cuh), as a model run on the CPU.

The kernel's roles hand buffers to one another through mbarriers waited on by
phase parity: a wait for phase i returns as soon as the barrier's completed
phase count k has the other parity than i.  It is therefore sound only if it
is never asked while k <= i - 1 (it would return at once, a phase early) and
never when k >= i + 2 (a whole phase was missed).  Per unit s the producer
waits for its A slot (MMAs of s - NA) and its B slot (MMAs of s - NOB), loads
A, and for an ra unit loads B by TMA (fullb completes on arrival) or for a
row unit arrives on fullb at once; the converters wait on fullb, widen the
codes of a row unit into B, and arrive on conv; the MMA thread waits on conv
and fulla and commits to opfree and emptya.  The model runs the roles and
the asynchronous completions (TMA arrival, MMA commit) under random
interleavings, with the slot counts read from the kernel's source, and
checks that every wait that returns has exactly its phase completed and that
no buffer is written while a reader of its previous contents is pending, for
random mixes of row units and ra units.  The mistake planted in the model,
a producer that waits for the B slot only before ra units, is harmless when
NA == NOB (the A-slot wait implies it) and must be caught with more A slots."""
import os
import random
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "sodabayes_gb300", "csrc", "update_tc.cuh")


def _consts():
    txt = open(SRC).read()
    out = {}
    for name in ("TV_NA", "TV_NOB"):
        m = re.search(r"constexpr int %s = (\d+);" % name, txt)
        assert m, name
        out[name] = int(m.group(1))
    # the producer waits for the B slot before every unit, row or ra
    out["bwait_all"] = "if (ok && s >= TV_NOB) ok = tc::mbar_wait(&s_opfree[ob]" in txt
    return out


class Unsound(AssertionError):
    pass


class Bar:
    def __init__(self):
        self.k = 0   # completed phases

    def ready(self, i):
        """try_wait.parity for phase i: true when k has the other parity than i.  With k >= i + 2 the
        waiter has missed a whole phase (on the GPU it would wait until its bounded wait gives up)."""
        if self.k >= i + 2:
            raise Unsound("parity wait for phase %d asked with %d phases complete" % (i, self.k))
        ok = (self.k & 1) != (i & 1)
        if ok and self.k != i + 1:
            raise Unsound("parity wait for phase %d returned with %d phases complete" % (i, self.k))
        return ok


def run(kinds, NA, NOB, bwait_all, seed):
    rnd = random.Random(seed)
    nu = len(kinds)
    fulla = [Bar() for _ in range(NA)]
    emptya = [Bar() for _ in range(NA)]
    fullb = [Bar() for _ in range(NOB)]
    conv = [Bar() for _ in range(NOB)]
    opfree = [Bar() for _ in range(NOB)]
    a_owner = [None] * NA        # unit whose A tile is in the slot, until its MMAs complete
    b_owner = [None] * NOB       # unit whose B operand is in the buffer, until its MMAs complete
    mma_done = set()
    landed_a, landed_b = set(), set()

    def write_a(s):
        a = s % NA
        if a_owner[a] is not None and a_owner[a] not in mma_done:
            raise Unsound("A slot %d overwritten by unit %d while unit %d's MMAs read it" % (a, s, a_owner[a]))
        a_owner[a] = s

    def write_b(s):
        ob = s % NOB
        if b_owner[ob] is not None and b_owner[ob] not in mma_done:
            raise Unsound("B operand %d overwritten by unit %d while unit %d's MMAs read it" % (ob, s, b_owner[ob]))
        b_owner[ob] = s

    pending = []   # asynchronous completions: callables

    def producer():
        for s in range(nu):
            a, ob = s % NA, s % NOB
            if s >= NA:
                yield emptya[a], s // NA - 1
            if s >= NOB and (bwait_all or kinds[s] == 1):
                yield opfree[ob], (s - NOB) // NOB
            write_a(s)

            def land_a(s=s, a=a):
                landed_a.add(s)
                fulla[a].k += 1
            pending.append(land_a)
            if kinds[s] == 1:
                write_b(s)   # TMA writes the B operand of an ra unit

                def land_b(s=s, ob=ob):
                    landed_b.add(s)
                    fullb[ob].k += 1
                pending.append(land_b)
            else:
                fullb[ob].k += 1   # the slot is the converters' to write

    def converter():
        for s in range(nu):
            ob = s % NOB
            yield fullb[ob], s // NOB
            if kinds[s] == 0:
                write_b(s)   # widened codes into the B operand
                landed_b.add(s)
            conv[ob].k += 1

    def mma():
        for s in range(nu):
            a, ob = s % NA, s % NOB
            yield conv[ob], s // NOB
            yield fulla[a], s // NA
            if s not in landed_a or s not in landed_b:
                raise Unsound("the MMAs of unit %d read an operand still in flight" % s)

            def commit(s=s, a=a, ob=ob):
                mma_done.add(s)
                opfree[ob].k += 1
                emptya[a].k += 1
            pending.append(commit)

    roles = [producer(), converter(), mma()]
    waits = [next(r, None) for r in roles]
    steps = 0
    while any(w is not None for w in waits) or pending:
        steps += 1
        assert steps < 100000
        choices = [("async", j) for j in range(len(pending))]
        for i, w in enumerate(waits):
            if w is not None and w[0].ready(w[1]):
                choices.append(("role", i))
        if not choices:
            raise AssertionError("deadlock")
        kind, j = rnd.choice(choices)
        if kind == "async":
            pending.pop(j)()
        else:
            waits[j] = next(roles[j], None)


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
    assert c["bwait_all"], "the producer's wait for the B slot before every unit is missing from update_tc.cuh"
    rnd = random.Random(7)
    for t, kinds in enumerate(_mixes(rnd, 300)):
        run(kinds, c["TV_NA"], c["TV_NOB"], True, seed=t)


def test_update_protocol_model_catches_a_missing_wait():
    """Six A slots: sound with the B-slot wait before every unit, caught when
    the producer waits for the B slot only before ra units."""
    c = _consts()
    rnd = random.Random(11)
    mixes = list(_mixes(rnd, 300))
    for t, kinds in enumerate(mixes):
        run(kinds, 6, c["TV_NOB"], True, seed=t)
    caught = 0
    for t, kinds in enumerate(mixes):
        try:
            run(kinds, 6, c["TV_NOB"], False, seed=t)
        except Unsound:
            caught += 1
    assert caught > 0
