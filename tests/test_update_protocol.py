"""The mbarrier protocol of the tensor-core residual update (k_update_tc in
sodabayes_gb300/csrc/update_tc.cuh), as a model run on the CPU.

The kernel's roles hand buffers to one another through mbarriers waited on by
phase parity: a wait for phase i returns as soon as the barrier's completed
phase count k has the other parity than i.  It is therefore sound only if it
is never asked while k <= i - 1 (it would return at once, a phase early) and
never when k >= i + 2 (a whole phase was missed).  A CTA's row units come
before its ra units; unit s uses operand slot s % NS.  A code loader streams
each row unit's packed codes into code slot s % NC (bulk copy; cfull
completes on arrival), waiting until every converter has read the slot's
previous unit (cfree).  The producer waits for
the slot (the MMAs of unit s - NS), loads A, and for an ra unit also loads B
by TMA (fullb completes on arrival); the converters, for row units only, wait
for the slot themselves, widen the codes into B and arrive on conv; the MMA
thread waits on conv (row unit) or on fullb (ra unit: phase = the slot's
earlier units less its row units) and on fulla, and commits once to free.
The model runs the roles and the asynchronous completions (TMA arrival, MMA
commit) under random interleavings, with the slot count read from the
kernel's source, and checks that every wait that returns has exactly its
phase completed and that no buffer is written while a reader of its previous
contents is pending.  Planted mistakes it must catch: converters that do not
wait for the slot, a code loader that does not wait for its slot, a fullb
phase that forgets the row units, and ra units placed before row units."""
import os
import random
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "sodabayes_gb300", "csrc", "update_tc.cuh")


def _consts():
    txt = open(SRC).read()
    m = re.search(r"constexpr int TV_NS = (\d+);", txt)
    assert m, "TV_NS"
    mc = re.search(r"constexpr int TV_NC = (\d+);", txt)
    assert mc, "TV_NC"
    return {
        "TV_NS": int(m.group(1)),
        "TV_NC": int(mc.group(1)),
        # the code loader waits until every converter has read the slot's previous unit
        "cfree_wait": "if (s >= TV_NC && !tc::mbar_wait(&s_cfree[cs], ((s / TV_NC) - 1) & 1)) {" in txt,
        # the converters wait for their unit's codes
        "cfull_wait": "bool ok = tc::mbar_wait(&s_cfull[cs], (s / TV_NC) & 1);" in txt,
        # the converters wait for the slot before writing B
        "conv_wait": "ok = s < TV_NS || tc::mbar_wait(&s_free[ob], ((s / TV_NS) - 1) & 1);" in txt,
        # the MMA thread's fullb phase discounts the slot's row units
        "ra_phase": "tc::mbar_wait(&s_fullb[sl], ra_phase(s, nrow) & 1)" in txt,
    }


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


def ra_phase(s, nrow, NS):
    sl = s % NS
    return s // NS - ((nrow - 1 - sl) // NS + 1 if nrow > sl else 0)


def run(kinds, NS, seed, conv_wait=True, naive_ra_phase=False, NC=6, cfree_wait=True):
    rnd = random.Random(seed)
    nu = len(kinds)
    nrow = 0
    while nrow < nu and kinds[nrow] == 0:
        nrow += 1
    fulla = [Bar() for _ in range(NS)]
    fullb = [Bar() for _ in range(NS)]
    conv = [Bar() for _ in range(NS)]
    free = [Bar() for _ in range(NS)]
    cfull = [Bar() for _ in range(NC)]
    cfree = [Bar() for _ in range(NC)]
    c_owner = [None] * NC        # unit whose packed codes are in the code slot, until the converters read them
    codes_read, landed_c = set(), set()
    a_owner = [None] * NS        # unit whose A tile is in the slot, until its MMAs complete
    b_owner = [None] * NS        # unit whose B operand is in the slot, until its MMAs complete
    mma_done = set()
    landed_a, landed_b = set(), set()

    def write(owner, s, what):
        sl = s % NS
        if owner[sl] is not None and owner[sl] not in mma_done:
            raise Unsound("%s slot %d overwritten by unit %d while unit %d's MMAs read it" % (what, sl, s, owner[sl]))
        owner[sl] = s

    pending = []   # asynchronous completions: callables

    def producer():
        for s in range(nu):
            sl = s % NS
            if s >= NS:
                yield free[sl], s // NS - 1
            write(a_owner, s, "A")

            def land_a(s=s, sl=sl):
                landed_a.add(s)
                fulla[sl].k += 1
            pending.append(land_a)
            if kinds[s] == 1:
                write(b_owner, s, "B")   # TMA writes the B operand of an ra unit

                def land_b(s=s, sl=sl):
                    landed_b.add(s)
                    fullb[sl].k += 1
                pending.append(land_b)

    def loader():
        for s in range(nrow):
            cs = s % NC
            if s >= NC and cfree_wait:
                yield cfree[cs], s // NC - 1
            if c_owner[cs] is not None and c_owner[cs] not in codes_read:
                raise Unsound("code slot %d overwritten by unit %d before unit %d was read" % (cs, s, c_owner[cs]))
            c_owner[cs] = s

            def land_c(s=s, cs=cs):
                landed_c.add(s)
                cfull[cs].k += 1
            pending.append(land_c)

    def converter():
        # the kernel's converters take the first nrow units as the row units
        for s in range(nrow):
            sl, cs = s % NS, s % NC
            yield cfull[cs], s // NC
            if s not in landed_c:
                raise Unsound("the converters read the codes of unit %d still in flight" % s)
            codes_read.add(s)
            cfree[cs].k += 1
            if s >= NS and conv_wait:
                yield free[sl], s // NS - 1
            write(b_owner, s, "B")   # widened codes into the B operand
            landed_b.add(s)
            conv[sl].k += 1

    def mma():
        for s in range(nu):
            sl = s % NS
            if s < nrow:
                yield conv[sl], s // NS
            else:
                yield fullb[sl], (s // NS if naive_ra_phase else ra_phase(s, nrow, NS))
            yield fulla[sl], s // NS
            if s not in landed_a or s not in landed_b:
                raise Unsound("the MMAs of unit %d read an operand still in flight" % s)

            def commit(s=s, sl=sl):
                mma_done.add(s)
                free[sl].k += 1
            pending.append(commit)

    roles = [producer(), loader(), converter(), mma()]
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


def _mixes(rnd, n, ordered=True):
    for _ in range(n):
        nu = rnd.randint(1, 40)
        split = rnd.randint(0, nu)
        if ordered:   # row units first, then ra units (the kernel's unit order)
            yield [0] * split + [1] * (nu - split)
        else:
            yield [rnd.randint(0, 1) for _ in range(nu)]


def _caught(mixes, NS, **kw):
    caught = 0
    for t, kinds in enumerate(mixes):
        try:
            run(kinds, NS, seed=t, NC=_consts()["TV_NC"], **kw)
        except (Unsound, AssertionError):
            caught += 1
    return caught


def test_update_protocol_is_sound():
    c = _consts()
    assert c["conv_wait"], "the converters' wait for the operand slot is missing from update_tc.cuh"
    assert c["ra_phase"], "the MMA thread's fullb phase (ra_phase) is missing from update_tc.cuh"
    assert c["cfree_wait"] and c["cfull_wait"], "the code ring's waits are missing from update_tc.cuh"
    rnd = random.Random(7)
    for t, kinds in enumerate(_mixes(rnd, 400)):
        run(kinds, c["TV_NS"], seed=t, NC=c["TV_NC"])


def test_update_protocol_model_catches_planted_mistakes():
    c = _consts()
    NS = c["TV_NS"]
    rnd = random.Random(11)
    mixes = list(_mixes(rnd, 300))
    assert _caught(mixes, NS) == 0
    # converters that write B without waiting for the slot
    assert _caught(mixes, NS, conv_wait=False) > 0
    # a code loader that refills a slot before the converters have read it
    assert _caught([k for k in mixes if k.count(0) > 8], NS, cfree_wait=False) > 0
    # a fullb phase that counts the slot's row units as ra uses
    assert _caught(mixes, NS, naive_ra_phase=True) > 0
    # ra units before row units: the kernel's converters and phases assume the opposite
    rnd = random.Random(13)
    shuffled = [k for k in _mixes(rnd, 300, ordered=False) if 0 in k and 1 in k and k.index(1) < len(k) - 1 - k[::-1].index(0)]
    assert _caught(shuffled, NS) > 0
