"""The mbarrier protocol of the tensor-core rhs (k_rhs_tc in
sodabayes_gb300/csrc/rhs_tc.cuh), as a model run on the CPU, like
test_update_protocol.py for the residual update.

Roles: the TMA thread loads each stage's B tile, and a U stage's A tile,
into raw buffer s % NS (one barrier phase per stage); a code loader streams
each genotype stage's packed codes into code slot s % NC (bulk copy, cfull
completes on arrival) once every converter has read the slot's previous stage
(cfree); the converter warps take a stage's codes from its slot and widen
them into tensor-memory operand s % NOB and take no part in the raw buffers; the MMA
thread reads that operand and the stage's B tile (genotype stages: it waits
for both) or both raw tiles (U stages, which follow the genotype stages).  A
raw buffer is free once the MMAs of its stage are done (MMA commit); an
operand once the MMAs of its stage completed.

Checked for every number of stages and genotype/U split, for the kernel's
NS (computed from its buffer sizes for 4, 8 and 16 chains) and NOB, under
random interleavings: no parity wait returns a phase early, and no raw
buffer or operand is overwritten while a reader of its previous contents is
pending.  Three mistakes planted in the model must be caught: converters that
do not wait for the MMAs of the operand's previous stage, a code loader that
refills a slot before it is read, and an MMA thread that takes a genotype
stage without waiting for its B tile."""
import os
import random
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "sodabayes_gb300", "csrc", "rhs_tc.cuh")


def _consts():
    txt = open(SRC).read()
    nob = int(re.search(r"constexpr int TC_NOB = (\d+);", txt).group(1))
    nc = int(re.search(r"constexpr int TC_NC = (\d+);", txt).group(1))
    tm = int(re.search(r"constexpr int TC_TM = (\d+);", txt).group(1))
    kc = int(re.search(r"constexpr int TC_KC = (\d+);", txt).group(1))
    ku = int(re.search(r"constexpr int TC_KU = (\d+);", txt).group(1))
    ns = {}
    for ct in (4, 8, 16):
        nb = ((3 * ct + 15) // 16) * 16
        raw = tm * ku * 2 + nb * kc * 2
        ns[ct] = min(8, (220 * 1024 - 1024 - nc * 4096) // raw)
    assert "if (s >= TC_NC && !tc::mbar_wait(&s_cfree[cs], ((s / TC_NC) - 1) & 1)) {" in txt
    assert "bool ok = tc::mbar_wait(&s_cfull[cs], (s / TC_NC) & 1);" in txt
    return nob, ns, nc


class Unsound(AssertionError):
    pass


class Bar:
    def __init__(self):
        self.k = 0

    def ready(self, i):
        if self.k >= i + 2:
            raise Unsound("parity wait for phase %d asked with %d phases complete" % (i, self.k))
        ok = (self.k & 1) != (i & 1)
        if ok and self.k != i + 1:
            raise Unsound("parity wait for phase %d returned with %d phases complete" % (i, self.k))
        return ok


def run(ns_total, nck, NS, NOB, seed, skip_opfree=False, skip_bwait=False, NC=6, skip_cfree=False):
    rnd = random.Random(seed)
    full = [Bar() for _ in range(NS)]
    empty = [Bar() for _ in range(NS)]   # MMA commit
    conv = [Bar() for _ in range(NOB)]
    opfree = [Bar() for _ in range(NOB)]
    raw_owner = [None] * NS
    op_owner = [None] * NOB
    mma_done, landed = set(), set()
    cfull = [Bar() for _ in range(NC)]
    cfree = [Bar() for _ in range(NC)]
    c_owner = [None] * NC
    codes_read, landed_c = set(), set()
    pending = []

    def loader():
        for s in range(nck):
            cs = s % NC
            if s >= NC and not skip_cfree:
                yield cfree[cs], s // NC - 1
            if c_owner[cs] is not None and c_owner[cs] not in codes_read:
                raise Unsound("code slot %d overwritten by stage %d before stage %d was read" % (cs, s, c_owner[cs]))
            c_owner[cs] = s

            def land_c(s=s, cs=cs):
                landed_c.add(s)
                cfull[cs].k += 1
            pending.append(land_c)

    def producer():
        for s in range(ns_total):
            buf = s % NS
            if s >= NS:
                yield empty[buf], s // NS - 1
            prev = raw_owner[buf]
            if prev is not None and prev not in mma_done:
                raise Unsound("raw buffer %d overwritten by stage %d while stage %d is read" % (buf, s, prev))
            raw_owner[buf] = s

            def land(s=s, buf=buf):
                landed.add(s)
                full[buf].k += 1
            pending.append(land)

    def converter():
        for s in range(nck):
            ob, cs = s % NOB, s % NC
            yield cfull[cs], s // NC
            if s not in landed_c:
                raise Unsound("the converters read the codes of stage %d still in flight" % s)
            codes_read.add(s)
            cfree[cs].k += 1
            if s >= NOB and not skip_opfree:
                yield opfree[ob], (s - NOB) // NOB
            prev = op_owner[ob]
            if prev is not None and prev not in mma_done:
                raise Unsound("operand %d overwritten by stage %d while stage %d's MMAs read it" % (ob, s, prev))
            op_owner[ob] = s
            conv[ob].k += 1

    def mma():
        for s in range(ns_total):
            buf, ob = s % NS, s % NOB
            if s < nck:
                yield conv[ob], s // NOB
                if not skip_bwait:
                    yield full[buf], s // NS
            else:
                yield full[buf], s // NS
            if s not in landed:
                raise Unsound("the MMAs of stage %d read a B tile still in flight" % s)

            def commit(s=s, buf=buf, ob=ob):
                mma_done.add(s)
                if s < nck:
                    opfree[ob].k += 1
                empty[buf].k += 1
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


def test_rhs_protocol_is_sound():
    nob, ns, nc = _consts()
    rnd = random.Random(3)
    t = 0
    for ct, NS in ns.items():
        assert NS >= 4
        for _ in range(150):
            total = rnd.randint(1, 48)
            nck = rnd.randint(0, total)
            run(total, nck, NS, nob, seed=t, NC=nc)
            t += 1


def test_rhs_protocol_model_catches_a_missing_wait():
    """The mistake planted in the model: converters that do not wait for the
    MMAs of the operand's previous stage."""
    nob, ns, nc = _consts()
    rnd = random.Random(5)
    caught = 0
    for t in range(200):
        total = rnd.randint(nob + 1, 48)
        try:
            run(total, total, ns[16], nob, seed=t, skip_opfree=True, NC=nc)
        except Unsound:
            caught += 1
    assert caught > 0


def test_rhs_protocol_model_catches_an_mma_before_its_b_tile():
    """An MMA thread that takes a genotype stage once its codes are converted,
    without waiting for the stage's B tile (the converters no longer wait for
    the raw buffer), must be caught."""
    nob, ns, nc = _consts()
    rnd = random.Random(9)
    caught = 0
    for t in range(200):
        total = rnd.randint(1, 48)
        try:
            run(total, total, ns[16], nob, seed=t, skip_bwait=True, NC=nc)
        except Unsound:
            caught += 1
    assert caught > 0


def test_rhs_protocol_model_catches_a_code_slot_refilled_too_early():
    nob, ns, nc = _consts()
    rnd = random.Random(17)
    caught = 0
    for t in range(200):
        total = rnd.randint(nc + 2, 48)
        try:
            run(total, total, ns[16], nob, seed=t, NC=nc, skip_cfree=True)
        except Unsound:
            caught += 1
    assert caught > 0
