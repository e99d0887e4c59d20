"""A CPU model of how the faster-evgen chunk passes find event starts
(csrc/tp_kernels.cu: fe_sub_chases, fe_walk, k_fe_map, k_fe_starts),
checked against the direct event-by-event chase on random accept bits.

The model follows the kernels' structure: a chunk of kFeChunk positions is
cut into kFeSubs sub-spans; the chase of sub-span s starts kFeLead positions
before it (sub-span 0: at the chunk's first entry offset), marks the event
starts that fall in it and keeps its first start past it; a walk from an
entry offset steps event by event until it stands on a marked start, then
takes the marks' count to the sub-span's end and jumps to that chase's exit.
The starts pass lists each sub-span's events from the walk's first start
in it. An event (src/evgen.rs:143-173, 221-249) takes random_array::<9>,
::<6>, then ::<2> per re-rolled point; for ranf a random_array::<N> skips
the rest of a 55-draw block holding fewer than N draws
(src/random/ranf.rs:78-102). Pairs: A[p] accepts (p, p+1), B[p] (p, p+3).
"""
import numpy as np
import pytest

CHUNK, SUB, SUBS, LEAD = 4096, 256, 16, 512  # the kernels' proportions, smaller
SPAN = CHUNK + 1024


def make_step(A, B, ranf, base):
    """The next event start after an event starting at P (None past the span)."""

    def step(P):
        r = (base + P) % 55

        def take(n):
            nonlocal P, r
            if ranf and 55 - r < n:
                P += 55 - r
                r = 0
            at = P
            P += n
            r = (r + n) % 55
            return at

        take(9)
        q = take(6)
        if q + 3 >= SPAN:
            return None
        rejected = 3 - int(B[q]) - int(B[q + 1]) - int(B[q + 2])
        while rejected:
            a = take(2)
            if a + 1 >= SPAN:
                return None
            rejected -= int(A[a])
        return P

    return step


def sub_chases(step, entry0):
    marks = np.zeros(CHUNK, bool)
    exits = []
    for s in range(SUBS):
        lo, hi = s * SUB, (s + 1) * SUB
        P = entry0 if s == 0 else max(lo - LEAD, 0)
        while P is not None and P < hi:
            if P >= lo:
                marks[P] = True
            P = step(P)
        exits.append(P)
    return marks, exits


def walk(step, marks, exits, P):
    """(exit, events, first start and events before it per sub-span, jumps)."""
    n, first, jumps = 0, {}, 0
    while P < CHUNK:
        s = P // SUB
        first.setdefault(s, (P, n))
        if marks[P]:
            n += int(marks[P:(s + 1) * SUB].sum())
            P = exits[s]
            jumps += 1
        else:
            P = step(P)
            n += 1
        assert P is not None
    return P, n, first, jumps


def starts_from_walk(step, marks, first):
    out = []
    for s in range(SUBS):
        if s not in first:
            continue
        P, _ = first[s]
        hi = (s + 1) * SUB
        while P < hi:
            if marks[P]:
                out += [P + int(i) for i in np.nonzero(marks[P:hi])[0]]
                break
            out.append(P)
            P = step(P)
    return out


def direct(step, P):
    starts = []
    while P < CHUNK:
        starts.append(P)
        P = step(P)
    return P, starts


@pytest.mark.parametrize("ranf", [False, True], ids=["xoshiro", "ranf"])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_walk_equals_direct_chase(ranf, seed):
    rng = np.random.default_rng(seed)
    acc = np.pi / 4  # the unit-circle acceptance
    A = rng.random(SPAN + 8) < acc
    B = rng.random(SPAN + 8) < acc
    base = int(rng.integers(0, 55))  # the chunk's first draw within its ranf block
    step = make_step(A, B, ranf, base)
    entry0 = int(rng.integers(0, 20)) if seed > 1 else 0
    marks, exits = sub_chases(step, entry0)
    total_jumps = 0
    for e in range(entry0, entry0 + 32):  # the map pass's 32 entry offsets
        exit_w, n, first, jumps = walk(step, marks, exits, e)
        total_jumps += jumps
        exit_d, starts = direct(step, e)
        assert (exit_w, n) == (exit_d, len(starts))
        assert starts_from_walk(step, marks, first) == starts
        # the walk's first start of every sub-span that has one, with its index
        for s, (P, k) in first.items():
            assert starts[k] == P and P // SUB == s
    # the walks do take the chases' shortcuts (most sub-spans are jumped)
    assert total_jumps > 32 * SUBS // 2
