"""A host model of the mixed sweeps' lagged convergence decisions (ssa_persistent, mixed
mode), run under random schedules: CTAs on a patch graph, each phase waiting for its neighbours'
progress counters, a ring of slots per sweep holding (sweep + 1) << 32 | residual keys folded
with max and a monotonic arrival count per slot, and sweep j decided at the end of sweep
j + lag. Checks that a reader never finds its slot already holding a later sweep when the ring
has more than 2 lag + 1 slots (and that the check fires with exactly 2 lag + 1 under a schedule
that keeps one end of a chain of patches far ahead), that every CTA stops at the same sweep,
and that the solve stops `lag` sweeps after the first sweep whose maximum residual is below the
tolerance."""
import random

import pytest


def grid(n):
    nbr = {}
    for i in range(n):
        for j in range(n):
            nbr[i * n + j] = [a * n + b for a, b in ((i - 1, j), (i + 1, j), (i, j - 1), (i, j + 1))
                              if 0 <= a < n and 0 <= b < n]
    return nbr


def chain(n):
    return {k: [q for q in (k - 1, k + 1) if 0 <= q < n] for k in range(n)}


class RingOverrun(AssertionError):
    pass


def run_model(nbr, lag, ring, residual, tol, seed, weights=None, max_sweeps=60):
    """Every CTA's stop sweep (1-based); all equal. `weights` biases the scheduler."""
    rng = random.Random(seed)
    n = len(nbr)
    ctas = list(range(n))
    prog = [0] * n            # published phases
    key = [0] * ring
    cnt = [0] * ring
    state = [dict(phases=0, sweep=0, stage=0, done=None) for _ in range(n)]
    # stage 0..4: colour phases, 5: arrive, 6: boundary phase, 7: decide
    steps = 0
    while any(s["done"] is None for s in state):
        steps += 1
        assert steps < 5_000_000, "no progress"
        c = rng.choices(ctas, weights=weights)[0] if weights else rng.randrange(n)
        s = state[c]
        if s["done"] is not None:
            continue
        st = s["stage"]
        if st in (0, 1, 2, 3, 4, 6):
            if not (st == 0 and s["sweep"] == 0) and any(prog[q] < s["phases"] for q in nbr[c]):
                continue      # waiting for a neighbour
            if st == 0:
                s["sweep"] += 1
            s["phases"] += 1
            prog[c] = s["phases"]
            s["stage"] = 5 if st == 4 else (7 if st == 6 else st + 1)
        elif st == 5:         # fold the residual into the slot, then count in
            g = s["sweep"] - 1
            key[g % ring] = max(key[g % ring], ((g + 1) << 32) | residual(c, g))
            cnt[g % ring] += 1
            s["stage"] = 6
        else:                 # decide sweep (sweep - lag) once every CTA is in
            d = s["sweep"] - lag
            if d >= 1:
                g = d - 1
                if cnt[g % ring] < n * (g // ring + 1):
                    continue
                k = key[g % ring]
                if k >> 32 != g + 1:
                    raise RingOverrun("slot holds sweep %d, reader wants %d" % ((k >> 32) - 1, g))
                if (k & 0xFFFFFFFF) < tol:
                    s["done"] = s["sweep"]
                    continue
            if s["sweep"] >= max_sweeps:
                s["done"] = s["sweep"]
                continue
            s["stage"] = 0
    return [s["done"] for s in state]


def _case(n, seed, lo, hi):
    rng = random.Random(1000 + seed)
    conv = rng.randrange(lo, hi)              # first sweep (1-based) below the tolerance (100)
    noise = {(c, g): rng.randrange(0, 50) for c in range(n) for g in range(80)}

    def residual(c, g):
        return 100 + 1000 // (g + 1) + noise[(c, g)] if g + 1 < conv else noise[(c, g)]
    return conv, residual


@pytest.mark.parametrize("lag,ring", [(1, 8), (2, 8), (3, 8), (1, 4), (2, 6)])
def test_lagged_decisions_are_safe_and_consistent(lag, ring):
    assert ring > 2 * lag + 1
    topologies = [(grid(4), None), (chain(40), [1.0 / (1 + k) ** 2 for k in range(40)])]
    for nbr, weights in topologies:
        for seed in range(4):
            conv, residual = _case(len(nbr), seed, 10, 25)
            stops = run_model(nbr, lag, ring, residual, 100, seed, weights)
            assert set(stops) == {conv + lag}, (seed, set(stops), conv)


@pytest.mark.parametrize("lag", [1, 2])
def test_ring_of_2lag_plus_1_is_caught(lag):
    """The negative control: one slot short of the bound, the chain's far end still reads a slot
    the near end has already refilled, and the reader's check reports it."""
    nbr = chain(40)
    conv, residual = _case(40, 0, 10, 25)
    with pytest.raises(RingOverrun):
        run_model(nbr, lag, 2 * lag + 1, residual, 100, 0, [1.0 / (1 + k) ** 2 for k in range(40)])
