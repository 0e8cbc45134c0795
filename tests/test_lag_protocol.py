"""A host model of the mixed sweeps' lagged convergence decisions (ssa_persistent and
ssa_batched, mixed mode), run under random schedules: CTAs on a patch graph, each phase waiting
for its neighbours' progress counters; a ring of slots, each with a monotonic 64-bit arrival word
to which every CTA adds, per sweep, 1 + (1 << 16 unless its residual is below the tolerance) +
(1 << 32 if above 1e6) + (1 << 48 if NaN); each CTA remembering the word of every slot as it last
read it, deciding sweep j at the end of sweep j + lag from the difference once its count is the
number of CTAs, and, at the end of a linear solve, reading (draining) the sweeps left
undecided; a barrier between linear solves. Checks, over several linear solves in a row, that
a reader's difference never holds an arrival of a later sweep when the ring has more than
2 lag + 1 slots (and that this is violated with exactly 2 lag + 1 under a schedule that keeps one
end of a chain of patches far ahead), that every CTA stops at the same sweep, and that each
solve stops `lag` sweeps after the first sweep whose maximum residual is below the
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


def increment(res, tol):
    inc = 1
    if not res < tol:
        inc += 1 << 16
    if res > 1e6:
        inc += 1 << 32
    if res != res:
        inc += 1 << 48
    return inc


def decision(d):
    nc, nd, nn = (d >> 16) & 0xFFFF, (d >> 32) & 0xFFFF, d >> 48
    return 0 if nn else 1 if nc == 0 else 2 if nd else 0


def run_model(nbr, lag, ring, residuals, tol, seed, weights=None, max_sweeps=60):
    """Every CTA's stop sweep per linear solve (1-based within the solve). `residuals` holds one
    function (cta, sweep) -> residual per linear solve; `weights` biases the scheduler."""
    rng = random.Random(seed)
    n = len(nbr)
    ctas = list(range(n))
    mask = (1 << 64) - 1
    prog = [0] * n                       # published phases
    word = [0] * ring
    arrivals = [[] for _ in range(ring)]  # (global sweep) of every arrival not yet read by all
    barrier = [0] * (len(residuals) + 1)
    state = [dict(phases=0, sweep=0, stage=0, solve=0, base=0, decided=0, prev=[0] * ring, seen=[0] * ring,
                  stops=[], finished=False) for _ in range(n)]
    # stage 0..4: colour phases, 5: arrive, 6: boundary phase, 7: decide, 8: drain, 9: barrier

    def read(s, g):
        """CTA state s reads sweep g (global, 0-based): None while incomplete, else the decision."""
        slot = g % ring
        d = (word[slot] - s["prev"][slot]) & mask
        if d & 0xFFFF < n:
            return None
        new = arrivals[slot][s["seen"][slot]:s["seen"][slot] + n]
        if d & 0xFFFF != n or any(x != g for x in new):
            raise RingOverrun("slot %d: reader of sweep %d finds arrivals of sweeps %s" % (slot, g, sorted(set(new))))
        s["prev"][slot] = word[slot]
        s["seen"][slot] += n
        return decision(d)

    steps = 0
    while not all(s["finished"] for s in state):
        steps += 1
        assert steps < 5_000_000, "no progress"
        c = rng.choices(ctas, weights=weights)[0] if weights else rng.randrange(n)
        s = state[c]
        if s["finished"]:
            continue
        st = s["stage"]
        if st in (0, 1, 2, 3, 4, 6):
            if not (st == 0 and s["phases"] == 0) and any(prog[q] < s["phases"] for q in nbr[c]):
                continue      # waiting for a neighbour
            if st == 0:
                s["sweep"] += 1
            s["phases"] += 1
            prog[c] = s["phases"]
            s["stage"] = 5 if st == 4 else (7 if st == 6 else st + 1)
        elif st == 5:         # fold the residual into the slot's word
            g = s["base"] + s["sweep"] - 1
            word[g % ring] = (word[g % ring] + increment(residuals[s["solve"]](c, s["sweep"] - 1), tol)) & mask
            arrivals[g % ring].append(g)
            s["stage"] = 6
        elif st == 7:         # decide up to sweep (sweep - lag), every sweep at the cap
            upto = s["sweep"] if s["sweep"] >= max_sweeps else s["sweep"] - lag
            act = 0
            while s["decided"] < upto and act == 0:
                r = read(s, s["base"] + s["decided"])
                if r is None:
                    break
                s["decided"] += 1
                act = r
            if act == 0 and s["decided"] < upto:
                continue      # waiting for the other CTAs' arrivals
            if act or s["sweep"] >= max_sweeps:
                s["stops"].append(s["sweep"])
                s["stage"] = 8
            else:
                s["stage"] = 0
        elif st == 8:         # drain the sweeps after the deciding one
            while s["decided"] < s["sweep"]:
                if read(s, s["base"] + s["decided"]) is None:
                    break
                s["decided"] += 1
            if s["decided"] == s["sweep"]:
                barrier[s["solve"]] += 1
                s["stage"] = 9
        else:                 # barrier between linear solves
            if barrier[s["solve"]] < n:
                continue
            s["base"] += s["sweep"]
            s["solve"] += 1
            s["sweep"] = s["decided"] = 0
            if s["solve"] == len(residuals):
                s["finished"] = True
            else:
                s["stage"] = 0
    return [s["stops"] for s in state]


def _case(n, seed, lo, hi, solves=3):
    rng = random.Random(1000 + seed)
    out = []
    for _ in range(solves):
        conv = rng.randrange(lo, hi)          # first sweep (1-based) below the tolerance (100)
        noise = {(c, g): rng.randrange(0, 50) for c in range(n) for g in range(80)}

        def residual(c, g, conv=conv, noise=noise):
            return 100 + 1000 // (g + 1) + noise[(c, g)] if g + 1 < conv else noise[(c, g)]
        out.append((conv, residual))
    return out


@pytest.mark.parametrize("lag,ring", [(1, 8), (2, 8), (3, 8), (1, 4), (2, 6)])
def test_lagged_decisions_are_safe_and_consistent(lag, ring):
    assert ring > 2 * lag + 1
    topologies = [(grid(4), None), (chain(40), [1.0 / (1 + k) ** 2 for k in range(40)])]
    for nbr, weights in topologies:
        for seed in range(2):
            case = _case(len(nbr), seed, 10, 25)
            stops = run_model(nbr, lag, ring, [r for _, r in case], 100, seed, weights)
            want = [conv + lag for conv, _ in case]
            assert all(s == want for s in stops), (seed, stops[0], want)


def test_decision_flags_follow_the_maximum():
    tol = 1e-4
    for vals in ([1e-5, 2e-5], [1e-5, 1e-3], [1e-3, 2e7], [1e-5, float("nan")], [2e7, float("nan")], [float("inf")]):
        d = sum(increment(v, tol) for v in vals)
        m = max(vals, key=lambda v: (v != v, v))   # the FP32 key order: NaN above everything
        want = 0 if m != m else 1 if m < tol else 2 if m > 1e6 else 0
        assert decision(d) == want and d & 0xFFFF == len(vals), vals


@pytest.mark.parametrize("lag", [1, 2])
def test_ring_of_2lag_plus_1_is_caught(lag):
    """The negative control: one slot short of the bound, the chain's far end reads a slot the
    near end has already refilled."""
    nbr = chain(40)
    case = _case(40, 0, 10, 25, solves=1)
    with pytest.raises(RingOverrun):
        run_model(nbr, lag, 2 * lag + 1, [r for _, r in case], 100, 0, [1.0 / (1 + k) ** 2 for k in range(40)])
