"""The device planner's choice-row walk (flam3_gb300/csrc/f3g_choice.h)
against the reference's 16384-step loop (flam3.c:165-224, host/prep.c), both
run on the host through flam3gpu_choice_breakpoints: identical breakpoints
and identical errors.

The walk replaces the loop's chain of r = fl(r + dr) by closed-form runs
inside each FP64 binade, so the cases aim at the rounding: random weights
(dr with a full 53-bit significand, so the first binades above dr round at
ties half the time), step sizes built to tie at every binade from the first
to the fourteenth, exact dyadic weights (no rounding at all), weights spread
over many orders of magnitude, zero and tiny weights (several breakpoints at
one step), chaos rows and a final xform's weight (only in the raw-weight
row)."""
import math

import numpy as np
import pytest

from flam3_gb300 import render


def both(d, c=None, nstd=None):
    out = []
    for walk in (False, True):
        try:
            out.append(("ok", render.choice_breakpoints(d, c, nstd, walk=walk)))
        except render.Flam3GpuError as e:
            out.append(("error", str(e).split(": ", 1)[1]))
    return out


MOVES = []


def check(d, c=None, nstd=None):
    ref, walk = both(d, c, nstd)
    assert ref == walk, (list(d), None if c is None else list(c), nstd, ref, walk)
    if ref[0] == "ok":
        MOVES.append(render.choice_breakpoints(d, c, nstd, walk=True, moves=True)[1])
    return ref


def test_random_rows():
    rng = np.random.default_rng(11)
    errors = ok = 0
    for k in range(1500):
        nx = int(rng.integers(1, 33))
        kind = k % 5
        if kind == 0:
            d = rng.uniform(0.0, 1.0, nx)
        elif kind == 1:
            d = 10.0 ** rng.uniform(-12, 12, nx)  # many orders of magnitude
        elif kind == 2:
            d = rng.integers(0, 8, nx) / 8.0  # exact dyadic weights, zeros included
            d[0] = max(d[0], 0.125)
        elif kind == 3:
            d = rng.uniform(0.0, 1.0, nx) * (rng.uniform(0, 1, nx) < 0.6)  # zero weights
            d[int(rng.integers(0, nx))] = rng.uniform(0.1, 1.0)
        else:
            d = rng.exponential(1.0, nx) * rng.choice([1e-6, 1.0, 1e6])
        nstd = nx - int(rng.integers(0, 2)) if nx > 1 else nx  # a final xform at the end
        c = None
        if rng.uniform() < 0.4:
            c = rng.uniform(0.0, 2.0, nstd) * (rng.uniform(0, 1, nstd) < 0.8)
            c[int(rng.integers(0, nstd))] = rng.uniform(0.5, 1.5)
        r = check(d, c, nstd)
        ok += r[0] == "ok"
        errors += r[0] == "error"
    assert ok > 1400
    # the walk takes a few dozen steps where the loop takes 16384
    assert max(MOVES) < 200 and float(np.mean(MOVES)) < 60, (max(MOVES), float(np.mean(MOVES)))


@pytest.mark.parametrize("tail", range(0, 16))
def test_ties_at_each_binade(tail):
    """dr = S / 16384 with S's significand ending in a one followed by `tail`
    zeros: the fraction dr/u is exactly one half in the binade `tail + 1`
    above dr's own."""
    rng = np.random.default_rng(100 + tail)
    for _ in range(40):
        M = (int(rng.integers(1 << 52, 1 << 53)) >> (tail + 1) << (tail + 1)) | (1 << tail)
        S = math.ldexp(M, -52 + int(rng.integers(-30, 30)))
        for split in (0.5, 0.25, 0.125):
            a = S * split  # exact scalings: a + b == S exactly
            b = S - a
            assert a + b == S
            check([a, b])
            check([a, b, 0.0, a], None, 2)  # final xform weight in the raw row only
            check([a, b], [1.0, 1.0])
            check([a, b], [0.5, 2.0])


def test_exact_and_degenerate_rows():
    check([1.0])
    check([1.0, 0.0, 0.0, 1.0])
    check([3.0, 5.0, 7.0])
    check([1e-300, 1.0])
    check([1.0, 1e-300, 1e-300, 1.0])
    check([1e300, 1e300])
    check([0.1, 0.2, 0.3], None, 3)
    # a negative final weight in the raw row: its threshold is never reached
    assert check([0.5, 0.5, -0.25], None, 2)[0] == "ok"
    # the reference's errors
    assert check([0.0, 0.0])[0] == "error"
    assert check([0.5, -0.1])[0] == "error"
    assert check([0.5, 0.5], [1.0, -1.0])[0] == "error"


def test_walk_counts_every_breakpoint_like_the_table():
    """The breakpoints of a row reproduce the reference's table: entry v is the
    number of breakpoints at or below v."""
    d = [0.3, 0.0, 0.45, 1e-9, 0.25]
    brk = render.choice_breakpoints(d, walk=True)
    dr = sum(d) / 16384
    table, r, j, t = [], 0.0, 0, d[0]
    for v in range(16384):
        while r >= t:
            j += 1
            t += d[j]
        table.append(j)
        r += dr
    assert table == [int(np.searchsorted(brk, v, side="right")) for v in range(16384)]
