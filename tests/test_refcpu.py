"""The CPU baseline (oracle/refcpu.c, the reference's threaded CPU data flow
restated in C) against the oracle: the same right-hand side, truncation and
RK4 steps to 1e-12 on uniform bricks in 1D to 3D, periodic and reflecting,
P = 1 to 7. The baseline's time stands for the reference's CPU path only if
it computes what the reference computes."""
import numpy as np
import pytest

from cases import smooth_data, state_from
from oracle.oracle import Oracle
from oracle.refcpu import RefCPU
from twoldg.forest import wave_forest

CASES = [(1, 3, 2, 3, False), (1, 5, 4, 2, True), (2, 2, 2, 3, False), (2, 4, 2, 4, True), (3, 3, 4, 2, False),
         (3, 2, 2, 2, True), (3, 1, 2, 3, False), (2, 6, 2, 2, False), (3, 7, 2, 1, True)]


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("case", CASES, ids=lambda c: "D%dP%dE%dr%d%s" % (c[:4] + ("-wall" if c[4] else "",)))
def test_refcpu_matches_the_oracle(case):
    D, P, E, roots, refl = case
    f = wave_forest(np.float64, D, P, E, roots=roots, reflecting=refl)
    o, r = Oracle(f, P), RefCPU(f, P)
    u = state_from(f, P, smooth_data(D))
    assert rel(r.rhs(u), o.rhs(u)) < 1e-12
    u0 = o.truncate(u)
    assert rel(r.truncate(u), u0) < 1e-13
    dt = 0.5 * f.minimum_spacing() / (P + 1)
    assert rel(r.rk4(u0, dt, 3), o.rk4(u0, dt, 3)) < 1e-12
    w = u0.copy()
    r.rk4(w, dt, 3, inplace=True)
    assert np.array_equal(w, r.rk4(u0, dt, 3))


def test_refcpu_takes_uniform_bricks_only():
    f = wave_forest(np.float64, 2, 3, 2, roots=4, refined=True)
    with pytest.raises(ValueError):
        RefCPU(f, 3)
