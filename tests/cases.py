"""Shared inputs of the test suite: forests, deterministic test data and the
state vectors the oracle and the library are compared on."""
import math

import numpy as np

import twoldg
from twoldg.forest import wave_forest


def smooth_data(D):
    """A smooth periodic state that is neither separable nor a single mode
    (test/evolution_tests.jl:9-19)."""
    def f(x, var):
        s = np.zeros_like(x[0])
        for d in range(D):
            s = s + np.sin(math.pi * (2 * (d + 1) * x[d] + var / 3)) * np.cos(math.pi * 2 * x[(d + 1) % D])
        return s
    return f


def scrambled(n, s):
    """A deterministic irregular sequence (test/refined_tests.jl:21)."""
    i = np.arange(1, n + 1, dtype=np.float64)
    return np.sin(math.pi * (s + 0.7548776662 * i ** 2 + 0.5698402910 * i))


def node_positions(forest, P, T=np.float64):
    """Host node coordinates (nblocks, D, N^D) from the golden tables' offsets."""
    from oracle.oracle import golden_tables
    offs = golden_tables(P)["offsets"]
    N, D = forest.N, forest.D
    P1 = P + 1
    n = np.arange(N)
    local = (n // P1) * P1
    grids = np.indices([N] * D).reshape(D, -1)[::-1]
    out = np.empty((len(forest.leaves), D, N ** D))
    for b, (lv, c) in enumerate(forest.leaves):
        h = forest.spacing((lv, c))
        for k in range(D):
            x1 = forest.lo[k] + h * ((c[k] * N + local) + offs[n % P1])
            out[b, k] = x1[grids[k]]
    return out


def state_from(forest, P, f):
    x = node_positions(forest, P)
    nb = len(forest.leaves)
    u = np.empty((nb, 2, forest.N ** forest.D))
    xs = tuple(x[:, k, :] for k in range(forest.D))
    u[:, 0] = f(xs, 1)
    u[:, 1] = f(xs, 2)
    return u.reshape(-1)


def refined_forest(D, P, reflecting=False):
    """The forests of test/refined_tests.jl:73-79: the middle refined in a
    periodic box, a corner touching two walls refined in a reflecting one."""
    roots = 3 if D == 3 else 4
    region = tuple((0.0, 0.5) for _ in range(D)) if reflecting else True
    return wave_forest(np.float64, D, P, 2, roots=roots, reflecting=reflecting, refined=region)
