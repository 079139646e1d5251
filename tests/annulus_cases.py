"""The annulus run on the oracle (test infrastructure): metric node values
from the geometry, the sqrt(g) factors along every element line for the
oracle's own projectors, and the rotating Bessel mode."""
import math

import numpy as np

from cases import node_positions
from oracle.oracle import Oracle, golden_tables
from twoldg.element import Element
from twoldg.geometry import annulus_exact, annulus_forest, annulus_wavenumber, metric_tables


def line_weights(forest, geo, P):
    """(D, nblocks, E, P+1): the sqrt(g) factor along each element line."""
    D, N = forest.D, forest.N
    P1 = P + 1
    E = N // P1
    offs = golden_tables(P)["offsets"]
    n = np.arange(N)
    local = (n // P1) * P1
    out = np.empty((D, len(forest.leaves), E, P1))
    for b, key in enumerate(forest.leaves):
        h = forest.spacing(key)
        for d in range(D):
            x = forest.lo[d] + h * ((key[1][d] * N + local) + offs[n % P1])
            out[d, b] = geo.jacobian_factor(d, x).reshape(E, P1)
    return out


def annulus_oracle(P, E, roots, truncate=True):
    forest, geo = annulus_forest(np.float64, P, E, roots=roots)
    coef, modes, duals, hspeed = metric_tables(forest, Element(np.float64, P), geo)
    o = Oracle(forest, P, truncate=truncate, coef=coef, line_weights=line_weights(forest, geo, P))
    return forest, geo, o, hspeed


def state_of(forest, P, f):
    x = node_positions(forest, P)
    nb = len(forest.leaves)
    u = np.empty((nb, 2, forest.N ** forest.D))
    xs = tuple(x[:, k, :] for k in range(forest.D))
    u[:, 0] = f(xs, 1)
    u[:, 1] = f(xs, 2)
    return u.reshape(-1)


def oracle_annulus_errors(P, E, roots, m=2, n=1, cfl=0.5, truncate=True):
    forest, geo, o, hspeed = annulus_oracle(P, E, roots, truncate)
    k = annulus_wavenumber(m, n, 1.0, 2.0)
    t_end = math.pi / 2 * max(m, 1) / k
    u0 = state_of(forest, P, annulus_exact(geo, m, k, 0.0))
    if truncate:
        u0 = o.truncate(u0)
    nsteps = int(math.ceil(t_end / (cfl * hspeed / (P + 1))))
    dt = t_end / nsteps
    u = o.rk4(u0, dt, nsteps)
    ue = state_of(forest, P, annulus_exact(geo, m, k, t_end))
    return dict(u=o.norm(u, 2, 1, ue), v=o.norm(u, 2, 2, ue), l2=o.norm(u, 2, 3, ue), nsteps=nsteps,
                energy0=o.energy(u0), energy=o.energy(u), dt=dt)
