"""The seven-patch ball run on the oracle (test infrastructure)."""
import math

import numpy as np

from oracle.oracle import BallOracle
from twoldg.ball import PlaneWave, ball_tables, node_logical, sevenpatch_forest


def ball_setup(P, E, roots, truncate=True, k=(1.1, -0.7, 0.5), phi=0.3):
    forest, geo = sevenpatch_forest(np.float64, P, E, roots=roots)
    wave = PlaneWave(k, phi)
    tables = ball_tables(forest, P, wave)
    o = BallOracle(forest, P, tables, wave, truncate=truncate)
    return forest, geo, wave, tables, o


def physical_nodes(forest, tables):
    xl = tables["xl"]
    out = np.empty(xl.shape)
    for b, (p, c) in enumerate(forest.blocks):
        x = forest.geo.position(tuple(xl[b, k] for k in range(3)), p)
        for k in range(3):
            out[b, k] = np.asarray(x[k])
    return out


def ball_state(forest, tables, f):
    X = physical_nodes(forest, tables)
    u = np.empty((forest.nleaves(), 2, forest.N ** 3))
    xs = tuple(X[:, k] for k in range(3))
    u[:, 0] = f(xs, 1)
    u[:, 1] = f(xs, 2)
    return u.reshape(-1)


def oracle_sevenpatch_errors(P, E, roots, cfl=0.5, tend=1.0, truncate=True):
    forest, geo, wave, tables, o = ball_setup(P, E, roots, truncate)
    u0 = ball_state(forest, tables, lambda x, v: wave.state(x, 0.0, v))
    if truncate:
        u0 = o.truncate(u0)
    nsteps = int(math.ceil(tend / (cfl * tables["hspeed"] / (P + 1))))
    dt = tend / nsteps
    u = o.rk4(u0, dt, nsteps, 0.0)
    ue = ball_state(forest, tables, lambda x, v: wave.state(x, tend, v))
    return dict(u=o.norm(u, 2, 1, ue), v=o.norm(u, 2, 2, ue), l2=o.norm(u, 2, 3, ue), nsteps=nsteps,
                energy0=o.energy(u0, 0.0), energy=o.energy(u, tend))
