"""The seven- and thirteen-patch balls run on the oracle (test infrastructure)."""
import math

import numpy as np

from oracle.oracle import BallOracle
from twoldg.ball import PlaneWave, ball_forest, ball_tables, node_logical, sevenpatch_forest


def ball_setup(P, E, roots, truncate=True, k=(1.1, -0.7, 0.5), phi=0.3, Rm=None, radiative=None, Lc=1.0, R1=3.0,
               grading=0.0, refined=False):
    """A ball (the thirteen-patch one with Rm, its cube refined by `refined`),
    its tables and its oracle; radiative = (kappa, inverse_r) replaces the
    Dirichlet wave."""
    forest, geo = ball_forest(np.float64, P, E, roots, Lc, R1, Rm=Rm, grading=grading, refined=refined)
    wave = PlaneWave(k, phi)
    tables = ball_tables(forest, P, wave)
    rad = None
    if radiative is not None:
        rad = (radiative[0], 1.0 / geo.outer_radius() if radiative[1] else 0.0)
    o = BallOracle(forest, P, tables, wave, truncate=truncate, radiative=rad)
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


def oracle_sevenpatch_errors(P, E, roots, cfl=0.5, tend=1.0, truncate=True, Rm=None):
    forest, geo, wave, tables, o = ball_setup(P, E, roots, truncate, Rm=Rm)
    u0 = ball_state(forest, tables, lambda x, v: wave.state(x, 0.0, v))
    if truncate:
        u0 = o.truncate(u0)
    nsteps = int(math.ceil(tend / (cfl * tables["hspeed"] / (P + 1))))
    dt = tend / nsteps
    u = o.rk4(u0, dt, nsteps, 0.0)
    ue = ball_state(forest, tables, lambda x, v: wave.state(x, tend, v))
    return dict(u=o.norm(u, 2, 1, ue), v=o.norm(u, 2, 2, ue), l2=o.norm(u, 2, 3, ue), nsteps=nsteps,
                energy0=o.energy(u0, 0.0), energy=o.energy(u, tend))


def oracle_radiative_errors(P, E, roots, kappa=1.0, inverse_r=True, w=0.5, cfl=0.5, tend=2.0, truncate=True,
                            Rm=None):
    """radiative_errors on the oracle: the outgoing pulse of width w under a
    radiative sphere; L2 errors and the energies (the boundary's term included)."""
    from twoldg.ball import OutgoingPulse
    forest, geo, wave, tables, o = ball_setup(P, E, roots, truncate, Rm=Rm, radiative=(kappa, inverse_r))
    pulse = OutgoingPulse(w)
    u0 = ball_state(forest, tables, lambda x, v: pulse.state(x, 0.0, v))
    if truncate:
        u0 = o.truncate(u0)
    nsteps = int(math.ceil(tend / (cfl * tables["hspeed"] / (P + 1))))
    dt = tend / nsteps
    u = o.rk4(u0, dt, nsteps, 0.0)
    ue = ball_state(forest, tables, lambda x, v: pulse.state(x, tend, v))
    return dict(l2=o.norm(u, 2, 3, ue), nsteps=nsteps, energy0=o.energy(u0, 0.0), energy=o.energy(u, tend))
