"""wave_errors run entirely on the oracle (test infrastructure): the
standing mode to a quarter period with RK4 and truncation limiters,
errors of u and v separately, as the reference's convergence tables list
them (reference CODE.md:4124-4169)."""
import math

import numpy as np

from cases import node_positions
from oracle.oracle import Oracle
from twoldg.forest import wave_forest


def exact(D, L, m, t, reflecting):
    if reflecting:
        om = math.pi * m * math.sqrt(D) / L
        def shape(x):
            s = np.ones_like(x[0])
            for d in range(D):
                s = s * np.cos(math.pi * (m * x[d] / L))
            return s
    else:
        om = 2 * math.pi * m * math.sqrt(D) / L
        def shape(x):
            s = np.ones_like(x[0])
            for d in range(D):
                s = s * np.sin(2 * math.pi * m * x[d] / L)
            return s
    def f(x, var):
        return math.cos(om * t) * shape(x) if var == 1 else -om * math.sin(om * t) * shape(x)
    return f, om


def oracle_errors(D, P, E, roots, cfl=0.5, periods=0.25, truncate=True, reflecting=False, refined=False):
    forest = wave_forest(np.float64, D, P, E, roots=roots, reflecting=reflecting, refined=refined)
    o = Oracle(forest, P, truncate=truncate)
    x = node_positions(forest, P)
    xs = tuple(x[:, k, :] for k in range(D))
    f0, om = exact(D, 1.0, 1, 0.0, reflecting)
    nb = len(forest.leaves)
    u0 = np.empty((nb, 2, forest.N ** D))
    u0[:, 0] = f0(xs, 1)
    u0[:, 1] = f0(xs, 2)
    u0 = o.truncate(u0.reshape(-1))
    t_end = periods * 2 * math.pi / om
    dt0 = cfl * forest.minimum_spacing() / (P + 1)
    nsteps = int(math.ceil(t_end / dt0))
    dt = t_end / nsteps
    u = o.rk4(u0, dt, nsteps)
    f1, _ = exact(D, 1.0, 1, t_end, reflecting)
    ue = np.empty((nb, 2, forest.N ** D))
    ue[:, 0] = f1(xs, 1)
    ue[:, 1] = f1(xs, 2)
    ue = ue.reshape(-1)
    return dict(eu=o.norm(u, 2, 1, ue), ev=o.norm(u, 2, 2, ue), l2=o.norm(u, 2, 3, ue),
                linf=o.norm(u, 0, 3, ue), nsteps=nsteps, energy0=o.energy(u0), energy=o.energy(u),
                h=forest.minimum_spacing(), forest=forest, oracle=o, u0=u0, state=u, dt=dt)
