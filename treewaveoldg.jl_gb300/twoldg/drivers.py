"""The standing-mode drivers of src/sinewave.jl, over libtwoldg.

wave_omega/wave_exact (src/sinewave.jl:17-39), reflect_omega/reflect_exact
(:50-75), wave_errors/reflect_errors (:228-274), convergence_rate
(src/evolution.jl:1534-1540). The exact solutions are numpy-vectorised
callbacks f(x, var) evaluated in the element's type.
"""
import math

import numpy as np

from .element import Element
from .forest import wave_forest
from .problem import (WaveProblem, initial_state, oldg_timestep, quadrature_norm, wave_energy,
                      wave_integrator)


def wave_omega(D, L, m, T=np.float64):
    T = np.dtype(T).type
    return T(2) * T(math.pi) * T(m) * T(math.sqrt(D)) / T(L)


def wave_exact(D, L, m, t, T=np.float64):
    """u = cos(wt) prod_d sin(2 pi m x_d / L), v = du/dt."""
    T = np.dtype(T).type
    om = wave_omega(D, L, m, T)
    twopi = T(2) * T(math.pi)
    t = T(t)

    def f(x, var):
        shape = np.ones_like(x[0])
        for d in range(D):
            shape = shape * np.sin(twopi * T(m) * x[d] / T(L))
        if var == 1:
            return np.cos(om * t) * shape
        return -om * np.sin(om * t) * shape
    return f


def reflect_omega(D, L, m, T=np.float64):
    T = np.dtype(T).type
    return T(math.pi) * T(m) * T(math.sqrt(D)) / T(L)


def reflect_exact(D, L, m, t, T=np.float64):
    """u = cos(wt) prod_d cos(m pi x_d / L), the Neumann standing mode."""
    T = np.dtype(T).type
    om = reflect_omega(D, L, m, T)
    t = T(t)

    def f(x, var):
        shape = np.ones_like(x[0])
        for d in range(D):
            shape = shape * np.cos(T(math.pi) * (T(m) * x[d] / T(L)))
        if var == 1:
            return np.cos(om * t) * shape
        return -om * np.sin(om * t) * shape
    return f


def convergence_rate(hs, errs):
    x = np.log(np.asarray(hs, dtype=np.float64))
    y = np.log(np.asarray(errs, dtype=np.float64))
    xb, yb = x.mean(), y.mean()
    return float(((x - xb) * (y - yb)).sum() / ((x - xb) ** 2).sum())


def wave_errors(T, D, P, E, roots=4, L=1.0, m=1, cfl=0.5, periods=0.25, truncate=True,
                reflecting=False, refined=False, precision=None):
    """wave_errors(T, Val(D); P, E, roots, ...) (src/sinewave.jl:228-261):
    evolve the standing mode to t_end and return the quadrature L2 and nodal
    Linf errors of u and v together, h, h_e, the step count, the block count
    and the initial and final energies."""
    T = np.dtype(T)
    Tt = T.type
    forest = wave_forest(T, D, P, E, roots=roots, L=L, reflecting=reflecting, refined=refined)
    el = Element(T, P)
    problem = WaveProblem(forest, el, truncate=truncate, precision=precision)
    exact_mode = reflect_exact if reflecting else wave_exact
    omega = reflect_omega if reflecting else wave_omega
    u0 = initial_state(problem, exact_mode(D, L, m, 0.0, T))
    t_end = Tt(periods) * Tt(2) * Tt(math.pi) / omega(D, L, m, T)
    nsteps = int(math.ceil(Tt(t_end / oldg_timestep(problem, cfl))))
    dt = Tt(t_end / Tt(nsteps))
    integ = wave_integrator(problem, u0, 0.0, float(t_end), float(dt))
    integ.solve()
    u = integ.u
    uexact = problem.to_device(problem.fill_at_nodes(exact_mode(D, L, m, t_end, T)))
    h = forest.minimum_spacing()
    return dict(l2=quadrature_norm(problem, u, 2, ref=uexact),
                linf=quadrature_norm(problem, u, math.inf, ref=uexact),
                h=h, he=(P + 1) * h, nsteps=nsteps, nblocks=forest.nleaves(),
                energy0=wave_energy(problem, u0), energy=wave_energy(problem, u))


def reflect_errors(T, D, **kw):
    """reflect_errors (src/sinewave.jl:263-274): wave_errors on a reflecting box."""
    kw["reflecting"] = True
    return wave_errors(T, D, **kw)
