"""Geometries with a diagonal metric, and the annulus driver.

A geometry maps a forest's logical coordinates to physical space; the wave
equation there is sqrt(g) v' = sum_d D_d (A_d D_d u) with A_d = sqrt(g) g^dd,
so a problem needs the node values of sqrt(g) and A_d, the truncation's
rank-one pair of every element line in the weight of the sqrt(g) factor along
it, and the largest logical wave speed for the time step
(src/evolution.jl:513-708, src/geometry.jl:176-268).

PolarAnnulus is the reference's four-patch annulus r0 <= r <= r1
(src/geometry.jl:176-268): theta = (p-1) pi/2 + theta' x1, r = r0 + r' x2 on
patch p. Its patches are glued in a ring by the identity, so its forest is
the unrolled brick: 4 n1 x n2 roots, periodic in x1 (the glue) and
reflecting in x2 (the walls), with theta = theta' x1 over the whole ring.
"""
import math

import numpy as np

from .forest import Forest


class PolarAnnulus:
    """The annulus map (src/geometry.jl:176-268): sqrt(g) = r theta' r',
    A_1 = r'/(r theta'), A_2 = r theta'/r'."""

    def __init__(self, r0, r1, roots):
        if not 0 < r0 < r1:
            raise ValueError("an annulus needs 0 < r0 < r1, got r0 = %r and r1 = %r" % (r0, r1))
        if not all(n > 0 for n in roots):
            raise ValueError("every patch of the annulus needs a positive number of roots along each "
                             "dimension, got %r" % (roots,))
        self.r0, self.r1 = float(r0), float(r1)
        self.roots = tuple(int(n) for n in roots)
        self.dtheta = (math.pi / 2) / self.roots[0]
        self.dr = (self.r1 - self.r0) / self.roots[1]

    def radius(self, x2):
        return self.r0 + self.dr * x2

    def angle(self, x1):
        return self.dtheta * x1

    def terms(self, x):
        """(sqrt(g), A_1, A_2) at logical positions x = (x1, x2)."""
        r = self.radius(x[1])
        J = r * self.dtheta * self.dr
        return J, self.dr / (r * self.dtheta), r * self.dtheta / self.dr

    def jacobian_factor(self, d, xd):
        """The factor of sqrt(g) along dimension d (0-based) at coordinate xd."""
        if d == 0:
            return np.full_like(np.asarray(xd, dtype=np.float64), self.dtheta)
        return self.radius(np.asarray(xd, dtype=np.float64)) * self.dr

    def physical_coordinates(self, x):
        r, th = self.radius(x[1]), self.angle(x[0])
        return r * np.cos(th), r * np.sin(th)


def annulus_forest(T, P, E, roots=(2, 1), r0=1.0, r1=2.0):
    """The annulus as the unrolled brick of its four patches and its map
    (src/geometry.jl:255-268)."""
    N = E * (P + 1)
    if E % 2:
        raise ValueError("E = %d elements of order P = %d per block is odd, and E must be even" % (E, P))
    n1, n2 = roots
    f = Forest([4 * n1, n2], N, [0.0, 0.0], [float(4 * n1), float(n2)], [True, False], [False, True])
    return f, PolarAnnulus(r0, r1, roots)


def _legendre_all(P, x):
    L = [np.ones_like(x), x]
    for k in range(2, P + 1):
        L.append(((2 * k - 1) * x * L[k - 1] - (k - 1) * L[k - 2]) / k)
    return L[:P + 1]


def projector_mode(nodes, weights, a, P):
    """The degree-P polynomial at the nodes orthogonal to every lower degree
    in sum_i w_i a_i f_i g_i: L_P less its projection on L_0 .. L_{P-1}
    (src/evolution.jl:578-592). a: (..., P+1) line weights."""
    L = np.array(_legendre_all(P, nodes))            # (P+1 modes, P+1 nodes)
    wa = weights * a                                 # (..., P+1)
    G = np.einsum("...i,ki,li->...kl", wa, L[:P], L[:P])
    rhs = np.einsum("...i,i,ki->...k", wa, L[P], L[:P])
    c = np.linalg.solve(G, rhs[..., None])[..., 0]
    return L[P] - np.einsum("...k,ki->...i", c, L[:P])


def metric_tables(forest, el, geo):
    """Node coefficients (N^D, 1+D, nblocks) and per-line truncation pairs
    (P+1, E, nblocks, D) of a diagonal-metric geometry, in float64, and the
    time step's spacing over speed (src/evolution.jl:594-708)."""
    D, N, P = forest.D, forest.N, el.P
    P1 = P + 1
    E = N // P1
    nodes = el.nodes.astype(np.float64)
    w = el.weights.astype(np.float64)
    offs = el.offsets.astype(np.float64)
    nb = len(forest.leaves)
    coef = np.empty((nb, 1 + D, N ** D))
    modes = np.empty((D, nb, E, P1))
    duals = np.empty((D, nb, E, P1))
    n = np.arange(N)
    local = (n // P1) * P1
    grids = np.indices([N] * D).reshape(D, -1)[::-1]
    hspeed = math.inf
    for b, key in enumerate(forest.leaves):
        lv, c = key
        h = forest.spacing(key)
        xs = []
        for k in range(D):
            x1 = forest.lo[k] + h * ((c[k] * N + local) + offs[n % P1])
            xs.append(x1)
        X = tuple(xs[k][grids[k]] for k in range(D))
        J, *A = geo.terms(X)
        coef[b, 0] = J
        for k in range(D):
            coef[b, 1 + k] = A[k]
        speed = np.max([np.sqrt(coef[b, 1 + k] / coef[b, 0]) for k in range(D)])
        hspeed = min(hspeed, h / speed)
        for d in range(D):
            for e in range(E):
                a = geo.jacobian_factor(d, xs[d][e * P1:(e + 1) * P1])
                phi = projector_mode(nodes, w, a, P)
                gamma = np.sum(w * a * phi ** 2)
                modes[d, b, e] = phi
                duals[d, b, e] = w * a * phi / gamma
    # (N^D, 1+D, nblocks) column-major == (nblocks, 1+D, N^D) row-major
    return (np.ascontiguousarray(coef.reshape(-1)), np.ascontiguousarray(modes.reshape(-1)),
            np.ascontiguousarray(duals.reshape(-1)), hspeed)


# --- the rotating Bessel mode (src/annulus.jl) --------------------------------

def _dbesselj(m, z):
    from scipy.special import jv
    return (jv(m - 1, z) - jv(m + 1, z)) / 2


def _dbessely(m, z):
    from scipy.special import yv
    return (yv(m - 1, z) - yv(m + 1, z)) / 2


def annulus_cross(m, k, r0, r1):
    return _dbesselj(m, k * r0) * _dbessely(m, k * r1) - _dbesselj(m, k * r1) * _dbessely(m, k * r0)


def annulus_wavenumber(m, n, r0, r1):
    """The n-th positive root of J_m'(k r0) Y_m'(k r1) - J_m'(k r1) Y_m'(k r0),
    bracketed by a scan in steps of pi/(r1-r0)/50 and bisected to the last bit
    (src/annulus.jl:23-59)."""
    if not (m >= 0 and n >= 1):
        raise ValueError("the mode needs m >= 0 and n >= 1, got m = %d and n = %d" % (m, n))
    if not 0 < r0 < r1:
        raise ValueError("the annulus needs 0 < r0 < r1")
    f = lambda k: annulus_cross(m, k, r0, r1)
    step = math.pi / (r1 - r0) / 50
    a = step / 8
    fa = f(a)
    found = 0
    while True:
        b = a + step
        fb = f(b)
        if fa == 0 or np.sign(fa) != np.sign(fb):
            found += 1
            if found == n:
                lo, hi, flo = a, b, fa
                while True:
                    mid = (lo + hi) / 2
                    if mid == lo or mid == hi:
                        return lo
                    fm = f(mid)
                    if fm == 0:
                        return mid
                    if np.sign(fm) == np.sign(flo):
                        lo, flo = mid, fm
                    else:
                        hi = mid
        a, fa = b, fb


def annulus_exact(geo, m, k, t, T=np.float64):
    """u = R(kr) cos(m theta - k t), v = k R(kr) sin(m theta - k t), R(k r0)
    scaled to 1 (src/annulus.jl:62-115); a callback f(x, var) of the logical
    position."""
    from scipy.special import jv, yv
    jr0, yr0 = _dbesselj(m, k * geo.r0), _dbessely(m, k * geo.r0)
    scale = math.pi * k * geo.r0 / 2

    def f(x, var):
        r = geo.radius(np.asarray(x[1], dtype=np.float64))
        th = geo.angle(np.asarray(x[0], dtype=np.float64))
        R = scale * (jv(m, k * r) * yr0 - yv(m, k * r) * jr0)
        ph = m * th - k * t
        val = R * np.cos(ph) if var == 1 else k * R * np.sin(ph)
        return val.astype(T)
    return f


def annulus_errors(T=np.float64, P=3, E=2, roots=(2, 1), r0=1.0, r1=2.0, m=1, n=1, cfl=0.5, tend=None,
                   truncate=True, precision=None):
    """annulus_errors (src/annulus.jl:117-162): the rotating Neumann mode to a
    quarter turn of its pattern, (pi/2) m/k, by default; sqrt(g)-weighted L2
    errors of u and v together and apart, nodal Linf, the physical radial
    spacing, the step count and the energies."""
    from .element import Element
    from .problem import (WaveProblem, initial_state, oldg_timestep, quadrature_norm, wave_energy,
                          wave_integrator)
    T = np.dtype(T)
    forest, geo = annulus_forest(T, P, E, roots=roots, r0=r0, r1=r1)
    el = Element(T, P)
    problem = WaveProblem(forest, el, truncate=truncate, geometry=geo, precision=precision)
    k = annulus_wavenumber(m, n, r0, r1)
    t_end = (math.pi / 2 * max(m, 1) / k) if tend is None else float(tend)
    t_end = float(T.type(t_end))
    u0 = initial_state(problem, annulus_exact(geo, m, k, 0.0, T))
    nsteps = int(math.ceil(T.type(t_end) / oldg_timestep(problem, cfl)))
    dt = float(T.type(T.type(t_end) / T.type(nsteps)))
    integ = wave_integrator(problem, u0, 0.0, t_end, dt)
    integ.nsteps = nsteps
    integ.solve()
    u = integ.u
    ue = problem.to_device(problem.fill_at_nodes(annulus_exact(geo, m, k, t_end, T)))
    h = forest.minimum_spacing() * geo.dr
    return dict(l2=quadrature_norm(problem, u, 2, ref=ue), l2u=quadrature_norm(problem, u, 2, (1,), ref=ue),
                l2v=quadrature_norm(problem, u, 2, (2,), ref=ue),
                linf=quadrature_norm(problem, u, math.inf, ref=ue), h=h, he=(P + 1) * h, nsteps=nsteps, dt=dt,
                tend=t_end, nblocks=forest.nleaves(), k=k, energy0=wave_energy(problem, u0),
                energy=wave_energy(problem, u))
