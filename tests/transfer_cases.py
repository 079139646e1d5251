"""Shared cases of the transfer tests (test/transfer_tests.jl): the
deterministic irregular grid function, the polynomial the pins integrate, the
graded composite reference integral, and the exact moments of a particle's
density by the ball rule in its rest frame."""
import math

import numpy as np

from oracle import transfer as T


def irregular(n):
    """sin(pi (0.1 + 0.7548776662 i^2)), i = 1..n (test/transfer_tests.jl:15-16)."""
    i = np.arange(1, n + 1, dtype=np.float64)
    return np.sin(np.pi * (0.1 + 0.7548776662 * i * i))


def poly(X):
    """1 + x - 2 y^2 z + x^3 y^3 z^3 (test/transfer_tests.jl:189)."""
    X = np.atleast_2d(X)
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    return 1 + x - 2 * y * y * z + x ** 3 * y ** 3 * z ** 3


def bump(r2, ell):
    """(1 - r^2/ell^2)^4 inside ell (test/transfer_tests.jl:76)."""
    return np.where(r2 < ell * ell, (1 - r2 / (ell * ell)) ** 4, 0.0)


def exact_moment(f, Q, ell, z, v, nr=12, nt=12):
    """int rho f by the ball rule in the rest frame (test/transfer_tests.jl:195-197):
    sum w Q rho0(ell^2 |y|^2, ell) f(z + L(v)^-1 ell y) ell^3 / gamma."""
    ys, ws = T.ball_rule(nr, nt)
    z = np.asarray(z, dtype=np.float64)
    v = np.asarray(v, dtype=np.float64)
    gamma = 1 / math.sqrt(1 - float(v @ v))
    Y = ell * ys
    lab = Y - (gamma / (gamma + 1) * (Y @ v))[:, None] * v[None, :]
    rho = T.particle_density(ys * ell + z[None, :], z, np.zeros(3), ell, Q)   # rest-frame profile
    return float(np.sum(ws * rho * f(z[None, :] + lab) * ell ** 3) / gamma)


REF_X, REF_W = np.polynomial.legendre.leggauss(16)


def _composite(g, a, b, breaks):
    pts = sorted(set([a, b] + [x for x in breaks if a < x < b]))
    acc = 0.0
    for k in range(len(pts) - 1):
        half = (pts[k + 1] - pts[k]) / 2
        xs = pts[k] + half * (1 + REF_X)
        acc += float(np.sum(REF_W * half * g(xs)))
    return acc


def reference_integral(f, lo, hi, z, scale, grades, ell, prefix=()):
    """An independent int f over a box (test/transfer_tests.jl:44-73): composite
    16-point Gauss-Legendre one dimension at a time, with breakpoints graded
    geometrically toward z on `scale` and, where the line crosses a bump of
    radius ell, at the crossing and graded toward it. f maps (n, D) points to
    n values; the innermost dimension is vectorised."""
    d = len(prefix)
    D = len(lo)
    breaks = [z[d] + s * scale * 2.0 ** k for k in grades for s in (-1, 1)]
    r2 = sum((prefix[j] - z[j]) ** 2 for j in range(d))
    if ell is not None and r2 < ell * ell:
        c = math.sqrt(ell * ell - r2)
        breaks += [z[d] + s * c * (1 - 2.0 ** -k) for k in range(13) for s in (-1, 1)]
    if d == D - 1:
        def g(xs):
            X = np.empty((len(xs), D))
            X[:, :d] = prefix
            X[:, d] = xs
            return f(X)
    else:
        def g(xs):
            return np.array([reference_integral(f, lo, hi, z, scale, grades, ell, prefix + (float(x),))
                             for x in xs])
    return _composite(g, lo[d], hi[d], breaks)


def grad_poly(X):
    """The gradient of poly, (npts, 3)."""
    X = np.atleast_2d(X)
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    return np.stack([1 + 3 * x ** 2 * y ** 3 * z ** 3, -4 * y * z + 3 * x ** 3 * y ** 2 * z ** 3,
                     -2 * y * y + 3 * x ** 3 * y ** 3 * z ** 2], axis=1)


def brick_values(mesh, t, f):
    """A state vector of the oracle's brick mesh with f at every node, in
    both variables."""
    u = np.zeros(mesh.nblocks * 2 * mesh.NN)
    P1 = mesh.P + 1
    for b, e in mesh.elements():
        lo, hi = mesh.element_box(b, e)
        xs = [lo[d] + (hi[d] - lo[d]) * (1 + t.nodes) / 2 for d in range(mesh.D)]
        X = np.array([[xs[d][K[mesh.D - 1 - d]] for d in range(mesh.D)] for K in np.ndindex(*([P1] * mesh.D))])
        for var in (1, 2):
            u[mesh.node_index(b, e, var)] = f(X)
    return u
