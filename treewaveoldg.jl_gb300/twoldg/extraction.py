"""Waveforms (src/extraction.jl): the field's spherical-harmonic modes on
spheres about a centre, read from the solution's own element polynomials.

The points are located on the host once: on a brick as they are, on the
seven-patch ball through the ball's inverse map (ball_patch_point); each
point's element and its Lagrange weights at the element's Gauss-Lobatto
nodes make a stencil of (P+1)^D state-vector positions and weights. The
reading itself is a gather and weighted sum on the device (twoldg_gather),
the modes a quadrature on the host: Gauss-Legendre in cos(theta) times an
equally spaced phi."""
import ctypes
import math

import numpy as np

from . import _lib
from .ball import SHELLS, SevenPatchBall
from .problem import _check_state, _dptr, _sync_torch


# --- spherical harmonics and the sphere rule ---------------------------------
def harmonic_modes(lmax):
    """(l, m), 0 <= m <= l <= lmax, l by l and m from 0 within each (src/extraction.jl:83-91)."""
    return [(l, m) for l in range(lmax + 1) for m in range(l + 1)]


def mode_index(l, m):
    """0-based position of (l, m) in harmonic_modes."""
    return l * (l + 1) // 2 + m


def spherical_harmonics(lmax, theta, phi):
    """The orthonormal Y_lm(theta, phi), 0 <= m <= l <= lmax, with the Condon-Shortley
    phase, in the order of harmonic_modes (src/extraction.jl:49-81): the normalised
    associated Legendre functions by the three-term recurrence in l from the sectoral
    P_m^m. theta and phi may be arrays; the result has the modes first."""
    theta = np.asarray(theta, dtype=np.float64)
    phi = np.asarray(phi, dtype=np.float64)
    x, y = np.cos(theta), np.sin(theta)
    out = np.empty(((lmax + 1) * (lmax + 2) // 2,) + theta.shape, dtype=np.complex128)
    pmm = np.full(theta.shape, math.sqrt(1 / (4 * math.pi)))
    for m in range(lmax + 1):
        if m > 0:
            pmm = pmm * (-math.sqrt((2 * m + 1) / (2 * m))) * y
        e = np.exp(1j * m * phi)
        out[mode_index(m, m)] = pmm * e
        if m == lmax:
            continue
        p1 = math.sqrt(2 * m + 3) * x * pmm
        out[mode_index(m + 1, m)] = p1 * e
        p0 = pmm
        for l in range(m + 2, lmax + 1):
            a = math.sqrt((4 * l * l - 1) / (l * l - m * m))
            b = math.sqrt(((l - 1) ** 2 - m * m) / (4 * (l - 1) ** 2 - 1))
            p0, p1 = p1, a * (x * p1 - b * p0)
            out[mode_index(l, m)] = p1 * e
    return out


def sphere_rule(lmax, ntheta):
    """The quadrature on the unit sphere (src/extraction.jl:93-119):
    Gauss-Legendre in cos(theta) at ntheta points times nphi = 2 ntheta equally
    spaced phi, point q = i nphi + j. Returns the table w_q conj(Y_lm) (modes x
    points) and the points' directions (points x 3)."""
    nphi = 2 * ntheta
    xg, wg = np.polynomial.legendre.leggauss(ntheta)
    th = np.arccos(xg)
    ph = 2 * math.pi * np.arange(nphi) / nphi
    TH, PH = np.meshgrid(th, ph, indexing="ij")
    W = np.repeat(wg, nphi).reshape(ntheta, nphi) * (2 * math.pi / nphi)
    Y = spherical_harmonics(lmax, TH, PH)                    # (modes, ntheta, nphi)
    table = (W[None] * np.conj(Y)).reshape(Y.shape[0], -1)
    dirs = np.stack([np.sin(TH) * np.cos(PH), np.sin(TH) * np.sin(PH), np.cos(TH)], axis=-1).reshape(-1, 3)
    return table, dirs


# --- the ball's inverse map ---------------------------------------------------
def ball_patch_point(geo, x):
    """The patch (0-based) and logical position of the physical point x of the
    seven-patch ball, the inverse of its map (src/extraction.jl:5-47): a point
    with every coordinate within Lc of the origin is the cube's; any other lies
    in the shell of its largest coordinate k and that coordinate's sign s, on
    the ray through its point f = x Lc / |x_k| on the cube's face, with the
    radial position inverting rho = (|x| - |f|) / (R1 - |f|) and the grading."""
    X = np.asarray(x, dtype=np.float64)
    n, m = geo.roots
    Lc, R1 = geo.Lc, geo.R1
    r = float(np.sqrt(X @ X))
    if r > R1 * (1 + 8 * np.finfo(np.float64).eps):
        raise ValueError("the point %r lies at |x| = %r, beyond the ball's sphere at R1 = %r" % (tuple(X), r, R1))
    a = np.abs(X)
    k = 0 if (a[0] >= a[1] and a[0] >= a[2]) else (1 if a[1] >= a[2] else 2)
    if a[k] <= Lc:
        return 0, tuple(np.clip((X + Lc) * (n / (2 * Lc)), 0.0, float(n)))
    s = 1 if X[k] > 0 else -1
    f = X * (Lc / a[k])
    rf = float(np.sqrt(f @ f))
    rho = min(max((r - rf) / (R1 - rf), 0.0), 1.0)
    al = geo.grading
    eta = rho if al == 0 else math.log1p(rho * math.expm1(al)) / al
    xi = [min(max(n * (f[j] / Lc + 1) / 2, 0.0), float(n)) for j in range(3)]
    xi[k] = min(max(m * eta if s == 1 else m * (1 - eta), 0.0), float(m))
    return 1 + SHELLS.index((k, s)), tuple(xi)


# --- element stencils ----------------------------------------------------------
def _lagrange(nodes, z):
    w = np.ones(len(nodes))
    for j in range(len(nodes)):
        for q in range(len(nodes)):
            if q != j:
                w[j] *= (z - nodes[q]) / (nodes[j] - nodes[q])
    return w


def _lagrange_derivative(nodes, z):
    """d/dz of every Lagrange polynomial through the nodes, at z (the
    product rule over the factors)."""
    n = len(nodes)
    out = np.zeros(n)
    for j in range(n):
        for k in range(n):
            if k == j:
                continue
            term = 1.0 / (nodes[j] - nodes[k])
            for q in range(n):
                if q != j and q != k:
                    term *= (z - nodes[q]) / (nodes[j] - nodes[q])
            out[j] += term
    return out


def _locate_brick(forest, x):
    """The leaf containing the physical point x of a brick and the point's
    position in it scaled to [0, 1]^D."""
    D = forest.D
    lmax = max(lv for lv, _ in forest.leaves)
    cell = []
    for d in range(D):
        lo, hi = forest.lo[d], forest.hi[d]
        if not (lo <= x[d] <= hi):
            raise ValueError("the point %r lies beyond the brick, whose periodic image would be read" % (tuple(x),))
        ext = forest.roots[d] << lmax
        c = min(int(math.floor((x[d] - lo) / (hi - lo) * ext)), ext - 1)
        cell.append(c)
    key = forest._find(lmax, cell)
    lv, c = key
    out = []
    for d in range(D):
        w = (forest.hi[d] - forest.lo[d]) / forest.roots[d] / (1 << lv)
        out.append(min(max((x[d] - (forest.lo[d] + c[d] * w)) / w, 0.0), 1.0))
    return forest._index[key], out


def element_stencils(forest, P, points, geometry=None, deriv=None):
    """Each point's element and its weights, the element's own degree-P
    polynomial through its Gauss-Lobatto nodes (src/extraction.jl:172-214):
    state-vector positions of the (P+1)^D nodes for variable 1 and the
    products of the 1D Lagrange weights, one row per point. With deriv = d
    (a brick only) the weights give the polynomial's derivative along
    dimension d instead (src/transfer.jl:2011-2030). `geometry` is a brick's
    diagonal-metric map, which the extraction cannot invert."""
    from .ball import BallForest
    from .element import Element
    D, N = forest.D, forest.N
    P1, E, NN = P + 1, N // (P + 1), N ** D
    nodes = Element(np.float64, P).nodes.astype(np.float64)
    ball = isinstance(forest, BallForest)
    if ball and not isinstance(forest.geo, SevenPatchBall):
        raise ValueError("the extraction maps physical points to the forest on a brick or the seven-patch "
                         "ball only, not on a %s" % type(forest.geo).__name__)
    if deriv is not None and (ball or not 0 <= deriv < D):
        raise ValueError("the gradient's stencils are a brick's, along a dimension 0..%d" % (D - 1))
    if geometry is not None and not ball:
        raise ValueError("the extraction maps physical points to the forest on a brick or the seven-patch "
                         "ball only, not on a %s" % type(geometry).__name__)
    index = np.empty((len(points), P1 ** D), dtype=np.int64)
    weights = np.empty((len(points), P1 ** D))
    # a ball's leaves by (patch, level, corner): the refined cube's finest
    # leaf holding a point is found from the finest level down
    bindex = ({(p, lv, c): i for i, ((p, c), lv) in enumerate(zip(forest.blocks, forest.levels))}
              if ball else None)
    top = max(forest.levels) if ball else 0
    for j, x in enumerate(points):
        if ball:
            patch, xi = ball_patch_point(forest.geo, x)
            r = forest.geo.patch_roots(patch)
            for lv in range(top, -1, -1):
                s = 1 << lv
                corner = tuple(min(int(math.floor(xi[d] * s)), r[d] * s - 1) for d in range(3))
                b = bindex.get((patch, lv, corner))
                if b is not None:
                    break
            local = [xi[d] * s - corner[d] for d in range(3)]
        else:
            b, local = _locate_brick(forest, x)
        e = [min(int(math.floor(local[d] * E)), E - 1) for d in range(D)]
        W = [_lagrange(nodes, 2 * (local[d] * E - e[d]) - 1) for d in range(D)]
        if deriv is not None:
            # d xi / d x = 2 E over the block's width along deriv
            lo, hi = forest.block_extent(forest.leaves[b])[deriv]
            W[deriv] = _lagrange_derivative(nodes, 2 * (local[deriv] * E - e[deriv]) - 1) * (2 * E / (hi - lo))
        q = 0
        for I in np.ndindex(*([P1] * D)):
            J = I[::-1]                      # first dimension fastest
            pos = sum((e[d] * P1 + J[d]) * N ** d for d in range(D))
            index[j, q] = b * 2 * NN + pos
            weights[j, q] = np.prod([W[d][J[d]] for d in range(D)])
            q += 1
    return index, weights


# --- the extractions ----------------------------------------------------------
class SphereExtraction:
    """SphereExtraction(wave, radii; lmax, ntheta, centre) (src/extraction.jl:121-170):
    the points of spheres of `radii` about `centre`, their stencils on the
    problem's device, and the rule that turns the values there into modes."""

    def __init__(self, p, radii, lmax=6, ntheta=None, centre=(0.0, 0.0, 0.0)):
        if lmax < 0:
            raise ValueError("lmax must be at least 0, got %r" % (lmax,))
        ntheta = 2 * lmax + 12 if ntheta is None else int(ntheta)
        if ntheta <= lmax:
            raise ValueError("ntheta = %d Gauss points in cos(theta) do not integrate the modes up to lmax = %d "
                             "exactly; ntheta must exceed lmax" % (ntheta, lmax))
        radii = [float(r) for r in radii]
        if not all(r > 0 for r in radii):
            raise ValueError("every radius must be positive, got %r" % (radii,))
        self.radii, self.lmax, self.ntheta, self.nphi = radii, int(lmax), ntheta, 2 * ntheta
        self.centre = np.asarray(centre, dtype=np.float64)
        self.table, dirs = sphere_rule(lmax, ntheta)
        self.points = np.concatenate([self.centre[None] + r * dirs for r in radii])
        self._stencil(p, self.points)

    def _stencil(self, p, points):
        import torch
        from .ball import BallForest
        geometry = None if isinstance(p.forest, BallForest) else p.geometry
        index, weights = element_stencils(p.forest, p.P, points, geometry)
        self.nper = index.shape[1]
        self.index = torch.from_numpy(np.ascontiguousarray(index.reshape(-1))).to(p.device)
        self.weights = torch.from_numpy(np.ascontiguousarray(weights.reshape(-1)).astype(p.dtype)).to(p.device)
        self.npoints = len(points)


def stencil_values(ex, p, u, var=1):
    """The gather of sphere_values and plane_values on the device (twoldg_gather):
    each point's nodes of variable `var`, weighted and summed; a host array."""
    import torch
    _check_state(p, u)
    out = torch.empty(ex.npoints, dtype=u.dtype, device=u.device)
    _sync_torch()
    _lib.check(_lib.lib().twoldg_gather(p.handle, _dptr(u), int(var), int(ex.npoints), int(ex.nper),
                                        ctypes.c_void_p(ex.index.data_ptr()), ctypes.c_void_p(ex.weights.data_ptr()),
                                        _dptr(out)))
    p.synchronize()
    return out.cpu().numpy().astype(np.float64)


def sphere_values(ex, p, u, var=1):
    """The values of variable `var` (1: u, 2: v) at the extraction's points
    (src/extraction.jl:216-245), the containing element's own polynomial there."""
    return stencil_values(ex, p, u, var)


def sphere_modes(ex, values_or_problem, u=None, var=1):
    """The modes Phi_lm, one row per mode of harmonic_modes(lmax) and one column
    per radius (src/extraction.jl:247-262), of values at the points or of a state."""
    values = sphere_values(ex, values_or_problem, u, var) if u is not None else np.asarray(values_or_problem)
    npts = ex.table.shape[1]
    if len(values) != npts * len(ex.radii):
        raise ValueError("%d values for %d spheres of %d points each" % (len(values), len(ex.radii), npts))
    return ex.table @ values.reshape(len(ex.radii), npts).T


class PlaneExtraction(SphereExtraction):
    """PlaneExtraction(wave, centre, halfwidth, n) (src/extraction.jl:264-330): the
    cell centres of an n x n grid in the plane z = centre[2], x fastest, and
    their stencils where the forest holds them (`inside`)."""

    def __init__(self, p, centre, halfwidth, n):
        self.centre = np.asarray(centre, dtype=np.float64)
        self.halfwidth, self.n = float(halfwidth), int(n)
        s = self.halfwidth * (2 * np.arange(1, n + 1) - 1 - n) / n
        pts = [(self.centre[0] + s[i], self.centre[1] + s[j], self.centre[2]) for j in range(n) for i in range(n)]
        self.points = np.array(pts)
        from .ball import BallForest
        if isinstance(p.forest, BallForest):
            self.inside = np.linalg.norm(self.points, axis=1) < p.forest.geo.R1
        else:
            f = p.forest
            self.inside = np.all([(self.points[:, d] >= f.lo[d]) & (self.points[:, d] <= f.hi[d])
                                  for d in range(p.D)], axis=0)
        self._stencil(p, self.points[self.inside])


def plane_values(ex, p, u, var=1):
    """The n x n values of the plane (NaN outside the forest), x fastest along the first axis."""
    out = np.full(ex.n * ex.n, np.nan)
    out[ex.inside] = stencil_values(ex, p, u, var)
    return out.reshape(ex.n, ex.n).T
