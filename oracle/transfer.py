"""CPU oracle of the particle-grid transfer (test infrastructure only: the
tests, smoke() and the bench's CPU baseline call it as the checker; the
library never does).

A numpy restatement of the reference's projection of a source onto the nodes
(src/transfer.jl): the far and graded tensor Gauss rules (:462-491, :520-680),
the nested rule split at a particle's support with Gauss points inside and
Johnston and Elliott's sinh rule outside (:233-455), the classification of
elements (:493-503, :1380-1415), the reconstruction (:1990-2009), the ball
rule (:2032-2048), the averaging over shared nodes (:1616-1714), and the
pairing with its support elements and continuous values (:1449-1500,
:1726-1797) for the density kernel (src/dynamic.jl:124-135). Tables come from tests/golden/transfer_tables.json and
element_tables.json (mpmath at 512 bits, rounded once), never from the library
under test. Sums run over flattened point lists where the reference nests
them, which moves results by rounding only.
"""
import json
import math
import os

import numpy as np

from .oracle import golden_tables

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(os.path.dirname(HERE), "tests", "golden", "transfer_tables.json")

RFAR = 9.0
GRADED = ((1.0, 14), (2.0, 10), (3.0, 8), (4.0, 7))
NSINH, NMID, NINNER = 48, 16, 24

_fixture = None


def _load():
    global _fixture
    if _fixture is None:
        with open(GOLDEN) as f:
            _fixture = json.load(f)
    return _fixture


def _f64(bits):
    a = np.asarray(bits, dtype=np.uint64)
    return a.view(np.float64).copy()


def gauss(n):
    """Gauss-Legendre nodes (ascending) and weights of n points (src/transfer.jl:44-62)."""
    r = _load()["rules"].get(str(n))
    if r is None:
        x, w = np.polynomial.legendre.leggauss(n)
        x = (x - x[::-1]) / 2
        return x, w
    return _f64(r["nodes"]["f64"]), _f64(r["weights"]["f64"])


def fixture_table(P, name, kind="f64"):
    """A transfer table of order P from the fixture ('bary', 'lagrange_q', 'contract_q')."""
    v = _load()["orders"][str(P)][name][kind]
    if kind == "f64":
        return _f64(v)
    return np.asarray(v, dtype=np.uint32).view(np.float32).copy()


def gauss_bits(n, what, kind):
    """The fixture's raw bits of rule n ('nodes' / 'weights', 'f64' / 'f32')."""
    return np.asarray(_load()["rules"][str(n)][what][kind], dtype=np.uint64 if kind == "f64" else np.uint32)


class Tables:
    """TransferTables(Float64, P) (src/transfer.jl:107-170) with the
    reference's defaults, or the quadrature given."""

    def __init__(self, P, q=None, graded=GRADED, rfar=RFAR, nsinh=NSINH, nmid=NMID, ninner=NINNER):
        el = golden_tables(P)
        self.P = P
        self.nodes = el["nodes"].astype(np.float64)
        self.weights = el["weights"].astype(np.float64)
        P1 = P + 1
        self.bary = np.array([1.0 / np.prod([self.nodes[i] - self.nodes[j] for j in range(P1) if j != i])
                              for i in range(P1)])
        self.q = q if q is not None else P + 3
        self.far = self.rule(self.q)
        self.graded = [self.rule(n) for _, n in graded]
        self.gradedfrom = [float(d) for d, _ in graded]
        self.rfar = float(rfar)
        self.sinh = gauss(nsinh)
        self.mid = gauss(nmid)
        self.inner = gauss(ninner)

    def rule(self, n):
        """(nodes, weights, contract[i][k] = w_k phi_i(x_k) / w^_i) of an n-point Gauss rule."""
        x, w = gauss(n)
        lag = self.lagrange_values(x)                 # (n, P+1)
        con = (w[:, None] * lag / self.weights[None, :]).T
        return x, w, con

    def lagrange_values(self, xi):
        """phi_i(xi) in the product form bary_i prod_{j != i} (xi - x^_j) (src/transfer.jl:171-182)."""
        xi = np.asarray(xi, dtype=np.float64)
        P1 = self.P + 1
        out = np.empty(xi.shape + (P1,))
        for i in range(P1):
            acc = np.full(xi.shape, self.bary[i])
            for j in range(P1):
                if j != i:
                    acc = acc * (xi - self.nodes[j])
            out[..., i] = acc
        return out

    def lagrange_derivatives(self, xi):
        xi = np.asarray(xi, dtype=np.float64)
        P1 = self.P + 1
        out = np.zeros(xi.shape + (P1,))
        for i in range(P1):
            for k in range(P1):
                if k == i:
                    continue
                term = np.full(xi.shape, self.bary[i])
                for j in range(P1):
                    if j != i and j != k:
                        term = term * (xi - self.nodes[j])
                out[..., i] += term
        return out

    def element_basis(self, lo, hi, X, deriv=-1):
        """phi_n(x) of every node of the element [lo, hi] at the points X
        (npts, D), node index with dimension 0 fastest (src/transfer.jl:204-217)."""
        X = np.atleast_2d(np.asarray(X, dtype=np.float64))
        D = X.shape[1]
        out = np.ones((X.shape[0], 1))
        for d in range(D):
            xi = (2 * X[:, d] - lo[d] - hi[d]) / (hi[d] - lo[d])
            f = (self.lagrange_derivatives(xi) * (2 / (hi[d] - lo[d]))) if d == deriv else self.lagrange_values(xi)
            # dimension d varies slower than every earlier one
            out = (f[:, :, None] * out[:, None, :]).reshape(X.shape[0], -1)
        return out

    def element_weights(self, he, D):
        w = self.weights * (he / 2)
        out = np.ones(1)
        for _ in range(D):
            out = (w[:, None] * out[None, :]).reshape(-1)
        return out


class Support:
    """ParticleSupport(z, v, ell) (src/transfer.jl:264-290)."""

    def __init__(self, z, v, ell):
        self.z = np.asarray(z, dtype=np.float64)
        self.v = np.asarray(v, dtype=np.float64)
        self.ell = float(ell)


def box_distance2(x, lo, hi, dims):
    acc = 0.0
    for d in dims:
        delta = max(lo[d] - x[d], x[d] - hi[d], 0.0)
        acc += delta * delta
    return acc


def support_breaks(s, prefix, lo, hi):
    """support_breaks (src/transfer.jl:302-366)."""
    D = len(s.z)
    F = len(prefix)
    d = F
    g2 = 1 / (1 - float(np.dot(s.v, s.v)))
    r2F = sum((prefix[j] - s.z[j]) ** 2 for j in range(F))
    vrF = sum(s.v[j] * (prefix[j] - s.z[j]) for j in range(F))
    breaks, extent = [], None
    for code in range(3 ** (D - d - 1)):
        r2, vr, vfree, c = r2F, vrF, 0.0, code
        for j in range(d + 1, D):
            c, k = divmod(c, 3)
            if k == 0:
                vfree += s.v[j] ** 2
            else:
                f = (lo[j] if k == 1 else hi[j]) - s.z[j]
                r2 += f * f
                vr += s.v[j] * f
        cc = g2 / (1 + g2 * vfree)
        A = 1 + cc * s.v[d] ** 2
        B = cc * vr * s.v[d]
        C = r2 + cc * vr ** 2 - s.ell ** 2
        disc = B * B - A * C
        if not disc > 0:
            continue
        q = math.sqrt(disc)
        x1 = s.z[d] + (-B - q) / A
        x2 = s.z[d] + (-B + q) / A
        if code == 0:
            extent = (x1, x2)
        if lo[d] < x1 < hi[d]:
            breaks.append(x1)
        if lo[d] < x2 < hi[d]:
            breaks.append(x2)
    return sorted(breaks), extent


def inner_points(t, a, b, plain):
    u, w = t.inner
    half = (b - a) / 2
    th = math.pi * (1 + u) / 2
    if plain:
        return a + half * (1 + u), w * half
    return a + half * (1 - np.cos(th)), w * math.pi / 2 * half * np.sin(th)


def sinh_points(rule, a, b, c, beta):
    nodes, weights = rule
    half, mid = (b - a) / 2, (a + b) / 2
    xc, eps = (c - mid) / half, beta / half
    lo_, hi_ = math.asinh((1 + xc) / eps), math.asinh((1 - xc) / eps)
    mu, eta = (hi_ + lo_) / 2, (lo_ - hi_) / 2
    return mid + half * (xc + eps * np.sinh(mu * nodes - eta)), weights * eps * mu * np.cosh(mu * nodes - eta) * half


def line_segments(s, t, lo, hi, prefix, innermost, compact):
    """The segments of one line of the nested rule (LINE_FOLD, src/transfer.jl:368-412)."""
    D = len(s.z)
    d = len(prefix)
    breaks, extent = support_breaks(s, prefix, lo, hi)
    off2 = box_distance2(s.z, lo, hi, range(d + 1, D)) + sum((prefix[j] - s.z[j]) ** 2 for j in range(d))
    out = []
    a = lo[d]
    for b in breaks + [hi[d]]:
        if b > a:
            mid = (a + b) / 2
            if extent is not None and extent[0] < mid < extent[1]:
                out.append(inner_points(t, a, b, innermost))
            elif not compact:
                c = min(max(s.z[d], a), b)
                beta = max(math.sqrt(off2 + (s.z[d] - c) ** 2), np.finfo(np.float64).eps * (b - a))
                out.append(sinh_points(t.mid if beta >= (b - a) / 2 else t.sinh, a, b, c, beta))
        a = b
    return out


def nested_points(s, t, lo, hi, D, compact=False):
    """Every point of the nested rule over the box and its weight, the
    product of its lines' weights (collect_points!, src/transfer.jl:1302-1328)."""
    xs, ws = [], []

    def visit(prefix, w, n):
        for lx, lw in line_segments(s, t, lo, hi, prefix, n == 1, compact):
            if n == 1:
                pts = np.empty((len(lx), D))
                pts[:, :len(prefix)] = prefix
                pts[:, len(prefix)] = lx
                xs.append(pts)
                ws.append(w * lw)
            else:
                for xk, wk in zip(lx, lw):
                    visit(prefix + [float(xk)], w * wk, n - 1)

    visit([], 1.0, D)
    if not xs:
        return np.zeros((0, D)), np.zeros(0)
    return np.concatenate(xs), np.concatenate(ws)


def nested_rule(f, s, t, lo, hi, D, compact=False):
    """sum w f(x) over the nested rule's points; f maps (npts, D) to (npts, ...)."""
    X, W = nested_points(s, t, lo, hi, D, compact)
    if len(W) == 0:
        return 0.0
    vals = f(X)
    return np.tensordot(W, vals, axes=(0, 0))


def tensor_rule(S, rule, lo, hi, D):
    """The tensor Gauss rule over [lo, hi], contracted one dimension at a time:
    P S at the element's nodes (src/transfer.jl:490-491, 592-621)."""
    x, _, con = rule
    q = len(x)
    grids = [lo[d] + (hi[d] - lo[d]) * (1 + x) / 2 for d in range(D)]
    mesh = np.meshgrid(*grids, indexing="ij")            # axis d = dimension d
    X = np.stack([m.reshape(-1) for m in mesh], axis=1)
    vals = np.asarray(S(X), dtype=np.float64).reshape((q,) * D)
    for d in range(D):
        vals = np.moveaxis(np.tensordot(con, vals, axes=(1, d)), 0, d)
    # node order with dimension 0 fastest
    return np.transpose(vals, tuple(range(D - 1, -1, -1))).reshape(-1)


def particle_density(X, z, v, ell, charge):
    """Q rho0(|L(v)(x - z)|^2, ell) (src/particle.jl:117-127; src/particle_forms.jl:29-37)."""
    X = np.atleast_2d(X)
    z = np.asarray(z, dtype=np.float64)
    v = np.asarray(v, dtype=np.float64)
    r = X - z[None, :]
    gamma = 1 / math.sqrt(1 - float(np.dot(v, v)))
    y = r + (gamma ** 2 / (gamma + 1) * (r @ v))[:, None] * v[None, :]
    q = np.sum(y * y, axis=1)
    u = 1 - q / ell ** 2
    rho = (3465 / 512) * u ** 4 / ell ** 3 / math.pi
    return charge * np.where(q < ell ** 2, rho, 0.0)


def ball_rule(n_r, n_theta):
    """ball_rule(T, n_r, n_theta) (src/transfer.jl:2032-2048): points and weights of
    a cubature of the unit ball, r^2 in the weights."""
    xr, wr = gauss(n_r)
    xm, wm = gauss(n_theta)
    n_phi = 2 * n_theta
    pts, wts = [], []
    for i in range(n_r):
        r = (1 + xr[i]) / 2
        for j in range(n_theta):
            st = math.sqrt(1 - xm[j] ** 2)
            for k in range(n_phi):
                phi = 2 * math.pi * k / n_phi
                pts.append((r * st * math.cos(phi), r * st * math.sin(phi), r * xm[j]))
                wts.append(wr[i] / 2 * r * r * wm[j] * 2 * math.pi / n_phi)
    return np.array(pts), np.array(wts)


class Mesh:
    """What the projection reads of a forest: each block's origin and node
    spacing in the particles' frame, N, P, E, D, and the frame's blocks."""

    def __init__(self, origins, spacings, P, E, mask=None):
        self.origins = np.asarray(origins, dtype=np.float64)
        self.spacings = np.asarray(spacings, dtype=np.float64)
        self.nblocks, self.D = self.origins.shape
        self.P, self.E = P, E
        self.N = E * (P + 1)
        self.NN = self.N ** self.D
        self.mask = np.ones(self.nblocks, dtype=bool) if mask is None else np.asarray(mask, dtype=bool)

    def element_box(self, b, e):
        P1 = self.P + 1
        lo = [self.origins[b, d] + self.spacings[b] * (e[d] * P1) for d in range(self.D)]
        hi = [self.origins[b, d] + self.spacings[b] * ((e[d] + 1) * P1) for d in range(self.D)]
        return lo, hi

    def node_index(self, b, e, var):
        """State-vector positions of the element's nodes, dimension 0 fastest."""
        P1, N, D = self.P + 1, self.N, self.D
        idx = np.zeros(1, dtype=np.int64)
        for d in range(D):
            col = (e[d] * P1 + np.arange(P1)) * N ** d
            idx = (col[:, None] + idx[None, :]).reshape(-1)
        return b * 2 * self.NN + (var - 1) * self.NN + idx

    def elements(self):
        for b in range(self.nblocks):
            for J in np.ndindex(*([self.E] * self.D)):
                yield b, tuple(reversed(J))


def classify(mesh, t, particles, ball, rnear, he):
    """host_elements (src/transfer.jl:1380-1415): far, graded per band, near (with its particle)."""
    D = mesh.D
    c, R = np.asarray(ball[0], dtype=np.float64), float(ball[1])
    rn, rf = rnear * he, t.rfar * he
    far, graded, near = [], [[] for _ in t.graded], []
    for b in range(mesh.nblocks):
        if not mesh.mask[b]:
            continue
        blo = mesh.origins[b]
        bhi = blo + mesh.spacings[b] * mesh.N
        if not box_distance2(c, blo, bhi, range(D)) < R * R:
            continue
        for J in np.ndindex(*([mesh.E] * D)):
            e = tuple(reversed(J))
            lo, hi = mesh.element_box(b, e)
            if box_distance2(c, lo, hi, range(D)) >= R * R:
                continue
            d2 = [box_distance2(s.z, lo, hi, range(D)) for s in particles]
            if not any(x < rf * rf for x in d2):
                far.append((b, e))
                continue
            k = int(np.argmin(d2))
            if d2[k] >= rn * rn:
                delta = math.sqrt(d2[k]) / he
                band = 0
                for i, f in enumerate(t.gradedfrom):
                    if f <= delta:
                        band = i
                graded[band].append((b, e))
                continue
            if sum(x < s.ell ** 2 for x, s in zip(d2, particles)) > 1:
                raise ValueError("the supports of two particles meet the element at %r" % (tuple(lo),))
            near.append((b, e, k))
    return far, graded, near


def project_source(du, mesh, t, S, particles, ball, rnear=1.0, factor=-1.0, var=2, he=None):
    """project_source!(du, p, t, S, particles; ball, rnear, factor, var)
    (src/transfer.jl:918-944) on a flat state vector du (numpy, float64): S
    maps points (npts, D) to values. Returns du."""
    D = mesh.D
    P1 = mesh.P + 1
    if he is None:
        he = float(np.min(mesh.spacings[mesh.mask])) * P1
    if not 0 <= rnear <= t.rfar:
        raise ValueError("rnear = %r must lie between 0 and rfar = %r" % (rnear, t.rfar))
    far, graded, near = classify(mesh, t, particles, ball, rnear, he)
    for rule, lst in [(t.far, far)] + list(zip(t.graded, graded)):
        for b, e in lst:
            lo, hi = mesh.element_box(b, e)
            du[mesh.node_index(b, e, var)] += factor * tensor_rule(S, rule, lo, hi, D)
    wn = t.element_weights(he, D)
    for b, e, k in near:
        lo, hi = mesh.element_box(b, e)
        vals = nested_rule(lambda X: np.asarray(S(X))[:, None] * t.element_basis(lo, hi, X),
                           particles[k], t, lo, hi, D)
        du[mesh.node_index(b, e, var)] += factor * vals / wn
    return du


def brick_mesh(D, P, E, roots, L=1.0, lo=0.0):
    """A uniform brick of roots^D blocks over [lo, lo + L]^D, blocks listed
    with dimension 0 fastest."""
    n = roots
    w = L / n
    origins, spacings = [], []
    for J in np.ndindex(*([n] * D)):
        c = tuple(reversed(J))
        origins.append([lo + c[d] * w for d in range(D)])
        spacings.append(w / (E * (P + 1)))
    return Mesh(origins, spacings, P, E)


def weighted_inner(mesh, t, a, b, var):
    """<a, b>_w over variable var: sum_n w_n a_n b_n with w_n the node's quadrature weight."""
    D = mesh.D
    P1 = mesh.P + 1
    acc = 0.0
    for blk in range(mesh.nblocks):
        he = mesh.spacings[blk] * P1
        wn = t.element_weights(he, D)
        for J in np.ndindex(*([mesh.E] * D)):
            e = tuple(reversed(J))
            idx = mesh.node_index(blk, e, var)
            acc += float(np.sum(wn * a[idx] * b[idx]))
    return acc


def average_shared(u, mesh, ball, var):
    """average_shared!(ua, sn, var) (src/transfer.jl:1616-1714) on the flat
    state vector u (numpy, in place): in the frame's blocks that the ball
    meets, D passes; in pass d every pair of coincident nodes across a face
    along d -- between a block's elements, and across its upper face to the
    ball's block there on the same level -- takes their mean, the lower
    node's value first. No periodic images."""
    D, N, P1, E = mesh.D, mesh.N, mesh.P + 1, mesh.E
    c, R = np.asarray(ball[0], dtype=np.float64), float(ball[1])
    lo = mesh.origins
    hi = mesh.origins + mesh.spacings[:, None] * N
    blocks = [b for b in range(mesh.nblocks)
              if mesh.mask[b] and box_distance2(c, lo[b], hi[b], range(D)) < R * R]
    member = set(blocks)

    def across(b, d):
        h = mesh.spacings[b]
        x = [lo[b, k] + h * N / 2 if k != d else lo[b, k] + h * (N + 0.5) for k in range(D)]
        for g in range(mesh.nblocks):
            if mesh.mask[g] and all(lo[g, k] <= x[k] < hi[g, k] for k in range(D)):
                return g if g in member and mesh.spacings[g] == h else None
        return None

    U = u.reshape(mesh.nblocks, 2, mesh.NN)
    for d in range(D):
        ax = D - 1 - d              # dimension d is axis D-1-d of a block's (N,)*D view
        for b in blocks:
            a = U[b, var - 1].reshape((N,) * D)
            for k in range(1, E):
                i1 = [slice(None)] * D
                i2 = [slice(None)] * D
                i1[ax], i2[ax] = k * P1 - 1, k * P1
                m = (a[tuple(i1)] + a[tuple(i2)]) / 2
                a[tuple(i1)] = m
                a[tuple(i2)] = m
            bn = across(b, d)
            if bn is not None:
                an = U[bn, var - 1].reshape((N,) * D)
                i1 = [slice(None)] * D
                i2 = [slice(None)] * D
                i1[ax], i2[ax] = N - 1, 0
                m = (a[tuple(i1)] + an[tuple(i2)]) / 2
                a[tuple(i1)] = m
                an[tuple(i2)] = m
    return u


def density_kernel(X, z, v, ell, charge):
    """(grad rho, rho) of one particle at the points X (npts, 3), as (npts, 4):
    particle_density and its gradient (src/particle.jl:117-127; density_kernel,
    src/dynamic.jl:124-135): y = L(v)(x - z), rho = Q rho0(y.y),
    grad rho = L(v)(2 Q rho0'(y.y) y), L symmetric."""
    X = np.atleast_2d(np.asarray(X, dtype=np.float64))
    z = np.asarray(z, dtype=np.float64)
    v = np.asarray(v, dtype=np.float64)
    gamma = 1 / math.sqrt(1 - float(np.dot(v, v)))
    g = gamma ** 2 / (gamma + 1)
    r = X - z[None, :]
    y = r + (g * (r @ v))[:, None] * v[None, :]
    q = np.sum(y * y, axis=1)
    inside = q < ell ** 2
    u = np.where(inside, 1 - q / ell ** 2, 0.0)
    c = (3465 / 512) / ell ** 3 / math.pi
    rho = charge * c * u ** 4
    drho = -4 * charge * c * u ** 3 / ell ** 2
    w = 2 * drho[:, None] * y
    grad = w + (g * (w @ v))[:, None] * v[None, :]
    return np.concatenate([grad, rho[:, None]], axis=1)


def frame_domain(mesh):
    """The frame's box: the hull of its blocks."""
    lo = mesh.origins[mesh.mask].min(axis=0)
    hi = (mesh.origins[mesh.mask] + mesh.spacings[mesh.mask][:, None] * mesh.N).max(axis=0)
    return lo, hi


def locate_element(mesh, x):
    """locate_element (src/transfer.jl:1417-1431): the frame's block that holds
    x, and the element there, clamped to the block."""
    P1 = mesh.P + 1
    for b in range(mesh.nblocks):
        if not mesh.mask[b]:
            continue
        lo = mesh.origins[b]
        hi = lo + mesh.spacings[b] * mesh.N
        if all(lo[d] <= x[d] < hi[d] for d in range(mesh.D)):
            e = tuple(min(max(int(math.floor((x[d] - lo[d]) / (mesh.spacings[b] * P1))), 0), mesh.E - 1)
                      for d in range(mesh.D))
            return b, e
    raise ValueError("the point %r is outside the domain" % (tuple(x),))


def support_elements(mesh, s, he):
    """support_elements (src/transfer.jl:1726-1758): the elements that hold a
    corner of the box [z - ell, z + ell], in the corners' order (dimension 0
    fastest, the lower side first)."""
    D = mesh.D
    if not 2 * s.ell < he:
        raise ValueError("the particle's support, 2l = %r across, is not smaller than an element, h_e = %r"
                         % (2 * s.ell, he))
    dlo, dhi = frame_domain(mesh)
    if not all(dlo[d] <= s.z[d] - s.ell and s.z[d] + s.ell < dhi[d] for d in range(D)):
        raise ValueError("the particle's support around z = %r reaches past the domain's faces; the transfer "
                         "does not look for periodic images" % (tuple(s.z),))
    out = []
    for corner in range(1 << D):
        x = [s.z[d] + (s.ell if (corner >> d) & 1 else -s.ell) for d in range(D)]
        be = locate_element(mesh, x)
        if be not in out:
            out.append(be)
    return out


def continuous_values(u, mesh, b, e, var):
    """continuous_values (src/transfer.jl:1449-1500): the element's nodal
    values of var with every node on its boundary replaced by the mean over
    the elements that share it (the element's own value first, then its
    neighbours with dimension 0 varying fastest); the neighbours on the same
    level, no periodic images."""
    D, E, P, P1 = mesh.D, mesh.E, mesh.P, mesh.P + 1
    lo, hi = mesh.element_box(b, e)
    dlo, dhi = frame_domain(mesh)

    def neighbour(s):
        en = tuple(e[d] + s[d] for d in range(D))
        if all(0 <= en[d] < E for d in range(D)):
            return b, en
        x = [(lo[d] + hi[d]) / 2 + s[d] * (hi[d] - lo[d]) for d in range(D)]
        if not all(dlo[d] < x[d] < dhi[d] for d in range(D)):
            raise ValueError("the element at %r is on the domain's face; the continuous reconstruction, like the "
                             "transfer, does not look for periodic images" % (tuple(lo),))
        bn, en = locate_element(mesh, x)
        if mesh.spacings[bn] != mesh.spacings[b]:
            raise ValueError("the element at %r has a neighbour on another level; the continuous reconstruction "
                             "needs the same level across every face" % (tuple(lo),))
        return bn, en

    U = u.reshape(mesh.nblocks, 2, mesh.NN)
    N = mesh.N

    def read(bn, en, K):
        return U[bn, var - 1, sum((en[d] * P1 + K[d]) * N ** d for d in range(D))]

    out = []
    for J in np.ndindex(*([P1] * D)):
        K = tuple(reversed(J))                   # dimension 0 fastest
        dirs = [-1 if K[d] == 0 else (1 if K[d] == P else 0) for d in range(D)]
        acc, count = read(b, e, K), 1
        free = [d for d in range(D) if dirs[d] != 0]
        for code in range(1, 1 << len(free)):
            s = [0] * D
            for i, d in enumerate(free):
                if (code >> i) & 1:
                    s[d] = dirs[d]
            bn, en = neighbour(s)
            Kn = tuple(K[d] if s[d] == 0 else (P if s[d] < 0 else 0) for d in range(D))
            acc += read(bn, en, Kn)
            count += 1
        out.append(acc / count)
    return np.array(out)


def pairing(u, mesh, t, K, s, var=1, continuous=False, he=None):
    """pairing(p, t, u, K, s; var, continuous) (src/transfer.jl:1779-1797):
    int K g_h over the support's elements, each by the nested rule kept to the
    support (compact), g_h the element's polynomial of var (made continuous
    first with continuous=True). K maps points (npts, D) to (npts, C)."""
    D = mesh.D
    if he is None:
        he = float(np.min(mesh.spacings[mesh.mask])) * (mesh.P + 1)
    acc = 0.0
    for b, e in support_elements(mesh, s, he):
        lo, hi = mesh.element_box(b, e)
        g = continuous_values(u, mesh, b, e, var) if continuous else u[mesh.node_index(b, e, var)]
        acc = acc + nested_rule(lambda X: np.asarray(K(X)) * (t.element_basis(lo, hi, X) @ g)[:, None],
                                s, t, lo, hi, D, compact=True)
    return acc
