"""The seven-patch ball: a full-metric geometry with quarter-turn glue.

SevenPatchBall (src/geometry.jl:270-553) maps a cube [-Lc, Lc]^3 (patch 1,
n^3 roots) and six shells over its faces (patches 2-7, m roots along the
radial dimension k and n along the others) onto the ball |x| <= R1. The
shells' metric is neither diagonal nor separable, so the problem holds the
gradient in Cartesian components, V = grad u, and the flux through a face
normal to d is S[d] . V with the area vectors S[d] = sqrt(g) grad xi^d
(src/evolution.jl:112-220). The outer sphere takes Dirichlet data: the plane
wave u = sin(k . x - |k| t + phi) (src/sevenpatch.jl:9-59).

The forest here is explicit: seven patches of root blocks, and for every
block face its neighbour block, the neighbour's face and the orientation
of the face plane across the glue, found by matching the physical
positions of the face nodes on both sides (the glue's axis maps are quarter
turns between shells; continuity of the physical coordinates across every
glued face is what fixes them). Faces on the sphere are boundary faces.
"""
import math

import numpy as np


class Dual:
    """Forward-mode dual numbers over numpy arrays: a value and its
    derivatives with respect to the three logical coordinates."""

    __array_priority__ = 1000

    def __init__(self, v, d):
        self.v = np.asarray(v, dtype=np.float64)
        self.d = [np.asarray(x, dtype=np.float64) for x in d]

    @staticmethod
    def lift(x):
        return x if isinstance(x, Dual) else Dual(x, [np.zeros_like(np.asarray(x, dtype=np.float64))] * 3)

    def __add__(self, o):
        o = Dual.lift(o)
        return Dual(self.v + o.v, [a + b for a, b in zip(self.d, o.d)])

    __radd__ = __add__

    def __neg__(self):
        return Dual(-self.v, [-a for a in self.d])

    def __sub__(self, o):
        return self + (-Dual.lift(o))

    def __rsub__(self, o):
        return Dual.lift(o) + (-self)

    def __mul__(self, o):
        o = Dual.lift(o)
        return Dual(self.v * o.v, [a * o.v + self.v * b for a, b in zip(self.d, o.d)])

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = Dual.lift(o)
        return Dual(self.v / o.v, [(a * o.v - self.v * b) / (o.v * o.v) for a, b in zip(self.d, o.d)])

    def __rtruediv__(self, o):
        return Dual.lift(o) / self


def dsqrt(x):
    if not isinstance(x, Dual):
        return np.sqrt(x)
    s = np.sqrt(x.v)
    return Dual(s, [a / (2 * s) for a in x.d])


def dexp(x):
    if not isinstance(x, Dual):
        return np.exp(x)
    e = np.exp(x.v)
    return Dual(e, [a * e for a in x.d])


# the shells' cube faces (k, s), in patch order 2-7 (src/geometry.jl:366)
SHELLS = ((0, -1), (0, 1), (1, -1), (1, 1), (2, -1), (2, 1))


class SevenPatchBall:
    """The seven-patch ball map (src/geometry.jl:270-455), dimensions 0-based."""

    def __init__(self, Lc, R1, roots, grading=0.0):
        if not Lc > 0:
            raise ValueError("the cube's half-width Lc must be positive, got %r" % (Lc,))
        if not R1 > math.sqrt(3) * Lc:
            raise ValueError("the outer radius R1 = %r must exceed sqrt(3) Lc = %r, so that the cube's corners "
                             "lie inside the sphere and every shell maps one to one" % (R1, math.sqrt(3) * Lc))
        if not all(r > 0 for r in roots):
            raise ValueError("every patch of the ball needs a positive number of roots, got %r" % (roots,))
        self.Lc, self.R1 = float(Lc), float(R1)
        self.roots = tuple(int(r) for r in roots)
        self.grading = float(grading)

    def patch_roots(self, p):
        n, m = self.roots
        if p == 0:
            return (n, n, n)
        k, _ = SHELLS[p - 1]
        return tuple(m if j == k else n for j in range(3))

    def shell_fraction(self, eta):
        a = self.grading
        if a == 0:
            return eta
        return (dexp(a * eta) - 1) / (math.exp(a) - 1)

    def position(self, xi, p):
        """Physical position of logical xi (a 3-tuple of arrays or Duals) of patch p (0-based)."""
        n, m = self.roots
        Lc = self.Lc
        if p == 0:
            return tuple((2 * Lc / n) * xi[j] - Lc for j in range(3))
        k, s = SHELLS[p - 1]
        f = [s * Lc * (xi[j] * 0 + 1) if j == k else Lc * (2 * xi[j] / n - 1) for j in range(3)]
        eta = xi[k] / m if s == 1 else 1 - xi[k] / m
        rho = self.shell_fraction(eta)
        norm = dsqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2])
        return tuple((1 - rho) * f[j] + (rho * self.R1 / norm) * f[j] for j in range(3))

    def frame(self, xi, p):
        return map_frame(self, xi, p)

    def outer_radius(self):
        return self.R1

    npatches = 7

    def affine_patch(self, p):
        return p == 0

    def factored_dim(self, p):
        """The dimension along which sqrt(g) splits on patch p, or -1: on no
        patch of the seven-patch ball (src/geometry.jl:123-135)."""
        return -1


def map_frame(geo, xi, p):
    """sqrt(g) and the area vectors S[d][i] = sqrt(g) d xi^d / d x^i at logical xi
    of patch p (src/geometry.jl:402-409, 655-662), by forward-mode
    differentiation of the geometry's map."""
    shape = np.shape(xi[0])
    duals = [Dual(xi[j], [np.ones(shape) if q == j else np.zeros(shape) for q in range(3)]) for j in range(3)]
    x = geo.position(duals, p)
    Jm = np.empty(shape + (3, 3))
    for i in range(3):
        xi_ = Dual.lift(x[i])
        for j in range(3):
            Jm[..., i, j] = np.broadcast_to(xi_.d[j], shape)
    J = np.abs(np.linalg.det(Jm))
    Ji = np.linalg.inv(Jm)               # Ji[d, i] = d xi^d / d x^i
    S = J[..., None, None] * Ji          # S[..., d, i]
    return J, S


class ThirteenPatchBall:
    """The thirteen-patch ball (src/geometry.jl:555-717), patches 0-based:
    the seven-patch ball out to the middle sphere |x| = Rm (patches 0-6,
    roots (n, m)), and six outer shells over the same cube faces (patches
    7-12, m' roots along the radial dimension k and n across it) whose
    radial coordinate is exactly radial: c_k = s, c_j = 2 xi_j / n - 1,
    rho = xi_k / m' (s = 1) or 1 - xi_k / m' (s = -1), x = (Rm + (R1 - Rm) rho)
    c / |c|. On an outer shell sqrt(g) = r^2 r' (2/n)^2 (1 + c_a^2 + c_b^2)^(-3/2),
    a radial factor times an angular one that is the same on all six."""

    npatches = 13

    def __init__(self, Lc, Rm, R1, roots):
        if not Lc > 0:
            raise ValueError("the cube's half-width Lc must be positive, got %r" % (Lc,))
        if not Rm > math.sqrt(3) * Lc:
            raise ValueError("the middle radius Rm = %r must exceed sqrt(3) Lc = %r, so that the cube's corners lie "
                             "inside the middle sphere and every inner shell maps one to one"
                             % (Rm, math.sqrt(3) * Lc))
        if not R1 > Rm:
            raise ValueError("the outer radius R1 = %r must exceed the middle radius Rm = %r" % (R1, Rm))
        if len(roots) != 3:
            raise ValueError("the thirteen-patch ball takes roots = (n, m, m'), the cube's per side and the inner "
                             "and outer shells' radial ones, got %r" % (tuple(roots),))
        if not all(r > 0 for r in roots):
            raise ValueError("every patch of the ball needs a positive number of roots along each dimension, "
                             "got %r" % (tuple(roots),))
        self.Lc, self.Rm, self.R1 = float(Lc), float(Rm), float(R1)
        self.roots = tuple(int(r) for r in roots)
        self.inner = SevenPatchBall(Lc, Rm, self.roots[:2])

    def patch_roots(self, p):
        if p < 7:
            return self.inner.patch_roots(p)
        n, _, m2 = self.roots
        k, _ = SHELLS[p - 7]
        return tuple(m2 if j == k else n for j in range(3))

    def outer_radius_at(self, xk, s):
        m2 = self.roots[2]
        rho = xk / m2 if s == 1 else 1 - xk / m2
        return self.Rm + (self.R1 - self.Rm) * rho

    def position(self, xi, p):
        if p < 7:
            return self.inner.position(xi, p)
        n = self.roots[0]
        k, s = SHELLS[p - 7]
        c = [s * (xi[j] * 0 + 1) if j == k else 2 * xi[j] / n - 1 for j in range(3)]
        norm = dsqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2])
        r = self.outer_radius_at(xi[k], s)
        return tuple((r / norm) * c[j] for j in range(3))

    def frame(self, xi, p):
        return map_frame(self, xi, p)

    def outer_radius(self):
        return self.R1

    def affine_patch(self, p):
        return p == 0

    def factored_dim(self, p):
        """The radial dimension of an outer shell, along which sqrt(g) splits
        (src/geometry.jl:671); -1 elsewhere."""
        return SHELLS[p - 7][0] if p >= 7 else -1

    def radial_volume(self, xk, p):
        """r^2 r' at the radial coordinate xk of outer shell p (src/geometry.jl:675-679)."""
        _, s = SHELLS[p - 7]
        r = self.outer_radius_at(xk, s)
        return r * r * ((self.R1 - self.Rm) / self.roots[2])

    def angular_volume(self, xa, xb):
        """(2/n)^2 (1 + c_a^2 + c_b^2)^(-3/2), the gnomonic area element, at the two
        coordinates across the radial one (src/geometry.jl:681-687)."""
        n = self.roots[0]
        ca, cb = 2 * xa / n - 1, 2 * xb / n - 1
        q = 1 + ca * ca + cb * cb
        return (2.0 / n) ** 2 / (q * np.sqrt(q))

class BallForest:
    """The forest of a ball: its patches' blocks and the explicit face table.
    Blocks are ordered patch by patch, and within a patch by corner with the
    first dimension fastest; a refined cube (patch 0) holds its leaves in the
    Morton order of a refined box. Every root block has logical extent 1, a
    block of level L 2^-L, and `levels` holds each block's level (only the
    affine cube refines); `leaves` pairs it with the corner, counted in
    blocks of that level."""

    def __init__(self, geo, N):
        self.geo = geo
        self.D = 3
        self.N = int(N)
        self.blocks = []                    # (patch, corner)
        for p in range(geo.npatches):
            r = geo.patch_roots(p)
            for c2 in range(r[2]):
                for c1 in range(r[1]):
                    for c0 in range(r[0]):
                        self.blocks.append((p, (c0, c1, c2)))
        self.levels = [0] * len(self.blocks)
        self.leaves = [(0, c) for _, c in self.blocks]
        self.refined = False
        self.face_nb = None
        self.face_code = None

    def nleaves(self):
        return len(self.blocks)

    def spacing(self, key=None):
        return (1.0 if key is None else 2.0 ** -key[0]) / self.N

    def minimum_spacing(self):
        return 2.0 ** -max(self.levels) / self.N

    def block_scale(self, b):
        """The logical extent of block b: 2^-level."""
        return 2.0 ** -self.levels[b]


def refine_cube(forest, refined):
    """The ball's cube (patch 0, n roots per side) refined as wave_forest
    refines a box (src/geometry.jl:540-553): `refined` is True (the middle
    half, (n/4, 3n/4)^3), a tuple of three intervals (one region), or a list
    of such tuples (one region per level), in the cube's logical coordinates
    [0, n]^3, each level balanced 2:1 across faces, edges and corners. The
    glue keeps the leaves across a glued face at one level, so a refinement
    that reaches the cube's faces would refine a shell, whose map is not
    affine, and is refused."""
    from .forest import Forest, refine_regions, refinement_regions
    n = forest.geo.patch_roots(0)[0]
    cube = Forest([n] * 3, forest.N, [0.0] * 3, [float(n)] * 3, [False] * 3, [True] * 3)
    refine_regions(cube, refinement_regions(refined, 3, float(n)), n)
    for lv, c in cube.leaves:
        if lv > 0 and any(c[k] == 0 or c[k] == (n << lv) - 1 for k in range(3)):
            raise ValueError("the refinement %r reaches the cube's faces, and the glue keeps the leaves across a "
                             "glued face at one level, so it would refine a shell, whose map is not affine: keep "
                             "the regions at least one root inside the cube [0, %d]^3" % (refined, n))
    shells = [(p, c) for p, c in forest.blocks if p != 0]
    forest.blocks = [(0, c) for _, c in cube.leaves] + shells
    forest.levels = [lv for lv, _ in cube.leaves] + [0] * len(shells)
    forest.leaves = [(lv, c) for lv, (_, c) in zip(forest.levels, forest.blocks)]
    forest.refined = max(forest.levels) > 0
    return forest


def face_plane_logical(corner, N, offs, f, scale=1.0):
    """Logical coordinates (3 arrays of N^2) of the face-node plane of face f of
    a block at integer corner and of extent `scale` (2^-level); tangential
    dims in increasing order, first fastest."""
    P1 = len(offs)
    n = np.arange(N)
    x1d = (n // P1) * P1 + offs[n % P1]
    d, side = f // 2, f % 2
    tang = [k for k in range(3) if k != d]
    a, b = np.meshgrid(x1d, x1d, indexing="xy")   # a varies fastest along columns
    coords = [None] * 3
    coords[tang[0]] = (corner[tang[0]] + a.reshape(-1) / N) * scale
    coords[tang[1]] = (corner[tang[1]] + b.reshape(-1) / N) * scale
    coords[d] = np.full(N * N, float(corner[d] + (1 if side else 0)) * scale)
    return coords


def orient(a, b, code, N):
    """The neighbour's tangential indices of our face point (a, b): bit 0
    swaps the two, bit 1 reverses the first, bit 2 the second."""
    if code & 1:
        a, b = b, a
    if code & 2:
        a = N - 1 - a
    if code & 4:
        b = N - 1 - b
    return a, b


# face_nb of a face between two blocks of a refined cube: the library finds
# the neighbour, or the coarse-fine partners, by level and corner
CUBE_FACE = -2


def build_ball_faces(forest, offsets):
    """The face table of a ball forest by matching face-node positions. In a
    refined cube every face between two cube blocks is CUBE_FACE, which the
    library's mesh compiler resolves by the blocks' levels and corners."""
    geo, N = forest.geo, forest.N
    nb = forest.nleaves()
    face_nb = np.full(nb * 6, -1, dtype=np.int32)
    face_code = np.zeros(nb * 6, dtype=np.int32)
    index = {blk: i for i, blk in enumerate(forest.blocks)}
    pos = {}
    centre = {}
    for bi, (p, c) in enumerate(forest.blocks):
        for f in range(6):
            x = geo.position(face_plane_logical(c, N, offsets, f, forest.block_scale(bi)), p)
            X = np.stack([np.asarray(v) for v in x], axis=-1)
            pos[(bi, f)] = X
            centre[(bi, f)] = X.mean(axis=0)
    # same-patch neighbours first
    for bi, (p, c) in enumerate(forest.blocks):
        r = geo.patch_roots(p)
        lv = forest.levels[bi]
        for f in range(6):
            d, side = f // 2, f % 2
            cn = list(c)
            cn[d] += 1 if side else -1
            if 0 <= cn[d] < (r[d] << lv):
                if forest.refined and p == 0:
                    face_nb[bi * 6 + f] = CUBE_FACE
                else:
                    face_nb[bi * 6 + f] = index[(p, tuple(cn))]
                    face_code[bi * 6 + f] = (f ^ 1)
    # glued faces: the unmatched faces whose face-node centres coincide
    open_faces = [(bi, f) for bi in range(nb) for f in range(6) if face_nb[bi * 6 + f] == -1]
    keys = {}
    scale = geo.R1
    for bf in open_faces:
        key = tuple(np.round(centre[bf] / scale, 9))
        keys.setdefault(key, []).append(bf)
    nn = np.arange(N)
    A, B = np.meshgrid(nn, nn, indexing="xy")
    A, B = A.reshape(-1), B.reshape(-1)
    for key, group in keys.items():
        if len(group) == 1:
            continue                       # an outer (sphere) face
        if len(group) != 2:
            raise ValueError("faces %r meet at one centre" % (group,))
        (b1, f1), (b2, f2) = group
        X1, X2 = pos[(b1, f1)], pos[(b2, f2)]
        found = None
        for code in range(8):
            a2, bb2 = orient(A, B, code, N)
            if np.allclose(X1, X2[a2 + N * bb2], atol=1e-10 * scale):
                found = code
                break
        if found is None:
            raise ValueError("glued faces (%d, %d) and (%d, %d) do not match" % (b1, f1, b2, f2))
        face_nb[b1 * 6 + f1] = b2
        face_code[b1 * 6 + f1] = f2 | (found << 4)
        # the inverse orientation for the other side
        inv = None
        for code in range(8):
            a1, bb1 = orient(A, B, code, N)
            if np.allclose(X2, X1[a1 + N * bb1], atol=1e-10 * scale):
                inv = code
                break
        face_nb[b2 * 6 + f2] = b1
        face_code[b2 * 6 + f2] = f1 | (inv << 4)
    forest.face_nb = face_nb
    forest.face_code = face_code
    return face_nb, face_code


def sevenpatch_forest(T, P, E, roots=(2, 2), Lc=1.0, R1=3.0, grading=0.0, refined=False):
    """The ball forest and its map (src/geometry.jl:494-538); `refined`
    refines the affine cube (refine_cube)."""
    from .element import Element
    if E % 2:
        raise ValueError("E = %d elements of order P = %d per block is odd, and E must be even" % (E, P))
    geo = SevenPatchBall(Lc, R1, roots, grading)
    forest = BallForest(geo, E * (P + 1))
    if refined is not False:
        refine_cube(forest, refined)
    build_ball_faces(forest, Element(np.float64, P).offsets.astype(np.float64))
    return forest, geo


def thirteenpatch_forest(T, P, E, roots=(2, 1, 1), Lc=1.0, Rm=2.0, R1=3.0, refined=False):
    """The thirteen-patch ball's forest and its map (src/geometry.jl:719-751):
    roots = (n, m, m'), the cube's per side and the inner and outer shells'
    radial ones; `refined` refines the affine cube (refine_cube)."""
    from .element import Element
    if E % 2:
        raise ValueError("E = %d elements of order P = %d per block is odd, and E must be even" % (E, P))
    if len(tuple(roots)) != 3:
        raise ValueError("the thirteen-patch ball takes roots = (n, m, m'), the cube's per side and the inner "
                         "and outer shells' radial ones, got %r" % (tuple(roots),))
    geo = ThirteenPatchBall(Lc, Rm, R1, roots)
    forest = BallForest(geo, E * (P + 1))
    if refined is not False:
        refine_cube(forest, refined)
    build_ball_faces(forest, Element(np.float64, P).offsets.astype(np.float64))
    return forest, geo


def ball_forest(T, P, E, roots, Lc, R1, Rm=None, grading=0.0, refined=False):
    """The seven-patch ball, or with a middle radius Rm the thirteen-patch one
    (src/sevenpatch.jl:119-128)."""
    if Rm is None:
        return sevenpatch_forest(T, P, E, roots=roots, Lc=Lc, R1=R1, grading=grading, refined=refined)
    if grading != 0:
        raise ValueError("the thirteen-patch ball's inner shells are ungraded: grading must be 0 with Rm")
    return thirteenpatch_forest(T, P, E, roots=roots, Lc=Lc, Rm=Rm, R1=R1, refined=refined)


def node_logical(forest, P, offsets):
    """Logical coordinates (nblocks, 3, N^3) of every node, patch-local."""
    N = forest.N
    P1 = P + 1
    n = np.arange(N)
    x1d = (n // P1) * P1 + offsets[n % P1]
    grids = np.indices([N] * 3).reshape(3, -1)[::-1]
    out = np.empty((forest.nleaves(), 3, N ** 3))
    for b, (p, c) in enumerate(forest.blocks):
        s = forest.block_scale(b)
        for k in range(3):
            out[b, k] = (c[k] + x1d[grids[k]] / N) * s
    return out


class PlaneWave:
    """u = sin(k . x - |k| t + phi) (src/sevenpatch.jl:9-59)."""

    def __init__(self, k, phi):
        self.k = tuple(float(x) for x in k)
        self.omega = math.sqrt(sum(x * x for x in self.k))
        self.phi = float(phi)

    def state(self, X, t, var):
        th = sum(self.k[j] * X[j] for j in range(3)) - self.omega * t + self.phi
        return np.sin(th) if var == 1 else -self.omega * np.cos(th)


class RadiativeBoundary:
    """The radiative, maximally dissipative condition on a ball's outer
    sphere (src/evolution.jl:1129-1160): n . grad u = -(kappa du/dt + u/R),
    R the geometry's outer radius; inverse_r = False drops the u/R term.
    kappa = 1 with u/R is Sommerfeld's condition; kappa = 0 without it a wall
    that holds the normal derivative at zero."""

    def __init__(self, kappa=1.0, inverse_r=True):
        if not kappa >= 0:
            raise ValueError("kappa = %r is negative, and a radiative boundary with kappa < 0 feeds energy in: "
                             "take kappa >= 0, kappa = 1 for Sommerfeld's condition" % (kappa,))
        self.kappa = float(kappa)
        self.inverse_r = bool(inverse_r)


class DirichletData:
    """Dirichlet data of any form on a ball's outer sphere: the reference's
    DirichletValues{:u} and {:grad} through boundary_by_coordinates
    (src/evolution.jl:1110-1127, 1303-1314), with `data(X, t)` returning u at
    the physical positions X (a (3, n) array) and the Cartesian gradient of u
    there ((3, n)). The problem evaluates it at the boundary face nodes for
    every stage time of a call and hands the library the table
    (twoldg_set_boundary_values)."""

    def __init__(self, data):
        self.data = data


class SphericalStandingWave(DirichletData):
    """u = j0(k r) cos(k t) with j0(x) = sin(x)/x, an exact solution of the
    wave equation regular at the origin, v = du/dt = -k j0(k r) sin(k t), and
    grad u = k j0'(k r) cos(k t) x/r with j0'(x) = (x cos x - sin x)/x^2; as
    Dirichlet data on the sphere it is a stand-in for any data(x, t)."""

    def __init__(self, k):
        self.k = float(k)
        super().__init__(self._data)

    def _radial(self, X):
        X = [np.asarray(x, dtype=np.float64) for x in X]
        r = np.sqrt(X[0] ** 2 + X[1] ** 2 + X[2] ** 2)
        kr = self.k * r
        small = kr < 1e-6
        krs = np.where(small, 1.0, kr)
        j0 = np.where(small, 1 - kr * kr / 6, np.sin(krs) / krs)
        dj0 = np.where(small, -kr / 3, (krs * np.cos(krs) - np.sin(krs)) / krs ** 2)
        return X, r, j0, dj0

    def state(self, X, t, var):
        _, _, j0, _ = self._radial(X)
        return j0 * math.cos(self.k * t) if var == 1 else -self.k * j0 * math.sin(self.k * t)

    def _data(self, X, t):
        X, r, j0, dj0 = self._radial(X)
        g = np.where(r > 0, self.k * dj0 * math.cos(self.k * t) / np.where(r > 0, r, 1.0), 0.0)
        return j0 * math.cos(self.k * t), np.stack([g * X[0], g * X[1], g * X[2]])


class OutgoingPulse:
    """u = (f(t - r) - f(t + r)) / r with f(s) = exp(-s^2/w^2), a solution of the
    wave equation regular at the origin, and v = du/dt (src/sevenpatch.jl:130-177);
    below r = w/1000 the series in r through r^4."""

    def __init__(self, w):
        self.w = float(w)

    def state(self, X, t, var):
        w = self.w
        X = [np.asarray(x, dtype=np.float64) for x in X]
        r = np.sqrt(X[0] ** 2 + X[1] ** 2 + X[2] ** 2)
        f = lambda s: np.exp(-(s / w) ** 2)
        df = lambda s: -2 * s / w ** 2 * f(s)
        rs = np.where(r > w / 1000, r, 1.0)
        if var == 1:
            far = (f(t - rs) - f(t + rs)) / rs
        else:
            far = (df(t - rs) - df(t + rs)) / rs
        y = t / w
        H = (2 * y, 4 * y ** 2 - 2, 8 * y ** 3 - 12 * y, 16 * y ** 4 - 48 * y ** 2 + 12,
             32 * y ** 5 - 160 * y ** 3 + 120 * y, 64 * y ** 6 - 480 * y ** 4 + 720 * y ** 2 - 120)
        dn = lambda k: (-1 / w) ** k * H[k - 1] * f(t)
        r2 = r * r
        if var == 1:
            near = -2 * (dn(1) + r2 * dn(3) / 6 + r2 ** 2 * dn(5) / 120)
        else:
            near = -2 * (dn(2) + r2 * dn(4) / 6 + r2 ** 2 * dn(6) / 120)
        return np.where(r > w / 1000, far, near)


def legendre_at(P, x):
    L = [np.ones_like(x), np.asarray(x, dtype=np.float64)]
    for k in range(2, P + 1):
        L.append(((2 * k - 1) * x * L[k - 1] - (k - 1) * L[k - 2]) / k)
    return np.array(L[:P + 1])


def ball_tables(forest, P, wave=None):
    """The full metric's host tables for a ball forest, in float64
    (src/evolution.jl:723-1018): coef (nblocks, 1 + 9, N^3) = sqrt(g) and
    S[d][i] at 1 + 3d + i; the per-element truncation of the shells (elem_slot,
    W_e = w_hat sqrt(g) and the upper Cholesky factor of G = Psi^T W Psi);
    the boundary face nodes' positions per slot (3, N^2); and the time step's
    spacing over speed."""
    from .element import Element
    cache = forest.__dict__.setdefault("_tables", {})
    if P in cache:
        return cache[P]
    geo, N = forest.geo, forest.N
    el = Element(np.float64, P)
    P1 = P + 1
    E = N // P1
    offs = el.offsets.astype(np.float64)
    xl = node_logical(forest, P, offs)                 # (nb, 3, N^3)
    nb = forest.nleaves()
    NN = N ** 3
    coef = np.empty((nb, 10, NN))
    hspeed = math.inf
    for b, (p, c) in enumerate(forest.blocks):
        # the time step is the CFL limit of the block that binds: its own
        # spacing over its own largest logical speed
        h = forest.block_scale(b) / N
        J, S = geo.frame(tuple(xl[b, k] for k in range(3)), p)
        coef[b, 0] = J
        for d in range(3):
            for i in range(3):
                coef[b, 1 + 3 * d + i] = S[:, d, i]
        g = np.einsum("ndi,nei->nde", S, S) / (J ** 2)[:, None, None]
        speed = np.sqrt(np.max(np.linalg.eigvalsh(g), axis=1)).max()
        hspeed = min(hspeed, h / speed)
    # per-element truncation tables for the shells whose sqrt(g) does not
    # factorize (the cube is affine: slot 0; factored shells: fac_slot)
    L = legendre_at(P, el.nodes.astype(np.float64))   # (P+1 modes, P+1 nodes)
    nodes = np.array([(n0, n1, n2) for n2 in range(P1) for n1 in range(P1) for n0 in range(P1)])
    basis = np.array([(q0, q1, q2) for q2 in range(P) for q1 in range(P) for q0 in range(P)])
    Psi = L[basis[:, 0]][:, nodes[:, 0]] * L[basis[:, 1]][:, nodes[:, 1]] * L[basis[:, 2]][:, nodes[:, 2]]
    Psi = Psi.T                                        # (n3, m3)
    what = el.weights[nodes[:, 0]] * el.weights[nodes[:, 1]] * el.weights[nodes[:, 2]]
    slot = np.zeros(nb, dtype=np.int32)
    ws, chols = [], []
    for b, (p, c) in enumerate(forest.blocks):
        if geo.affine_patch(p) or geo.factored_dim(p) >= 0:
            continue
        slot[b] = len(ws) + 1
        Wb = np.empty((E ** 3, P1 ** 3))
        Cb = np.empty((E ** 3, P ** 3, P ** 3))
        for e2 in range(E):
            for e1 in range(E):
                for e0 in range(E):
                    e = e0 + E * (e1 + E * e2)
                    idx = (e0 * P1 + nodes[:, 0]) + N * (e1 * P1 + nodes[:, 1]) + N * N * (e2 * P1 + nodes[:, 2])
                    W = what * coef[b, 0, idx]
                    G = Psi.T @ (W[:, None] * Psi)
                    U = np.linalg.cholesky(G).T            # upper, G = U^T U
                    Wb[e] = W
                    Cb[e] = U
        ws.append(Wb)
        chols.append(Cb)
    # (n3, E^3, ntab) column-major == (ntab, E^3, n3) row-major; U column-major per element
    ew = np.ascontiguousarray(np.array(ws)).reshape(-1) if ws else np.zeros(1)
    echol = np.ascontiguousarray(np.array(chols).transpose(0, 1, 3, 2)).reshape(-1) if chols else np.zeros(1)
    fac = factored_tables(forest, P, el)
    # boundary face nodes' positions per slot, (3, N^2)
    bnd = np.zeros((nb * 6, 3, N * N))
    for b, (p, c) in enumerate(forest.blocks):
        for f in range(6):
            if forest.face_nb[b * 6 + f] < 0:
                x = geo.position(face_plane_logical(c, N, offs, f, forest.block_scale(b)), p)
                bnd[b * 6 + f] = np.stack([np.asarray(v) for v in x])
    out = dict(coef=np.ascontiguousarray(coef.reshape(-1)), elem_slot=slot, elem_w=ew, elem_chol=echol,
               ntab=len(ws), bnd_x=np.ascontiguousarray(bnd.reshape(-1)), hspeed=hspeed, xl=xl)
    out.update(fac)
    cache[P] = out       # one forest, one set of tables: problems of any precision share them
    return out


def factored_tables(forest, P, el):
    """The factored truncation's tables (src/evolution.jl:840-899) for the
    blocks of patches whose sqrt(g) splits as R(x_k) Omega(x_across): per such
    block f its radial dimension k and the rank-one pair (projector_mode in
    the weight w_hat R) of each element along k; per distinct position
    across k the in-plane weights w_hat_a w_hat_b Omega and the upper Cholesky
    factor of the in-plane Gram matrix, shared by every block of a radial
    column and by all shells of one angular factor. Float64, rounded once to
    the field type by the library."""
    from .geometry import projector_mode
    geo, N = forest.geo, forest.N
    P1 = P + 1
    E = N // P1
    nb = forest.nleaves()
    wq = el.weights.astype(np.float64)
    offs = el.offsets.astype(np.float64)
    n = np.arange(N)
    x1d = (n // P1) * P1 + offs[n % P1]
    fslot = np.zeros(nb, dtype=np.int32)
    radial, rmodes, rduals, aslot = [], [], [], []
    keys = {}
    firsts = []
    for b, (p, c) in enumerate(forest.blocks):
        k = geo.factored_dim(p)
        if geo.affine_patch(p) or k < 0:
            continue
        fslot[b] = len(radial) + 1
        radial.append(k)
        rm = np.empty((E, P1))
        rd = np.empty((E, P1))
        for e in range(E):
            R = geo.radial_volume(c[k] + x1d[e * P1:(e + 1) * P1] / N, p)
            phi = projector_mode(el.nodes.astype(np.float64), wq, R, P)
            gamma = np.sum(wq * R * phi ** 2)
            rm[e] = phi
            rd[e] = wq * R * phi / gamma
        rmodes.append(rm)
        rduals.append(rd)
        across = tuple(c[j] for j in range(3) if j != k)
        if across not in keys:
            keys[across] = len(keys)
            firsts.append(across)
        aslot.append(keys[across])
    if not radial:
        return dict(fac_slot=fslot, fac_radial=None, fac_rmodes=None, fac_rduals=None, fac_aslot=None,
                    fac_aw=None, fac_achol=None, fac_ntab=0)
    L = legendre_at(P, el.nodes.astype(np.float64))
    nodes2 = np.array([(na, nb_) for nb_ in range(P1) for na in range(P1)])
    basis2 = np.array([(q0, q1) for q1 in range(P) for q0 in range(P)])
    Psi = (L[basis2[:, 0]][:, nodes2[:, 0]] * L[basis2[:, 1]][:, nodes2[:, 1]]).T      # (n2, m2)
    w2 = wq[nodes2[:, 0]] * wq[nodes2[:, 1]]
    aw = np.empty((len(firsts), E * E, P1 * P1))
    ach = np.empty((len(firsts), E * E, P * P, P * P))
    for A, (ca, cb) in enumerate(firsts):
        for eb in range(E):
            for ea in range(E):
                xa = ca + x1d[ea * P1 + nodes2[:, 0]] / N
                xb = cb + x1d[eb * P1 + nodes2[:, 1]] / N
                W = w2 * geo.angular_volume(xa, xb)
                G = Psi.T @ (W[:, None] * Psi)
                U = np.linalg.cholesky(G).T
                aw[A, ea + E * eb] = W
                ach[A, ea + E * eb] = U
    return dict(fac_slot=fslot, fac_radial=np.array(radial, dtype=np.int32),
                fac_rmodes=np.ascontiguousarray(np.array(rmodes)).reshape(-1),
                fac_rduals=np.ascontiguousarray(np.array(rduals)).reshape(-1),
                fac_aslot=np.array(aslot, dtype=np.int32),
                fac_aw=np.ascontiguousarray(aw).reshape(-1),
                fac_achol=np.ascontiguousarray(ach.transpose(0, 1, 3, 2)).reshape(-1), fac_ntab=len(firsts))


def ball_desc(forest, P, truncate, precision, tables, wave):
    """The twoldg_desc of a ball problem (an explicit face table and the full
    metric); `wave` is the Dirichlet PlaneWave, Dirichlet data of any form
    (DirichletData) or a RadiativeBoundary."""
    import ctypes
    from . import _lib
    nb = forest.nleaves()
    d = _lib.Desc()
    d.dim, d.order, d.elems = 3, P, forest.N // (P + 1)
    d.precision = precision
    d.truncate = 1 if truncate else 0
    d.nblocks = nb
    # a root block has logical extent 1: the cube's n roots per side span [0, n]
    n = forest.geo.patch_roots(0)[0]
    for k in range(3):
        d.roots[k] = n
        d.periodic[k] = 0
        d.reflecting[k] = 0
        d.lo[k] = 0.0
        d.hi[k] = float(n)
    # the blocks' levels, and the cube's corners (in blocks of their level),
    # by which the library resolves the refined cube's faces
    levels = np.array(forest.levels, dtype=np.int32)
    corners = np.array([c if p == 0 else (0, 0, 0) for p, c in forest.blocks], dtype=np.int64).reshape(-1)
    ip, dp = ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)
    d.level = levels.ctypes.data_as(ip)
    d.corner = corners.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    d.metric = 2
    d.coef = tables["coef"].ctypes.data_as(dp)
    d.face_nb = forest.face_nb.ctypes.data_as(ip)
    d.face_code = forest.face_code.ctypes.data_as(ip)
    d.elem_slot = tables["elem_slot"].ctypes.data_as(ip)
    d.elem_w = tables["elem_w"].ctypes.data_as(dp)
    d.elem_chol = tables["elem_chol"].ctypes.data_as(dp)
    d.elem_ntab = tables["ntab"]
    if isinstance(wave, RadiativeBoundary):
        d.boundary = 1
        d.kappa = wave.kappa
        d.inv_r = 1.0 / forest.geo.outer_radius() if wave.inverse_r else 0.0
    elif isinstance(wave, DirichletData):
        d.boundary = 2
    else:
        for k in range(3):
            d.wave_k[k] = wave.k[k]
        d.wave_phi = wave.phi
    d.bnd_x = tables["bnd_x"].ctypes.data_as(dp)
    if tables.get("fac_ntab", 0) > 0:
        d.fac_slot = tables["fac_slot"].ctypes.data_as(ip)
        d.fac_radial = tables["fac_radial"].ctypes.data_as(ip)
        d.fac_rmodes = tables["fac_rmodes"].ctypes.data_as(dp)
        d.fac_rduals = tables["fac_rduals"].ctypes.data_as(dp)
        d.fac_aslot = tables["fac_aslot"].ctypes.data_as(ip)
        d.fac_aw = tables["fac_aw"].ctypes.data_as(dp)
        d.fac_achol = tables["fac_achol"].ctypes.data_as(dp)
        d.fac_ntab = tables["fac_ntab"]
    keep = (levels, corners, tables, forest.face_nb, forest.face_code)
    return d, keep


def sevenpatch_exact(geo, wave, t, forest=None):
    """u and v = du/dt of the plane wave at time t (src/sevenpatch.jl:38-59), as a
    callback f(x, var) of physical positions."""
    def f(x, var):
        return wave.state(x, t, var)
    return f


def sevenpatch_errors(T=np.float64, P=3, E=2, roots=(2, 2), Lc=1.0, R1=3.0, k=(1.1, -0.7, 0.5), phi=0.3, cfl=0.5,
                      tend=1.0, truncate=True, precision=None, Rm=None, refined=False):
    """sevenpatch_errors (src/sevenpatch.jl:61-117): the plane wave on the ball
    (its cube refined by `refined`) to tend with itself as the Dirichlet data
    on the sphere; sqrt(g)-weighted L2 errors of u and v together and apart,
    Linf, the cube's physical spacing, the step count and the energies."""
    from .element import Element
    from .problem import WaveProblem, initial_state, oldg_timestep, quadrature_norm, wave_energy, wave_integrator
    T = np.dtype(T)
    forest, geo = ball_forest(T, P, E, roots, Lc, R1, Rm=Rm, refined=refined)
    wave = PlaneWave(k, phi)
    problem = WaveProblem(forest, Element(T, P), truncate=truncate, geometry=geo, boundary=wave,
                          precision=precision)
    t_end = float(T.type(tend))
    u0 = initial_state(problem, sevenpatch_exact(geo, wave, 0.0))
    nsteps = int(math.ceil(T.type(t_end) / oldg_timestep(problem, cfl)))
    dt = float(T.type(T.type(t_end) / T.type(nsteps)))
    integ = wave_integrator(problem, u0, 0.0, t_end, dt)
    integ.nsteps = nsteps
    integ.solve()
    u = integ.u
    ue = problem.to_device(problem.fill_at_nodes(sevenpatch_exact(geo, wave, t_end)))
    h = forest.minimum_spacing() * 2 * geo.Lc / geo.roots[0]
    return dict(l2=quadrature_norm(problem, u, 2, ref=ue), l2u=quadrature_norm(problem, u, 2, (1,), ref=ue),
                l2v=quadrature_norm(problem, u, 2, (2,), ref=ue), linf=quadrature_norm(problem, u, math.inf, ref=ue),
                h=h, he=(P + 1) * h, nsteps=nsteps, dt=dt, tend=t_end, nblocks=forest.nleaves(),
                energy0=wave_energy(problem, u0, t=0.0), energy=wave_energy(problem, u, t=t_end))


def radiative_errors(T=np.float64, P=3, E=2, roots=(2, 2), Lc=1.0, R1=3.0, w=0.5, kappa=1.0, inverse_r=True,
                     cfl=0.5, tend=2.0, truncate=True, precision=None, Rm=None, refined=False):
    """radiative_errors (src/sevenpatch.jl:186-237): the outgoing pulse of width
    w from the origin to tend under a radiative boundary of kappa (and u/R) on
    the outer sphere; sqrt(g)-weighted L2 errors of u and v together and apart,
    Linf, the cube's physical spacing, the step count and the energies, the
    boundary's own term included."""
    from .element import Element
    from .problem import WaveProblem, initial_state, oldg_timestep, quadrature_norm, wave_energy, wave_integrator
    T = np.dtype(T)
    forest, geo = ball_forest(T, P, E, roots, Lc, R1, Rm=Rm, refined=refined)
    pulse = OutgoingPulse(w)
    problem = WaveProblem(forest, Element(T, P), truncate=truncate, geometry=geo,
                          boundary=RadiativeBoundary(kappa, inverse_r), precision=precision)
    t_end = float(T.type(tend))
    u0 = initial_state(problem, lambda x, var: pulse.state(x, 0.0, var))
    nsteps = int(math.ceil(T.type(t_end) / oldg_timestep(problem, cfl)))
    dt = float(T.type(T.type(t_end) / T.type(nsteps)))
    integ = wave_integrator(problem, u0, 0.0, t_end, dt)
    integ.nsteps = nsteps
    integ.solve()
    u = integ.u
    ue = problem.to_device(problem.fill_at_nodes(lambda x, var: pulse.state(x, t_end, var)))
    h = forest.minimum_spacing() * 2 * geo.Lc / geo.roots[0]
    return dict(l2=quadrature_norm(problem, u, 2, ref=ue), l2u=quadrature_norm(problem, u, 2, (1,), ref=ue),
                l2v=quadrature_norm(problem, u, 2, (2,), ref=ue), linf=quadrature_norm(problem, u, math.inf, ref=ue),
                h=h, he=(P + 1) * h, nsteps=nsteps, dt=dt, tend=t_end, nblocks=forest.nleaves(),
                energy0=wave_energy(problem, u0, t=0.0), energy=wave_energy(problem, u, t=t_end))
