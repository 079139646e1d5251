"""ctypes wrapper of the C oracle (oracle.c). Test infrastructure only.

Tables come from tests/golden/element_tables.json (the mpmath restatement of
the reference's Element), never from the library under test.
"""
import ctypes
import json
import os
import struct

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(os.path.dirname(HERE), "tests", "golden", "element_tables.json")


class OracleMesh(ctypes.Structure):
    _fields_ = [
        ("D", ctypes.c_int), ("P", ctypes.c_int), ("E", ctypes.c_int), ("nblocks", ctypes.c_int),
        ("truncate", ctypes.c_int), ("roots", ctypes.c_int * 3), ("periodic", ctypes.c_int * 3),
        ("reflecting", ctypes.c_int * 3), ("lo", ctypes.c_double * 3), ("hi", ctypes.c_double * 3),
        ("level", ctypes.POINTER(ctypes.c_int32)), ("corner", ctypes.POINTER(ctypes.c_int64)),
        ("nodes", ctypes.POINTER(ctypes.c_double)), ("weights", ctypes.POINTER(ctypes.c_double)),
        ("stencil", ctypes.POINTER(ctypes.c_double)), ("projector", ctypes.POINTER(ctypes.c_double)),
        ("duals", ctypes.POINTER(ctypes.c_double)), ("coef", ctypes.POINTER(ctypes.c_double)),
        ("line_weights", ctypes.POINTER(ctypes.c_double)), ("metric", ctypes.c_int),
        ("face_nb", ctypes.POINTER(ctypes.c_int32)), ("face_code", ctypes.POINTER(ctypes.c_int32)),
        ("elem_slot", ctypes.POINTER(ctypes.c_int32)), ("bnd_x", ctypes.POINTER(ctypes.c_double)),
        ("wave_k", ctypes.c_double * 3), ("wave_phi", ctypes.c_double), ("t", ctypes.c_double),
        ("boundary", ctypes.c_int), ("kappa", ctypes.c_double), ("inv_r", ctypes.c_double),
        ("cache", ctypes.c_void_p), ("brick", ctypes.c_void_p),
    ]


_lib = None
_tables = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(_build.build())
        vp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
        mp = ctypes.POINTER(OracleMesh)
        L.oracle_rhs.argtypes = [mp, vp, vp]
        L.oracle_truncate.argtypes = [mp, vp]
        L.oracle_rk4.argtypes = [mp, vp, ctypes.c_double, ctypes.c_int]
        L.oracle_energy.argtypes = [mp, vp, dp]
        L.oracle_norm.argtypes = [mp, vp, vp, ctypes.c_int, ctypes.c_int, dp]
        L.oracle_modes.argtypes = [mp, vp, ctypes.c_int, ctypes.c_int, vp, vp, vp, ctypes.c_double, vp]
        L.oracle_threads.restype = ctypes.c_int
        L.oracle_rhs_full.argtypes = [mp, vp, vp]
        L.oracle_truncate_full2.argtypes = [mp, vp]
        L.oracle_rk4_full.argtypes = [mp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.oracle_full_prepare.argtypes = [mp]
        L.oracle_full_release.argtypes = [mp]
        L.oracle_full_release.restype = None
        L.oracle_energy_full.argtypes = [mp, vp, dp]
        L.oracle_norm_full.argtypes = [mp, vp, vp, ctypes.c_int, ctypes.c_int, dp]
        _lib = L
    return _lib


def golden_tables(P, kind="f64"):
    """Tables of order P from the golden fixture, as float64 (or float32) arrays."""
    global _tables
    if _tables is None:
        with open(GOLDEN) as f:
            _tables = json.load(f)
    raw = _tables["orders"][str(P)][kind]
    out = {}
    for k, v in raw.items():
        if kind == "f64":
            conv = lambda b: struct.unpack("<d", struct.pack("<Q", b))[0]
        else:
            conv = lambda b: struct.unpack("<f", struct.pack("<I", b))[0]
        a = np.array([[conv(x) for x in row] for row in v] if isinstance(v[0], list) else [conv(x) for x in v])
        out[k] = a.astype(np.float64 if kind == "f64" else np.float32)
    return out


class Oracle:
    """The oracle over one forest (a twoldg Forest-like object with D, roots,
    N, lo, hi, periodic, reflecting and leaves), in FP64."""

    def __init__(self, forest, P, truncate=True, coef=None, line_weights=None):
        """coef: (nblocks, 1+D, N^D) metric node values; line_weights: (D,
        nblocks, E, P+1) sqrt(g) factors along each element line (a
        diagonal-metric geometry), or None for the flat problem."""
        self.forest = forest
        self.P = P
        self.D = forest.D
        self.N = forest.N
        self.E = forest.N // (P + 1)
        self.NN = self.N ** self.D
        self.nblocks = len(forest.leaves)
        t = golden_tables(P)
        self.tables = t
        self._arrays = dict(
            level=np.array([lv for lv, _ in forest.leaves], dtype=np.int32),
            corner=np.array([c for _, c in forest.leaves], dtype=np.int64).reshape(-1),
            nodes=np.ascontiguousarray(t["nodes"]), weights=np.ascontiguousarray(t["weights"]),
            stencil=np.ascontiguousarray(t["stencil"]).reshape(-1),
            projector=np.ascontiguousarray(t["truncate"]).reshape(-1),
            duals=np.ascontiguousarray(t["duals"]).reshape(-1))
        m = OracleMesh()
        m.D, m.P, m.E, m.nblocks, m.truncate = self.D, P, self.E, self.nblocks, 1 if truncate else 0
        for k in range(3):
            m.roots[k] = forest.roots[k] if k < self.D else 1
            m.periodic[k] = int(forest.periodic[k]) if k < self.D else 1
            m.reflecting[k] = int(forest.reflecting[k]) if k < self.D else 0
            m.lo[k] = forest.lo[k] if k < self.D else 0.0
            m.hi[k] = forest.hi[k] if k < self.D else 1.0
        a = self._arrays
        m.level = a["level"].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        m.corner = a["corner"].ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        for k in ("nodes", "weights", "stencil", "projector", "duals"):
            setattr(m, k, a[k].ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        if coef is not None:
            a["coef"] = np.ascontiguousarray(coef, dtype=np.float64).reshape(-1)
            a["line_weights"] = np.ascontiguousarray(line_weights, dtype=np.float64).reshape(-1)
            m.coef = a["coef"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            m.line_weights = a["line_weights"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self.mesh = m

    def _vec(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        if u.size != 2 * self.NN * self.nblocks:
            raise ValueError("state size %d != %d" % (u.size, 2 * self.NN * self.nblocks))
        return u

    def rhs(self, u):
        u = self._vec(u)
        du = np.zeros_like(u)
        if lib().oracle_rhs(ctypes.byref(self.mesh), u.ctypes.data, du.ctypes.data):
            raise MemoryError("oracle_rhs failed")
        return du

    def truncate(self, u):
        u = self._vec(u).copy()
        lib().oracle_truncate(ctypes.byref(self.mesh), u.ctypes.data)
        return u

    def rk4(self, u, dt, nsteps):
        u = self._vec(u).copy()
        if lib().oracle_rk4(ctypes.byref(self.mesh), u.ctypes.data, float(dt), int(nsteps)):
            raise MemoryError("oracle_rk4 failed")
        return u

    def energy(self, u):
        u = self._vec(u)
        e = ctypes.c_double()
        lib().oracle_energy(ctypes.byref(self.mesh), u.ctypes.data, ctypes.byref(e))
        return e.value

    def norm(self, u, p=2, vars_mask=3, ref=None):
        u = self._vec(u)
        r = None if ref is None else self._vec(ref)
        out = ctypes.c_double()
        lib().oracle_norm(ctypes.byref(self.mesh), u.ctypes.data, None if r is None else r.ctypes.data,
                          int(p), int(vars_mask), ctypes.byref(out))
        return out.value

    def modes(self, u, var, modes, weights, pows, post):
        u = self._vec(u)
        nq = len(modes)
        mo = np.array(modes, dtype=np.int32)
        w = np.array(weights, dtype=np.float64)
        pw = np.array(pows, dtype=np.float64)
        tau = np.zeros(self.nblocks * self.E ** self.D)
        lib().oracle_modes(ctypes.byref(self.mesh), u.ctypes.data, int(var), nq, mo.ctypes.data, w.ctypes.data,
                           pw.ctypes.data, float(post), tau.ctypes.data)
        return tau

    def modal_indicator(self, u, mode, var=1):
        df = lambda m: float(np.prod(np.arange(1, 2 * m, 2))) if m > 0 else 1.0
        modes = list(range(1, mode + 1))
        return self.modes(u, var - 1, modes, [df(m) for m in modes], [mode / m for m in modes], 1.0 / df(mode))


def threads():
    return lib().oracle_threads()


class BallOracle(Oracle):
    """The oracle on a ball forest (full metric, glue, Dirichlet plane wave or
    radiative boundary): coef (sqrt(g), S) from the geometry, the face table,
    the blocks whose truncation is the sqrt(g)-orthogonal projection per
    element (every block off the affine cube, the factored ones included:
    the oracle solves each element's projection from sqrt(g) itself, so the
    factored tables are checked against it); `radiative` is (kappa, inv_r)
    or None; `standing` is k of the spherical standing wave j0(k r) cos(k t)
    as the Dirichlet data (evaluated here, from the formula), or None."""

    def __init__(self, forest, P, tables, wave, truncate=True, radiative=None, standing=None):
        self.forest = forest
        self.P = P
        self.D = 3
        self.N = forest.N
        self.E = forest.N // (P + 1)
        self.NN = self.N ** 3
        self.nblocks = forest.nleaves()
        t = golden_tables(P)
        a = dict(nodes=np.ascontiguousarray(t["nodes"]), weights=np.ascontiguousarray(t["weights"]),
                 stencil=np.ascontiguousarray(t["stencil"]).reshape(-1),
                 projector=np.ascontiguousarray(t["truncate"]).reshape(-1),
                 duals=np.ascontiguousarray(t["duals"]).reshape(-1),
                 level=np.array(getattr(forest, "levels", [0] * self.nblocks), dtype=np.int32),
                 corner=np.array([c if p == 0 else (0, 0, 0) for p, c in forest.blocks], dtype=np.int64).reshape(-1),
                 coef=np.ascontiguousarray(tables["coef"], dtype=np.float64),
                 face_nb=np.ascontiguousarray(forest.face_nb, dtype=np.int32),
                 face_code=np.ascontiguousarray(forest.face_code, dtype=np.int32),
                 elem_slot=np.ascontiguousarray((np.asarray(tables["elem_slot"]) != 0) |
                                                (np.asarray(tables.get("fac_slot", 0)) != 0), dtype=np.int32),
                 bnd_x=np.ascontiguousarray(tables["bnd_x"], dtype=np.float64))
        self._arrays = a
        m = OracleMesh()
        m.D, m.P, m.E, m.nblocks, m.truncate = 3, P, self.E, self.nblocks, 1 if truncate else 0
        n = forest.geo.patch_roots(0)[0]
        for k in range(3):
            # a root block spans 1: the cube's n roots, a brick for a refined cube
            m.roots[k], m.periodic[k], m.reflecting[k], m.lo[k], m.hi[k] = n, 0, 0, 0.0, float(n)
            m.wave_k[k] = wave.k[k] if wave is not None else 0.0
        m.wave_phi = wave.phi if wave is not None else 0.0
        m.metric = 2
        if radiative is not None:
            m.boundary, m.kappa, m.inv_r = 1, float(radiative[0]), float(radiative[1])
        if standing is not None:
            # the spherical standing wave j0(k r) cos(k t) as the Dirichlet data
            m.boundary, m.wave_k[0] = 2, float(standing)
        dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)
        m.level = a["level"].ctypes.data_as(ip)
        m.corner = a["corner"].ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        for k in ("nodes", "weights", "stencil", "projector", "duals", "coef", "bnd_x"):
            setattr(m, k, a[k].ctypes.data_as(dp))
        for k in ("face_nb", "face_code", "elem_slot"):
            setattr(m, k, a[k].ctypes.data_as(ip))
        self.mesh = m
        # factor every projected element's Gram matrix once (long double LU)
        if lib().oracle_full_prepare(ctypes.byref(m)):
            raise MemoryError("oracle_full_prepare failed")

    def __del__(self):
        m = getattr(self, "mesh", None)
        if m is not None and m.cache:
            lib().oracle_full_release(ctypes.byref(m))

    def rhs(self, u, t=0.0):
        u = self._vec(u)
        du = np.zeros_like(u)
        self.mesh.t = t
        if lib().oracle_rhs_full(ctypes.byref(self.mesh), u.ctypes.data, du.ctypes.data):
            raise MemoryError("oracle_rhs_full failed")
        return du

    def truncate(self, u):
        u = self._vec(u).copy()
        lib().oracle_truncate_full2(ctypes.byref(self.mesh), u.ctypes.data)
        return u

    def rk4(self, u, dt, nsteps, t0=0.0):
        u = self._vec(u).copy()
        if lib().oracle_rk4_full(ctypes.byref(self.mesh), u.ctypes.data, float(t0), float(dt), int(nsteps)):
            raise MemoryError("oracle_rk4_full failed")
        return u

    def energy(self, u, t=0.0):
        u = self._vec(u)
        e = ctypes.c_double()
        self.mesh.t = t
        lib().oracle_energy_full(ctypes.byref(self.mesh), u.ctypes.data, ctypes.byref(e))
        return e.value

    def norm(self, u, p=2, vars_mask=3, ref=None):
        u = self._vec(u)
        r = None if ref is None else self._vec(ref)
        out = ctypes.c_double()
        lib().oracle_norm_full(ctypes.byref(self.mesh), u.ctypes.data, None if r is None else r.ctypes.data,
                               int(p), int(vars_mask), ctypes.byref(out))
        return out.value


# --- the regrid transfer, restated (test infrastructure) ----------------------
def transfer_operators(P):
    """The 1D prolongation I (2(P+1) x (P+1): the coarse element's Lagrange
    polynomial at the nodes of its two halves) and the L2 restriction
    R = M_c^-1 I^T M_f in the Gauss-Lobatto inner product ((P+1) x 2(P+1)),
    evaluated here from the golden nodes and weights in long double."""
    t = golden_tables(P)
    x = np.array(t["nodes"], dtype=np.longdouble)
    w = np.array(t["weights"], dtype=np.longdouble)
    P1 = P + 1
    I = np.zeros((2 * P1, P1), dtype=np.longdouble)
    for h in range(2):
        for i in range(P1):
            xf = (x[i] + 2 * h - 1) / 2
            for j in range(P1):
                lj = np.longdouble(1)
                for m in range(P1):
                    if m != j:
                        lj *= (xf - x[m]) / (x[j] - x[m])
                I[h * P1 + i, j] = lj
    wf = np.concatenate([w / 2, w / 2])
    R = (I * wf[:, None]).T / w[:, None]
    return I.astype(np.float64), R.astype(np.float64)


def _along(A, op, d, D):
    """Apply a matrix along dimension d of a block array (axis D-1-d)."""
    ax = D - 1 - d
    return np.moveaxis(np.tensordot(op, A, axes=([1], [ax])), 0, ax)


def oracle_transfer(old_leaves, u_old, new_leaves, D, P, E):
    """The state on leaves `old_leaves` ((level, corner) per block, the state
    layout's order) moved onto `new_leaves`: copy, refine by I, coarsen by R,
    dimension by dimension."""
    P1, N = P + 1, E * (P + 1)
    NN = N ** D
    I, R = transfer_operators(P)
    half = E // 2
    index = {k: b for b, k in enumerate(old_leaves)}
    u_old = np.asarray(u_old, dtype=np.float64).reshape(len(old_leaves), 2, *([N] * D))
    out = np.empty((len(new_leaves), 2) + (N,) * D)
    # refine: fine node i of the half s takes row (ef % 2) P1 + i % P1 of I over coarse element s E/2 + ef/2
    up = []
    for s in range(2):
        op = np.zeros((N, N))
        for i in range(N):
            ef = i // P1
            ec = s * half + ef // 2
            op[i, ec * P1:(ec + 1) * P1] = I[(ef % 2) * P1 + i % P1]
        up.append(op)
    # coarsen: coarse node i of element ec reads R's row over the two fine
    # elements 2 (ec % (E/2)) and the next of the child half ec // (E/2)
    down = np.zeros((N, 2 * N))
    for i in range(N):
        ec = i // P1
        h = ec // half
        f0 = h * N + 2 * (ec % half) * P1
        down[i, f0:f0 + 2 * P1] = R[i % P1]
    for b, (lv, c) in enumerate(new_leaves):
        if (lv, c) in index:
            out[b] = u_old[index[(lv, c)]]
            continue
        parent = (lv - 1, tuple(x >> 1 for x in c))
        if lv > 0 and parent in index:
            A = u_old[index[parent]]
            for var in range(2):
                X = A[var]
                for d in range(D):
                    X = _along(X, up[c[d] & 1], d, D)
                out[b, var] = X
            continue
        kids = {}
        for q in np.ndindex(*([2] * D)):
            kids[q] = index[(lv + 1, tuple(2 * c[d] + q[d] for d in range(D)))]
        for var in range(2):
            big = np.empty((2 * N,) * D)
            for q, kb in kids.items():
                sl = tuple(slice(q[D - 1 - ax] * N, (q[D - 1 - ax] + 1) * N) for ax in range(D))
                big[sl] = u_old[kb, var]
            for d in range(D):
                big = _along(big, down, d, D)
            out[b, var] = big
    return out.reshape(-1)


# --- the extraction's reading, restated (test infrastructure) -----------------
def oracle_point_values(forest, P, u, points, var=1, locate=None):
    """The element polynomial of variable `var` at physical points of a brick
    (or, with `locate(x) -> (block, local coordinates in [0, 1]^D)`, of any
    forest): the block found by scanning the leaves' extents, the element by
    the position in it, the value by the Lagrange form through the golden
    Gauss-Lobatto nodes in long double."""
    t = golden_tables(P)
    nodes = np.array(t["nodes"], dtype=np.longdouble)
    D, N = forest.D, forest.N
    P1, E, NN = P + 1, N // (P + 1), N ** D
    u = np.asarray(u, dtype=np.float64).reshape(-1, 2, *([N] * D))
    out = np.empty(len(points))
    for j, x in enumerate(points):
        if locate is None:
            b, local = None, None
            for q, key in enumerate(forest.leaves):
                ext = forest.block_extent(key)
                if all(ext[d][0] <= x[d] <= ext[d][1] for d in range(D)):
                    b, local = q, [(x[d] - ext[d][0]) / (ext[d][1] - ext[d][0]) for d in range(D)]
                    if forest.leaves[q][0] == max(lv for lv, _ in forest.leaves):
                        break
            if b is None:
                raise ValueError("point %r is outside the forest" % (tuple(x),))
        else:
            b, local = locate(x)
        acc = np.longdouble(0)
        e = [min(int(local[d] * E), E - 1) for d in range(D)]
        z = [np.longdouble(2) * (np.longdouble(local[d]) * E - e[d]) - 1 for d in range(D)]
        L = []
        for d in range(D):
            row = []
            for i in range(P1):
                v = np.longdouble(1)
                for m in range(P1):
                    if m != i:
                        v *= (z[d] - nodes[m]) / (nodes[i] - nodes[m])
                row.append(v)
            L.append(row)
        for I in np.ndindex(*([P1] * D)):
            J = I[::-1]
            w = np.longdouble(1)
            for d in range(D):
                w *= L[d][J[d]]
            idx = tuple(e[d] * P1 + J[d] for d in range(D))[::-1]
            acc += w * np.longdouble(u[(b, var - 1) + idx])
        out[j] = float(acc)
    return out
