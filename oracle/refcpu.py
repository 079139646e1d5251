"""ctypes wrapper of refcpu.c, the reference's threaded CPU field step
restated in C. Test infrastructure only: it is the timed CPU baseline of
bench.py (cpu_baseline, --impl reference), held to the oracle by tests/.
Tables come from tests/golden/element_tables.json."""
import ctypes

import numpy as np

from . import build as _build
from .oracle import golden_tables


class RefDesc(ctypes.Structure):
    _fields_ = [
        ("D", ctypes.c_int), ("P", ctypes.c_int), ("E", ctypes.c_int), ("nblocks", ctypes.c_int),
        ("truncate", ctypes.c_int), ("roots", ctypes.c_int * 3), ("reflecting", ctypes.c_int * 3),
        ("corner", ctypes.POINTER(ctypes.c_int64)), ("h", ctypes.c_double),
        ("stencil", ctypes.POINTER(ctypes.c_double)), ("topmode", ctypes.POINTER(ctypes.c_double)),
        ("topdual", ctypes.POINTER(ctypes.c_double)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(_build.build_refcpu())
        vp = ctypes.c_void_p
        L.refcpu_create.restype = vp
        L.refcpu_create.argtypes = [ctypes.POINTER(RefDesc)]
        L.refcpu_destroy.argtypes = [vp]
        L.refcpu_destroy.restype = None
        L.refcpu_rhs.argtypes = [vp, vp, vp]
        L.refcpu_rhs.restype = None
        L.refcpu_truncate.argtypes = [vp, vp]
        L.refcpu_truncate.restype = None
        L.refcpu_rk4.argtypes = [vp, vp, ctypes.c_double, ctypes.c_int]
        L.refcpu_rk4.restype = None
        L.refcpu_threads.restype = ctypes.c_int
        L.refcpu_set_threads.argtypes = [ctypes.c_int]
        L.refcpu_set_threads.restype = None
        _lib = L
    return _lib


def threads():
    return lib().refcpu_threads()


def set_threads(n):
    lib().refcpu_set_threads(int(n))


class RefCPU:
    """The reference's CPU step over a uniform brick forest (all leaves at
    level 0), FP64."""

    def __init__(self, forest, P, truncate=True):
        if any(lv != 0 for lv, _ in forest.leaves):
            raise ValueError("the CPU baseline steps uniform bricks (level-0 leaves) only")
        self.forest, self.P, self.D, self.N = forest, P, forest.D, forest.N
        self.NN = forest.N ** forest.D
        self.nblocks = len(forest.leaves)
        t = golden_tables(P)
        self._keep = dict(corner=np.array([c for _, c in forest.leaves], dtype=np.int64).reshape(-1),
                          stencil=np.ascontiguousarray(t["stencil"]).reshape(-1),
                          topmode=np.ascontiguousarray(t["topmode"]), topdual=np.ascontiguousarray(t["topdual"]))
        d = RefDesc()
        d.D, d.P, d.E, d.nblocks = self.D, P, forest.N // (P + 1), self.nblocks
        d.truncate = 1 if truncate else 0
        for k in range(3):
            d.roots[k] = forest.roots[k] if k < self.D else 1
            d.reflecting[k] = int(forest.reflecting[k]) if k < self.D else 0
        d.h = forest.minimum_spacing()
        k = self._keep
        d.corner = k["corner"].ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        for name in ("stencil", "topmode", "topdual"):
            setattr(d, name, k[name].ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        self._desc = d
        self._h = lib().refcpu_create(ctypes.byref(d))
        if not self._h:
            raise MemoryError("refcpu_create failed")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().refcpu_destroy(h)
            self._h = None

    def _vec(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        if u.size != 2 * self.NN * self.nblocks:
            raise ValueError("state size %d != %d" % (u.size, 2 * self.NN * self.nblocks))
        return u

    def rhs(self, u):
        u = self._vec(u)
        du = np.empty_like(u)
        lib().refcpu_rhs(self._h, u.ctypes.data, du.ctypes.data)
        return du

    def truncate(self, u):
        u = self._vec(u).copy()
        lib().refcpu_truncate(self._h, u.ctypes.data)
        return u

    def rk4(self, u, dt, nsteps, inplace=False):
        """nsteps RK4 steps; with inplace the caller's float64 contiguous
        array is stepped without a copy (the timed baseline)."""
        u = u if inplace else self._vec(u).copy()
        lib().refcpu_rk4(self._h, u.ctypes.data, float(dt), int(nsteps))
        return u
