"""Block forests: the host-side stand-in for TreeAMR's Forest on the path.

A forest is a brick of roots^D root blocks, each leaf a block at a level
with an integer corner counted in blocks of that level, N = E(P+1) nodes
per block and dimension. This module builds the forests the reference's
drivers build (wave_forest, nested_cubes: src/sinewave.jl:114-199): uniform,
periodic or reflecting boxes, refined by regions level by level and
balanced after each. Leaves are kept in Morton order of their corners, which
is the block order of the state layout.
"""
import numpy as np


def _morton(c, bits=21):
    key = 0
    D = len(c)
    for bit in range(bits):
        for k in range(D):
            key |= ((int(c[k]) >> bit) & 1) << (bit * D + k)
    return key


class Forest:
    """A forest of blocks: `roots` per dimension, extents [lo, hi) per
    dimension, N points per block and dimension, periodic or reflecting
    faces per dimension, and its leaves as (level, corner) pairs."""

    def __init__(self, roots, N, lo, hi, periodic, reflecting):
        self.D = len(roots)
        self.roots = tuple(int(r) for r in roots)
        self.N = int(N)
        self.lo = tuple(float(x) for x in lo)
        self.hi = tuple(float(x) for x in hi)
        self.periodic = tuple(bool(p) for p in periodic)
        self.reflecting = tuple(bool(r) for r in reflecting)
        leaves = []
        for idx in np.ndindex(*self.roots):
            leaves.append((0, tuple(int(i) for i in idx)))
        self.leaves = leaves
        self._sort()

    # -- structure ---------------------------------------------------------
    def _sort(self):
        lmax = max((lv for lv, _ in self.leaves), default=0)
        self.leaves.sort(key=lambda k: (_morton([c << (lmax - k[0]) for c in k[1]]), k[0]))
        self._index = {k: i for i, k in enumerate(self.leaves)}

    def nleaves(self):
        return len(self.leaves)

    def block_extent(self, key):
        """((lo, hi) per dimension) of a leaf, in physical coordinates."""
        lv, c = key
        out = []
        for k in range(self.D):
            w = (self.hi[k] - self.lo[k]) / self.roots[k] / (1 << lv)
            out.append((self.lo[k] + c[k] * w, self.lo[k] + (c[k] + 1) * w))
        return tuple(out)

    def spacing(self, key):
        lv = key[0]
        return (self.hi[0] - self.lo[0]) / self.roots[0] / (1 << lv) / self.N

    def minimum_spacing(self):
        return min(self.spacing(k) for k in self.leaves)

    def refine(self, targets):
        """Replace each target leaf by its 2^D children."""
        targets = set(targets)
        out = []
        for lv, c in self.leaves:
            if (lv, c) in targets:
                for q in np.ndindex(*([2] * self.D)):
                    out.append((lv + 1, tuple(2 * c[k] + q[k] for k in range(self.D))))
            else:
                out.append((lv, c))
        self.leaves = out
        self._sort()

    def _find(self, level, corner):
        """The leaf covering cell `corner` of `level`: (key) or None."""
        lv = level
        c = list(corner)
        while lv >= 0:
            k = (lv, tuple(c))
            if k in self._index:
                return k
            lv -= 1
            c = [x >> 1 for x in c]
        return None

    def _wrap(self, level, c):
        out = []
        for k in range(self.D):
            ext = self.roots[k] << level
            x = c[k]
            if x < 0 or x >= ext:
                if not self.periodic[k]:
                    return None
                x %= ext
            out.append(x)
        return tuple(out)

    def balance(self):
        """2:1 balance across faces, edges and corners: refine any leaf that
        has a neighbouring leaf more than one level finer, until none has."""
        offsets = [o for o in np.ndindex(*([3] * self.D)) if any(x != 1 for x in o)]
        while True:
            leafset = set(self.leaves)
            lmax = max(lv for lv, _ in self.leaves)
            refine = set()
            for lv, c in self.leaves:
                if lv < 2:
                    continue
                for o in offsets:
                    n = self._wrap(lv, [c[k] + o[k] - 1 for k in range(self.D)])
                    if n is None:
                        continue
                    # the coarser leaf covering that neighbouring cell
                    k2 = self._find(lv, n)
                    if k2 is not None and k2[0] < lv - 1 and k2 in leafset:
                        refine.add(k2)
            if not refine:
                return self
            self.refine(refine)
            del lmax


def refinement_regions(refined, D, L):
    """The regions `wave_forest`'s `refined` stands for (src/sinewave.jl:170-183)."""
    def isregion(r):
        return (isinstance(r, tuple) and len(r) == D and
                all(isinstance(i, tuple) and len(i) == 2 and i[0] < i[1] for i in r))
    if refined is True:
        return [tuple((L / 4, 3 * L / 4) for _ in range(D))]
    if isregion(refined):
        return [refined]
    if isinstance(refined, list) and all(isregion(r) for r in refined):
        return refined
    raise ValueError("refined must be False, True, a tuple of %d intervals (lo, hi) with lo < hi, "
                     "one per dimension, or a list of such tuples, one per level; got %r" % (D, refined))


def refine_regions(forest, regions, roots):
    """Refine level by level (src/sinewave.jl:144-160)."""
    D = forest.D
    for k, region in enumerate(regions, start=1):
        targets = []
        for key in forest.leaves:
            if key[0] != k - 1:
                continue
            ext = forest.block_extent(key)
            if all(region[d][0] < (ext[d][0] + ext[d][1]) / 2 < region[d][1] for d in range(D)):
                targets.append(key)
        if not targets:
            raise ValueError("no block centre of level %d lies inside the region %r that is to refine it "
                             "to level %d; with refined=True the region is the middle half of the box, "
                             "which holds a block centre only from roots = 3 on (roots = %d)"
                             % (k - 1, region, k, roots))
        forest.refine(targets)
        forest.balance()
    return forest


def wave_forest(T, D, P, E, roots=4, L=1.0, reflecting=False, refined=False):
    """A box of roots^D blocks of E^D elements of order P (src/sinewave.jl:114-135)."""
    N = E * (P + 1)
    if E % 2:
        raise ValueError("E = %d elements of order P = %d per block is odd, and E must be even: a block of "
                         "a refined forest covers half of its parent and has to cover whole elements of it, "
                         "so element centering needs N = %d to be a multiple of 2(P+1) = %d"
                         % (E, P, N, 2 * (P + 1)))
    f = Forest([roots] * D, N, [0.0] * D, [float(L)] * D, [not reflecting] * D, [reflecting] * D)
    if refined is False:
        return f
    refine_regions(f, refinement_regions(refined, D, float(L)), roots)
    return f


def nested_cubes(D, w0, levels):
    """Regions of `levels` nested cubes about the centre of a box of side
    2^levels w0 (src/sinewave.jl:192-199)."""
    if levels < 1:
        raise ValueError("a forest has at least one level, got %d" % levels)
    if not w0 > 0:
        raise ValueError("the finest cube's half-width w0 = %r must be positive" % (w0,))
    c = 2 ** (levels - 1) * w0
    return [tuple((c - 2 ** (levels - 1 - k) * w0, c + 2 ** (levels - 1 - k) * w0) for _ in range(D))
            for k in range(1, levels)]
