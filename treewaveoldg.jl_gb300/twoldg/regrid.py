"""Adaptive refinement on the path (src/refinement.jl:190-286; the regrid
itself is TreeAMR's regrid!, which the reference's adaptive_blast drives):
the regrid mark of a block from its modal indicator, the flags of a
problem's state, a regrid of the forest by them, and the transfer of the
state onto the new forest through twoldg_transfer, which refines by the
coarse element's polynomial and coarsens by the L2 projection in the
Gauss-Lobatto inner product, so that sum w u of each variable is kept."""
import ctypes

import numpy as np

from . import _lib
from .forest import Forest
from .problem import _check_state, _dptr, _sync_torch

REFINE, KEEP, COARSEN = "refine", "keep", "coarsen"


def check_thresholds(refine_tol, coarsen_tol):
    if not coarsen_tol < refine_tol:
        raise ValueError("coarsen_tol (%r) must lie below refine_tol (%r): the gap between them is the dead "
                         "band that stops blocks from flipping between levels on alternate regrids"
                         % (coarsen_tol, refine_tol))


def refine_mark(tau_b, P, level, refine_tol, coarsen_tol, maxlevel_cap):
    """refine_mark(tau, el, b, k; refine_tol, coarsen_tol, maxlevel_cap)
    (src/refinement.jl:223-250) for one block: tau_b holds its elements'
    indicator with axis d the element index along dimension d. Returns
    (REFINE, box), (KEEP, box), COARSEN or KEEP, with box the bounding box of
    the nodes of the elements above coarsen_tol, per dimension the owned node
    range [start, stop) (0-based)."""
    check_thresholds(refine_tol, coarsen_tol)
    tau_b = np.asarray(tau_b, dtype=np.float64)
    P1 = P + 1
    fire = bool((tau_b > refine_tol).any())
    hot = tau_b > coarsen_tol
    box = None
    if hot.any():
        idx = np.argwhere(hot)
        lo, hi = idx.min(axis=0), idx.max(axis=0)
        box = tuple((int(lo[d]) * P1, (int(hi[d]) + 1) * P1) for d in range(tau_b.ndim))
    if fire and level < maxlevel_cap:
        return (REFINE, box)
    if box is not None:
        return (KEEP, box)
    if level > 0:
        return COARSEN
    return KEEP


def refine_flags(p, u, mode, refine_tol, coarsen_tol, maxlevel_cap, var=1):
    """refine_flags(fs, el; mode, refine_tol, coarsen_tol, maxlevel_cap, var)
    (src/refinement.jl:269-286): the modal indicator of u's variable `var` up
    to `mode`, computed once on the device, and refine_mark for every block."""
    from .indicator import modal_indicator
    check_thresholds(refine_tol, coarsen_tol)
    tau = modal_indicator(p, u, mode, var).cpu().numpy().astype(np.float64)
    D = p.D
    flags = []
    for b, (lv, _) in enumerate(p.forest.leaves):
        tb = np.transpose(tau[b], tuple(range(D - 1, -1, -1)))   # axis d: dimension d
        flags.append(refine_mark(tb, p.P, lv, refine_tol, coarsen_tol, maxlevel_cap))
    return flags


def _flag_kind(f):
    return f[0] if isinstance(f, tuple) else f


def regrid(forest, flags, buffer=0):
    """The forest regridded by one flag per leaf (REFINE, KEEP or COARSEN, or
    (flag, box)): a flagged box dilated by `buffer` points of its block's
    spacing asks for its block's level around it (one more with REFINE), so
    the leaves it reaches are not coarsened and a coarser one is refined, and
    the margin travels with the feature; a complete set of
    2^D sibling leaves all flagged COARSEN and not recruited is merged when
    no leaf beside their parent is finer than they are; then the forest is
    refined back to 2:1 balance. Returns a new Forest; each of its blocks is
    a leaf of the old one, a child of one, or the parent of 2^D of them."""
    if len(flags) != forest.nleaves():
        raise ValueError("one flag per leaf: %d flags for %d leaves" % (len(flags), forest.nleaves()))
    D = forest.D
    kinds = [_flag_kind(f) for f in flags]
    for k in kinds:
        if k not in (REFINE, KEEP, COARSEN):
            raise ValueError("a flag is REFINE, KEEP or COARSEN (or one of the first two with a box), got %r" % (k,))
    leaves = list(forest.leaves)
    extents = [forest.block_extent(k) for k in leaves]
    refine = {leaves[b] for b in range(len(leaves)) if kinds[b] == REFINE}
    hold = set()
    for b, f in enumerate(flags):
        if not isinstance(f, tuple) or f[1] is None:
            continue
        key = leaves[b]
        h = forest.spacing(key)
        ext = extents[b]
        box = [(ext[d][0] + (f[1][d][0] - buffer) * h, ext[d][0] + (f[1][d][1] + buffer) * h) for d in range(D)]
        for q, other in enumerate(leaves):
            if q == b:
                continue
            oe = extents[q]
            if all(oe[d][0] < box[d][1] and box[d][0] < oe[d][1] for d in range(D)):
                hold.add(other)
                if other[0] < key[0] + (1 if f[0] == REFINE else 0):
                    refine.add(other)
    new = Forest.__new__(Forest)
    new.__dict__.update({k: v for k, v in forest.__dict__.items() if not k.startswith("_tables")})
    new.leaves = list(leaves)
    new._sort()
    # coarsening: complete sibling sets, all COARSEN, none held or refined
    index = {k: b for b, k in enumerate(leaves)}
    parents = {}
    for b, (lv, c) in enumerate(leaves):
        if lv > 0 and kinds[b] == COARSEN and (lv, c) not in hold and (lv, c) not in refine:
            parents.setdefault((lv - 1, tuple(x >> 1 for x in c)), []).append((lv, c))
    merged = []
    for (plv, pc), kids in parents.items():
        if len(kids) != 1 << D:
            continue
        # no leaf beside the parent finer than the children
        ok = True
        pext = [(forest.lo[d] + pc[d] * (forest.hi[d] - forest.lo[d]) / forest.roots[d] / (1 << plv),
                 forest.lo[d] + (pc[d] + 1) * (forest.hi[d] - forest.lo[d]) / forest.roots[d] / (1 << plv))
                for d in range(D)]
        for q, other in enumerate(leaves):
            if other[0] <= plv + 1:
                continue
            oe = extents[q]
            touch = True
            for d in range(D):
                L = forest.hi[d] - forest.lo[d]
                a0, a1 = pext[d]
                b0, b1 = oe[d]
                near = b0 <= a1 + 1e-12 * L and a0 <= b1 + 1e-12 * L
                if forest.periodic[d]:
                    near = near or b0 <= a1 - L + 1e-12 * L or b1 >= a0 + L - 1e-12 * L
                touch = touch and near
            if touch:
                ok = False
                break
        if ok:
            merged.append(((plv, pc), kids))
    out = [k for k in leaves if k not in refine]
    for key in refine:
        lv, c = key
        for q in np.ndindex(*([2] * D)):
            out.append((lv + 1, tuple(2 * c[k] + q[k] for k in range(D))))
    for parent, kids in merged:
        kids = set(kids)
        out = [k for k in out if k not in kids]
        out.append(parent)
    new.leaves = out
    new._sort()
    new.balance()
    return new


def transfer_state(old, u_old, new):
    """The state u_old of problem `old` moved onto problem `new`'s forest
    (twoldg_transfer): a new device state vector of `new`."""
    _check_state(old, u_old)
    if old.precision != new.precision:
        raise ValueError("the transfer keeps the precision: %s onto %s" % (old.precision, new.precision))
    u_new = new.statevector()
    _sync_torch()
    _lib.check(_lib.lib().twoldg_transfer(ctypes.byref(old._desc), _dptr(u_old), ctypes.byref(new._desc),
                                          _dptr(u_new), None))
    return u_new
