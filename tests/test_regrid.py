"""Adaptive refinement on the host and the oracle: the block verdict, the
regrid of a forest by flags, and the transfer restated in the oracle, which
keeps sum w u, reproduces the coarse polynomial on refinement and is
undone by coarsening on data of degree P - 1 or less. No GPU."""
import numpy as np
import pytest

from cases import scrambled
from oracle.oracle import golden_tables, oracle_transfer, transfer_operators
from twoldg.forest import wave_forest
from twoldg.regrid import COARSEN, KEEP, REFINE, check_thresholds, refine_mark, regrid


def test_refine_mark_is_treewaves_verdict_with_the_box_in_nodes():
    # test/adaptive_tests.jl:175-196 with 0-based, half-open node ranges:
    # element e of P + 1 = 4 nodes holds the nodes [4e, 4e + 4)
    P = 3
    tols = dict(refine_tol=0.01, coarsen_tol=0.001)
    t1 = np.zeros((2, 2))
    t1[1, 0] = 0.5
    t2 = np.zeros((2, 2))
    t2[0, 1] = 0.005
    assert refine_mark(t1, P, 0, maxlevel_cap=1, **tols) == (REFINE, ((4, 8), (0, 4)))
    assert refine_mark(t1, P, 1, maxlevel_cap=1, **tols) == (KEEP, ((4, 8), (0, 4)))
    assert refine_mark(t2, P, 1, maxlevel_cap=2, **tols) == (KEEP, ((0, 4), (4, 8)))
    t2[1, 1] = 0.002
    assert refine_mark(t2, P, 1, maxlevel_cap=2, **tols) == (KEEP, ((0, 8), (4, 8)))
    t2[:, :] = 0.0005
    assert refine_mark(t2, P, 1, maxlevel_cap=2, **tols) == COARSEN
    assert refine_mark(t2, P, 0, maxlevel_cap=2, **tols) == KEEP
    with pytest.raises(ValueError, match="dead band"):
        check_thresholds(0.01, 0.01)


def test_regrid_refines_coarsens_and_balances():
    f = wave_forest(np.float64, 2, 2, 2, roots=4)
    # refine the block at the corner (1, 1) and its neighbours through a box
    flags = [KEEP] * f.nleaves()
    b = f.leaves.index((0, (1, 1)))
    flags[b] = (REFINE, ((0, 6), (0, 6)))
    g = regrid(f, flags, buffer=0)
    assert (1, (2, 2)) in g.leaves and (0, (1, 1)) not in g.leaves
    assert g.nleaves() == 16 - 1 + 4
    # the buffer recruits the neighbours its dilated box reaches
    g2 = regrid(f, flags, buffer=1)
    assert g2.nleaves() == 16 - 9 + 36
    # coarsen the four children back
    flags = [COARSEN if lv == 1 else KEEP for lv, _ in g.leaves]
    h = regrid(g, flags)
    assert sorted(h.leaves) == sorted(f.leaves)
    # a sibling set is kept when one of them is held
    flags = [COARSEN if lv == 1 else KEEP for lv, _ in g.leaves]
    flags[g.leaves.index((1, (2, 2)))] = KEEP
    assert sorted(regrid(g, flags).leaves) == sorted(g.leaves)
    # a KEEP box asks for its own level around it: a coarser leaf it reaches
    # is refined, one at the same level is only held
    flags = [KEEP] * g.nleaves()
    flags[g.leaves.index((1, (3, 3)))] = (KEEP, ((0, 6), (0, 6)))
    k = regrid(g, flags, buffer=1)
    assert (1, (2, 4)) in k.leaves and (0, (1, 2)) not in k.leaves
    assert (1, (2, 2)) in k.leaves
    # refining next to a refined block keeps 2:1 balance
    flags = [REFINE if k == (1, (3, 3)) else KEEP for k in g.leaves]
    r = regrid(g, flags)
    assert (2, (6, 6)) in r.leaves
    for lv, c in r.leaves:
        assert lv <= 2


def mass(leaves, u, D, P, E, L=1.0, roots=4, scale=False):
    """sum w u per variable: w the Gauss-Lobatto weights times h (P+1)/2 per
    dimension (with scale: also sum w |u|, the size its rounding is measured by)."""
    w = np.array(golden_tables(P)["weights"])
    P1, N = P + 1, E * (P + 1)
    u = np.asarray(u).reshape(len(leaves), 2, N ** D)
    out, size = np.zeros(2), np.zeros(2)
    for b, (lv, c) in enumerate(leaves):
        h = L / roots / (1 << lv) / N
        w1 = h * P1 / 2 * w[np.arange(N) % P1]
        wb = w1
        for _ in range(D - 1):
            wb = np.kron(w1, wb)
        out += u[b] @ wb
        size += np.abs(u[b]) @ wb
    return (out, size) if scale else out


def same_mass(leaves, u, m0, D, P, E):
    m, size = mass(leaves, u, D, P, E, scale=True)
    return bool(np.all(np.abs(m - m0) <= 1e-13 * size))


@pytest.mark.parametrize("D,P", [(1, 3), (2, 3), (3, 2), (2, 4)])
def test_oracle_transfer_keeps_mass_and_polynomials(D, P):
    # test/adaptive_tests.jl:216-255: a regrid keeps the Gauss-Lobatto
    # integral of each variable to 1e-13; refinement evaluates the coarse
    # polynomial, so coarsening after it is the identity on each element's
    # degree-P data that the restriction reproduces (degree <= P - 1 here)
    E = 2
    f = wave_forest(np.float64, D, P, E, roots=4, refined=True)
    nb, N = f.nleaves(), E * (P + 1)
    u = scrambled(nb * 2 * N ** D, 0.2)
    m0 = mass(f.leaves, u, D, P, E)
    coarse = [(lv, c) for lv, c in f.leaves if lv == 0]
    parents = sorted({(0, tuple(x >> 1 for x in c)) for lv, c in f.leaves if lv == 1})
    down = coarse + parents
    u1 = oracle_transfer(f.leaves, u, down, D, P, E)
    assert same_mass(down, u1, m0, D, P, E)
    up = wave_forest(np.float64, D, P, E, roots=4, refined=True).leaves
    u2 = oracle_transfer(down, u1, up, D, P, E)
    assert same_mass(up, u2, m0, D, P, E)
    # refine a field of degree P - 1 per element and coarsen it back: unchanged
    from twoldg.element import Element
    offs = Element(np.float64, P).offsets
    x1 = (np.arange(N) // (P + 1)) * (P + 1) + offs[np.arange(N) % (P + 1)]
    poly = []
    for lv, c in down:
        h = 1.0 / 4 / (1 << lv) / N
        xs = [h * (c[d] * N + x1) for d in range(D)]
        grids = np.meshgrid(*xs[::-1], indexing="ij")
        val = sum((g - 0.3) ** (P - 1) for g in grids) + 0.5
        poly.append(np.stack([val.reshape(-1), 2 * val.reshape(-1)]))
    poly = np.concatenate([p.reshape(-1) for p in poly])
    back = oracle_transfer(up, oracle_transfer(down, poly, up, D, P, E), down, D, P, E)
    assert np.abs(back - poly).max() < 1e-12 * np.abs(poly).max()


def test_transfer_operators_left_inverse_on_lower_degrees():
    # R I is the identity on polynomials of degree <= P - 1 (the fine
    # quadrature integrates their products with the coarse basis exactly)
    for P in (1, 2, 3, 4, 5):
        I, R = transfer_operators(P)
        x = np.array(golden_tables(P)["nodes"])
        for k in range(P):
            v = x ** k
            assert np.abs(R @ (I @ v) - v).max() < 1e-13
