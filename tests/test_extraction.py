"""Waveform extraction on the host and the oracle: the spherical harmonics
and the sphere rule, the ball's inverse map, and the element stencils, whose
reading equals the oracle's own element polynomials and converges at order
P + 1. No GPU."""
import math

import numpy as np
import pytest

from ball_cases import ball_state
from cases import state_from
from oracle.oracle import oracle_point_values
from twoldg.ball import SevenPatchBall, ball_tables, sevenpatch_forest
from twoldg.extraction import (ball_patch_point, element_stencils, harmonic_modes, mode_index, sphere_rule,
                               spherical_harmonics)
from twoldg.forest import wave_forest


def extraction_f(x):
    # a smooth function that is no polynomial (test/extraction_tests.jl:13-15)
    return np.sin(0.7 * x[0] + 0.3) * np.cos(0.5 * x[1]) * np.exp(0.2 * x[2]) + 0.3 * x[0] * x[2]


def fill(x, var):
    return extraction_f(x) if var == 1 else 2 * extraction_f(x)


def test_spherical_harmonics_closed_forms_and_exact_rule():
    # test/extraction_tests.jl:25-58
    th, ph = 0.7, 1.9
    Y = spherical_harmonics(2, th, ph)
    cis = lambda a: np.exp(1j * a)
    assert Y[mode_index(0, 0)] == pytest.approx(1 / math.sqrt(4 * math.pi))
    assert Y[mode_index(1, 0)] == pytest.approx(math.sqrt(3 / (4 * math.pi)) * math.cos(th))
    assert Y[mode_index(1, 1)] == pytest.approx(-math.sqrt(3 / (8 * math.pi)) * math.sin(th) * cis(ph))
    assert Y[mode_index(2, 0)] == pytest.approx(math.sqrt(5 / (16 * math.pi)) * (3 * math.cos(th) ** 2 - 1))
    assert Y[mode_index(2, 1)] == pytest.approx(-math.sqrt(15 / (8 * math.pi)) * math.sin(th) * math.cos(th) * cis(ph))
    assert Y[mode_index(2, 2)] == pytest.approx(math.sqrt(15 / (32 * math.pi)) * math.sin(th) ** 2 * cis(2 * ph))
    assert harmonic_modes(2) == [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2)]
    lmax, nth = 6, 7
    table, dirs = sphere_rule(lmax, nth)
    assert len(dirs) == 2 * nth ** 2 and np.allclose(np.linalg.norm(dirs, axis=1), 1)
    th = np.arccos(dirs[:, 2])
    ph = np.arctan2(dirs[:, 1], dirs[:, 0])
    Ys = spherical_harmonics(lmax, th, ph)
    assert np.abs(table @ Ys.T - np.eye(len(table))).max() < 1e-13
    # a real band-limited field's modes, the negative m by symmetry
    rng = np.random.default_rng(5)
    coef = {lm: complex(*rng.normal(size=2)) for lm in harmonic_modes(lmax)}
    for l in range(lmax + 1):
        coef[(l, 0)] = coef[(l, 0)].real
    vals = sum(2 * np.real(coef[(l, m)] * Ys[mode_index(l, m)]) if m > 0 else coef[(l, m)].real * Ys[mode_index(l, m)].real
               for (l, m) in harmonic_modes(lmax))
    modes = table @ vals
    for (l, m) in harmonic_modes(lmax):
        assert abs(modes[mode_index(l, m)] - coef[(l, m)]) < 1e-13


@pytest.mark.parametrize("grading", [0.0, 1.5])
def test_ball_inverse_map(grading):
    # test/extraction_tests.jl:60-93: the forward map of what is found gives
    # the point back, inside its patch's box, in every patch
    geo = SevenPatchBall(1.0, 3.0, (4, 3), grading=grading)
    rng = np.random.default_rng(11)
    pts = rng.normal(size=(4000, 3))
    pts = pts / np.linalg.norm(pts, axis=1)[:, None] * 3 * rng.random(4000)[:, None] ** (1 / 3)
    pts = np.concatenate([pts, [[1.0, 0.3, -0.2], [1.0, 1.0, 0.5], [-1, -1, -1], [0, 0, 3.0],
                                np.array([3, 3, 3]) / math.sqrt(3), [0, -2.0, 0], [0, 0, 0]]])
    worst, patches = 0.0, set()
    for x in pts:
        p, xi = ball_patch_point(geo, x)
        patches.add(p)
        y = np.array([np.asarray(v, dtype=np.float64).reshape(-1)[0]
                      for v in geo.position(tuple(np.array([c]) for c in xi), p)])
        worst = max(worst, float(np.linalg.norm(y - x)))
        r = geo.patch_roots(p)
        assert all(0 <= xi[d] <= r[d] for d in range(3))
    assert worst < 1e-13
    assert patches == set(range(7))
    assert ball_patch_point(geo, (0.5, -0.25, 1.0))[0] == 0
    assert ball_patch_point(geo, (0.0, 0.0, 2.0))[0] == 6
    assert ball_patch_point(geo, (-2.0, 0.0, 0.0))[0] == 1
    with pytest.raises(ValueError, match="beyond the ball's sphere"):
        ball_patch_point(geo, (0.0, 3.1, 0.0))


def gather(index, weights, u, var, NN):
    return (weights * u[index + (var - 1) * NN]).sum(axis=1)


def test_brick_stencils_are_the_oracle_polynomials_and_converge():
    # test/extraction_tests.jl:133-147 on the host: the stencils' reading is
    # the oracle's own element polynomial, and converges at order P + 1
    P = 3
    table, dirs = sphere_rule(3, 9)
    errs = []
    for s in (1, 2):
        f = wave_forest(np.float64, 3, P, 2, roots=4 * s, L=4.0)
        u = state_from(f, P, fill)
        pts = np.concatenate([np.array([2.0, 2.0, 2.0]) + r * dirs for r in (0.5, 1.5)])
        index, weights = element_stencils(f, P, pts)
        NN = f.N ** 3
        vals = gather(index, weights, u, 1, NN)
        if s == 1:
            ref = oracle_point_values(f, P, u, pts[:300], var=2)
            assert np.abs(gather(index[:300], weights[:300], u, 2, NN) - ref).max() < 1e-13 * np.abs(ref).max()
        errs.append(np.abs(vals - extraction_f(pts.T)).max())
    assert math.log2(errs[0] / errs[1]) > P + 0.5


@pytest.mark.parametrize("refined", [False, True])
def test_ball_stencils_converge_across_the_patches(refined):
    # the seven-patch ball: spheres inside the cube's refined region, across
    # its coarse-fine faces, across the cube-shell faces and in the shells
    # converge at order P + 1 (test/extraction_tests.jl:95-131); refined, the
    # cube's (s, 3s)^3 is one level finer, and a point read from the wrong
    # level's leaf stops the error from falling
    P = 3
    table, dirs = sphere_rule(4, 10)
    errs = []
    for s in (1, 2):
        f, geo = sevenpatch_forest(np.float64, P, 2, roots=(4 * s, 2 * s),
                                   refined=((s, 3 * s),) * 3 if refined else False)
        if refined:
            assert max(f.levels) == 1
        tables = ball_tables(f, P)
        u = ball_state(f, tables, fill)
        pts = np.concatenate([r * dirs for r in (0.3, 0.7, 1.3, 2.2)])
        index, weights = element_stencils(f, P, pts)
        vals = gather(index, weights, u, 1, f.N ** 3)
        errs.append(np.abs(vals - extraction_f(pts.T)).max())
    assert math.log2(errs[0] / errs[1]) > P + 0.5


def test_extraction_refuses_what_it_cannot_read():
    f = wave_forest(np.float64, 3, 2, 2, roots=4, L=4.0)
    with pytest.raises(ValueError, match="periodic image"):
        element_stencils(f, 2, [np.array([2.0, 2.0, 5.1])])
    from twoldg.geometry import annulus_forest
    g, geo = annulus_forest(np.float64, 2, 2)
    with pytest.raises(ValueError, match="brick or the seven-patch ball"):
        element_stencils(g, 2, [np.array([0.5, 0.5])], geometry=geo)


@pytest.mark.parametrize("D,P", [(2, 3), (3, 2), (3, 4)])
def test_gradient_stencils_are_the_basis_derivatives(D, P):
    # reconstruct_gradient (src/transfer.jl:2011-2030) reads the element's
    # polynomial through derivative weights: they are the oracle's basis
    # derivatives at the point, and a polynomial of degree P per dimension
    # filled at the nodes gives its exact gradient
    from oracle import transfer as OT
    from twoldg.extraction import element_stencils
    from twoldg.forest import wave_forest
    forest = wave_forest(np.float64, D, P, 2, roots=2)
    t = OT.Tables(P)
    rng = np.random.default_rng(7)
    pts = rng.uniform(0.02, 0.98, size=(6, D))
    P1, N = P + 1, forest.N
    coef = rng.standard_normal(D)

    def g(X):
        return sum(coef[d] * X[..., d] ** P for d in range(D)) + np.prod(X, axis=-1)

    def grad(X):
        out = np.stack([coef[d] * P * X[..., d] ** (P - 1) for d in range(D)], axis=-1)
        for d in range(D):
            out[..., d] += np.prod(np.delete(X, d, axis=-1), axis=-1)
        return out

    from cases import node_positions
    x = node_positions(forest, P)
    nb = len(forest.leaves)
    u = np.zeros((nb, 2, N ** D))
    u[:, 0] = g(np.moveaxis(x, 1, 2))
    u = u.reshape(-1)
    for d in range(D):
        index, weights = element_stencils(forest, P, pts, deriv=d)
        for j, X in enumerate(pts):
            b = int(index[j, 0] // (2 * N ** D))
            pos = index[j, 0] - b * 2 * N ** D
            e = [(pos // N ** k) % N // P1 for k in range(D)]
            lo = [forest.block_extent(forest.leaves[b])[k][0] + forest.spacing(forest.leaves[b]) * e[k] * P1
                  for k in range(D)]
            hi = [lo[k] + forest.spacing(forest.leaves[b]) * P1 for k in range(D)]
            ref = t.element_basis(lo, hi, X[None, :], deriv=d)[0]
            assert np.abs(weights[j] - ref).max() <= 1e-12 * np.abs(ref).max()
        got = np.sum(weights * u[index], axis=1)
        assert np.abs(got - grad(pts)[:, d]).max() <= 1e-11 * np.abs(grad(pts)).max()
    with pytest.raises(ValueError, match="brick"):
        element_stencils(forest, P, pts, deriv=D)
