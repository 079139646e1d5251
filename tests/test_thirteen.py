"""The thirteen-patch ball and the radiative sphere on the host and the
oracle: the map, its frame and factorization, the glue, the factored
truncation tables against the oracle's per-element projection, the energy
identities, and the reference's published tables. No GPU."""
import math

import numpy as np
import pytest

from ball_cases import ball_setup, oracle_radiative_errors, oracle_sevenpatch_errors
from cases import scrambled
from twoldg.ball import (SHELLS, RadiativeBoundary, ThirteenPatchBall, face_plane_logical, orient,
                         thirteenpatch_forest)
from twoldg.element import Element


def test_thirteen_forest_glue_and_sphere():
    # roots (2, 1, 2): 8 cube + 6 * 4 inner + 6 * 8 outer blocks; the outer
    # sphere is the 6 * 2^2 outer faces of the outer shells
    # (test/thirteenpatch_tests.jl:201-212)
    f, geo = thirteenpatch_forest(np.float64, 2, 2, roots=(2, 1, 2), Lc=1.0, Rm=2.0, R1=3.5)
    assert f.nleaves() == 80
    assert (f.face_nb < 0).sum() == 24
    offs = Element(np.float64, 2).offsets.astype(np.float64)
    N = f.N
    A, B = np.meshgrid(np.arange(N), np.arange(N), indexing="xy")
    A, B = A.reshape(-1), B.reshape(-1)
    turns = 0
    for b, (p, c) in enumerate(f.blocks):
        for face in range(6):
            X1 = np.stack(geo.position(face_plane_logical(c, N, offs, face), p), axis=-1)
            nb = f.face_nb[b * 6 + face]
            if nb < 0:
                assert p >= 7
                assert np.allclose(np.linalg.norm(X1, axis=1), 3.5, rtol=1e-15)
                continue
            code = f.face_code[b * 6 + face]
            nf, o = code & 15, code >> 4
            assert f.face_nb[nb * 6 + nf] == b
            turns += o & 1
            pn, cn = f.blocks[nb]
            X2 = np.stack(geo.position(face_plane_logical(cn, N, offs, nf), pn), axis=-1)
            a2, b2 = orient(A, B, o, N)
            assert np.allclose(X1, X2[a2 + N * b2], atol=1e-12)
    assert turns > 0


def test_thirteen_map_frame_and_factors():
    # the frame is the map's inverse Jacobian (finite differences); on the
    # middle sphere the inner shells end where the outer ones start; on the
    # outer shells x is radial along k, S[k] is radial and S across it
    # tangential, and sqrt(g) is the radial factor times the angular one
    # (test/thirteenpatch_tests.jl:51-138)
    geo = ThirteenPatchBall(1.0, 2.0, 3.5, (2, 1, 2))
    xi = (np.array([0.3, 1.7, 1.2]), np.array([0.9, 0.2, 1.6]), np.array([1.1, 1.5, 0.4]))
    for p in range(13):
        r = geo.patch_roots(p)
        x = tuple(xi[j] * r[j] / 2.0 for j in range(3))
        J, S = geo.frame(x, p)
        eps = 1e-6
        x0 = np.array(geo.position(x, p))
        Jm = np.empty((3, 3, 3))
        for j in range(3):
            xp = list(x)
            xp[j] = x[j] + eps
            Jm[:, :, j] = ((np.array(geo.position(tuple(xp), p)) - x0) / eps).T
        assert np.all(J > 0)
        assert np.allclose(J, np.abs(np.linalg.det(Jm)), rtol=1e-5)
        for q in range(3):
            assert np.allclose(S[q] @ Jm[q], J[q] * np.eye(3), atol=1e-4 * J[q])
        if p >= 7:
            k, s = SHELLS[p - 7]
            X = x0.T
            for q in range(3):
                assert np.linalg.norm(np.cross(S[q, k], X[q])) < 1e-13 * np.linalg.norm(S[q, k]) * np.linalg.norm(X[q])
                for d in range(3):
                    if d != k:
                        assert abs(S[q, d] @ X[q]) < 1e-13 * np.linalg.norm(S[q, d]) * np.linalg.norm(X[q])
            ac = [j for j in range(3) if j != k]
            R = geo.radial_volume(x[k], p)
            Om = geo.angular_volume(x[ac[0]], x[ac[1]])
            assert np.allclose(R * Om, J, rtol=1e-14)
    for k, s in SHELLS:
        pi, po = 1 + SHELLS.index((k, s)), 7 + SHELLS.index((k, s))
        xi_in = [np.array([0.6]), np.array([1.3]), np.array([0.9])]
        xi_out = list(xi_in)
        xi_in[k] = np.array([1.0 if s == 1 else 0.0])          # the inner shell's outer face (m = 1)
        xi_out[k] = np.array([0.0 if s == 1 else 2.0])         # the outer shell's inner face (m' = 2)
        Xi = np.array(geo.position(tuple(xi_in), pi))
        Xo = np.array(geo.position(tuple(xi_out), po))
        assert np.allclose(Xi, Xo, atol=1e-15)
        assert np.linalg.norm(Xi) == pytest.approx(2.0, rel=1e-15)


def test_thirteen_refuses_what_it_cannot_map():
    with pytest.raises(ValueError, match="odd"):
        thirteenpatch_forest(np.float64, 2, 3)
    with pytest.raises(ValueError, match="sqrt\\(3\\) Lc"):
        thirteenpatch_forest(np.float64, 2, 2, Lc=1.0, Rm=1.5, R1=3.0)
    with pytest.raises(ValueError, match="must exceed the middle radius"):
        thirteenpatch_forest(np.float64, 2, 2, Lc=1.0, Rm=2.0, R1=2.0)
    with pytest.raises(ValueError, match="\\(n, m, m'\\)"):
        thirteenpatch_forest(np.float64, 2, 2, roots=(2, 2))
    with pytest.raises(ValueError, match="positive number of roots"):
        thirteenpatch_forest(np.float64, 2, 2, roots=(2, 0, 1))
    with pytest.raises(ValueError, match="negative"):
        RadiativeBoundary(kappa=-1.0)


def factored_apply(tables, P, E, nb, v):
    """The factored truncation restated from the host tables (radial pair along
    k, then the in-plane projection per plane), for the blocks with fac_slot."""
    from twoldg.ball import legendre_at
    el = Element(np.float64, P)
    L = legendre_at(P, el.nodes.astype(np.float64))
    P1, N = P + 1, E * (P + 1)
    v = v.reshape(nb, N, N, N).copy()           # [b, z, y, x]
    rm = tables["fac_rmodes"].reshape(-1, E, P1)
    rd = tables["fac_rduals"].reshape(-1, E, P1)
    aw = tables["fac_aw"].reshape(tables["fac_ntab"], E * E, P1 * P1)
    ach = tables["fac_achol"].reshape(tables["fac_ntab"], E * E, P * P, P * P)   # [.., q, r] = U[r, q]
    Psi = np.array([[L[q % P][n % P1] * L[q // P][n // P1] for q in range(P * P)] for n in range(P1 * P1)])
    for b in range(nb):
        f = tables["fac_slot"][b] - 1
        if f < 0:
            continue
        k, A = tables["fac_radial"][f], tables["fac_aslot"][f]
        d0, d1 = [j for j in range(3) if j != k]
        a = np.moveaxis(v[b], [2 - d0, 2 - d1, 2 - k], [0, 1, 2])   # [x_d0, x_d1, x_k]
        for e in range(E):
            sl = slice(e * P1, (e + 1) * P1)
            c = a[:, :, sl] @ rd[f, e]
            a[:, :, sl] -= c[:, :, None] * rm[f, e][None, None, :]
        for ea in range(E):
            for eb in range(E):
                U = ach[A, ea + E * eb].T
                W = aw[A, ea + E * eb]
                G = U.T @ U
                blk = a[ea * P1:(ea + 1) * P1, eb * P1:(eb + 1) * P1, :]     # [na, nb, x_k]
                flat = blk.transpose(1, 0, 2).reshape(P1 * P1, N)          # node index na + P1 nb
                z = np.linalg.solve(G, Psi.T @ (W[:, None] * flat))
                blk[:] = (Psi @ z).reshape(P1, P1, N).transpose(1, 0, 2)
        v[b] = np.moveaxis(a, [0, 1, 2], [2 - d0, 2 - d1, 2 - k])
    return v.reshape(-1)


@pytest.mark.parametrize("P", [2, 3])
def test_factored_tables_are_the_element_projection(P):
    # on the outer shells the radial pair times the in-plane projection of the
    # host's tables equals the oracle's per-element sqrt(g)-orthogonal
    # projection, solved from sqrt(g) itself (test/thirteenpatch_tests.jl:140-176)
    forest, geo, wave, tables, o = ball_setup(P, 2, (2, 1, 2), Rm=2.0, R1=3.5)
    nb, NN = forest.nleaves(), forest.N ** 3
    assert (tables["fac_slot"] > 0).sum() == 48 and tables["fac_ntab"] == 4 and tables["ntab"] == 24
    u = scrambled(nb * 2 * NN, 0.4)
    ref = o.truncate(u).reshape(nb, 2, NN)
    got = factored_apply(tables, P, 2, nb, u.reshape(nb, 2, NN)[:, 1].copy()).reshape(nb, NN)
    outer = tables["fac_slot"] > 0
    scale = np.abs(ref[outer, 1]).max()
    assert np.abs(got[outer] - ref[outer, 1]).max() < 1e-12 * scale


def energy_rate(o, u):
    # the energy is quadratic: its central difference along du is its rate
    du = o.rhs(u)
    e = 1e-3
    return (o.energy(u + e * du) - o.energy(u - e * du)) / (2 * e), o.energy(u)


def boundary_rate(forest, tables, P, u, kappa):
    # -kappa sum w |S[d]| v^2 over the sphere's nodes: the rate of the energy
    # with the boundary's term (its u v / R part is that term's own rate)
    N, NN, P1 = forest.N, forest.N ** 3, P + 1
    wq = Element(np.float64, P).weights.astype(np.float64)
    coef = tables["coef"].reshape(-1, 10, NN)
    u = u.reshape(-1, 2, NN)
    r = 0.0
    for b in range(forest.nleaves()):
        for f in range(6):
            if forest.face_nb[b * 6 + f] >= 0:
                continue
            d, side = f // 2, f % 2
            tang = [q for q in range(3) if q != d]
            for t in range(N * N):
                x = [0, 0, 0]
                x[d] = N - 1 if side else 0
                x[tang[0]], x[tang[1]] = t % N, t // N
                n = x[0] + N * (x[1] + N * x[2])
                w = np.prod([(1.0 / N) * P1 / 2 * wq[x[q] % P1] for q in tang])
                S = coef[b, 1 + 3 * d:4 + 3 * d, n]
                r -= w * np.linalg.norm(S) * kappa * u[b, 1, n] ** 2
    return r


@pytest.mark.parametrize("P", [2, 3])
@pytest.mark.parametrize("truncate", [False, True])
def test_thirteen_energy_invariant_across_the_glues(P, truncate):
    # zero Dirichlet data and a state vanishing in the outer shells' outermost
    # elements: nothing crosses the sphere, so the energy's rate vanishes
    # across the identity and quarter-turn glues of both layers and the
    # factored truncation (test/thirteenpatch_tests.jl:214-233)
    forest, geo, wave, tables, o = ball_setup(P, 2, (2, 1, 2), truncate, k=(0.0, 0.0, 0.0), phi=0.0, Rm=2.0)
    nb, N = forest.nleaves(), forest.N
    u = scrambled(nb * 2 * N ** 3, 0.2).reshape(nb, 2, N ** 3)
    he = (P + 1) / N
    for b, (p, c) in enumerate(forest.blocks):
        if p >= 7:
            k, s = SHELLS[p - 7]
            xk = tables["xl"][b, k]
            u[b][:, (xk >= 2 - he - 1e-12) if s == 1 else (xk <= he + 1e-12)] = 0
    u = o.truncate(u.reshape(-1))
    rate, E = energy_rate(o, u)
    assert E > 1
    assert abs(rate) < 1e-12 * E


@pytest.mark.parametrize("ball", ["seven", "thirteen"])
@pytest.mark.parametrize("kappa,inverse_r", [(1.0, True), (1.0, False), (0.5, True), (0.0, False)])
@pytest.mark.parametrize("truncate", [False, True])
def test_radiative_sphere_changes_the_energy_by_its_boundary_term(ball, kappa, inverse_r, truncate):
    # the ghosts set u's face value to the face node's and the flux to
    # -sigma |S| (kappa v + u/R), so the energy with the boundary's own term
    # changes at -kappa sum w |S| v^2 (test/sevenpatch_tests.jl:314-341,
    # test/thirteenpatch_tests.jl:235-252)
    P = 3 if kappa == 0.5 else 2
    roots, Rm = ((2, 2), None) if ball == "seven" else ((2, 1, 1), 2.0)
    forest, geo, wave, tables, o = ball_setup(P, 2, roots, truncate, Rm=Rm, radiative=(kappa, inverse_r))
    u = o.truncate(scrambled(forest.nleaves() * 2 * forest.N ** 3, 0.3))
    rate, E = energy_rate(o, u)
    expect = boundary_rate(forest, tables, P, u, kappa)
    assert abs(rate - expect) < 1e-12 * E
    if kappa > 0:
        assert expect < -1e-3 * E


@pytest.mark.parametrize("P,row", [(2, (6.28e-2, 8.09e-2, 239)), (3, (9.37e-3, 1.24e-2, 424))])
def test_thirteen_published_table(P, row):
    # reference CODE.md:4521-4533: the plane wave of the seven-patch table on
    # the thirteen-patch ball Lc = 1, Rm = 2, R1 = 3, roots (2, 1, 1), E = 2,
    # to t = 1, truncated: sqrt(g)-weighted L2 errors of u and v and the steps
    r = oracle_sevenpatch_errors(P, 2, (2, 1, 1), Rm=2.0)
    assert r["nsteps"] == row[2]
    assert r["u"] == pytest.approx(row[0], rel=0.01)
    assert r["v"] == pytest.approx(row[1], rel=0.01)


@pytest.mark.parametrize("kappa,inverse_r,left,l2", [(1.0, True, 3.5e-3, 2.5e-2), (0.0, False, None, 0.54)])
def test_radiative_published_table(kappa, inverse_r, left, l2):
    # reference CODE.md:4268-4281: the outgoing pulse of width 1/2 on the
    # seven-patch ball, roots (2, 2), E = 2, P = 3, to t = 5: the energy left
    # (the boundary's term included) and the L2 error; Sommerfeld's condition
    # lets the pulse out, the wall (kappa = 0, no u/R) keeps it to 1 - 2.3e-9
    r = oracle_radiative_errors(3, 2, (2, 2), kappa=kappa, inverse_r=inverse_r, tend=5.0)
    ratio = r["energy"] / r["energy0"]
    if left is None:
        assert 1 - ratio == pytest.approx(2.3e-9, rel=0.05)
    else:
        assert ratio == pytest.approx(left, rel=0.03)
    assert r["l2"] == pytest.approx(l2, rel=0.02)


def test_outer_shells_sqrtg_is_the_product_of_the_declared_factors():
    # test/thirteenpatch_tests.jl:116-138: the factored truncation is
    # sqrt(g)-orthogonal only if the radial factor r^2 r' and the angular one
    # (2/n)^2 (1 + c_a^2 + c_b^2)^(-3/2) multiply to the frame's sqrt(g), with
    # one angular function shared by the six shells; the cube and the inner
    # shells do not factorize
    from twoldg.ball import thirteenpatch_forest
    forest, geo = thirteenpatch_forest(np.float64, 2, 2, roots=(3, 1, 2), Lc=1.0, Rm=2.0, R1=3.5)
    assert all(geo.factored_dim(q) == -1 for q in range(7))
    for xi in ((0.3, 0.7, 0.9), (2.9, 0.1, 1.2), (1.5, 1.5, 1.5)):
        for q in range(7, 13):
            k = geo.factored_dim(q)
            assert k == (q - 7) // 2
            xa, xb = (xi[j] for j in range(3) if j != k)
            J = float(geo.frame(xi, q)[0])
            assert geo.radial_volume(xi[k], q) * geo.angular_volume(xa, xb) == pytest.approx(J, rel=1e-14)
