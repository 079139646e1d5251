"""The seven-patch ball (full metric, quarter-turn glue, Dirichlet sphere):
the host geometry and glue, and the oracle against the reference's published
table. No GPU."""
import math

import numpy as np
import pytest

from ball_cases import ball_setup, oracle_sevenpatch_errors
from twoldg.ball import face_plane_logical, orient, sevenpatch_forest
from twoldg.element import Element


def test_ball_forest_and_glue_continuity():
    # 8 + 6 * 8 blocks at roots (2, 2); 448 at (4, 4); every glued face's
    # nodes coincide with the neighbour's under the face table's orientation
    # (the property the reference fixes the quarter turns by)
    for roots, nb, nbnd in (((2, 2), 56, 24), ((4, 4), 448, 96)):
        f, geo = sevenpatch_forest(np.float64, 3, 2, roots=roots)
        assert f.nleaves() == nb
        assert (f.face_nb < 0).sum() == nbnd
    f, geo = sevenpatch_forest(np.float64, 2, 2, roots=(2, 2))
    offs = Element(np.float64, 2).offsets.astype(np.float64)
    N = f.N
    A, B = np.meshgrid(np.arange(N), np.arange(N), indexing="xy")
    A, B = A.reshape(-1), B.reshape(-1)
    quarter_turns = 0
    for b, (p, c) in enumerate(f.blocks):
        for face in range(6):
            nb = f.face_nb[b * 6 + face]
            if nb < 0:
                X = np.stack(geo.position(face_plane_logical(c, N, offs, face), p), axis=-1)
                assert np.allclose(np.linalg.norm(X, axis=1), geo.R1)
                continue
            code = f.face_code[b * 6 + face]
            nf, o = code & 15, code >> 4
            quarter_turns += (o & 1)
            pn, cn = f.blocks[nb]
            X1 = np.stack(geo.position(face_plane_logical(c, N, offs, face), p), axis=-1)
            X2 = np.stack(geo.position(face_plane_logical(cn, N, offs, nf), pn), axis=-1)
            a2, b2 = orient(A, B, o, N)
            assert np.allclose(X1, X2[a2 + N * b2], atol=1e-12)
    assert quarter_turns > 0


def test_frame_is_the_inverse_jacobian():
    f, geo = sevenpatch_forest(np.float64, 2, 2, roots=(2, 2))
    xi = (np.array([0.3, 1.7]), np.array([0.9, 0.2]), np.array([1.1, 1.5]))
    for p in range(7):
        J, S = geo.frame(xi, p)
        eps = 1e-6
        x0 = np.array(geo.position(xi, p))
        Jm = np.empty((2, 3, 3))
        for j in range(3):
            xp = list(xi)
            xp[j] = xi[j] + eps
            Jm[:, :, j] = ((np.array(geo.position(tuple(xp), p)) - x0) / eps).T
        assert np.allclose(J, np.abs(np.linalg.det(Jm)), rtol=1e-5)
        for k in range(2):
            assert np.allclose(S[k] @ Jm[k], J[k] * np.eye(3), atol=1e-4 * J[k])


# reference CODE.md:4247-4252: k = (1.1, -0.7, 0.5), phi = 0.3, Lc = 1, R1 = 3,
# t = 1, patches of (2s, 2s) roots, E = 2, cfl 1/2: the sqrt(g)-weighted L2
# errors of u and of v, and 1 - E1/E0 (the energy the wave carries out), at
# s = 1, 2 for P = 2 and s = 1 for P = 3 (the larger runs left out for time)
SEVENPATCH = [
    (2, True, (6.07e-2, 1.63e-2), (7.81e-2, 2.25e-2), (0.016, 0.030)),
    (2, False, (4.97e-2, 3.87e-3), (9.33e-2, 1.45e-2), (0.032, 0.035)),
    (3, True, (8.83e-3,), (1.14e-2,), (0.035,)),
    (3, False, (2.32e-3,), (6.85e-3,), (0.035,)),
]


def _printed(value, printed, digits=3):
    """value rounds to the significant digits printed."""
    e = np.floor(np.log10(abs(printed)))
    return abs(value - printed) <= 0.5001 * 10.0 ** (e - digits + 1)


@pytest.mark.parametrize("row", SEVENPATCH, ids=["P%d-%s" % (r[0], "trunc" if r[1] else "plain") for r in SEVENPATCH])
def test_sevenpatch_published_table(row):
    # every printed digit (two for the energy carried out)
    P, truncate, us, vs, des = row
    for i in range(len(us)):
        s = i + 1
        r = oracle_sevenpatch_errors(P, 2, (2 * s, 2 * s), truncate=truncate)
        assert _printed(r["u"], us[i]), (s, r["u"])
        assert _printed(r["v"], vs[i]), (s, r["v"])
        assert _printed(1 - r["energy"] / r["energy0"], des[i], digits=2), (s, r["energy"] / r["energy0"])


@pytest.mark.parametrize("P", [2, 3])
@pytest.mark.parametrize("grading", [0.0, 1.5])
def test_ball_laplacian_is_self_adjoint_away_from_the_sphere(P, grading):
    # with homogeneous data (a field vanishing on the sphere's ghosts), the
    # full-metric Laplacian is self-adjoint in sqrt(g)-weighted quadrature over
    # the cube and its glued shells, graded or not, to the 1e-13 of
    # test/sevenpatch_tests.jl:182-226: checked on fields supported inside
    # |x| < 1.5
    forest, geo, wave, tables, o = ball_setup(P, 2, (2, 2), truncate=False, k=(0.0, 0.0, 0.0), phi=0.0,
                                              grading=grading)
    from ball_cases import physical_nodes
    X = physical_nodes(forest, tables)
    r = np.linalg.norm(X, axis=1)
    bump = lambda c: np.where(r < 1.5, np.cos(np.pi * r / 3.0) ** 4, 0.0) * (1 + 0.3 * X[:, c])
    nb, NN = forest.nleaves(), forest.N ** 3

    def lap(a):
        s = np.zeros((nb, 2, NN))
        s[:, 0] = a
        return o.rhs(s.reshape(-1)).reshape(nb, 2, NN)[:, 1]
    P1 = P + 1
    N = forest.N
    wq = Element(np.float64, P).weights
    w1 = (1.0 / N) * P1 / 2 * wq[np.arange(N) % P1]
    w = np.kron(np.kron(w1, w1), w1)[None, :] * tables["coef"].reshape(nb, 10, NN)[:, 0]
    a, b = bump(0), bump(1)
    la, lb = lap(a), lap(b)
    lhs, rhs = np.sum(w * b * la), np.sum(w * lb * a)
    assert abs(lhs - rhs) < 1e-13 * np.sum(np.abs(w * b * la))



def _flat_truncate(s, nb, N, el):
    """The element's own tensor projector on v, line by line along each
    dimension in order: the identity on Q_{P-1} and on nothing else."""
    P1 = el.P + 1
    mode, dual = el.topmode.astype(np.float64), el.topdual.astype(np.float64)
    out = s.reshape(nb, 2, N, N, N).copy()                      # [b, var, i2, i1, i0]
    v = out[:, 1]
    for d in range(3):
        w = np.moveaxis(v, 3 - d, -1)                          # a view, dimension d last
        for e in range(N // P1):
            line = w[..., e * P1:(e + 1) * P1]
            line -= (line @ dual)[..., None] * mode
    return out.reshape(-1)


@pytest.mark.parametrize("P", [2, 3])
def test_ball_truncation_is_the_sqrtg_orthogonal_projection(P):
    # test/sevenpatch_tests.jl:128-158 on the oracle's projector (each
    # element's solved directly from sqrt(g)): self-adjoint in the sqrt(g)
    # weights, a projection, onto Q_{P-1} (the element's own projector leaves
    # its result and not the data's), u left alone, the kinetic energy not
    # raised
    forest, geo, wave, tables, o = ball_setup(P, 2, (2, 2), truncate=True, k=(0.0, 0.0, 0.0), phi=0.0)
    el = Element(np.float64, P)
    nb, N = forest.nleaves(), forest.N
    NN = N ** 3
    P1 = P + 1
    w1 = (1.0 / N) * P1 / 2 * el.weights.astype(np.float64)[np.arange(N) % P1]
    wg = (np.kron(np.kron(w1, w1), w1)[None, :] * tables["coef"].reshape(nb, 10, NN)[:, 0]).reshape(-1)
    rng = np.random.default_rng(3)
    a, b = rng.standard_normal(nb * 2 * NN), rng.standard_normal(nb * 2 * NN)

    def v(x):
        return x.reshape(nb, 2, NN)[:, 1].reshape(-1)

    def inner(x, y):
        return float(np.sum(wg * x * y))

    ta, tb = o.truncate(a), o.truncate(b)
    scale = math.sqrt(inner(v(a), v(a)) * inner(v(b), v(b)))
    assert abs(inner(v(ta), v(b)) - inner(v(a), v(tb))) < 1e-14 * scale
    assert np.allclose(o.truncate(ta), ta, rtol=0, atol=1e-13 * np.abs(ta).max())
    assert np.allclose(_flat_truncate(ta, nb, N, el), ta, rtol=0, atol=1e-12 * np.abs(ta).max())
    assert not np.allclose(_flat_truncate(a, nb, N, el), a)
    assert np.array_equal(ta.reshape(nb, 2, NN)[:, 0], a.reshape(nb, 2, NN)[:, 0])
    assert inner(v(ta), v(ta)) <= inner(v(a), v(a))


def test_dirichlet_data_of_any_form_converge_at_order_P():
    """Dirichlet data other than the plane wave (the reference's
    DirichletValues takes any data(x, t), src/evolution.jl:1110-1127): the
    spherical standing wave j0(k r) cos(k t), k = 2, as the data on the
    seven-patch ball's sphere, P = 3 truncated, to t = 1/2 at cfl 1/2. The
    oracle's run converges at order P between roots (2, 2) and (3, 3)."""
    import math
    from twoldg.ball import SphericalStandingWave, ball_forest, ball_tables
    from oracle.oracle import BallOracle
    from ball_cases import ball_state
    w = SphericalStandingWave(2.0)
    errs, hs = [], []
    for roots in ((2, 2), (3, 3)):
        forest, geo = ball_forest(np.float64, 3, 2, roots, 1.0, 3.0)
        tables = ball_tables(forest, 3, w)
        o = BallOracle(forest, 3, tables, None, truncate=True, standing=2.0)
        u0 = o.truncate(ball_state(forest, tables, lambda x, v: w.state(x, 0.0, v)))
        n = int(math.ceil(0.5 / (0.5 * tables["hspeed"] / 4)))
        u = o.rk4(u0, 0.5 / n, n, 0.0)
        ue = ball_state(forest, tables, lambda x, v: w.state(x, 0.5, v))
        errs.append(o.norm(u, 2, 3, ue))
        hs.append(1.0 / roots[0])
    assert errs[0] < 1.2e-3
    rate = math.log(errs[0] / errs[1]) / math.log(hs[0] / hs[1])
    assert rate > 2.7, (errs, rate)


# --- the refined cube (src/geometry.jl:494-553, test/sevenpatch_tests.jl:421-535) ---

def _refined(P, roots=(4, 1), refined=True, Rm=None, k=(0.0, 0.0, 0.0), phi=0.0, truncate=False):
    from twoldg.ball import ball_forest, ball_tables, PlaneWave
    from oracle.oracle import BallOracle
    forest, geo = ball_forest(np.float64, P, 2, roots, 1.0, 3.0, Rm=Rm, refined=refined)
    wave = PlaneWave(k, phi)
    tables = ball_tables(forest, P, wave)
    return forest, geo, wave, tables, BallOracle(forest, P, tables, wave, truncate=truncate)


def test_refined_ball_forest_and_its_refusals():
    # refined=True refines the cube's middle half to level 1 and nothing else;
    # a region reaching the cube's faces would refine a shell across the glue,
    # and a region with no block centre in it refines nothing: both refused
    from twoldg.ball import CUBE_FACE, sevenpatch_forest
    f, geo = sevenpatch_forest(np.float64, 2, 2, roots=(4, 1), refined=True)
    assert max(f.levels) == 1
    assert all(p == 0 or lv == 0 for (p, _), lv in zip(f.blocks, f.levels))
    assert f.nleaves() == 64 - 8 + 64 + 6 * 16
    assert f.minimum_spacing() == pytest.approx(0.5 / f.N)
    # the cube's inner faces are resolved by the library; the glue and the sphere as before
    assert np.sum(f.face_nb == CUBE_FACE) > 0 and np.sum(f.face_nb == -1) == 6 * 16
    with pytest.raises(ValueError, match="reaches the cube's faces"):
        sevenpatch_forest(np.float64, 2, 2, roots=(4, 1), refined=((0.0, 2.0), (1.0, 3.0), (1.0, 3.0)))
    with pytest.raises(ValueError, match="no block centre"):
        sevenpatch_forest(np.float64, 2, 2, roots=(2, 1), refined=True)
    # the inspiral's nested cubes inside the ball: two levels about the centre
    from twoldg.forest import nested_cubes
    g, _ = sevenpatch_forest(np.float64, 2, 2, roots=(8, 1), refined=nested_cubes(3, 1.0, 3))
    assert max(g.levels) == 2


@pytest.mark.parametrize("P", [2, 3])
@pytest.mark.parametrize("truncate", [False, True])
def test_refined_ball_energy_is_invariant(P, truncate):
    # test/sevenpatch_tests.jl:421-444 on the oracle: with homogeneous data the
    # Laplacian of the refined ball is self-adjoint in the sqrt(g)-weighted
    # quadrature across the cube's coarse-fine faces and the glues (the coarse
    # ghost of the Cartesian gradient the adjoint of the fine one), and with
    # the truncation so is the projected operator, to 1e-13 of the terms
    from ball_cases import physical_nodes
    forest, geo, wave, tables, o = _refined(P, truncate=truncate)
    X = physical_nodes(forest, tables)
    r = np.linalg.norm(X, axis=1)
    nb, N = forest.nleaves(), forest.N
    NN = N ** 3
    bump = lambda c: np.where(r < 1.5, np.cos(np.pi * r / 3.0) ** 4, 0.0) * (1 + 0.3 * X[:, c])

    def op(a):
        s = np.zeros((nb, 2, NN))
        s[:, 1] = a
        s = o.truncate(s.reshape(-1)) if truncate else s.reshape(-1)
        s = s.reshape(nb, 2, NN)
        s[:, 0], s[:, 1] = s[:, 1].copy(), 0.0
        out = o.rhs(s.reshape(-1)).reshape(nb, 2, NN)
        t = np.zeros((nb, 2, NN))
        t[:, 1] = out[:, 1]
        return (o.truncate(t.reshape(-1)) if truncate else t.reshape(-1)).reshape(nb, 2, NN)[:, 1]
    P1 = P + 1
    wq = Element(np.float64, P).weights
    hs = np.array([forest.block_scale(b) / N for b in range(nb)])
    w1 = hs[:, None] * P1 / 2 * wq[np.arange(N) % P1][None, :]
    w = np.einsum("bi,bj,bk->bkji", w1, w1, w1).reshape(nb, NN) * tables["coef"].reshape(nb, 10, NN)[:, 0]
    a, b = bump(0), bump(1)
    la, lb = op(a), op(b)
    lhs, rhs = np.sum(w * b * la), np.sum(w * lb * a)
    scale = np.sum(np.abs(w * b * la))
    assert scale > 1
    assert abs(lhs - rhs) < 1e-13 * scale


def test_refined_ball_time_step_is_the_binding_blocks():
    # test/sevenpatch_tests.jl:480-497: the step is the smaller of each block's
    # own spacing over its own speed, here the cube's finest blocks',
    # h/(n/2Lc), and above the finest spacing over the fastest speed
    P = 2
    forest, geo, wave, tables, o = _refined(P)
    h = forest.minimum_spacing()
    assert tables["hspeed"] == pytest.approx(h / (4 / 2), rel=1e-14)
    from twoldg.ball import ball_forest, ball_tables
    uniform, _ = ball_forest(np.float64, P, 2, (4, 1), 1.0, 3.0)
    t0 = ball_tables(uniform, P, wave)
    speed = uniform.minimum_spacing() / t0["hspeed"]      # the fastest logical speed, uniform ball
    assert tables["hspeed"] > 1.5 * h / speed


def test_refined_ball_cube_takes_the_element_projector():
    # test/sevenpatch_tests.jl:446-470: the cube's blocks hold no tables
    # (slot 0, the element's tensor projector), the shells' theirs
    forest, geo, wave, tables, o = _refined(3, truncate=True)
    cube = np.array([p == 0 for p, _ in forest.blocks])
    slot = np.asarray(tables["elem_slot"])
    assert np.all((slot == 0) == cube)
    assert sorted(slot[~cube]) == list(range(1, int(np.sum(~cube)) + 1))


def test_refined_ball_plane_wave_as_accurate_as_uniform():
    # test/sevenpatch_tests.jl:499-535 on the oracle: refining the cube adds
    # resolution there and nothing else, so the error cannot grow
    from ball_cases import ball_state
    for P in (2, 3):
        res = {}
        for refined in (False, True):
            forest, geo, wave, tables, o = _refined(P, refined=refined, k=(1.1, -0.7, 0.5), phi=0.3,
                                                    truncate=True)
            u0 = o.truncate(ball_state(forest, tables, lambda x, v: wave.state(x, 0.0, v)))
            n = int(math.ceil(0.25 / (0.5 * tables["hspeed"] / (P + 1))))
            u = o.rk4(u0, 0.25 / n, n, 0.0)
            ue = ball_state(forest, tables, lambda x, v: wave.state(x, 0.25, v))
            res[refined] = (o.norm(u, 2, 3, ue), forest.nleaves(), forest.minimum_spacing())
        assert res[True][1] > res[False][1]
        assert res[True][0] <= 1.01 * res[False][0]
        assert res[True][2] == res[False][2] / 2
