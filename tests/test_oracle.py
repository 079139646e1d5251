"""The oracle pinned: against the reference's dense-matrix reference
(test/reference.jl via tests/dense.py), its property tests and its published
convergence numbers. No GPU."""
import math

import numpy as np
import pytest

from cases import refined_forest, scrambled, state_from, smooth_data
from dense import along, from_global, global_array, global_operators
from oracle.oracle import Oracle, golden_tables
from oracle_drivers import exact
from oracle_drivers import oracle_errors as _oracle_errors
import functools

# runs that several tests read are made once (the results are only read)
oracle_errors = functools.lru_cache(maxsize=None)(_oracle_errors)
from twoldg.forest import wave_forest


@pytest.mark.parametrize("D,P,E,roots", [(1, 3, 2, 3), (2, 2, 2, 3), (2, 3, 2, 2), (3, 1, 2, 3)])
def test_rhs_is_the_global_operator(D, P, E, roots):
    # test/evolution_tests.jl:22-59: du_u = v and du_v = sum_d along(Dm,d)^2 U to 1e-12
    forest = wave_forest(np.float64, D, P, E, roots=roots)
    o = Oracle(forest, P)
    u = state_from(forest, P, smooth_data(D))
    du = o.rhs(u)
    t = golden_tables(P)
    Dm, _, _ = global_operators(t["stencil"], t["truncate"], t["weights"], P, roots * E, forest.minimum_spacing())
    lap = sum(along(Dm, d, D) @ along(Dm, d, D) for d in range(D))
    U, V = global_array(forest, u, 0), global_array(forest, u, 1)
    assert np.array_equal(global_array(forest, du, 0), V)
    ref = lap @ U
    assert np.abs(global_array(forest, du, 1) - ref).max() < 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("D,P,E,roots", [(1, 3, 2, 2), (2, 2, 2, 2), (2, 4, 2, 1), (3, 3, 2, 1)])
def test_truncation_is_the_tensor_projector(D, P, E, roots):
    # test/evolution_tests.jl:83-103
    forest = wave_forest(np.float64, D, P, E, roots=roots)
    o = Oracle(forest, P)
    u = state_from(forest, P, smooth_data(D))
    w = o.truncate(u)
    t = golden_tables(P)
    _, Pim, _ = global_operators(t["stencil"], t["truncate"], t["weights"], P, roots * E, 1.0)
    Pi = Pim
    for _ in range(D - 1):
        Pi = np.kron(Pi, Pim)
    V = global_array(forest, u, 1)
    assert np.abs(global_array(forest, w, 1) - Pi @ V).max() < 1e-13 * np.abs(V).max()
    assert np.array_equal(global_array(forest, w, 0), global_array(forest, u, 0))
    assert np.abs(o.truncate(w) - w).max() < 1e-14 * np.abs(V).max()


def test_rhs_neither_writes_u_nor_remembers():
    # test/evolution_tests.jl:61-75
    forest = wave_forest(np.float64, 2, 2, 2, roots=2)
    o = Oracle(forest, 2)
    u = state_from(forest, 2, smooth_data(2))
    u0 = u.copy()
    a = o.rhs(u)
    o.rhs(2 * u)
    b = o.rhs(u)
    assert np.array_equal(u, u0) and np.array_equal(a, b)


def _weights(o, forest, P):
    t = golden_tables(P)
    N, D = forest.N, forest.D
    P1 = P + 1
    out = []
    for key in forest.leaves:
        h = forest.spacing(key)
        w1 = h * P1 / 2 * t["weights"][np.arange(N) % P1]
        w = np.ones(1)
        for _ in range(D):
            w = np.kron(w1, w)
        out.append(w)
    return np.array(out)


def _skew_residual(o, forest, P, a_u, b_u):
    """<b, Lap a>_w - <Lap b, a>_w relative: the Laplacian's self-adjointness,
    which is what makes the energy invariant (test/refined_tests.jl:82-143)."""
    nb = len(forest.leaves)
    NN = forest.N ** forest.D
    def lap(x):
        s = np.zeros((nb, 2, NN))
        s[:, 0] = x
        return o.rhs(s.reshape(-1)).reshape(nb, 2, NN)[:, 1]
    w = _weights(o, forest, P)
    la, lb = lap(a_u), lap(b_u)
    lhs = np.sum(w * b_u * la)
    rhs = np.sum(w * lb * a_u)
    return abs(lhs - rhs) / (np.sum(np.abs(w * b_u * la)) + np.sum(np.abs(w * lb * a_u)))


@pytest.mark.parametrize("D,P,reflecting", [(1, 3, False), (2, 2, False), (2, 3, True), (3, 2, False),
                                            (3, 1, True)])
def test_refined_laplacian_is_self_adjoint(D, P, reflecting):
    # A coarse ghost that is not the adjoint of the fine one breaks this;
    # measured residual ~1e-18 relative in the reference (CODE.md "The energy").
    forest = refined_forest(D, P, reflecting)
    assert len({lv for lv, _ in forest.leaves}) == 2
    o = Oracle(forest, P)
    n = len(forest.leaves) * forest.N ** D
    a = scrambled(n, 0.1).reshape(len(forest.leaves), -1)
    b = scrambled(n, 0.37).reshape(len(forest.leaves), -1)
    assert _skew_residual(o, forest, P, a, b) < 1e-13


@pytest.mark.parametrize("D,P", [(2, 3), (3, 3)])
def test_refined_exact_to_degree_P_along_and_P_minus_1_across(D, P):
    # test/refined_tests.jl:163-210 in the form the RHS exposes: the coarse
    # ghost R is exact to degree P-1 tangentially (not P), so on a two-level
    # forest the Laplacian is exact for data of degree P-1 in every dimension,
    # and not for degree P across a coarse-fine face. Checked on the blocks
    # around the refined middle, away from the periodic box's faces where a
    # polynomial is not periodic.
    forest = refined_forest(D, P)
    o = Oracle(forest, P)
    from cases import node_positions
    x = node_positions(forest, P)
    nb = len(forest.leaves)
    inner = [b for b, (lv, c) in enumerate(forest.leaves)
             if all(0.3 < (lo + hi) / 2 < 0.7 for lo, hi in forest.block_extent((lv, c)))]
    assert inner
    u = np.zeros((nb, 2, forest.N ** D))
    u[:, 0] = sum((x[:, k] - 0.5) ** 2 for k in range(D))
    du = o.rhs(u.reshape(-1)).reshape(nb, 2, -1)[:, 1]
    assert np.abs(du[inner] - 2.0 * D).max() < 1e-9
    # degree P tangentially is not reproduced by the coarse ghosts
    u[:, 0] = (x[:, 0] - 0.5) ** P
    du = o.rhs(u.reshape(-1)).reshape(nb, 2, -1)[:, 1]
    assert np.abs(du - P * (P - 1) * (x[:, 0] - 0.5) ** (P - 2))[inner].max() > 1e-6


def test_reflecting_wall_mirrors_with_parity():
    # On a reflecting box the Neumann cos mode's u has zero normal gradient at
    # the wall; the RHS of a field even about every wall is the global
    # operator of the box mirrored into a periodic box of twice the side.
    D, P, E, roots = 2, 3, 2, 2
    fr = wave_forest(np.float64, D, P, E, roots=roots, reflecting=True)
    fp = wave_forest(np.float64, D, P, E, roots=2 * roots, L=2.0)
    orf, op = Oracle(fr, P), Oracle(fp, P)
    f = lambda x, var: np.cos(math.pi * x[0]) * np.cos(2 * math.pi * x[1]) + 0.3 * np.cos(3 * math.pi * x[0]) * var
    ur = state_from(fr, P, f)
    # the mirrored field on [0,2)^2 with nodes mirrored as well: build it from the
    # reflecting box's global array by reflection of node order
    n = roots * fr.N
    Ur = global_array(fr, ur, 0).reshape(n, n, order="F")
    Vr = global_array(fr, ur, 1).reshape(n, n, order="F")
    mirror = lambda A: np.block([[A, A[::-1, :]], [A[:, ::-1], A[::-1, ::-1]]]).T.T
    def mir(A):
        top = np.concatenate([A, A[::-1, :]], axis=0)
        return np.concatenate([top, top[:, ::-1]], axis=1)
    up = np.zeros(2 * len(fp.leaves) * fp.N ** D)
    from_global(fp, mir(Ur).reshape(-1, order="F"), up, 0)
    from_global(fp, mir(Vr).reshape(-1, order="F"), up, 1)
    dr = global_array(fr, orf.rhs(ur), 1).reshape(n, n, order="F")
    dp = global_array(fp, op.rhs(up), 1).reshape(2 * n, 2 * n, order="F")
    assert np.abs(dr - dp[:n, :n]).max() < 1e-10 * np.abs(dp).max()
    del mirror


# reference CODE.md:4124-4145: the standing sine mode to a quarter period,
# E = 2, roots 2, 4, 8, cfl 1/2: D, P, truncate, the L2 errors of u and of v
CONVERGENCE = [
    (1, 1, True, (5.06e-1, 2.72e-1, 1.38e-1), (3.16, 1.70, 8.67e-1)),
    (1, 1, False, (1.10e-1, 2.83e-2, 7.12e-3), (4.92e-1, 1.17e-1, 2.87e-2)),
    (1, 2, True, (1.00e-1, 2.69e-2, 6.65e-3), (7.76e-1, 1.88e-1, 5.45e-2)),
    (1, 2, False, (8.08e-2, 3.46e-3, 4.38e-4), (6.93e-1, 1.13e-1, 2.48e-2)),
    (1, 3, True, (1.48e-2, 1.70e-3, 2.08e-4), (9.37e-2, 1.15e-2, 1.29e-3)),
    (1, 3, False, (2.77e-3, 8.41e-5, 2.59e-6), (4.38e-2, 1.01e-2, 1.29e-3)),
    (1, 4, True, (1.42e-3, 1.02e-4, 6.63e-6), (1.12e-2, 7.99e-4, 4.90e-5)),
    (1, 4, False, (2.32e-4, 6.90e-6, 1.44e-7), (1.00e-2, 1.08e-4, 2.49e-5)),
    (1, 5, True, (1.12e-4, 3.23e-6, 9.85e-8), (7.21e-4, 1.98e-5, 6.26e-7)),
    (1, 5, False, (1.36e-5, 1.44e-7, 1.10e-9), (2.56e-4, 1.20e-5, 4.08e-7)),
    (2, 1, True, (4.35e-1, 2.61e-1, 1.37e-1), (3.86, 2.32, 1.21)),
    (2, 1, False, (7.80e-2, 2.00e-2, 5.04e-3), (4.92e-1, 1.17e-1, 2.87e-2)),
    (2, 2, True, (1.04e-1, 2.56e-2, 6.54e-3), (8.95e-1, 2.58e-1, 7.34e-2)),
    (2, 2, False, (6.73e-2, 4.68e-3, 3.67e-4), (2.59e-1, 8.05e-2, 2.66e-2)),
    (2, 3, True, (1.47e-2, 1.71e-3, 2.08e-4), (1.43e-1, 1.55e-2, 1.87e-3)),
    (2, 3, False, (2.89e-3, 3.99e-4, 4.85e-5), (5.23e-2, 5.70e-3, 8.05e-4)),
    (2, 4, True, (1.46e-3, 1.02e-4, 6.61e-6), (1.20e-2, 9.31e-4, 6.38e-5)),
    (2, 4, False, (2.87e-4, 5.15e-6, 1.05e-7), (1.01e-2, 4.11e-4, 2.69e-5)),
    (2, 5, True, (1.12e-4, 3.23e-6, 9.86e-8), (1.03e-3, 2.90e-5, 8.78e-7)),
    (2, 5, False, (5.42e-6, 3.55e-7, 1.28e-8), (5.99e-4, 1.66e-5, 4.65e-7)),
]


@pytest.mark.parametrize("row", CONVERGENCE, ids=["D%d-P%d-%s" % (r[0], r[1], "trunc" if r[2] else "plain")
                                                  for r in CONVERGENCE])
def test_convergence_table(row):
    # every printed digit
    D, P, truncate, us, vs = row
    for i, roots in enumerate((2, 4, 8)):
        r = oracle_errors(D, P, 2, roots, truncate=truncate)
        assert _printed(r["eu"], us[i]), ("u", roots, r["eu"])
        assert _printed(r["ev"], vs[i]), ("v", roots, r["ev"])


def test_reflecting_convergence_table():
    # reference CODE.md:4165-4169: the Neumann mode on the reflecting box, l2
    # errors at roots 2, 4, 8, every printed digit (two or three)
    rows = [(1, 2, ((6.9e-2, 2), (1.98e-2, 3), (5.72e-3, 3))), (1, 3, ((4.23e-3, 3), (4.81e-4, 3), (6.0e-5, 2))),
            (2, 2, ((9.31e-2, 3), (2.64e-2, 3), (6.05e-3, 3)))]
    for D, P, refs in rows:
        for roots, (ref, digits) in zip((2, 4, 8), refs):
            r = oracle_errors(D, P, 2, roots, reflecting=True)
            assert _printed(r["l2"], ref, digits), (D, P, roots, r["l2"])
            assert r["energy"] <= r["energy0"]


def test_energy_lost_at_rk4_rate():
    # test/evolution_tests.jl:172-195
    for D, P, truncate in ((1, 3, True), (2, 2, True), (2, 3, False)):
        forest = wave_forest(np.float64, D, P, 2, roots=2)
        o = Oracle(forest, P, truncate=truncate)
        u0 = o.truncate(state_from(forest, P, smooth_data(D)))
        losses = []
        for cfl in (1.0, 0.5):
            dt = cfl * forest.minimum_spacing() / (P + 1)
            u = o.rk4(u0, dt, 200)
            E0, E1 = o.energy(u0), o.energy(u)
            assert E1 <= E0
            losses.append((E0 - E1) / E0)
        assert 0 < losses[1] < losses[0]
        assert losses[0] / losses[1] > 2 ** 5


def test_reflecting_energy_is_kept_but_for_rk4():
    # test/reflect_tests.jl:33-49: on the reflecting box the discrete energy,
    # with the gradient carrying the wall's parity, is an invariant of the
    # semi-discrete system; 50 steps at cfl 1/2 lose RK4's own share, never gain
    for D, P in ((1, 2), (2, 2)):
        forest = wave_forest(np.float64, D, P, 2, roots=2, reflecting=True)
        o = Oracle(forest, P)
        f0, _ = exact(D, 1.0, 1, 0.0, True)
        u0 = o.truncate(state_from(forest, P, f0))
        dt = 0.5 * forest.minimum_spacing() / (P + 1)
        u = o.rk4(u0, dt, 50)
        E0, E1 = o.energy(u0), o.energy(u)
        assert E1 <= E0
        assert E1 == pytest.approx(E0, rel=1e-6)


def test_reflecting_forest_declares_walls():
    # test/reflect_tests.jl:51-64: periodic stays the default, and a
    # reflecting forest has walls on every face and no periodic direction
    periodic = wave_forest(np.float64, 2, 2, 2, roots=2)
    assert all(periodic.periodic) and not any(periodic.reflecting)
    walls = wave_forest(np.float64, 2, 2, 2, roots=2, reflecting=True)
    assert not any(walls.periodic) and all(walls.reflecting)


def _rates(D, P, truncate=True, reflecting=False, roots=(2, 4, 8)):
    from twoldg.drivers import convergence_rate
    rs = [oracle_errors(D, P, 2, r, truncate=truncate, reflecting=reflecting) for r in roots]
    hs = [r["h"] for r in rs]
    return (convergence_rate(hs, [r["l2"] for r in rs]), convergence_rate(hs, [r["linf"] for r in rs]),
            [r["l2"] for r in rs])


@pytest.mark.parametrize("D", [1, 2])
@pytest.mark.parametrize("P", [2, 3, 4])
def test_truncated_error_converges_at_order_P(D, P):
    # test/sinewave_tests.jl:16-26, the paper's bound O(h_e^P)
    l2, linf, _ = _rates(D, P)
    assert P - 0.25 < l2 < P + 0.2
    assert P - 0.8 < linf < P + 0.4


@pytest.mark.parametrize("P", [3, 4])
def test_untruncated_u_is_more_accurate_but_irregular(P):
    # test/sinewave_tests.jl:28-39
    plain, _, errs = _rates(1, P, truncate=False)
    _, _, terrs = _rates(1, P)
    assert plain > P - 1
    assert errs[-1] < terrs[-1]


def test_first_order_at_P_1():
    # test/sinewave_tests.jl:41-47
    l2, _, _ = _rates(1, 1)
    assert 0.8 < l2 < 1.1


@pytest.mark.parametrize("D,P", [(1, 2), (1, 3), (2, 2), (2, 3)])
def test_reflecting_mode_converges_at_order_P(D, P):
    # test/reflect_tests.jl:21-31
    l2, linf, _ = _rates(D, P, reflecting=True)
    assert P - 0.35 < l2 < P + 0.4
    assert P - 1.0 < linf < P + 0.6


@pytest.mark.parametrize("D,P", [(1, 1), (1, 2), (1, 4), (2, 1), (2, 2), (2, 4)])
def test_rk4_is_stable_to_cfl_5_over_root_D(D, P):
    # test/evolution_tests.jl:196-222: the largest eigenvalue of the
    # truncated semi-discrete Laplacian, by power iteration through the
    # right-hand side and the truncation, puts RK4's limit |lambda dt| <= 2
    # sqrt 2 at the same cfl for every P, which pins oldg_timestep's
    # h_min / (P + 1) = h_e / (P + 1)^2
    import types
    from twoldg.problem import oldg_timestep
    forest = wave_forest(np.float64, D, P, 2, roots=2)
    o = Oracle(forest, P)
    x = o.truncate(state_from(forest, P, lambda y, var: np.sin(np.pi * (37 * sum(y) + 0.1)) if var == 1
                              else 0 * y[0]))
    nb = len(forest.leaves)
    X = x.reshape(nb, 2, -1)
    lam = 0.0
    for _ in range(300):
        Y = o.truncate(o.rhs(X.reshape(-1))).reshape(nb, 2, -1)
        lap = Y[:, 1]
        lam = np.linalg.norm(lap) / np.linalg.norm(X[:, 0])
        X[:, 0] = lap / np.linalg.norm(lap)
    p = types.SimpleNamespace(dtype=np.dtype(np.float64), forest=forest, hspeed=None, P=P)
    cflmax = 2 * math.sqrt(2) / math.sqrt(lam) / oldg_timestep(p, 1.0)
    assert 4.8 < cflmax * math.sqrt(D) < 5.8


def _standing(D, P, roots, refined=False, reflecting=False):
    """standing_errors (test/refined_tests.jl:311-331) on the oracle: the
    standing mode to a quarter period, its quadrature L2 error over the box,
    over the ball of radius 1/4 about the refined region's centre (nodes
    strictly inside), its largest error there, and the energy lost."""
    from cases import node_positions
    r = oracle_errors(D, P, 2, roots, refined=refined, reflecting=reflecting)
    forest = r["forest"]
    nb, NN = len(forest.leaves), forest.N ** D
    f1, _ = exact(D, 1.0, 1, r["dt"] * r["nsteps"], reflecting)
    x = node_positions(forest, P)
    xs = tuple(x[:, k, :] for k in range(D))
    err = r["state"].reshape(nb, 2, NN) - np.stack([f1(xs, 1), f1(xs, 2)], axis=1)
    wh = golden_tables(P)["weights"].astype(np.float64)
    grids = np.indices([forest.N] * D).reshape(D, -1)[::-1]
    w = np.empty((nb, NN))
    for b, key in enumerate(forest.leaves):
        ww = np.ones(NN)
        for d in range(D):
            ww = ww * (forest.spacing(key) * (P + 1) / 2 * wh[grids[d] % (P + 1)])
        w[b] = ww
    centre = np.full(D, 0.25 if reflecting else 0.5)
    inside = np.sum((x - centre[None, :, None]) ** 2, axis=1) < 0.25 ** 2
    W = np.stack([w, w], axis=1)
    B = np.stack([inside, inside], axis=1)
    e2 = err ** 2
    return dict(l2=math.sqrt(np.sum(W * e2) / np.sum(W)), ball_l2=math.sqrt(np.sum((W * e2)[B]) / np.sum(W[B])),
                ball_linf=float(np.abs(err)[B].max()), loss=(r["energy0"] - r["energy"]) / r["energy0"])


@pytest.mark.parametrize("D", [1, 2])
@pytest.mark.parametrize("P", [2, 3, 4])
def test_standing_mode_converges_at_order_P_on_two_levels(D, P):
    # test/refined_tests.jl:333-354: doubling every level, the box's error
    # falls at order P, and inside the refined middle it lies between the
    # uniform coarse and fine runs' (its largest error too, in 1D)
    c, f = _standing(D, P, 4), _standing(D, P, 8)
    m4, m8 = _standing(D, P, 4, refined=True), _standing(D, P, 8, refined=True)
    assert P - 0.25 < math.log2(m4["l2"] / m8["l2"]) < P + 0.2
    assert f["l2"] < m4["l2"] < c["l2"]
    assert f["ball_l2"] < m4["ball_l2"] < c["ball_l2"]
    if D == 1:
        assert f["ball_linf"] < m4["ball_linf"] < c["ball_linf"]


@pytest.mark.parametrize("D,P,truncate,reflecting", [(1, 3, True, False), (2, 2, True, False), (2, 3, False, False),
                                                     (2, 3, True, True)])
def test_energy_on_two_levels_is_lost_only_to_rk4(D, P, truncate, reflecting):
    # test/refined_tests.jl:356-376
    forest = refined_forest(D, P, reflecting=reflecting)
    o = Oracle(forest, P, truncate=truncate)

    def f(x, var):
        return sum(np.sin(np.pi * (2 * (d + 1) * x[d] + var / 3)) * np.cos(2 * np.pi * x[(d + 1) % D])
                   for d in range(D))

    u0 = o.truncate(state_from(forest, P, f)) if truncate else state_from(forest, P, f)
    E0 = o.energy(u0)
    losses = []
    for cfl in (1.0, 0.5):
        dt = cfl * forest.minimum_spacing() / (P + 1)
        losses.append((E0 - o.energy(o.rk4(u0, dt, 200))) / E0)
    assert 0 < losses[1] < losses[0]
    assert losses[0] / losses[1] > 2 ** 5


def _cflmax(forest, P):
    import types
    from twoldg.problem import oldg_timestep
    D = forest.D
    o = Oracle(forest, P)
    x = o.truncate(state_from(forest, P, lambda y, var: np.sin(np.pi * (37 * sum(y) + 0.1)) if var == 1
                              else 0 * y[0]))
    nb = len(forest.leaves)
    X = x.reshape(nb, 2, -1)
    lam = 0.0
    for _ in range(300):
        lap = o.truncate(o.rhs(X.reshape(-1))).reshape(nb, 2, -1)[:, 1]
        lam = np.linalg.norm(lap) / np.linalg.norm(X[:, 0])
        X[:, 0] = lap / np.linalg.norm(lap)
    p = types.SimpleNamespace(dtype=np.dtype(np.float64), forest=forest, hspeed=None, P=P)
    return 2 * math.sqrt(2) / math.sqrt(lam) / oldg_timestep(p, 1.0)


@pytest.mark.parametrize("D,P", [(1, 1), (1, 2), (1, 4), (2, 1), (2, 2), (2, 4), (3, 1)])
def test_rk4_limit_on_two_levels_is_the_uniform_one(D, P):
    # test/refined_tests.jl:378-409: the coarse-fine faces add no mode
    # stiffer than a uniform forest at the finest spacing has
    uniform = _cflmax(wave_forest(np.float64, D, P, 2, roots=3 if D == 3 else 4), P)
    twolevel = _cflmax(refined_forest(D, P), P)
    assert 0.99 < twolevel / uniform < 1.1
    assert 4.8 < twolevel * math.sqrt(D) < 6.2


@pytest.mark.parametrize("D", [1, 2])
@pytest.mark.parametrize("P", [2, 3])
def test_reflecting_box_refined_at_its_walls(D, P):
    # test/refined_tests.jl:411-431
    corner = tuple((0.0, 0.5) for _ in range(D))
    c, f = _standing(D, P, 4, reflecting=True), _standing(D, P, 8, reflecting=True)
    m4 = _standing(D, P, 4, refined=corner, reflecting=True)
    m8 = _standing(D, P, 8, refined=corner, reflecting=True)
    assert P - 0.25 < math.log2(m4["l2"] / m8["l2"]) < P + 0.2
    assert f["l2"] < m4["l2"] < c["l2"]
    assert f["ball_l2"] < m4["ball_l2"] < c["ball_l2"]
    assert 0 <= m4["loss"] < 1e-8


def test_coarse_ghost_degree_loss_in_2d():
    # test/refined_tests.jl:433-447 records, as a broken test, that in 2D at
    # P = 3 the refined middle's largest error falls by about 2^1.77 from
    # roots 8 to 16, not 2^(P - 1/2): the coarse ghost, the adjoint
    # restriction, is exact only to degree P - 1 tangentially. The shortfall
    # shows here too, which pins that ghost; the box's L2 keeps order P.
    P = 3
    m8, m16 = _standing(2, P, 8, refined=True), _standing(2, P, 16, refined=True)
    assert math.log2(m8["ball_linf"] / m16["ball_linf"]) < P - 0.5
    assert P - 0.25 < math.log2(m8["l2"] / m16["l2"]) < P + 0.2


# The reference's measured errors inside the refined region (1/4, 3/4)^D
# (CODE.md:4646-4662): D, P, roots, then L2 and L-infinity of the uniform
# coarse run (roots), the two-level forest (roots, the middle refined) and
# the uniform fine run (2 roots), the standing mode at a quarter period.
REFINED_REGION = [
    (1, 2, 8, (3.93e-02, 1.25e-02, 1.13e-02), (8.21e-02, 5.03e-02, 2.75e-02)),
    (1, 2, 16, (1.13e-02, 2.51e-03, 2.23e-03), (2.75e-02, 8.64e-03, 5.01e-03)),
    (1, 3, 8, (9.36e-04, 2.10e-04, 1.16e-04), (3.04e-03, 1.14e-03, 3.93e-04)),
    (1, 3, 16, (1.16e-04, 1.96e-05, 1.45e-05), (3.93e-04, 1.28e-04, 4.96e-05)),
    (1, 4, 8, (3.52e-05, 4.68e-06, 2.35e-06), (8.43e-05, 1.53e-05, 8.15e-06)),
    (1, 4, 16, (2.35e-06, 2.12e-07, 1.19e-07), (8.15e-06, 8.94e-07, 2.93e-07)),
    (2, 2, 8, (5.21e-02, 1.51e-02, 1.19e-02), (2.05e-01, 1.38e-01, 4.62e-02)),
    (2, 2, 16, (1.19e-02, 4.24e-03, 3.25e-03), (4.62e-02, 4.00e-02, 1.31e-02)),
    (2, 3, 8, (1.33e-03, 3.69e-04, 1.63e-04), (5.02e-03, 3.42e-03, 5.84e-04)),
    (2, 3, 16, (1.63e-04, 6.67e-05, 2.04e-05), (5.84e-04, 9.65e-04, 7.18e-05)),
    (2, 4, 8, (4.53e-05, 1.39e-05, 2.91e-06), (2.14e-04, 1.98e-04, 1.30e-05)),
    (2, 4, 16, (2.91e-06, 1.15e-06, 1.77e-07), (1.30e-05, 1.42e-05, 8.65e-07)),
]


def _region_errors(D, P, roots, refined):
    """L2 and L-infinity of the error at the nodes strictly inside (1/4, 3/4)^D,
    both variables, weighted by each node's quadrature weight."""
    from cases import node_positions
    r = oracle_errors(D, P, 2, roots, refined=refined)
    forest = r["forest"]
    nb, NN = len(forest.leaves), forest.N ** D
    f1, _ = exact(D, 1.0, 1, r["dt"] * r["nsteps"], False)
    x = node_positions(forest, P)
    xs = tuple(x[:, k, :] for k in range(D))
    err = r["state"].reshape(nb, 2, NN) - np.stack([f1(xs, 1), f1(xs, 2)], axis=1)
    wh = golden_tables(P)["weights"].astype(np.float64)
    grids = np.indices([forest.N] * D).reshape(D, -1)[::-1]
    w = np.empty((nb, NN))
    for b, key in enumerate(forest.leaves):
        ww = np.ones(NN)
        for d in range(D):
            ww = ww * (forest.spacing(key) * (P + 1) / 2 * wh[grids[d] % (P + 1)])
        w[b] = ww
    inside = np.all((x > 0.25) & (x < 0.75), axis=1)
    W, S = np.stack([w, w], axis=1), np.stack([inside, inside], axis=1)
    return math.sqrt(np.sum((W * err * err)[S]) / np.sum(W[S])), float(np.abs(err)[S].max())


def _printed(value, printed, digits=3):
    """value rounds to the significant digits printed."""
    e = math.floor(math.log10(abs(printed)))
    return abs(value - printed) <= 0.5001 * 10.0 ** (e - digits + 1)


@pytest.mark.parametrize("row", REFINED_REGION, ids=["D%d-P%d-roots%d" % r[:3] for r in REFINED_REGION])
def test_refined_region_table(row):
    # the two-level forest's coupling (coarse-fine ghosts by injection in
    # 1D, by I and R tangentially in 2D) pinned by the reference's own
    # measurements, every printed digit
    D, P, roots, l2, linf = row
    runs = [_region_errors(D, P, roots, False), _region_errors(D, P, roots, True),
            _region_errors(D, P, 2 * roots, False)]
    for k, (a, b) in enumerate(runs):
        assert _printed(a, l2[k]), ("L2", k, a, l2[k])
        assert _printed(b, linf[k]), ("Linf", k, b, linf[k])


# The reference's two-level convergence tables (CODE.md:4616-4636): D, P,
# the L2 and the L-infinity errors over the box of the two-level forest (the
# middle half refined) and of the uniform forest, at roots 4, 8, 16, 32.
REFINED_BOX = [
    (1, 2, (1.12e-01, 3.26e-02, 9.12e-03, 1.95e-03), (1.34e-01, 3.88e-02, 1.13e-02, 2.22e-03),
     (3.10e-01, 8.52e-02, 2.64e-02, 6.07e-03), (2.75e-01, 8.21e-02, 2.75e-02, 5.01e-03)),
    (1, 3, (5.66e-03, 6.75e-04, 8.32e-05, 1.04e-05), (8.20e-03, 9.27e-04, 1.16e-04, 1.45e-05),
     (2.83e-02, 3.06e-03, 3.93e-04, 4.98e-05), (2.94e-02, 3.04e-03, 3.93e-04, 4.96e-05)),
    (1, 4, (3.70e-04, 2.37e-05, 1.64e-06, 8.38e-08), (5.70e-04, 3.50e-05, 2.34e-06, 1.19e-07),
     (2.31e-03, 7.52e-05, 8.22e-06, 2.90e-07), (2.23e-03, 8.43e-05, 8.15e-06, 2.93e-07)),
    (2, 2, (1.67e-01, 4.70e-02, 1.09e-02, 2.97e-03), (1.83e-01, 5.21e-02, 1.19e-02, 3.26e-03),
     (6.81e-01, 1.97e-01, 4.73e-02, 1.32e-02), (6.59e-01, 2.05e-01, 4.62e-02, 1.31e-02)),
    (2, 3, (9.63e-03, 1.17e-03, 1.45e-04, 1.86e-05), (1.11e-02, 1.33e-03, 1.63e-04, 2.04e-05),
     (4.83e-02, 4.94e-03, 9.65e-04, 1.90e-04), (4.28e-02, 5.02e-03, 5.84e-04, 7.18e-05)),
    (2, 4, (5.68e-04, 3.97e-05, 2.58e-06, 1.60e-07), (6.62e-04, 4.54e-05, 2.91e-06, 1.77e-07),
     (3.58e-03, 4.40e-04, 3.15e-05, 2.77e-06), (2.31e-03, 2.14e-04, 1.30e-05, 8.65e-07)),
]


@pytest.mark.parametrize("row", REFINED_BOX, ids=["D%d-P%d" % r[:2] for r in REFINED_BOX])
def test_refined_box_tables(row):
    # the standing mode on two-level and uniform forests at roots 4 to 32,
    # RK4 at cfl 1/2 at the finest spacing, truncated: every printed digit
    D, P, two_l2, uni_l2, two_linf, uni_linf = row
    for i, roots in enumerate((4, 8, 16, 32)):
        two, uni = oracle_errors(D, P, 2, roots, refined=True), oracle_errors(D, P, 2, roots)
        assert _printed(two["l2"], two_l2[i]) and _printed(uni["l2"], uni_l2[i]), (roots, two["l2"], uni["l2"])
        assert _printed(two["linf"], two_linf[i]) and _printed(uni["linf"], uni_linf[i]), (roots, two["linf"],
                                                                                          uni["linf"])


def _line_limit(P, truncate):
    """The largest cfl at which RK4 is stable on the 1D periodic line:
    2 sqrt 2 over the square root of the spectral radius of the semi-discrete
    Laplacian (truncated as the limiter truncates, or plain), from its dense
    matrix, in units of h_min / (P + 1)."""
    forest = wave_forest(np.float64, 1, P, 2, roots=4)
    o = Oracle(forest, P, truncate=truncate)
    nb, NN = len(forest.leaves), forest.N
    A = np.empty((nb * NN, nb * NN))
    for j in range(nb * NN):
        X = np.zeros((nb, 2, NN))
        X[j // NN, 0, j % NN] = 1.0
        Y = o.rhs(X.reshape(-1))
        A[:, j] = (o.truncate(Y) if truncate else Y).reshape(nb, 2, NN)[:, 1].reshape(-1)
    lam = np.max(np.abs(np.linalg.eigvals(A)))
    return 2 * math.sqrt(2) / math.sqrt(lam) / (forest.minimum_spacing() / (P + 1))


def test_rk4_limit_on_the_line():
    # CODE.md:4727-4730, "The RK4 limit": every printed digit, P = 1..6
    truncated = (5.66, 5.20, 5.24, 5.17, 5.10, 5.03)
    plain = (5.66, 5.03, 4.99, 4.97, 4.94, 4.90)
    for P in range(1, 7):
        assert _printed(_line_limit(P, True), truncated[P - 1]), P
        assert _printed(_line_limit(P, False), plain[P - 1]), P


# CODE.md:4739-4750: cfl times sqrt D at the finest spacing, by the power
# iteration of test/evolution_tests.jl (300 steps through the right-hand side
# and the truncation), on the uniform forest, the two-level forest (the
# middle half refined) and the reflecting box with its corner refined, at
# roots 4 (3 in 3D). At 300 steps the iteration is 0.5 % from its limit in
# a few rows (2D, P = 3: 5.27 where the spectral radius gives 5.24); the
# table is reproduced as it was measured.
RK4_LIMIT_TWO_LEVEL = [(1, 1, 5.66, 5.75, 5.76), (1, 2, 5.20, 5.21, 5.21), (1, 3, 5.24, 5.24, 5.24),
                       (1, 4, 5.17, 5.18, 5.18), (2, 1, 5.66, 5.76, 5.76), (2, 2, 5.20, 5.22, 5.21),
                       (2, 3, 5.24, 5.27, 5.24), (2, 4, 5.17, 5.18, 5.18), (3, 1, 5.66, 6.04, 6.08),
                       (3, 2, 5.20, 5.29, 5.28)]


@pytest.mark.parametrize("row", RK4_LIMIT_TWO_LEVEL, ids=["D%d-P%d" % r[:2] for r in RK4_LIMIT_TWO_LEVEL])
def test_rk4_limit_on_two_levels_table(row):
    D, P, uniform, twolevel, walls = row
    r = math.sqrt(D)
    assert _printed(_cflmax(wave_forest(np.float64, D, P, 2, roots=3 if D == 3 else 4), P) * r, uniform)
    assert _printed(_cflmax(refined_forest(D, P), P) * r, twolevel)
    assert _printed(_cflmax(refined_forest(D, P, reflecting=True), P) * r, walls)


# CODE.md:4707-4715: the Neumann mode on the reflecting box with the corner
# (0, 1/2)^D refined: D, P, the L2 errors over the box at roots 4, 8, 16,
# the L2 and the L-infinity rates between them, and E1/E0 - 1 at roots 4.
REFINED_WALLS = [
    (1, 2, (1.43e-02, 3.93e-03, 8.77e-04), (1.86, 2.17), (1.27, 2.73), -3.1e-09),
    (1, 3, (3.57e-04, 4.36e-05, 5.40e-06), (3.03, 3.01), (2.85, 2.97), -2.1e-13),
    (1, 4, (1.22e-05, 8.16e-07, 4.44e-08), (3.90, 4.20), (3.02, 5.06), -2.2e-14),
    (2, 2, (2.27e-02, 5.33e-03, 1.44e-03), (2.09, 1.89), (2.19, 1.83), -1.4e-09),
    (2, 3, (5.95e-04, 7.25e-05, 9.03e-06), (3.04, 3.00), (3.11, 2.99), -1.1e-12),
    (2, 4, (1.98e-05, 1.28e-06, 7.78e-08), (3.95, 4.04), (4.04, 3.91), -1.2e-13),
]


@pytest.mark.parametrize("row", REFINED_WALLS, ids=["D%d-P%d" % r[:2] for r in REFINED_WALLS])
def test_refined_walls_table(row):
    # Every printed digit, but for two kinds of entry. The 1D, P = 4 error at
    # roots 4 comes out 1.21492e-05 (400 steps or 401 alike), against 1.22e-05
    # printed, 0.4 % off: that one is held to 0.5 %. An energy change below
    # 1e-12 is rounding in E1/E0 - 1, held to its sign and size only.
    D, P, l2, rates, linf_rates, loss = row
    corner = tuple((0.0, 0.5) for _ in range(D))
    rs = [oracle_errors(D, P, 2, roots, reflecting=True, refined=corner) for roots in (4, 8, 16)]
    for i, r in enumerate(rs):
        if (D, P, i) == (1, 4, 0):
            assert r["l2"] == pytest.approx(l2[i], rel=5e-3)
        else:
            assert _printed(r["l2"], l2[i]), (i, r["l2"])
    for i in range(2):
        assert abs(math.log2(rs[i]["l2"] / rs[i + 1]["l2"]) - rates[i]) <= 0.005001
        assert abs(math.log2(rs[i]["linf"] / rs[i + 1]["linf"]) - linf_rates[i]) <= 0.005001
    change = rs[0]["energy"] / rs[0]["energy0"] - 1
    if abs(loss) >= 1e-12:
        e = math.floor(math.log10(abs(loss)))
        assert abs(change - loss) <= 0.5001 * 10.0 ** (e - 1), change
    else:
        assert -1e-12 < change <= 0


def test_full_period_on_two_levels():
    # CODE.md:4688-4690: 2D, P = 3, the middle half refined, a full period:
    # the uniform and the two-level L2 over the box at roots 4, 8, 16
    uniform = (6.85e-04, 7.22e-05, 4.22e-06)
    twolevel = (1.54e-03, 2.05e-04, 3.25e-05)
    for i, roots in enumerate((4, 8, 16)):
        assert _printed(oracle_errors(2, 3, 2, roots, periods=1.0)["l2"], uniform[i])
        assert _printed(oracle_errors(2, 3, 2, roots, periods=1.0, refined=True)["l2"], twolevel[i])


def _bloch_blocks(P, truncate, M=6):
    """The semi-discrete operator (the right-hand side, then the truncation)
    on a periodic line of M elements of width 1, cut into the blocks by
    which an element hears its neighbours: A_k couples element g to g + k,
    u then v in each. Also the largest coupling beyond the neighbours."""
    E = 2
    forest = wave_forest(np.float64, 1, P, E, roots=M // E, L=float(M))
    o = Oracle(forest, P, truncate=truncate)
    nb, N, P1 = len(forest.leaves), forest.N, P + 1
    n = 2 * nb * N
    A = np.empty((n, n))
    for j in range(n):
        X = np.zeros(n)
        X[j] = 1.0
        Y = o.rhs(X)
        A[:, j] = o.truncate(Y) if truncate else Y

    def idx(g):
        b, e = divmod(g % M, E)
        base = b * 2 * N + e * P1
        return np.concatenate([base + np.arange(P1), base + N + np.arange(P1)])

    blocks = {k: A[np.ix_(idx(2), idx(2 + k))] for k in (-1, 0, 1)}
    beyond = max(np.abs(A[np.ix_(idx(2), idx(2 + k))]).max() for k in range(2, M - 1))
    return blocks, beyond


def _bloch(blocks, theta):
    """The eigenvalues of A(theta) = sum_k A_k e^{i k theta}."""
    return np.linalg.eigvals(sum(b * np.exp(1j * k * theta) for k, b in blocks.items()))


def test_dispersion_relation():
    # CODE.md:4766-4801 ("Why the error outruns light"), P = 3, h_e = 1: the
    # Bloch eigenvalues are +-i omega (energy kept mode by mode); with the
    # truncation two branches are frozen, the physical one has a gap at
    # k h = pi from 3.113 to 3.464, the branches meet at 7.746 at 2 pi, and the
    # spectral radius is 8.641; without it a spurious branch leaves 0 at
    # three times the speed of light, and the spectral radius is 9.105
    def rho(blocks):
        grid = np.linspace(0, 2 * np.pi, 721)
        best = max(grid, key=lambda t: np.abs(_bloch(blocks, t)).max())
        from scipy.optimize import minimize_scalar
        r = minimize_scalar(lambda t: -np.abs(_bloch(blocks, t)).max(), bounds=(best - 0.01, best + 0.01),
                            method="bounded", options={"xatol": 1e-10})
        return -r.fun

    for truncate in (True, False):
        blocks, beyond = _bloch_blocks(3, truncate)
        assert beyond == 0
        for t in np.linspace(0, 2 * np.pi, 37):
            assert np.abs(_bloch(blocks, t).real).max() < 2e-7
        w_pi = np.sort(np.abs(_bloch(blocks, np.pi)))
        w_0 = np.sort(np.abs(_bloch(blocks, 0.0)))
        slow = np.sort(np.abs(_bloch(blocks, 0.01)))
        if truncate:
            assert np.all(w_pi[:2] < 1e-7) and _printed(w_pi[2], 3.113, 4) and _printed(w_pi[4], 3.464, 4)
            assert _printed(w_0[-1], 7.746, 4) and _printed(rho(blocks), 8.641, 4)
            assert not np.any(np.abs(slow / 0.01 - 3) < 0.05)
        else:
            assert _printed(w_0[-1], 7.746, 4) and _printed(rho(blocks), 9.105, 4)
            assert np.any(np.abs(slow / 0.01 - 3) < 0.05)


@pytest.mark.parametrize("D,P", [(1, 3), (2, 2), (2, 3)])
def test_quadrature_norm_integrates_what_the_element_represents(D, P):
    # test/layout_tests.jl:41-60: a constant has norm one (p = 2 and 1), the
    # mean of |prod x^k|^2 over the unit box is exact while its degree 2k is
    # within the element's quadrature, and the largest value is 1
    forest = wave_forest(np.float64, D, P, 2, roots=2)
    o = Oracle(forest, P)
    one = state_from(forest, P, lambda x, var: 1.0 + 0 * x[0])
    assert o.norm(one, 2, 1) == pytest.approx(1.0, abs=1e-14)
    assert o.norm(one, 1, 1) == pytest.approx(1.0, abs=1e-14)
    k = P - 1
    mono = state_from(forest, P, lambda x, var: np.prod(x, axis=0) ** k)
    assert o.norm(mono, 2, 1) == pytest.approx(math.sqrt(1 / (2 * k + 1)) ** D, abs=1e-13)
    assert o.norm(mono, 0, 1) == pytest.approx(1.0, abs=1e-14)
