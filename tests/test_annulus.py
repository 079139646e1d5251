"""The annulus (a diagonal metric): the oracle against the reference's
published convergence table, and the metric's projector properties. No GPU."""
import math

import numpy as np
import pytest

from annulus_cases import annulus_oracle, line_weights, oracle_annulus_errors, state_of
from twoldg.element import Element
from twoldg.geometry import annulus_forest, metric_tables, projector_mode


# reference CODE.md:4190-4199: m = 2, n = 1, 1 <= r <= 2, to t = pi/k, patches
# of (2s, s) roots, E = 2, cfl 1/2: the sqrt(g)-weighted L2 errors of u and of v
# at s = 1, 2, 4, truncated and not (the table's s = 8 column is left out for
# time)
ANNULUS = [
    (2, True, (1.13e-1, 3.13e-2, 8.08e-3), (9.57e-2, 2.65e-2, 6.78e-3)),
    (2, False, (5.05e-3, 1.18e-3, 1.31e-4), (3.77e-2, 1.13e-2, 2.40e-3)),
    (3, True, (5.06e-3, 6.30e-4, 7.77e-5), (3.35e-3, 4.23e-4, 5.35e-5)),
    (3, False, (4.32e-4, 4.15e-5, 4.99e-6), (1.94e-3, 2.49e-4, 2.72e-5)),
    (4, True, (3.77e-4, 2.73e-5, 1.81e-6), (3.26e-4, 2.80e-5, 2.10e-6)),
    (4, False, (4.73e-5, 1.68e-6, 9.68e-8), (1.80e-4, 2.33e-5, 1.84e-6)),
    (5, True, (3.06e-5, 1.28e-6, 4.27e-8), (2.59e-5, 1.31e-6, 3.45e-8)),
    (5, False, (4.38e-6, 6.87e-8, 5.70e-9), (2.35e-5, 1.75e-6, 7.69e-8)),
]


def _printed(value, printed):
    """value rounds to the three significant digits printed."""
    e = np.floor(np.log10(abs(printed)))
    return abs(value - printed) <= 0.5001 * 10.0 ** (e - 2)


@pytest.mark.parametrize("row", ANNULUS, ids=["P%d-%s" % (r[0], "trunc" if r[1] else "plain") for r in ANNULUS])
def test_annulus_convergence_table(row):
    # every printed digit
    P, truncate, us, vs = row
    for i, s in enumerate((1, 2, 4)):
        r = oracle_annulus_errors(P, 2, (2 * s, s), truncate=truncate)
        assert _printed(r["u"], us[i]), (s, r["u"])
        assert _printed(r["v"], vs[i]), (s, r["v"])
        # RK4's loss, down to the energy sum's rounding at the finest runs
        assert r["energy"] <= r["energy0"] * (1 + 1e-13)


def test_metric_projector_is_orthogonal_in_the_weighted_product():
    el = Element(np.float64, 4)
    a = 1.0 + 0.3 * el.nodes
    phi = projector_mode(el.nodes, el.weights, a, 4)
    for k in range(4):
        assert abs(np.sum(el.weights * a * phi * el.nodes ** k)) < 1e-13
    # constant weight: L_P itself
    phi1 = projector_mode(el.nodes, el.weights, np.full(5, 2.5), 4)
    assert np.allclose(phi1, el.topmode, atol=1e-14)


def test_annulus_rhs_is_self_adjoint_and_rotation_free():
    # sqrt(g)-weighted SBP: <b, Lap a> = <Lap b, a> with the metric weights
    forest, geo, o, _ = annulus_oracle(3, 2, (2, 1), truncate=False)
    nb = len(forest.leaves)
    NN = forest.N ** 2
    rng = np.random.default_rng(1)
    a = rng.standard_normal((nb, NN))
    b = rng.standard_normal((nb, NN))
    coef = metric_tables(forest, Element(np.float64, 3), geo)[0].reshape(nb, 3, NN)

    def lap(x):
        s = np.zeros((nb, 2, NN))
        s[:, 0] = x
        return o.rhs(s.reshape(-1)).reshape(nb, 2, NN)[:, 1]
    from test_oracle import _weights
    w = _weights(o, forest, 3) * coef[:, 0]
    la, lb = lap(a), lap(b)
    assert abs(np.sum(w * b * la) - np.sum(w * lb * a)) < 1e-12 * np.sum(np.abs(w * b * la))


def test_annulus_energy_changes_by_rk4_loss_alone():
    # test/annulus_tests.jl:165-185: P = 3, roots (2, 1), the rotating mode to
    # t = pi/k at cfl 1/2 and 1/4: never a gain, a loss below 1e-8, falling by
    # more than 16 as the step halves
    losses = []
    for cfl in (0.5, 0.25):
        r = oracle_annulus_errors(3, 2, (2, 1), cfl=cfl)
        assert r["energy"] <= r["energy0"]
        losses.append((r["energy0"] - r["energy"]) / r["energy0"])
    assert losses[0] < 1e-8
    assert losses[0] / losses[1] > 16


def _host_truncation(forest, P, modes, duals, s):
    """The truncation the kernels apply from the host's per-line tables: on
    v, along dimension 0 then 1, each element line's v -= mode (dual . v)."""
    nb, N, P1 = len(forest.leaves), forest.N, P + 1
    E = N // P1
    modes = modes.reshape(2, nb, E, P1)
    duals = duals.reshape(2, nb, E, P1)
    out = s.reshape(nb, 2, N, N).copy()              # [b, var, i1, i0]
    for b in range(nb):
        v = out[b, 1]
        for e in range(E):
            sl = slice(e * P1, (e + 1) * P1)
            v[:, sl] -= np.outer(v[:, sl] @ duals[0, b, e], modes[0, b, e])
        for e in range(E):
            sl = slice(e * P1, (e + 1) * P1)
            v[sl, :] -= np.outer(modes[1, b, e], duals[1, b, e] @ v[sl, :])
    return out.reshape(-1)


@pytest.mark.parametrize("P", [2, 3, 4])
def test_annulus_truncation_is_the_sqrtg_orthogonal_projection(P):
    # test/annulus_tests.jl:95-131, for the library's host tables (which the
    # kernels read) and for the oracle's own projector (long double from the
    # sqrt(g) factors): self-adjoint in the sqrt(g) weights, a projection onto
    # Q_{P-1} (the flat projector leaves its result), u left alone, the
    # kinetic energy not raised; along the angle the tables are the element's
    from annulus_cases import line_weights
    from oracle.oracle import Oracle
    from test_oracle import _weights
    el = Element(np.float64, P)
    forest, geo = annulus_forest(np.float64, P, 2, roots=(2, 2), r0=0.25, r1=2.0)
    coef, modes, duals, _ = metric_tables(forest, el, geo)
    o = Oracle(forest, P, coef=coef, line_weights=line_weights(forest, geo, P))
    flat = Oracle(forest, P)
    nb, NN = len(forest.leaves), forest.N ** 2
    wg = (_weights(o, forest, P) * coef.reshape(nb, 3, NN)[:, 0]).reshape(-1)
    rng = np.random.default_rng(5)
    a, b = rng.standard_normal(nb * 2 * NN), rng.standard_normal(nb * 2 * NN)

    def v(x):
        return x.reshape(nb, 2, NN)[:, 1].reshape(-1)

    def inner(x, y):
        return float(np.sum(wg * x * y))

    for trunc in (lambda s: _host_truncation(forest, P, modes, duals, s), o.truncate):
        ta, tb = trunc(a), trunc(b)
        scale = math.sqrt(inner(v(a), v(a)) * inner(v(b), v(b)))
        assert abs(inner(v(ta), v(b)) - inner(v(a), v(tb))) < 1e-14 * scale
        assert np.allclose(trunc(ta), ta, rtol=0, atol=1e-13 * np.abs(ta).max())
        assert np.allclose(flat.truncate(ta), ta, rtol=0, atol=1e-12 * np.abs(ta).max())
        assert np.array_equal(ta.reshape(nb, 2, NN)[:, 0], a.reshape(nb, 2, NN)[:, 0])
        assert inner(v(ta), v(ta)) <= inner(v(a), v(a))
    assert np.allclose(_host_truncation(forest, P, modes, duals, a), o.truncate(a), rtol=0, atol=1e-13 * np.abs(a).max())
    m = modes.reshape(2, nb, 2, P + 1)[0]
    assert np.allclose(m, np.broadcast_to(el.topmode.astype(np.float64), m.shape), rtol=1e-13, atol=1e-14)


def test_bessel_mode_is_the_annulus_neumann_mode():
    # test/annulus_tests.jl:200-216: the exact solution has d_r u = 0 on both
    # walls and R(k r0) = 1 by its scaling; the roots are ordered
    from scipy.special import jv, yv
    from twoldg.geometry import _dbesselj, _dbessely, annulus_wavenumber
    r0, r1 = 0.5, 2.0
    for m, n in ((0, 1), (1, 1), (2, 1), (3, 2)):
        k = annulus_wavenumber(m, n, r0, r1)
        assert k > 0
        jr0, yr0 = _dbesselj(m, k * r0), _dbessely(m, k * r0)
        scale = math.pi * k * r0 / 2
        for r in (r0, r1):
            assert abs(scale * (_dbesselj(m, k * r) * yr0 - _dbessely(m, k * r) * jr0)) < 1e-12
        assert scale * (jv(m, k * r0) * yr0 - yv(m, k * r0) * jr0) == pytest.approx(1.0, rel=1e-12)
    assert annulus_wavenumber(1, 1, 1, 2) < annulus_wavenumber(1, 2, 1, 2)


def test_annulus_forest_refuses_what_it_does_not_map():
    # test/annulus_tests.jl:218-230, the forest's own refusals
    with pytest.raises(ValueError, match="odd"):
        annulus_forest(np.float64, 2, 3)
    with pytest.raises(ValueError, match="0 < r0 < r1"):
        annulus_forest(np.float64, 2, 2, r0=2, r1=1)
