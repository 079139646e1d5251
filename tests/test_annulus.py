"""The annulus (a diagonal metric): the oracle against the reference's
published convergence table, and the metric's projector properties. No GPU."""
import numpy as np
import pytest

from annulus_cases import annulus_oracle, line_weights, oracle_annulus_errors, state_of
from twoldg.element import Element
from twoldg.geometry import annulus_forest, metric_tables, projector_mode


@pytest.mark.parametrize("P,row", [
    (2, (1.13e-1, 3.13e-2, 9.57e-2, 2.65e-2)),
    (3, (5.06e-3, 6.30e-4, 3.35e-3, 4.23e-4)),
    (4, (3.77e-4, 2.73e-5, 3.26e-4, 2.80e-5)),
])
def test_annulus_convergence_table(P, row):
    # reference CODE.md:4177-4199: m = 2, n = 1, 1 <= r <= 2, to t = pi/k,
    # patches of (2s, s) roots, E = 2, truncated, cfl 1/2; sqrt(g)-weighted
    # L2 errors of u and v at s = 1, 2
    for i, s in enumerate((1, 2)):
        r = oracle_annulus_errors(P, 2, (2 * s, s))
        assert r["u"] == pytest.approx(row[i], rel=0.01), (s, r["u"])
        assert r["v"] == pytest.approx(row[2 + i], rel=0.01), (s, r["v"])
        assert r["energy"] <= r["energy0"]


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
