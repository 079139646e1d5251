"""Element tables: the library's double-double build against the golden
512-bit restatement (bit for bit), and the reference's own known answers
and properties (test/element_tests.jl)."""
import numpy as np
import pytest

from oracle.oracle import golden_tables
from twoldg.element import Element, element_table
from dense import global_operators

NAMES = ["nodes", "weights", "offsets", "stencil", "truncate", "topmode", "topdual", "duals", "prolong",
         "restrict"]


@pytest.mark.parametrize("P", range(1, 9))
@pytest.mark.parametrize("kind", ["f64", "f32"])
def test_tables_bit_exact_against_512_bit_restatement(P, kind):
    # The precision rule (test/element_tests.jl:122-137): each type's table is
    # the 512-bit value rounded once, so a double-double build must give the
    # same bits in float64 and float32.
    g = golden_tables(P, kind)
    dt = np.float64 if kind == "f64" else np.float32
    for name in NAMES:
        lib = element_table(P, dt, name)
        ref = g[name].reshape(lib.shape).astype(dt)
        assert np.array_equal(lib.view(np.uint64 if kind == "f64" else np.uint32),
                              ref.view(np.uint64 if kind == "f64" else np.uint32)), (P, kind, name)


def test_wide_derivative_is_the_papers():
    # test/element_tests.jl:38-56: the paper's printed matrices h_e D for P = 2, 3, 4
    W2 = element_table(2, np.float64, "stencil") * 3
    assert np.allclose(W2, [[-3, 0, 4, -1, 0], [0, -1, 0, 1, 0], [0, 1, -4, 0, 3]], atol=1e-14)
    W3 = np.round(element_table(3, np.float64, "stencil") * 4, 2)
    assert np.array_equal(W3, [[-6, 0, 8.09, -3.09, 1, 0], [0, -1.62, 0, 2.24, -0.62, 0],
                               [0, 0.62, -2.24, 0, 1.62, 0], [0, -1, 3.09, -8.09, 0, 6]])
    W4 = np.round(element_table(4, np.float64, "stencil") * 5, 2)
    assert np.array_equal(W4, [[-10, 0, 13.51, -5.33, 2.82, -1, 0], [0, -2.48, 0, 3.49, -1.53, 0.52, 0],
                               [0, 0.75, -2.67, 0, 2.67, -0.75, 0], [0, -0.52, 1.53, -3.49, 0, 2.48, 0],
                               [0, 1, -2.82, 5.33, -13.51, 0, 10]])


@pytest.mark.parametrize("P", range(1, 9))
def test_nodes_and_structure(P):
    # test/element_tests.jl:19-36 and :58-69
    el = Element(np.float64, P)
    x = el.nodes
    assert x[0] == -1 and x[-1] == 1
    assert all(x[i] == -x[P - i] for i in range(P + 1))
    assert np.all(np.diff(x) > 0)
    assert el.offsets[0] == 0 and el.offsets[-1] == P + 1
    for k in range(2 * P):
        exact = 2 / (k + 1) if k % 2 == 0 else 0.0
        assert abs(np.sum(el.weights * x ** k) - exact) < 1e-14
    assert abs(np.sum(el.weights * x ** (2 * P)) - 2 / (2 * P + 1)) > 1e-14
    W = el.stencil
    assert np.all(W[1:, 0] == 0) and np.all(W[:-1, -1] == 0)
    assert W[0, 0] != 0 and W[-1, -1] != 0
    assert all(abs(W[i, i + 1]) < 1e-12 for i in range(P + 1))
    assert np.allclose(W, -W[::-1, ::-1], atol=1e-12)


@pytest.mark.parametrize("P", range(1, 9))
def test_exact_to_degree_P_and_projector(P):
    # test/element_tests.jl:71-87 and :103-120
    el = Element(np.float64, P)
    W = el.stencil
    h = 2 / (P + 1)
    for k in range(P + 1):
        u = el.nodes ** k
        du = k * el.nodes ** (k - 1) if k else np.zeros_like(u)
        window = np.concatenate([[u[0]], u, [u[-1]]])
        assert np.allclose(W @ window / h, du, atol=1e-11 * max(1, P * P))
    Pi = el.truncate
    for k in range(P):
        assert np.allclose(Pi @ el.nodes ** k, el.nodes ** k, atol=1e-12)
    assert np.linalg.norm(Pi @ el.topmode) < 1e-12
    assert np.allclose(Pi @ Pi, Pi, atol=1e-12)
    w = el.weights
    assert np.allclose(w[:, None] * Pi, (w[:, None] * Pi).T, atol=1e-12)
    # the rank-one form the kernels apply is the same projector
    assert np.allclose(np.eye(P + 1) - np.outer(el.topmode, el.topdual), Pi, atol=1e-13)


@pytest.mark.parametrize("P", range(1, 7))
@pytest.mark.parametrize("K", [1, 3])
def test_summation_by_parts_on_a_periodic_line(P, K):
    # test/element_tests.jl:89-101: w D + (w D)^T = 0
    el = Element(np.float64, P)
    Dm, _, w = global_operators(el.stencil, el.truncate, el.weights, P, K, 0.1)
    WD = w[:, None] * Dm
    assert np.linalg.norm(WD + WD.T) <= 1e-12 * np.linalg.norm(WD)


@pytest.mark.parametrize("P", range(1, 7))
def test_coarse_fine_operators(P):
    # I is exact to degree P; R = M_c^-1 I^T M_f conserves sum w u and is exact
    # to degree P-1 but not P (reference CODE.md, "The coupling").
    el = Element(np.float64, P)
    I = element_table(P, np.float64, "prolong")
    R = element_table(P, np.float64, "restrict")
    x = el.nodes
    xf = np.concatenate([(x - 1) / 2, (x + 1) / 2])
    for k in range(P + 1):
        assert np.allclose(I @ x ** k, xf ** k, atol=1e-12)
    for k in range(P):
        assert np.allclose(R @ xf ** k, x ** k, atol=1e-12)
    assert not np.allclose(R @ xf ** P, x ** P, atol=1e-9)
    wf = np.concatenate([el.weights, el.weights]) / 2
    u = np.sin(3 * xf) + xf ** P
    assert abs(np.sum(el.weights * (R @ u)) - np.sum(wf * u)) < 1e-13
    # the adjoint relation: M_c R = I^T M_f
    assert np.allclose(el.weights[:, None] * R, I.T * wf[None, :], atol=1e-14)
