"""The particle-grid transfer on the CPU: the library's tables against the
512-bit fixture, the quadrature rules' own properties, and the oracle against
the reference's assertions (test/transfer_tests.jl) where they are cheap."""
import math

import numpy as np
import pytest

from oracle import transfer as T
from transfer_cases import brick_values, exact_moment, grad_poly, irregular, poly, reference_integral


def _lib_table(P, dtype, name, q=None):
    from twoldg.transfer import transfer_table
    return transfer_table(P, dtype, name, q)


@pytest.mark.parametrize("kind", ["f64", "f32"])
def test_tables_are_the_512_bit_ones_rounded_once(kind):
    # test/transfer_tests.jl:78-106: every table is the BigFloat one rounded once
    dt, it = (np.float64, np.uint64) if kind == "f64" else (np.float32, np.uint32)
    for n in (1, 2, 5, 7, 8, 10, 12, 14, 16, 24, 48, 80):
        for what in ("nodes", "weights"):
            lib = _lib_table(1, dt, "gauss_" + what, n)
            assert np.array_equal(lib.view(it), T.gauss_bits(n, what, kind)), (n, what)
    for P in range(1, 7):
        lib = _lib_table(P, dt, "bary")
        assert np.array_equal(lib.view(it), T.fixture_table(P, "bary", kind).view(it))
        for q in sorted({P + 3, 14, 10, 8, 7}):
            for name in ("lagrange", "contract"):
                lib = _lib_table(P, dt, name, q)
                ref = T.fixture_table(P, "%s_%d" % (name, q), kind).reshape(lib.shape)
                assert np.array_equal(lib.view(it), ref.view(it)), (P, q, name)


def test_gauss_rules_are_exact_to_degree_2n_minus_1():
    # test/transfer_tests.jl:82-90
    for n in (1, 2, 5, 12):
        x, w = T.gauss(n)
        for k in range(2 * n):
            assert abs(np.sum(w * x ** k) - (2 / (k + 1) if k % 2 == 0 else 0)) < 1e-14
        assert np.sum(w * x ** (2 * n)) - 2 / (2 * n + 1) < -1e-10
        assert np.array_equal(x, -x[::-1])


def test_contraction_is_the_weighted_lagrange_table():
    # test/transfer_tests.jl:100-105
    P = 3
    con = T.fixture_table(P, "contract_6").reshape(4, 6)
    lag = T.fixture_table(P, "lagrange_6").reshape(6, 4)
    gw = T.gauss(6)[1]
    w = T.Tables(P).weights
    for i in range(4):
        for k in range(6):
            assert con[i, k] == pytest.approx(gw[k] * lag[k, i] / w[i], rel=1e-15)


def test_graded_rule_is_the_tensor_gauss_rule_contracted():
    # test/transfer_tests.jl:330-346: contraction one dimension at a time
    # against the tensor Gauss rule applied point by point with the basis
    for D, P in ((1, 4), (2, 3), (3, 3)):
        t = T.Tables(P)
        g = t.graded[1]
        lo = [0.1 * (d + 1) for d in range(D)]
        hi = [x + 0.3 for x in lo]

        def S(X):
            out = np.exp(X[:, 0])
            for d in range(D):
                out = out * np.cos(3 * X[:, d] + d + 1)
            return out

        x, w, _ = g
        grids = [lo[d] + 0.3 * (1 + x) / 2 for d in range(D)]
        mesh = np.meshgrid(*grids, indexing="ij")
        X = np.stack([m.reshape(-1) for m in mesh], axis=1)
        W = np.ones(1)
        for d in range(D):
            W = (W[:, None] * (w * 0.15)[None, :]).reshape(-1)
        ref = (W[:, None] * S(X)[:, None] * t.element_basis(lo, hi, X)).sum(axis=0) / t.element_weights(0.3, D)
        got = T.tensor_rule(S, g, lo, hi, D)
        assert np.allclose(got, ref, rtol=1e-14, atol=1e-14 * np.abs(ref).max())


def _oracle_projection_error(D, P, roots):
    mesh = T.brick_mesh(D, P, 2, roots)
    t = T.Tables(P)

    def S(X):
        out = np.sin(2 * np.pi * X[:, 0])
        for d in range(1, D):
            out = out * np.cos(2 * np.pi * X[:, d])
        return out + 0.3

    du = np.zeros(mesh.nblocks * 2 * mesh.NN)
    T.project_source(du, mesh, t, S, [], (np.full(D, 0.5), 2.0), factor=1.0)
    ref = np.zeros_like(du)
    nodes = t.nodes
    for b in range(mesh.nblocks):
        for J in np.ndindex(*([2] * D)):
            e = tuple(reversed(J))
            lo, hi = mesh.element_box(b, e)
            grids = [lo[d] + (hi[d] - lo[d]) * (1 + nodes) / 2 for d in range(D)]
            m = np.meshgrid(*grids, indexing="ij")
            X = np.stack([a.reshape(-1) for a in m], axis=1)
            vals = S(X).reshape((P + 1,) * D)
            ref[mesh.node_index(b, e, 2)] = np.transpose(vals, tuple(range(D - 1, -1, -1))).reshape(-1)
    err = du - ref
    return math.sqrt(T.weighted_inner(mesh, t, err, err, 2) / T.weighted_inner(mesh, t, np.ones_like(du),
                                                                               np.ones_like(du), 2))


def test_oracle_projection_is_consistent_at_order_P():
    # test/transfer_tests.jl:108-133: (P S)_n - S(x_n) falls at the scheme's order
    for D, P in ((1, 2), (1, 3), (1, 4), (2, 2), (2, 3), (2, 4)):
        errs = [_oracle_projection_error(D, P, r) for r in (2, 4, 8)]
        rate = np.polyfit(np.log([1 / 2, 1 / 4, 1 / 8]), np.log(errs), 1)[0]
        assert rate > P - 0.1, (D, P, errs)
    e = [_oracle_projection_error(3, 2, r) for r in (2, 4)]
    assert math.log2(e[0] / e[1]) > 2 - 0.2


def test_oracle_near_rule_integrates_the_particle():
    # test/transfer_tests.jl:172-214, one moving case: the nested rule split
    # at the support gives Q / gamma and the polynomial moment to 1e-12
    mesh = T.brick_mesh(3, 3, 2, 1)
    t = T.Tables(3)
    he = 0.5
    ell = 1e-2 * he
    Q = 1e-3
    v = np.array([0.1, -0.15, 0.05])
    z = np.array([0.5, 0.5, 0.5]) + ell * np.array([0.3, -0.2, 0.1])
    s = T.Support(z, v, ell)
    du = np.zeros(mesh.nblocks * 2 * mesh.NN)
    T.project_source(du, mesh, t, lambda X: T.particle_density(X, z, v, ell, Q), [s], (z, 2 * ell),
                     factor=1.0, var=1, he=he)
    gamma = 1 / math.sqrt(1 - v @ v)
    one = np.ones_like(du)
    assert T.weighted_inner(mesh, t, du, one, 1) == pytest.approx(Q / gamma, rel=1e-12)
    # g = poly at the nodes
    g = np.zeros_like(du)
    for b in range(mesh.nblocks):
        for J in np.ndindex(2, 2, 2):
            e = tuple(reversed(J))
            lo, hi = mesh.element_box(b, e)
            grids = [lo[d] + (hi[d] - lo[d]) * (1 + t.nodes) / 2 for d in range(3)]
            m = np.meshgrid(*grids, indexing="ij")
            X = np.stack([a.reshape(-1) for a in m], axis=1)
            g[mesh.node_index(b, e, 1)] = np.transpose(poly(X).reshape(4, 4, 4), (2, 1, 0)).reshape(-1)
    assert T.weighted_inner(mesh, t, du, g, 1) == pytest.approx(exact_moment(poly, Q, ell, z, v), rel=1e-12)
    # the adjoint pairing over the support's elements, compact (src/transfer.jl:1779-1815)
    acc = 0.0
    for b in range(mesh.nblocks):
        for J in np.ndindex(2, 2, 2):
            e = tuple(reversed(J))
            lo, hi = mesh.element_box(b, e)
            gv = g[mesh.node_index(b, e, 1)]
            acc += T.nested_rule(lambda X: T.particle_density(X, z, v, ell, Q) * (t.element_basis(lo, hi, X) @ gv),
                                 s, t, lo, hi, 3, compact=True)
    assert acc == pytest.approx(exact_moment(poly, Q, ell, z, v), rel=1e-12)


def test_oracle_projection_is_adjoint_to_the_reconstruction_1d():
    # test/transfer_tests.jl:135-170, D = 1: <P S, g>_w = int S g_h for a
    # bump straddling a face, a Lorentzian peak and a smooth part
    D, roots, eps, grades, tol = 1, 8, 0.1, range(-12, 7), 1e-13
    P = 3
    mesh = T.brick_mesh(D, P, 2, roots)
    t = T.Tables(P)
    he = 1 / roots / 2
    ell = 0.05 * he
    z = np.array([0.5 + 0.3 * ell])

    def S(X):
        r2 = np.sum((X - z[None, :]) ** 2, axis=1)
        return np.cos(X[:, 0]) + np.where(r2 < ell * ell, (1 - r2 / ell ** 2) ** 4, 0.0) / ell ** D + \
            eps * he / (r2 + (eps * he) ** 2) ** 0.5

    du = np.zeros(mesh.nblocks * 2 * mesh.NN)
    T.project_source(du, mesh, t, S, [T.Support(z, np.zeros(1), ell)], (z, 10.0), factor=1.0)
    g = irregular(len(du))
    lhs = T.weighted_inner(mesh, t, du, g, 2)
    rhs = 0.0
    for b in range(mesh.nblocks):
        for e in ((0,), (1,)):
            lo, hi = mesh.element_box(b, e)
            gv = g[mesh.node_index(b, e, 2)]
            rhs += reference_integral(lambda X: S(X) * (t.element_basis(lo, hi, X) @ gv), lo, hi, z, ell,
                                      grades, ell)
    assert lhs == pytest.approx(rhs, rel=tol)


def first_run_window(he=0.125):
    """The first run's particles and window at h_e = 1/8 (bin/projection.jl):
    opposite charges on a circle of diameter 1 at v = 0.2, off the element
    corners by (0.31, 0.17, 0.43) h_e, ell = 1e-3, in a box of side 5 (origin at a
    corner), P = 3, E = 4, the window's ball R2 = 2.5 about the centre."""
    c = np.array([2.5] * 3)
    off = np.array([0.31, 0.17, 0.43]) * he
    parts = [T.Support(c + np.array([0.5, 0, 0]) + off, [0, 0.2, 0], 1e-3),
             T.Support(c - np.array([0.5, 0, 0]) + off, [0, -0.2, 0], 1e-3)]
    n = int(round(5 / (4 * he)))
    w = 5.0 / n
    origins = [[c_[d] * w for d in range(3)] for c_ in [tuple(reversed(J)) for J in np.ndindex(n, n, n)]]
    return T.Mesh(origins, [w / 16] * len(origins), 3, 4), parts, (c, 2.5)


def test_first_run_window_has_the_reference_far_count():
    # CODE.md "Quadrature": "of the first run's 31 102 [far elements] at
    # h_e = d/8, off the grid" -- the classification by r_far = 9 h_e,
    # r_near = h_e and the window's ball
    mesh, parts, ball = first_run_window()
    far, graded, near = T.classify(mesh, T.Tables(3), parts, ball, 1.0, 0.125)
    assert len(far) == 31102
    assert [len(g) for g in graded] == [134, 266, 438, 5240] and len(near) == 44


def test_oracle_averaging_is_the_projection_onto_continuous_fields():
    # average_shared! (src/transfer.jl:1616-1714): shared nodes end equal,
    # a second averaging changes nothing, sum w u is kept, and a continuous
    # field (a polynomial at the nodes) is left as it is
    for D in (2, 3):
        mesh = T.brick_mesh(D, 3, 2, 2)
        t = T.Tables(3)
        rng = np.random.default_rng(5)
        u = rng.standard_normal(mesh.nblocks * 2 * mesh.NN)
        w0 = T.weighted_inner(mesh, t, u, np.ones_like(u), 2)
        ball = (np.full(D, 0.5), 10.0)
        a = T.average_shared(u.copy(), mesh, ball, 2)
        assert np.array_equal(T.average_shared(a.copy(), mesh, ball, 2), a)
        assert T.weighted_inner(mesh, t, a, np.ones_like(a), 2) == pytest.approx(w0, rel=1e-13)
        # coincident nodes across the face between blocks 0 and its upper
        # neighbour along dimension 0 (blocks listed with dimension 0 fastest)
        N = mesh.N
        A = a.reshape(mesh.nblocks, 2, mesh.NN)[:, 1]
        f0 = A[0].reshape((N,) * D)[..., N - 1]
        f1 = A[1].reshape((N,) * D)[..., 0]
        assert np.array_equal(f0, f1)
        # a continuous field
        g = np.zeros_like(u)
        for b in range(mesh.nblocks):
            for J in np.ndindex(*([2] * D)):
                e = tuple(reversed(J))
                lo, hi = mesh.element_box(b, e)
                grids = [lo[d] + (hi[d] - lo[d]) * (1 + t.nodes) / 2 for d in range(D)]
                m = np.meshgrid(*grids, indexing="ij")
                X = np.stack([x.reshape(-1) for x in m], axis=1)
                vals = (1 + X[:, 0] * X[:, -1]).reshape((4,) * D)
                g[mesh.node_index(b, e, 2)] = np.transpose(vals, tuple(range(D - 1, -1, -1))).reshape(-1)
        assert np.allclose(T.average_shared(g.copy(), mesh, ball, 2), g, rtol=0, atol=1e-15)


@pytest.mark.parametrize("ratio", [1e-1, 1e-3])
@pytest.mark.parametrize("moving", [False, True])
def test_oracle_pairing_integrates_the_particle(ratio, moving):
    # test/transfer_tests.jl:172-214: the pairing of the particle's density
    # with a polynomial is exact to 1e-12 at any size; the gradient's, whose
    # integrand is of size Q/ell and cancels to Q |grad g|, to 1e-12 Q/ell
    # and the points' rounding in absolute coordinates, eps |z| / ell of the
    # support, times the integrand's slope Q/ell^2
    P = 3
    mesh = T.brick_mesh(3, P, 2, 1)
    t = T.Tables(P)
    he = 0.5
    ell, Q = ratio * he, 1e-3
    v = np.array([0.1, -0.15, 0.05]) if moving else np.zeros(3)
    z = np.array([0.5, 0.5, 0.5]) + ell * np.array([0.3, -0.2, 0.1])
    s = T.Support(z, v, ell)
    g = brick_values(mesh, t, poly)
    got = T.pairing(g, mesh, t, lambda X: T.density_kernel(X, z, v, ell, Q), s, var=1)
    assert got[3] == pytest.approx(exact_moment(poly, Q, ell, z, v), rel=1e-12)
    for d in range(3):
        exact = -exact_moment(lambda X: grad_poly(X)[:, d], Q, ell, z, v)
        assert abs(got[d] - exact) <= 1e-12 * Q / ell + 10 * np.finfo(np.float64).eps * np.linalg.norm(z) * Q / ell ** 2
    assert len(T.support_elements(mesh, s, he)) == 8


def test_oracle_pairing_is_the_projection_folded():
    # test/transfer_tests.jl:398-425: the pairing over the support equals the
    # projection of the kernel over the mesh folded with the grid function
    P = 3
    mesh = T.brick_mesh(3, P, 2, 1)
    t = T.Tables(P)
    he = 0.5
    ell, Q = 0.01 * he, 0.07
    g = irregular(mesh.nblocks * 2 * mesh.NN)
    z = np.array([0.5, 0.5 + 0.004 * he, 0.3])
    for v, comps in ((np.zeros(3), (3,)), (np.array([0.2, 0.1, 0.0]), (0, 1, 2, 3))):
        s = T.Support(z, v, ell)
        got = T.pairing(g, mesh, t, lambda X: T.density_kernel(X, z, v, ell, Q), s, var=1)
        for c in comps:
            du = T.project_source(np.zeros_like(g), mesh, t, lambda X: T.density_kernel(X, z, v, ell, Q)[:, c], [s],
                                  (z, 2 * ell), factor=1.0, var=1, he=he)
            fold = T.weighted_inner(mesh, t, du, g, 1)
            assert got[c] == pytest.approx(fold, rel=1e-13 if c == 3 else 1e-12)


def test_oracle_continuous_pairing():
    # test/transfer_tests.jl:427-472: the continuous pairing reads a field
    # filled at the nodes as it is, takes away most of a face jump, and
    # refuses to look across the domain's faces
    P = 3
    mesh = T.brick_mesh(3, P, 2, 2)
    t = T.Tables(P)
    he = 0.25
    ell, Q = 0.01 * he, 0.07

    def smooth(X):
        return np.sin(np.pi * (2 * X[:, 0] + 0.3)) * np.cos(np.pi * (3 * X[:, 1] - 0.1)) + X[:, 2] ** 2

    g = brick_values(mesh, t, smooth)
    g.reshape(mesh.nblocks, 2, mesh.NN)[:, 1] *= 2
    z = np.array([0.5 - 0.2 * ell, 0.5 + 0.3 * ell, 0.625 + 0.1 * ell])
    s = T.Support(z, np.zeros(3), ell)

    def K(X):
        return T.density_kernel(X, z, np.zeros(3), ell, Q)

    for var in (1, 2):
        a = T.pairing(g, mesh, t, K, s, var=var, continuous=True)
        b = T.pairing(g, mesh, t, K, s, var=var)
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    b0, e0 = T.support_elements(mesh, s, he)[0]
    g2 = g.copy()
    g2[mesh.node_index(b0, e0, 1)] += 1

    def jump(continuous):
        return (T.pairing(g2, mesh, t, K, s, var=1, continuous=continuous) -
                T.pairing(g, mesh, t, K, s, var=1, continuous=continuous))[:3]

    plain, cont = np.linalg.norm(jump(False)), np.linalg.norm(jump(True))
    assert plain > 0.1 * Q / ell
    assert cont < 0.15 * plain and cont < 10 * Q / he
    s = T.Support(np.array([0.5, 0.125 - 0.4 * ell, 0.6]), np.zeros(3), ell)
    with pytest.raises(ValueError, match="does not look for periodic images"):
        T.pairing(g, mesh, t, lambda X: np.ones((len(X), 1)), s, continuous=True)


def test_transfer_entry_points_refuse_bad_arguments_on_the_host():
    # the C ABI's argument checks run before any device work
    import ctypes
    from twoldg import _lib
    lib = _lib.lib()
    out = (ctypes.c_double * 8)()
    n = ctypes.c_int32()
    h = ctypes.c_void_p()
    assert lib.twoldg_pairing(None, None, 1, 0, out) == _lib.TWOLDG_EINVAL
    assert b"must not be NULL" in lib.twoldg_last_error()
    assert lib.twoldg_support_elements(None, 0, out, ctypes.byref(n)) == _lib.TWOLDG_EINVAL
    assert lib.twoldg_transfer_plan_create(None, None, ctypes.byref(h)) == _lib.TWOLDG_EINVAL
    assert lib.twoldg_project_density(None, None, 1.0, 1) == _lib.TWOLDG_EINVAL
    assert lib.twoldg_average_shared(None, None, 2) == _lib.TWOLDG_EINVAL
    assert lib.twoldg_transfer_table(3, 0, b"nodes", 6, out) == _lib.TWOLDG_EINVAL
    assert b"unknown transfer table" in lib.twoldg_last_error()
    assert lib.twoldg_transfer_table(0, 0, b"bary", 6, out) == _lib.TWOLDG_EINVAL


def test_ball_rule_is_exact_on_what_it_should_be():
    # test/transfer_tests.jl:585-600: the volume and moments of the unit
    # ball, and the particle profile's unit charge
    ys, ws = T.ball_rule(8, 8)
    assert np.sum(ws) == pytest.approx(4 * math.pi / 3, rel=1e-14)
    assert np.sum(ws * ys[:, 0] ** 2) == pytest.approx(4 * math.pi / 15, rel=1e-14)
    assert np.sum(ws * ys[:, 0] ** 2 * ys[:, 1] ** 2 * ys[:, 2] ** 2) == pytest.approx(4 * math.pi / 945, rel=1e-13)
    assert abs(np.sum(ws * ys[:, 0] ** 3 * ys[:, 1])) < 1e-15
    ell = 1e-3
    rho = T.particle_density(ys * ell, np.zeros(3), np.zeros(3), ell, 1.0)
    assert np.sum(ws * rho * ell ** 3) == pytest.approx(1.0, rel=1e-14)


@pytest.mark.parametrize("D,P", [(1, 4), (2, 3), (3, 2)])
def test_reconstruction_is_the_element_polynomial(D, P):
    # test/transfer_tests.jl:554-583 through the host stencils the device
    # gather reads: exact on a polynomial of degree P per dimension, with its
    # gradient, and the stored value at a node (a face node reconstructs the
    # upper element, so those are left out)
    from cases import node_positions
    from twoldg.extraction import element_stencils
    from twoldg.forest import wave_forest
    forest = wave_forest(np.float64, D, P, 2, roots=2)
    N, nb = forest.N, len(forest.leaves)
    x = np.moveaxis(node_positions(forest, P), 1, 2)            # (nb, N^D, D)

    def poly(X):
        return np.prod([1 + (d + 1) * X[..., d] - X[..., d] ** P for d in range(D)], axis=0)

    def grad(X):
        out = []
        for d in range(D):
            g = (d + 1) - P * X[..., d] ** (P - 1)
            for k in range(D):
                if k != d:
                    g = g * (1 + (k + 1) * X[..., k] - X[..., k] ** P)
            out.append(g)
        return np.stack(out, axis=-1)

    u = np.zeros((nb, 2, N ** D))
    u[:, 0] = poly(x)
    u = u.reshape(-1)
    pts = np.array([[(0.3 + 0.618 * k * (d + 1)) % 1.0 for d in range(D)] for k in range(1, 21)])
    index, weights = element_stencils(forest, P, pts)
    assert np.allclose(np.sum(weights * u[index], axis=1), poly(pts), rtol=1e-13, atol=0)
    for d in range(D):
        index, weights = element_stencils(forest, P, pts, deriv=d)
        assert np.abs(np.sum(weights * u[index], axis=1) - grad(pts)[:, d]).max() <= 1e-12 * np.abs(grad(pts)).max()
    w = irregular(nb * 2 * N ** D).reshape(nb, 2, N ** D)
    grids = np.indices([N] * D).reshape(D, -1)[::-1]
    interior = np.all(grids % (P + 1) != P, axis=0)
    for b in (0, nb - 1):
        X = x[b][interior]
        index, weights = element_stencils(forest, P, X)
        got = np.sum(weights * w.reshape(-1)[index + N ** D], axis=1)
        assert np.abs(got - w[b, 1][interior]).max() <= 1e-14


@pytest.mark.parametrize("ratio", [1e-1, 1e-2, 1e-3, 1e-4])
def test_sinh_points_grow_like_log_of_he_over_ell(ratio):
    # test/transfer_tests.jl:216-240: for the field of a particle of size ell
    # just outside a face of the unit element, a sinh rule of
    # 16 + 8 log10(h_e/ell) points per line reaches 1e-12 of an 80-point one
    P = 3
    lo, hi = [0.0, 0.0, 0.0], [1.0, 1.0, 1.0]
    ell = ratio
    z = np.array([1 + 1.01 * ell, 0.3, 0.6])
    s = T.Support(z, np.zeros(3), ell)

    def field(t):
        def g(X):
            r2 = np.sum((X - z) ** 2, axis=1)
            val = np.where(r2 < ell ** 2, (3 - r2 / ell ** 2) / (2 * ell), 1 / np.sqrt(r2))
            return val[:, None] * t.element_basis(lo, hi, X)
        return g

    tref = T.Tables(P, nsinh=80)
    ref = T.nested_rule(field(tref), s, tref, lo, hi, 3)
    t = T.Tables(P, nsinh=16 + 8 * round(math.log10(1 / ratio)))
    assert np.abs(T.nested_rule(field(t), s, t, lo, hi, 3) - ref).max() < 1e-12 * np.abs(ref).max()
