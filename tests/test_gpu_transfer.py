"""The particle-grid transfer on the GPU, through the C ABI: the projection
of the particles' density and of a caller's source against the oracle, and
the reference's own assertions (test/transfer_tests.jl) through the device:
the nested rule integrates a particle to 1e-12 at any size and speed, the
projection is consistent at order P and adjoint to the reconstruction, and
it does not jump as a particle crosses r_near or a face."""
import math

import numpy as np
import pytest

from oracle import transfer as T
from transfer_cases import exact_moment, irregular, poly, reference_integral

pytestmark = pytest.mark.gpu


def _problem(D, P, roots, dtype=np.float64, E=2):
    import twoldg
    f = twoldg.wave_forest(dtype, D, P, E, roots=roots)
    return twoldg.WaveProblem(f, twoldg.Element(dtype, P))


def _mesh(p):
    """The oracle's view of problem p's forest, in the state's block order."""
    f = p.forest
    origins = [[f.block_extent(k)[d][0] for d in range(p.D)] for k in f.leaves]
    spacings = [f.spacing(k) for k in f.leaves]
    return T.Mesh(origins, spacings, p.P, p.E)


def _node_weights(p):
    """w_n of every node of the state vector, for var 1 and var 2 alike."""
    P1 = p.P + 1
    w1 = np.tile(T.Tables(p.P).weights, p.E)
    out = np.empty((p.nblocks, p.NN))
    for b, k in enumerate(p.forest.leaves):
        h = p.forest.spacing(k)
        w = np.ones(1)
        for _ in range(p.D):
            w = ((w1 * h * P1 / 2)[:, None] * w[None, :]).reshape(-1)
        out[b] = w
    return np.repeat(out[:, None, :], 2, axis=1).reshape(-1)


def _inner(p, a, b, var):
    w = _node_weights(p).reshape(p.nblocks, 2, p.NN)[:, var - 1]
    a = np.asarray(a, dtype=np.float64).reshape(p.nblocks, 2, p.NN)[:, var - 1]
    b = np.asarray(b, dtype=np.float64).reshape(p.nblocks, 2, p.NN)[:, var - 1]
    return float(np.sum(w * a * b))


def _host(u):
    return u.double().cpu().numpy()


def test_density_projection_matches_the_oracle(native):
    from twoldg import ParticleSupport, project_source
    D, P = 3, 3
    p = _problem(D, P, 2)
    z = np.array([0.53, 0.47, 0.51])
    v = np.array([0.1, -0.15, 0.05])
    ell, Q = 0.02, 0.3
    ball = (z, 0.45)
    du = p.statevector()
    project_source(du, p, "density", [ParticleSupport(z, v, ell, charge=Q)], ball, rnear=1.0, factor=0.7, var=2)
    got = _host(du)
    ref = T.project_source(np.zeros(p.state_words), _mesh(p), T.Tables(P),
                           lambda X: T.particle_density(X, z, v, ell, Q), [T.Support(z, v, ell)], ball,
                           rnear=1.0, factor=0.7, var=2, he=0.25)
    assert np.abs(ref).max() > 0
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.all(got.reshape(p.nblocks, 2, -1)[:, 0] == 0)


@pytest.mark.parametrize("D,P", [(1, 3), (2, 2), (3, 3)])
def test_caller_source_projection_matches_the_oracle(native, D, P):
    # the source of test/transfer_tests.jl:295-328, evaluated by the caller
    # at the plan's points (the launch_points! role)
    import torch
    from twoldg import ParticleSupport, TransferPlan
    p = _problem(D, P, 2)
    z = np.array([0.5 + 0.03 * (d + 1) for d in range(D)])
    v = np.array([0.1 / (d + 1) for d in range(D)])
    s = ParticleSupport(z, v, 0.01)
    rnear = 1.5 if D < 3 else 1.0
    plan = TransferPlan(p, [s], (z, 1.0), rnear)
    assert plan.counts["near_elements"] > 2 ** D

    zt = torch.tensor(z, dtype=torch.float64, device="cuda")

    def S(xs):
        return 1 / (((xs - zt[:, None]) ** 2).sum(0) + 1e-4) + xs[0]

    du = p.statevector()
    plan.project(du, S, factor=1.0, var=2)
    got = _host(du)

    def Sn(X):
        return 1 / (np.sum((X - z[None, :]) ** 2, axis=1) + 1e-4) + X[:, 0]

    ref = T.project_source(np.zeros(p.state_words), _mesh(p), T.Tables(P), Sn, [T.Support(z, v, 0.01)], (z, 1.0),
                           rnear=rnear, factor=1.0, var=2)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("ratio", [1e-1, 1e-2, 1e-3, 1e-4])
@pytest.mark.parametrize("moving", [False, True])
def test_near_rule_integrates_the_particle_at_any_size(native, ratio, moving):
    # test/transfer_tests.jl:172-214 through the device
    from twoldg import ParticleSupport, TransferPlan
    p = _problem(3, 3, 1)
    he = 0.5
    ell = ratio * he
    Q = 1e-3
    v = np.array([0.1, -0.15, 0.05]) if moving else np.zeros(3)
    z = np.array([0.5, 0.5, 0.5]) + ell * np.array([0.3, -0.2, 0.1])
    plan = TransferPlan(p, [ParticleSupport(z, v, ell, charge=Q)], (z, 2 * ell))
    assert plan.counts["near_elements"] == 8 and plan.counts["far_elements"] == 0
    du = p.statevector()
    plan.project(du, "density", factor=1.0, var=1)
    got = _host(du)
    gamma = 1 / math.sqrt(1 - v @ v)
    assert _inner(p, got, np.ones_like(got), 1) == pytest.approx(Q / gamma, rel=1e-12)
    g = p.fill_at_nodes(lambda x, var: poly(np.stack([x[0].reshape(-1), x[1].reshape(-1), x[2].reshape(-1)],
                                                     axis=1)).reshape(x[0].shape)).reshape(-1)
    assert _inner(p, got, g, 1) == pytest.approx(exact_moment(poly, Q, ell, z, v), rel=1e-12)


def test_float32_density_keeps_the_charge(native):
    from twoldg import ParticleSupport, project_source
    p = _problem(3, 3, 1, dtype=np.float32)
    ell, Q = 5e-3, 1e-3
    v = np.array([0.1, -0.15, 0.05])
    z = np.array([0.5, 0.5, 0.5]) + ell * np.array([0.3, -0.2, 0.1])
    du = p.statevector()
    project_source(du, p, "density", [ParticleSupport(z, v, ell, charge=Q)], (z, 2 * ell), factor=1.0, var=1)
    got = _host(du)
    gamma = 1 / math.sqrt(1 - v @ v)
    assert _inner(p, got, np.ones_like(got), 1) == pytest.approx(Q / gamma, rel=1e-5)


def _projection_error(D, P, roots):
    import torch
    from twoldg import project_source
    p = _problem(D, P, roots)

    def S(xs):
        out = torch.sin(2 * math.pi * xs[0])
        for d in range(1, D):
            out = out * torch.cos(2 * math.pi * xs[d])
        return out + 0.3

    du = p.statevector()
    project_source(du, p, S, [], (np.full(D, 0.5), 2.0), factor=1.0)

    def Sn(x, var):
        out = np.sin(2 * np.pi * x[0])
        for d in range(1, D):
            out = out * np.cos(2 * np.pi * x[d])
        return (out + 0.3) if var == 2 else 0 * out

    err = _host(du) - p.fill_at_nodes(Sn).reshape(-1)
    one = np.ones_like(err)
    return math.sqrt(_inner(p, err, err, 2) / _inner(p, one, one, 2))


def test_projection_is_consistent_at_order_P(native):
    # test/transfer_tests.jl:108-133 through the device
    for D, P in ((1, 2), (1, 3), (1, 4), (2, 2), (2, 3), (2, 4)):
        errs = [_projection_error(D, P, r) for r in (2, 4, 8)]
        rate = np.polyfit(np.log([1 / 2, 1 / 4, 1 / 8]), np.log(errs), 1)[0]
        assert rate > P - 0.1, (D, P, errs)
    e = [_projection_error(3, 2, r) for r in (2, 4)]
    assert math.log2(e[0] / e[1]) > 2 - 0.2


def test_projection_is_adjoint_to_the_reconstruction_2d(native):
    # test/transfer_tests.jl:135-170, D = 2: <P S, g>_w = int S g_h for a bump
    # straddling a face (the nested rule split at its support), a Lorentzian
    # peak (the sinh rule) and a smooth part (the far rule)
    import torch
    from twoldg import ParticleSupport, project_source
    D, roots, eps, grades, tol = 2, 4, 0.1, range(-10, 5), 1e-12
    P = 3
    p = _problem(D, P, roots)
    he = 1 / roots / 2
    ell = 0.05 * he
    z = np.array([0.5 + 0.3 * ell, 0.5 + 0.22 * he])
    zt = torch.tensor(z, dtype=torch.float64, device="cuda")

    def S(xs):
        r2 = ((xs - zt[:, None]) ** 2).sum(0)
        b = torch.where(r2 < ell * ell, (1 - r2 / ell ** 2) ** 4, torch.zeros_like(r2))
        return torch.cos(xs[0]) + b / ell ** D + eps * he / (r2 + (eps * he) ** 2) ** 0.5

    def Sn(X):
        r2 = np.sum((X - z[None, :]) ** 2, axis=1)
        return np.cos(X[:, 0]) + np.where(r2 < ell * ell, (1 - r2 / ell ** 2) ** 4, 0.0) / ell ** D + \
            eps * he / (r2 + (eps * he) ** 2) ** 0.5

    du = p.statevector()
    project_source(du, p, S, [ParticleSupport(z, [0.0, 0.0], ell)], (z, 10.0), factor=1.0)
    got = _host(du)
    g = irregular(len(got))
    lhs = _inner(p, got, g, 2)
    mesh = _mesh(p)
    t = T.Tables(P)
    rhs = 0.0
    for b in range(mesh.nblocks):
        for J in np.ndindex(2, 2):
            e = tuple(reversed(J))
            lo, hi = mesh.element_box(b, e)
            gv = g[mesh.node_index(b, e, 2)]
            rhs += reference_integral(lambda X: Sn(X) * (t.element_basis(lo, hi, X) @ gv), lo, hi, z, ell, grades,
                                      ell)
    assert lhs == pytest.approx(rhs, rel=tol)


def test_projection_does_not_jump_across_rnear_or_faces(native):
    # test/transfer_tests.jl:281-293: a source that does not move, projected
    # with a particle that does, stays put to 1e-12
    import torch
    from twoldg import ParticleSupport, project_source
    p = _problem(3, 3, 1)
    he = 0.5
    ell = 1e-3

    def S(xs):
        return torch.cos(xs[0] - xs[1] / 2) * torch.exp(xs[2] / 2)

    def project(z):
        du = p.statevector()
        project_source(du, p, S, [ParticleSupport(z, [0.0] * 3, ell)], ((0.5, 0.5, 0.5), 2.0), rnear=1.5,
                       factor=1.0)
        return _host(du)

    base = project((5.0, 5.0, 5.0))
    for z in ((0.5 + 1.5 * he + 1e-6, 0.3, 0.2), (0.5 + 1.5 * he - 1e-6, 0.3, 0.2), (0.5 - 0.3 * ell, 0.3, 0.2),
              (0.5 + 0.3 * ell, 0.5 - 0.2 * ell, 0.2)):
        assert np.abs(project(z) - base).max() < 1e-12 * np.abs(base).max()


def test_points_are_the_rules_points(native):
    from twoldg import ParticleSupport, TransferPlan
    p = _problem(2, 3, 2)
    z = np.array([0.52, 0.49])
    plan = TransferPlan(p, [ParticleSupport(z, [0.0, 0.0], 0.01)], (z, 1.0))
    xs = plan.points().double().cpu().numpy()
    c = plan.counts
    assert xs.shape == (2, c["points"])
    assert c["points"] == c["far_points"] + c["graded_points"] + c["near_points"]
    mesh = _mesh(p)
    t = T.Tables(3)
    far, graded, near = T.classify(mesh, t, [T.Support(z, np.zeros(2), 0.01)], (z, 1.0), 1.0, 0.25)
    assert (len(far), sum(map(len, graded)), len(near)) == (c["far_elements"], c["graded_elements"],
                                                           c["near_elements"])
    # the first far element's Gauss points, dimension 0 fastest
    if far:
        b, e = far[0]
        lo, hi = mesh.element_box(b, e)
        x, _, _ = t.far
        q = len(x)
        for j in range(q * q):
            j0, j1 = j % q, j // q
            assert xs[0, j] == pytest.approx(lo[0] + (hi[0] - lo[0]) * (1 + x[j0]) / 2, abs=1e-15)
            assert xs[1, j] == pytest.approx(lo[1] + (hi[1] - lo[1]) * (1 + x[j1]) / 2, abs=1e-15)
    # the nested rule's points, element by element, as the oracle lists them
    X = np.concatenate([T.nested_points(T.Support(z, np.zeros(2), 0.01), t, *mesh.element_box(b, e), 2)[0]
                        for b, e, _ in near])
    assert np.allclose(xs[:, c["far_points"] + c["graded_points"]:].T, X, rtol=0, atol=1e-15)


def test_refusals(native):
    import twoldg
    from twoldg import ParticleSupport, TransferPlan
    p = _problem(3, 3, 1)
    s = ParticleSupport((0.5, 0.5, 0.5), (0, 0, 0), 1e-3)
    with pytest.raises(ValueError, match="rnear"):
        TransferPlan(p, [s], ((0.5,) * 3, 1.0), rnear=10.0)
    a = ParticleSupport((0.26, 0.26, 0.26), (0, 0, 0), 0.02)
    b = ParticleSupport((0.27, 0.27, 0.27), (0, 0, 0), 0.02)
    with pytest.raises(ValueError, match="two particles"):
        TransferPlan(p, [a, b], ((0.5,) * 3, 1.0))
    with pytest.raises(ValueError, match="below 1"):
        ParticleSupport((0.5,) * 3, (0.8, 0.7, 0.0), 1e-3)
    # a ball that reaches a coarser block
    f = twoldg.wave_forest(np.float64, 2, 3, 2, roots=2)
    f.refine([f.leaves[0]])
    q = twoldg.WaveProblem(f, twoldg.Element(np.float64, 3))
    with pytest.raises(ValueError, match="finest level"):
        TransferPlan(q, [], ((0.75, 0.75), 0.1))
    TransferPlan(q, [], ((0.1, 0.1), 0.05)).close()


def test_first_run_plan_counts_match_the_oracle(native):
    # the library's classification of the first run's window: the oracle's
    # counts, which hold the reference's 31 102 far elements (CODE.md
    # "Quadrature")
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from bench import transfer_setup
    import twoldg
    p, parts, ball = transfer_setup(twoldg)
    plan = twoldg.TransferPlan(p, parts, ball)
    c = plan.counts
    assert c["far_elements"] == 31102 and c["graded_elements"] == 134 + 266 + 438 + 5240
    assert c["near_elements"] == 44
    assert c["far_points"] == 31102 * 216
    assert c["graded_points"] == 134 * 14 ** 3 + 266 * 10 ** 3 + 438 * 8 ** 3 + 5240 * 7 ** 3
    plan.close()


def test_updated_plan_projects_as_a_fresh_one(native):
    # the reference holds a projection through a kept SourceBall to a fresh
    # one's bit for bit (CODE.md "What the projection reads of the forest is
    # built once"): an updated plan, likewise, for the density and for values
    import torch
    from twoldg import ParticleSupport, TransferPlan
    p = _problem(3, 3, 2)
    ball = ((0.5, 0.5, 0.5), 0.6)
    a = [ParticleSupport((0.41, 0.52, 0.47), (0.1, 0.0, 0.0), 0.02, charge=0.5),
         ParticleSupport((0.7, 0.33, 0.61), (0.0, -0.2, 0.05), 0.015, charge=-0.5)]
    b = [ParticleSupport((0.43, 0.51, 0.49), (0.1, 0.02, 0.0), 0.02, charge=0.5),
         ParticleSupport((0.69, 0.35, 0.6), (0.0, -0.2, 0.05), 0.015, charge=-0.5)]

    def S(xs):
        return torch.cos(3 * xs[0]) * torch.exp(xs[1] - xs[2])

    plan = TransferPlan(p, a, ball)
    plan.update(b)
    fresh = TransferPlan(p, b, ball)
    assert plan.counts == fresh.counts
    for src in ("density", S):
        d1, d2 = p.statevector(), p.statevector()
        plan.project(d1, src)
        fresh.project(d2, src)
        assert torch.equal(d1, d2)


@pytest.mark.parametrize("D,roots,ball", [(2, 3, ((0.4, 0.55), 0.5)), (3, 2, ((0.5, 0.5, 0.5), 2.0))])
def test_averaging_matches_the_oracle_bit_for_bit(native, D, roots, ball):
    # average_shared! (src/transfer.jl:1616-1714): each pair of coincident
    # nodes takes (lower + upper) / 2, in the ball's blocks
    import torch
    from twoldg import TransferPlan
    p = _problem(D, 3, roots)
    rng = np.random.default_rng(11)
    host = rng.standard_normal(p.state_words)
    u = torch.from_numpy(host.copy()).cuda()
    plan = TransferPlan(p, [], ball)
    plan.average_shared(u, var=2)
    ref = T.average_shared(host.copy(), _mesh(p), ball, 2)
    assert np.array_equal(_host(u), ref)
    plan.average_shared(u, var=1)
    assert np.array_equal(_host(u), T.average_shared(ref.copy(), _mesh(p), ball, 1))


def test_source_rhs_is_the_wave_rhs_less_the_averaged_projection(native):
    # inspiral_rhs!'s field part (src/inspiral.jl): wave_rhs!, the projected
    # source subtracted from v's rate, the averaging over shared nodes
    import torch
    import twoldg
    from oracle.oracle import Oracle
    from cases import smooth_data, state_from
    p = _problem(3, 3, 2)
    o = Oracle(p.forest, 3)
    u0 = o.truncate(state_from(p.forest, 3, smooth_data(3)))
    z = np.array([0.52, 0.46, 0.49])
    v = np.array([0.05, 0.1, -0.02])
    s = twoldg.ParticleSupport(z, v, 0.03, charge=0.4)
    ball = ((0.5, 0.5, 0.5), 0.7)
    plan = twoldg.TransferPlan(p, [s], ball)
    du = p.statevector()
    twoldg.source_rhs(du, torch.from_numpy(u0).cuda(), p, plan, "density")
    ref = o.rhs(u0)
    T.project_source(ref, _mesh(p), T.Tables(3), lambda X: T.particle_density(X, z, v, 0.03, 0.4),
                     [T.Support(z, v, 0.03)], ball, factor=-1.0, var=2, he=0.25)
    T.average_shared(ref, _mesh(p), ball, 2)
    assert np.abs(_host(du) - ref).max() <= 1e-12 * np.abs(ref).max()


def test_projection_in_the_ball_cube_keeps_the_charge(native):
    # the particles' frame on the seven-patch ball is its affine cube
    # (ParticleFrame, src/transfer.jl:705-766): a particle there projects
    # its charge Q / gamma onto the cube's nodes
    import twoldg
    forest, geo = twoldg.sevenpatch_forest(np.float64, 3, 2, roots=(4, 4), Lc=1.0, R1=3.0)
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, 3), truncate=True, geometry=geo,
                           boundary=twoldg.RadiativeBoundary())
    v = np.array([0.1, 0.05, -0.2])
    z = np.array([0.013, -0.021, 0.008])
    Q, ell = 0.2, 0.01
    du = p.statevector()
    twoldg.project_source(du, p, "density", [twoldg.ParticleSupport(z, v, ell, charge=Q)], (z, 3 * ell),
                          factor=1.0, var=1)
    got = _host(du).reshape(p.nblocks, 2, p.NN)
    scale = 2 * geo.Lc / 4
    w1 = np.tile(T.Tables(3).weights, 2) * (scale / p.N * 4 / 2)
    w = (w1[:, None, None] * w1[None, :, None] * w1[None, None, :]).reshape(-1)
    total = sum(float(np.sum(w * got[b, 0])) for b, (patch, _) in enumerate(forest.blocks) if patch == 0)
    assert np.abs(got[[b for b, (q, _) in enumerate(forest.blocks) if q != 0], 0]).max() == 0
    gamma = 1 / math.sqrt(1 - v @ v)
    assert total == pytest.approx(Q / gamma, rel=1e-12)
    with pytest.raises(ValueError, match="cube"):
        twoldg.TransferPlan(p, [twoldg.ParticleSupport((0.99, 0.0, 0.0), (0, 0, 0), 0.05)], ((0.5, 0, 0), 0.2))


# The pairing (src/transfer.jl:1779-1797) of each particle's density kernel
# (grad rho, rho) with a field, on the device against the oracle's nested
# rule. The gradient's integrand is of size Q/ell, the density's of size Q:
# each component is held to 1e-12 of its own scale times max |g|.
def _grad_tolerance(Q, ell, z):
    # The gradient's integrand is of size Q/ell and cancels to Q |grad g|.
    # Each point's position is rounded to eps |z| in absolute coordinates,
    # eps |z| / ell of the support, which the integrand's slope Q/ell^2 turns
    # into an error of that order: 1e-12 Q/ell, and ten times eps |z| Q/ell^2.
    return 1e-12 * Q / ell + 10 * np.finfo(np.float64).eps * float(np.linalg.norm(z)) * Q / ell ** 2


def _pair_scale(s, Q):
    return np.array([Q / s.ell] * 3 + [Q])


def _oracle_pairs(p, g, parts, Q, var, continuous):
    mesh, t = _mesh(p), T.Tables(p.P)
    he = min(p.forest.spacing(k) for k in p.forest.leaves) * (p.P + 1)
    return np.array([T.pairing(g, mesh, t, lambda X, s=s: T.density_kernel(X, s.z, s.v, s.ell, Q),
                               T.Support(s.z, s.v, s.ell), var=var, continuous=continuous, he=he) for s in parts])


@pytest.mark.parametrize("moving", [False, True])
def test_pairing_matches_the_oracle(native, moving):
    import torch
    from twoldg import ParticleSupport, TransferPlan
    p = _problem(3, 3, 4)
    he, Q = 0.125, 0.07
    ell = 0.05 * he
    v = np.array([0.2, -0.1, 0.05]) if moving else np.zeros(3)
    # one support on the corner of eight blocks, one across an element face
    parts = [ParticleSupport((0.5 + 0.3 * ell, 0.5 - 0.2 * ell, 0.5 + 0.1 * ell), v, ell, charge=Q),
             ParticleSupport((0.3, 0.375 - 0.4 * ell, 0.7), -v, ell, charge=Q)]
    plan = TransferPlan(p, parts, ((0.5, 0.5, 0.5), 0.6))
    assert [len(plan.support_elements(k)) for k in range(2)] == [8, 2]
    mesh = _mesh(p)
    for k, s in enumerate(parts):
        assert plan.support_elements(k) == T.support_elements(mesh, T.Support(s.z, s.v, s.ell), he)
    g = irregular(p.state_words)
    u = torch.from_numpy(g.copy()).cuda()
    for var in (1, 2):
        for continuous in (False, True):
            got = plan.pairing(u, var=var, continuous=continuous)
            ref = _oracle_pairs(p, g, parts, Q, var, continuous)
            for k, s in enumerate(parts):
                assert np.all(np.abs(got[k] - ref[k]) <= 1e-12 * _pair_scale(s, Q)), (var, continuous, k)


@pytest.mark.parametrize("ratio", [1e-1, 1e-2, 1e-3, 1e-4])
@pytest.mark.parametrize("moving", [False, True])
def test_pairing_integrates_the_particle_at_any_size(native, ratio, moving):
    # test/transfer_tests.jl:172-214 through the device: the pairing with a
    # polynomial is its exact moment (the ball rule in the rest frame), and
    # the gradient's is minus the moment of the polynomial's gradient
    import torch
    from twoldg import ParticleSupport, TransferPlan
    from transfer_cases import grad_poly
    p = _problem(3, 3, 1)
    he, Q = 0.5, 1e-3
    ell = ratio * he
    v = np.array([0.1, -0.15, 0.05]) if moving else np.zeros(3)
    z = np.array([0.5, 0.5, 0.5]) + ell * np.array([0.3, -0.2, 0.1])
    plan = TransferPlan(p, [ParticleSupport(z, v, ell, charge=Q)], (z, 2 * ell))
    assert len(plan.support_elements(0)) == 8
    g = p.fill_at_nodes(lambda x, var: poly(np.stack([x[0].reshape(-1), x[1].reshape(-1), x[2].reshape(-1)],
                                                     axis=1)).reshape(x[0].shape)).reshape(-1)
    got = plan.pairing(torch.from_numpy(g.copy()).cuda(), var=1)[0]
    assert got[3] == pytest.approx(exact_moment(poly, Q, ell, z, v), rel=1e-12)
    for d in range(3):
        assert abs(got[d] + exact_moment(lambda X: grad_poly(X)[:, d], Q, ell, z, v)) <= _grad_tolerance(Q, ell, z)


def test_pairing_is_the_density_projection_folded(native):
    # test/transfer_tests.jl:398-425: <P rho, g>_w, the projection of the
    # density over the mesh folded with g, is the pairing of rho with g
    import torch
    from twoldg import ParticleSupport, TransferPlan
    p = _problem(3, 3, 2)
    he, Q = 0.25, 0.07
    ell = 0.01 * he
    g = irregular(p.state_words)
    for v in (np.zeros(3), np.array([0.2, 0.1, 0.0])):
        z = np.array([0.5, 0.5 + 0.004 * he, 0.3])
        plan = TransferPlan(p, [ParticleSupport(z, v, ell, charge=Q)], (z, 2 * ell))
        du = p.statevector()
        plan.project(du, "density", factor=1.0, var=1)
        fold = _inner(p, _host(du), g, 1)
        got = plan.pairing(torch.from_numpy(g.copy()).cuda(), var=1)[0]
        assert got[3] == pytest.approx(fold, rel=1e-13)


def test_continuous_pairing_reads_a_continuous_field_as_it_is(native):
    # test/transfer_tests.jl:427-472 through the device
    import torch
    from twoldg import ParticleSupport, TransferPlan
    p = _problem(3, 3, 4)
    he, Q = 0.125, 0.07
    ell = 0.01 * he

    def smooth(x, var):
        return var * (np.sin(np.pi * (2 * x[0] + 0.3)) * np.cos(np.pi * (3 * x[1] - 0.1)) + x[2] ** 2)

    g = p.fill_at_nodes(smooth).reshape(-1)
    u = torch.from_numpy(g.copy()).cuda()
    for z in ((0.5 + 0.3 * ell, 0.375 - 0.4 * ell, 0.6), (0.5 - 0.2 * ell, 0.5 + 0.3 * ell, 0.625 + 0.1 * ell)):
        plan = TransferPlan(p, [ParticleSupport(z, (0, 0, 0), ell, charge=Q)], (z, 2 * ell))
        for var in (1, 2):
            a = plan.pairing(u, var=var, continuous=True)[0]
            b = plan.pairing(u, var=var)[0]
            assert np.all(np.abs(a - b) <= 1e-12 * np.abs(b).max()), var
        b0, e0 = plan.support_elements(0)[0]
        g2 = g.copy().reshape(p.nblocks, 2, -1)
        P1, N = p.P + 1, p.N
        for K in np.ndindex(P1, P1, P1):
            i = sum((e0[d] * P1 + K[d]) * N ** d for d in range(3))
            g2[b0, 0, i] += 1
        u2 = torch.from_numpy(g2.reshape(-1).copy()).cuda()

        def jump(continuous):
            return np.linalg.norm((plan.pairing(u2, 1, continuous) - plan.pairing(u, 1, continuous))[0, :3])

        assert jump(False) > 0.1 * Q / ell
        assert jump(True) < 0.15 * jump(False) and jump(True) < 10 * Q / he
    plan = TransferPlan(p, [ParticleSupport((0.5, 0.125 - 0.4 * ell, 0.6), (0, 0, 0), ell)], ((0.5, 0.5, 0.5), 0.6))
    plan.pairing(u, 1)
    with pytest.raises(ValueError, match="does not look for periodic images"):
        plan.pairing(u, 1, continuous=True)


def test_pairing_refusals(native):
    import torch
    from twoldg import ParticleSupport, TransferPlan
    p = _problem(3, 3, 1)
    u = torch.zeros(p.state_words, dtype=torch.float64, device="cuda")
    plan = TransferPlan(p, [ParticleSupport((0.3, 0.3, 0.3), (0, 0, 0), 0.3)], ((0.3, 0.3, 0.3), 0.5))
    with pytest.raises(ValueError, match="not smaller than an element"):
        plan.pairing(u)
    plan.update([ParticleSupport((0.01, 0.3, 0.3), (0, 0, 0), 0.02)])
    with pytest.raises(ValueError, match="periodic images"):
        plan.pairing(u)
    # the projection still runs on the refused plan
    plan.project(p.statevector(), "density")


def test_float32_pairing_matches_the_oracle_of_its_values(native):
    # the moments are FP64 whatever the field type: the pairing of an FP32
    # state is the oracle's pairing of the same (rounded) values
    import torch
    from twoldg import ParticleSupport, TransferPlan
    p = _problem(3, 3, 2, dtype=np.float32)
    he, Q = 0.25, 0.07
    ell = 0.05 * he
    s = ParticleSupport((0.5 + 0.3 * ell, 0.5 - 0.2 * ell, 0.4), (0.1, 0.2, 0.0), ell, charge=Q)
    plan = TransferPlan(p, [s], ((0.5, 0.5, 0.5), 0.6))
    g = irregular(p.state_words).astype(np.float32)
    u = torch.from_numpy(g.copy()).cuda()
    ref = _oracle_pairs(p, g.astype(np.float64), [s], Q, 2, True)
    got = plan.pairing(u, var=2, continuous=True)
    assert np.all(np.abs(got[0] - ref[0]) <= 1e-12 * _pair_scale(s, Q))


def test_pairing_repeats_and_follows_the_particles(native):
    # a pairing is the same to the bit on every call, and an updated plan's is
    # a fresh plan's; particle_forces is grad rho paired with u less v times
    # rho paired with v
    import torch
    import twoldg
    from twoldg import ParticleSupport, TransferPlan
    p = _problem(3, 3, 2)
    ball = ((0.5, 0.5, 0.5), 0.6)
    a = [ParticleSupport((0.41, 0.52, 0.47), (0.1, 0.0, 0.0), 0.02, charge=0.5),
         ParticleSupport((0.7, 0.33, 0.61), (0.0, -0.2, 0.05), 0.015, charge=-0.5)]
    b = [ParticleSupport((0.5, 0.56, 0.44), (0.1, 0.02, 0.0), 0.02, charge=0.5),
         ParticleSupport((0.69, 0.375, 0.6), (0.0, -0.2, 0.05), 0.015, charge=-0.5)]
    u = torch.from_numpy(irregular(p.state_words)).cuda()
    plan = TransferPlan(p, a, ball)
    first = plan.pairing(u, 1, True)
    assert np.array_equal(first, plan.pairing(u, 1, True))
    plan.update(b)
    fresh = TransferPlan(p, b, ball)
    for var in (1, 2):
        assert np.array_equal(plan.pairing(u, var, True), fresh.pairing(u, var, True))
    F = twoldg.particle_forces(plan, u)
    phi, pi = plan.pairing(u, 1, True), plan.pairing(u, 2, True)
    v = np.array([s.v for s in b])
    assert np.array_equal(F, phi[:, :3] - v * pi[:, 3:4])
    # source_pairing: the pairing of the density's own projection, averaged
    du = p.statevector()
    plan.project(du, "density", factor=1.0, var=1)
    assert np.array_equal(twoldg.source_pairing(plan, "density"), plan.pairing(du, 1, True))


def test_pairing_in_the_ball_cube(native):
    # in the seven-patch ball's cube a constant field pairs to Q / gamma with
    # rho and to zero with grad rho
    import torch
    import twoldg
    forest, geo = twoldg.sevenpatch_forest(np.float64, 3, 2, roots=(4, 4), Lc=1.0, R1=3.0)
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, 3), truncate=True, geometry=geo,
                           boundary=twoldg.RadiativeBoundary())
    v = np.array([0.1, 0.05, -0.2])
    z = np.array([0.013, -0.021, 0.008])
    Q, ell = 0.2, 0.01
    plan = twoldg.TransferPlan(p, [twoldg.ParticleSupport(z, v, ell, charge=Q)], (z, 3 * ell))
    u = torch.ones(p.state_words, dtype=torch.float64, device="cuda")
    got = plan.pairing(u, var=1, continuous=True)[0]
    gamma = 1 / math.sqrt(1 - v @ v)
    assert got[3] == pytest.approx(Q / gamma, rel=1e-12)
    assert np.abs(got[:3]).max() <= 1e-12 * Q / ell


def test_reconstruct_gradient_is_the_polynomial_gradient(native):
    # reconstruct_gradient (src/transfer.jl:2011-2030) through the device
    # gather: a polynomial of degree P per dimension filled at the nodes gives
    # its exact gradient, inside an element and on its faces
    import torch
    import twoldg
    p = _problem(3, 3, 2)
    g = p.fill_at_nodes(lambda x, var: var * (x[0] ** 3 + x[0] * x[1] * x[2] - 2 * x[1] ** 2)).reshape(-1)
    u = torch.from_numpy(g.copy()).cuda()
    for X in ((0.31, 0.52, 0.77), (0.5, 0.25, 0.9)):
        exact = np.array([3 * X[0] ** 2 + X[1] * X[2], X[0] * X[2] - 4 * X[1], X[0] * X[1]])
        for var in (1, 2):
            got = twoldg.reconstruct_gradient(p, u, X, var=var)
            assert np.abs(got - var * exact).max() <= 1e-12 * np.abs(exact).max()
