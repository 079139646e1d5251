"""The seven-patch ball through libtwoldg (full metric, quarter-turn glue,
Dirichlet plane wave) against the oracle, and sevenpatch_errors against the
reference's published table. Marked gpu."""
import math

import numpy as np
import pytest

from ball_cases import ball_setup, ball_state

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a, dtype=np.float64) - b).max() / np.abs(b).max())


def problem(forest, P, wave, truncate=True, dtype=np.float64, precision=None):
    import twoldg
    return twoldg.WaveProblem(forest, twoldg.Element(dtype, P), truncate=truncate, geometry=forest.geo,
                              boundary=wave, precision=precision)


@pytest.mark.parametrize("P,E,roots", [(2, 2, (2, 2)), (3, 2, (2, 2))])
@pytest.mark.parametrize("truncate", [True, False])
def test_ball_parity_f64(native, P, E, roots, truncate):
    import torch
    import twoldg
    forest, geo, wave, tables, o = ball_setup(P, E, roots, truncate)
    p = problem(forest, P, wave, truncate)
    f = lambda x, v: np.sin(0.4 * x[0] + v) * np.cos(0.3 * x[1] - 0.2 * x[2]) + 0.1 * x[2] * v
    u = ball_state(forest, tables, f)
    ud = torch.from_numpy(u).cuda()
    du = p.statevector()
    twoldg.wave_rhs(du, ud, p, 0.25)
    assert rel(du.cpu().numpy(), o.rhs(u, 0.25)) < 1e-12
    if truncate:
        w = ud.clone()
        twoldg.truncate_state(w, p)
        assert rel(w.cpu().numpy(), o.truncate(u)) < 1e-12
    u0 = o.truncate(u) if truncate else u
    dt = 0.5 * tables["hspeed"] / (P + 1)
    integ = twoldg.wave_integrator(p, torch.from_numpy(u0).cuda(), 0.1, 0.1 + 4 * dt, dt)
    integ.nsteps = 4
    integ.solve()
    ref = o.rk4(u0, dt, 4, 0.1)
    assert rel(integ.u.cpu().numpy(), ref) < 1e-12
    t1 = 0.1 + 4 * dt
    assert twoldg.wave_energy(p, integ.u, t=t1) == pytest.approx(o.energy(ref, t1), rel=1e-12)
    r = torch.from_numpy(ball_state(forest, tables, lambda x, v: wave.state(x, t1, v))).cuda()
    assert twoldg.quadrature_norm(p, integ.u, 2, ref=r) == pytest.approx(o.norm(ref, 2, 3, r.cpu().numpy()),
                                                                          rel=1e-12)


def test_ball_steps_past_one_graph(native):
    # 19 steps in one call: a graph of 16 steps and one of 3, the problem's
    # time advanced on the device after each step inside the graph, the
    # passes chained as programmatic dependent launches; against the oracle
    import torch
    import twoldg
    P, E, roots = 3, 2, (2, 2)
    forest, geo, wave, tables, o = ball_setup(P, E, roots, True)
    p = problem(forest, P, wave, True)
    f = lambda x, v: np.sin(0.4 * x[0] + v) * np.cos(0.3 * x[1] - 0.2 * x[2]) + 0.1 * x[2] * v
    u0 = o.truncate(ball_state(forest, tables, f))
    dt = 0.5 * tables["hspeed"] / (P + 1)
    integ = twoldg.wave_integrator(p, torch.from_numpy(u0).cuda(), 0.1, 0.1 + 19 * dt, dt)
    integ.nsteps = 19
    integ.solve()
    assert rel(integ.u.cpu().numpy(), o.rk4(u0, dt, 19, 0.1)) < 1e-12


def test_sevenpatch_errors_match_published(native):
    # reference CODE.md:4247-4252, P = 3, truncated, roots (2, 2): u 8.83e-3, v 1.14e-2
    import twoldg
    r = twoldg.sevenpatch_errors(np.float64, P=3, E=2, roots=(2, 2))
    assert r["nblocks"] == 56
    assert r["l2u"] == pytest.approx(8.83e-3, rel=0.01)
    assert r["l2v"] == pytest.approx(1.14e-2, rel=0.01)
    assert 1 - r["energy"] / r["energy0"] == pytest.approx(0.035, abs=0.0015)
    r32 = twoldg.sevenpatch_errors(np.float32, P=3, E=2, roots=(2, 2), precision="f32c")
    assert r32["l2"] == pytest.approx(r["l2"], rel=1e-3)


# reference CODE.md:4247-4252, the ball's larger runs (the oracle's tests
# leave them out for time): s = 2 (448 blocks, roots (4, 4)) for P = 2, 3
# with and without truncation, and s = 3 (1512 blocks) for P = 3 truncated;
# u and v errors, and the energy carried out, 1 - E1/E0, to the printed digits
PUBLISHED_S23 = [
    # (P, truncate, s, u error, v error, dE)
    (2, True, 2, 1.63e-2, 2.25e-2, 0.030),
    (2, False, 2, 3.87e-3, 1.45e-2, 0.035),
    (3, True, 2, 1.15e-3, 1.38e-3, 0.036),
    (3, False, 2, 2.38e-4, 9.03e-4, 0.036),
    (3, True, 3, 3.36e-4, 3.84e-4, 0.036),
]


@pytest.mark.parametrize("P,truncate,s,eu,ev,de", PUBLISHED_S23,
                         ids=["P%d%s-s%d" % (c[0], "-trunc" if c[1] else "", c[2]) for c in PUBLISHED_S23])
def test_sevenpatch_errors_published_larger_runs(native, P, truncate, s, eu, ev, de):
    import twoldg
    r = twoldg.sevenpatch_errors(np.float64, P=P, E=2, roots=(2 * s, 2 * s), truncate=truncate)
    assert r["nblocks"] == {2: 448, 3: 1512}[s]
    # printed to three digits: hold each to half a unit of its last digit
    assert abs(r["l2u"] - eu) <= 0.5 * 10 ** (math.floor(math.log10(eu)) - 2)
    assert abs(r["l2v"] - ev) <= 0.5 * 10 ** (math.floor(math.log10(ev)) - 2)
    assert abs((1 - r["energy"] / r["energy0"]) - de) <= 0.0005


@pytest.mark.parametrize("truncate", [True, False])
def test_dirichlet_data_of_any_form_parity_f64(native, truncate):
    """Dirichlet data of any form (boundary kind 2): the spherical standing
    wave j0(k r) cos(k t), evaluated by the caller at every stage time into the
    library's table, against the oracle, which evaluates the formula itself:
    the right-hand side, four RK4 steps and the energy to 1e-12."""
    import torch
    import twoldg
    from twoldg.ball import SphericalStandingWave, ball_forest, ball_tables
    from oracle.oracle import BallOracle
    w = SphericalStandingWave(2.0)
    forest, geo = ball_forest(np.float64, 3, 2, (2, 2), 1.0, 3.0)
    tables = ball_tables(forest, 3, w)
    o = BallOracle(forest, 3, tables, None, truncate=truncate, standing=2.0)
    p = problem(forest, 3, w, truncate)
    f = lambda x, v: np.sin(0.4 * x[0] + v) * np.cos(0.3 * x[1] - 0.2 * x[2]) + 0.1 * x[2] * v
    u = ball_state(forest, tables, f)
    du = p.statevector()
    twoldg.wave_rhs(du, torch.from_numpy(u).cuda(), p, 0.3)
    assert rel(du.cpu().numpy(), o.rhs(u, 0.3)) < 1e-12
    u0 = o.truncate(u) if truncate else u
    dt = 0.5 * tables["hspeed"] / 4
    integ = twoldg.wave_integrator(p, torch.from_numpy(u0).cuda(), 0.1, 0.1 + 4 * dt, dt)
    integ.nsteps = 4
    integ.solve()
    ref = o.rk4(u0, dt, 4, 0.1)
    assert rel(integ.u.cpu().numpy(), ref) < 1e-12
    t1 = 0.1 + 4 * dt
    assert twoldg.wave_energy(p, integ.u, t=t1) == pytest.approx(o.energy(ref, t1), rel=1e-12)


def test_dirichlet_data_of_any_form_refusals(native):
    """A call whose stage times the caller's table does not hold is refused
    before any work: no table yet, a time between levels, a step size other
    than the table's, a run past its last level."""
    import ctypes
    import torch
    import twoldg
    from twoldg import _lib
    from twoldg.ball import SphericalStandingWave, ball_forest
    w = SphericalStandingWave(2.0)
    forest, geo = ball_forest(np.float64, 2, 2, (2, 2), 1.0, 3.0)
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, 2), geometry=geo, boundary=w)
    L = _lib.lib()
    u = p.statevector()
    du = p.statevector()
    up, dup = ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(du.data_ptr())
    assert L.twoldg_rhs(p.handle, dup, up, 0.0) == _lib.TWOLDG_EINVAL
    assert b"twoldg_set_boundary_values" in L.twoldg_last_error()
    n = ctypes.c_int32()
    _lib.check(L.twoldg_boundary_faces(p.handle, None, ctypes.byref(n)))
    assert n.value == 6 * 4                  # the six shells' outer faces at roots (2, 2)
    dt = 0.01
    p.boundary_window(0.0, dt, 5)            # levels t = 0, dt/2, ..., 2 dt
    _lib.check(L.twoldg_rhs(p.handle, dup, up, 0.015))
    assert L.twoldg_rhs(p.handle, dup, up, 0.012) == _lib.TWOLDG_EINVAL
    _lib.check(L.twoldg_rk4_step(p.handle, up, 0.0, dt, 2))
    assert L.twoldg_rk4_step(p.handle, up, 0.0, dt, 3) == _lib.TWOLDG_EINVAL
    assert L.twoldg_rk4_step(p.handle, up, 0.0, 0.5 * dt, 1) == _lib.TWOLDG_EINVAL
    assert L.twoldg_rk4_step(p.handle, up, 0.01, dt, 1) == _lib.TWOLDG_OK
    p.synchronize()
    torch.cuda.synchronize()


# --- the refined cube (src/geometry.jl:494-553): coarse-fine faces under the full metric ---

@pytest.mark.parametrize("P,truncate,Rm,radiative", [(2, True, None, None), (3, False, None, None),
                                                     (3, True, None, None), (3, True, 2.0, (1.0, True))],
                         ids=["P2-trunc", "P3", "P3-trunc", "P3-thirteen-radiative"])
def test_refined_ball_parity_f64(native, P, truncate, Rm, radiative):
    """The ball with its cube refined (the middle half to level 1) through the
    library against the oracle: right-hand side, truncation, four RK4 steps,
    energy and norm to 1e-12; the seven-patch ball with the plane wave, and
    the thirteen-patch one (roots (4, 1, 1)) under Sommerfeld's condition."""
    import torch
    import twoldg
    from twoldg.ball import RadiativeBoundary
    roots = (4, 1) if Rm is None else (4, 1, 1)
    forest, geo, wave, tables, o = ball_setup(P, 2, roots, truncate, Rm=Rm, radiative=radiative, refined=True)
    assert max(forest.levels) == 1
    bnd = wave if radiative is None else RadiativeBoundary(*radiative)
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, P), truncate=truncate, geometry=forest.geo,
                           boundary=bnd)
    f = lambda x, v: np.sin(0.4 * x[0] + v) * np.cos(0.3 * x[1] - 0.2 * x[2]) + 0.1 * x[2] * v
    u = ball_state(forest, tables, f)
    ud = torch.from_numpy(u).cuda()
    du = p.statevector()
    twoldg.wave_rhs(du, ud, p, 0.25)
    assert rel(du.cpu().numpy(), o.rhs(u, 0.25)) < 1e-12
    if truncate:
        w = ud.clone()
        twoldg.truncate_state(w, p)
        assert rel(w.cpu().numpy(), o.truncate(u)) < 1e-12
    u0 = o.truncate(u) if truncate else u
    dt = 0.5 * tables["hspeed"] / (P + 1)
    integ = twoldg.wave_integrator(p, torch.from_numpy(u0).cuda(), 0.1, 0.1 + 4 * dt, dt)
    integ.nsteps = 4
    integ.solve()
    ref = o.rk4(u0, dt, 4, 0.1)
    assert rel(integ.u.cpu().numpy(), ref) < 1e-12
    t1 = 0.1 + 4 * dt
    assert twoldg.wave_energy(p, integ.u, t=t1) == pytest.approx(o.energy(ref, t1), rel=1e-12)
    r = torch.from_numpy(u).cuda()
    assert twoldg.quadrature_norm(p, integ.u, 2, ref=r) == pytest.approx(o.norm(ref, 2, 3, u), rel=1e-12)


def test_refined_ball_plane_wave_accuracy(native):
    # test/sevenpatch_tests.jl:499-535 through the library: refining the cube
    # does not raise the plane wave's error, and halves the finest spacing
    import twoldg
    for P in (2, 3):
        r0 = twoldg.sevenpatch_errors(np.float64, P=P, E=2, roots=(4, 1), tend=0.25)
        r1 = twoldg.sevenpatch_errors(np.float64, P=P, E=2, roots=(4, 1), tend=0.25, refined=True)
        assert r1["nblocks"] > r0["nblocks"]
        assert r1["l2"] <= 1.01 * r0["l2"]
        assert r1["h"] == r0["h"] / 2
    r32 = twoldg.sevenpatch_errors(np.float32, P=3, E=2, roots=(4, 1), tend=0.25, refined=True, precision="f32c")
    assert r32["l2"] == pytest.approx(r1["l2"], rel=1e-3)
