"""The seven-patch ball through libtwoldg (full metric, quarter-turn glue,
Dirichlet plane wave) against the oracle, and sevenpatch_errors against the
reference's published table. Marked gpu."""
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
