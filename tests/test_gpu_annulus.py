"""The annulus (diagonal metric) through libtwoldg against the oracle, and
annulus_errors against the reference's published table. Marked gpu."""
import math

import numpy as np
import pytest

from annulus_cases import annulus_oracle, state_of
from cases import scrambled

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a, dtype=np.float64) - b).max() / np.abs(b).max())


def smooth(x, var):
    return np.sin(0.7 * x[0] + var) * np.cos(1.3 * x[1]) + 0.2 * x[1] * var


@pytest.mark.parametrize("P,E,roots", [(3, 2, (2, 1)), (2, 4, (1, 2)), (4, 2, (2, 2))])
@pytest.mark.parametrize("truncate", [True, False])
def test_annulus_parity_f64(native, P, E, roots, truncate):
    import torch
    import twoldg
    forest, geo, o, hspeed = annulus_oracle(P, E, roots, truncate)
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, P), truncate=truncate, geometry=geo)
    u = state_of(forest, P, smooth)
    ud = torch.from_numpy(u).cuda()
    du = p.statevector()
    twoldg.wave_rhs(du, ud, p)
    assert rel(du.cpu().numpy(), o.rhs(u)) < 1e-12
    if truncate:
        w = ud.clone()
        twoldg.truncate_state(w, p)
        assert rel(w.cpu().numpy(), o.truncate(u)) < 1e-12
    u0 = o.truncate(u) if truncate else u
    dt = 0.5 * hspeed / (P + 1)
    integ = twoldg.wave_integrator(p, torch.from_numpy(u0).cuda(), 0.0, 5 * dt, dt)
    integ.solve()
    ref = o.rk4(u0, dt, 5)
    assert rel(integ.u.cpu().numpy(), ref) < 1e-12
    assert twoldg.wave_energy(p, integ.u) == pytest.approx(o.energy(ref), rel=1e-12)
    r = torch.from_numpy(state_of(forest, P, lambda x, v: np.cos(x[0]) * v)).cuda()
    for pn, po in ((2, 2), (math.inf, 0)):
        assert twoldg.quadrature_norm(p, integ.u, pn, ref=r) == pytest.approx(
            o.norm(ref, po, 3, r.cpu().numpy()), rel=1e-12)


def test_annulus_errors_match_published(native):
    # reference CODE.md:4177-4199, P = 3, truncated, s = 1: u 5.06e-3, v 3.35e-3
    import twoldg
    r = twoldg.annulus_errors(np.float64, P=3, E=2, roots=(2, 1), m=2, n=1)
    assert r["k"] == pytest.approx(1.3406, abs=1e-4)
    assert r["l2u"] == pytest.approx(5.06e-3, rel=0.01)
    assert r["l2v"] == pytest.approx(3.35e-3, rel=0.01)
    assert r["energy"] <= r["energy0"]
    r32 = twoldg.annulus_errors(np.float32, P=3, E=2, roots=(2, 1), m=2, n=1, precision="f32c")
    assert r32["l2"] == pytest.approx(r["l2"], rel=1e-3)


def test_annulus_energy_rate_is_zero(native):
    # the metric operator is skew in the sqrt(g)-weighted product: dE/dt = 0
    import torch
    import twoldg
    forest, geo, o, _ = annulus_oracle(3, 2, (2, 1), truncate=False)
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, 3), truncate=False, geometry=geo)
    n = len(forest.leaves) * forest.N ** 2
    u = np.stack([scrambled(n, 0.2).reshape(len(forest.leaves), -1),
                  scrambled(n, 0.6).reshape(len(forest.leaves), -1)], axis=1).reshape(-1)
    ud = torch.from_numpy(u).cuda()
    du = p.statevector()
    twoldg.wave_rhs(du, ud, p)
    eps = 1e-6
    rate = (twoldg.wave_energy(p, ud + eps * du) - twoldg.wave_energy(p, ud - eps * du)) / (2 * eps)
    scale = twoldg.wave_energy(p, ud) * float(np.abs(du.cpu().numpy()).max())
    assert abs(rate) < 1e-8 * scale
