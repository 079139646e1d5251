"""The blast wave on the oracle: the exact solution by the inverse Hankel
transform and the uniform run against the reference's published errors,
and the adaptive driver's argument checks. No GPU."""
import math

import numpy as np
import pytest

from cases import state_from
from oracle.oracle import Oracle
from twoldg.blast import adaptive_blast, blast_exact, blast_initial, blast_reference, refinement_buffer
from twoldg.forest import wave_forest


def oracle_uniform_blast(P, E, roots, t_end, sigma=0.08, cfl=0.5):
    f = wave_forest(np.float64, 2, P, E, roots=roots)
    o = Oracle(f, P)
    u0 = o.truncate(state_from(f, P, blast_initial(1.0, (0.5, 0.5), sigma)))
    nsteps = int(math.ceil(t_end / (cfl * f.minimum_spacing() / (P + 1))))
    u = o.rk4(u0, t_end / nsteps, nsteps)
    ref = blast_reference(1.0, (0.5, 0.5), sigma, rmax=t_end + 6 * sigma)
    ue = state_from(f, P, blast_exact(ref, t_end))
    return o.norm(u, 0, 3, ue), nsteps


def oracle_uniform_run(P, E, roots, t_end=0.4, sigma=0.08, cfl=0.5):
    """uniform_blast (src/blast.jl:153-186) on the oracle: the errors of u and
    v together (L-infinity and L2) at t_end and the energies."""
    f = wave_forest(np.float64, 2, P, E, roots=roots)
    o = Oracle(f, P)
    u0 = o.truncate(state_from(f, P, blast_initial(1.0, (0.5, 0.5), sigma)))
    nsteps = int(math.ceil(t_end / (cfl * f.minimum_spacing() / (P + 1))))
    u = o.rk4(u0, t_end / nsteps, nsteps)
    ue = state_from(f, P, blast_exact(blast_reference(1.0, (0.5, 0.5), sigma, rmax=t_end + 6 * sigma), t_end))
    return dict(err=o.norm(u, 0, 3, ue), l2=o.norm(u, 2, 3, ue), energy0=o.energy(u0), energy=o.energy(u))


def _printed(value, printed):
    """value rounds to the three significant digits printed."""
    e = math.floor(math.log10(abs(printed)))
    return abs(value - printed) <= 0.5001 * 10.0 ** (e - 2)


@pytest.mark.parametrize("P,roots,t,linf", [(3, 16, 0.2, 5.59e-2), (3, 16, 0.4, 2.06e-2), (4, 16, 0.2, 5.43e-3),
                                             (3, 32, 0.2, 3.99e-3)])
def test_uniform_blast_published_errors(P, roots, t, linf):
    # reference CODE.md:4935-4937: the uniform runs at the adaptive runs' cap
    # (sigma = 0.08, E = 2, truncated, cfl 1/2): L-infinity of u and v
    # together, every printed digit
    err, _ = oracle_uniform_blast(P, 2, roots, t)
    assert _printed(err, linf), err


def test_blast_exact_is_the_initial_data_at_t0_and_periodic():
    # the Hankel transform of the Gaussian reproduces it at t = 0 (to its
    # midpoint rule's 1e-6), with v = 0, and the images make it periodic
    ref = blast_reference(1.0, (0.5, 0.5), 0.08, rmax=0.2 + 6 * 0.08)
    x = (np.linspace(0.0, 1.0, 57), np.linspace(0.1, 0.9, 57))
    u0 = blast_exact(ref, 0.0)
    assert np.abs(u0(x, 1) - blast_initial(1.0, (0.5, 0.5), 0.08)(x, 1)).max() < 1e-5
    assert np.abs(u0(x, 2)).max() < 1e-12
    ut = blast_exact(ref, 0.2)
    xa = (np.array([0.05, 0.3]), np.array([0.2, 0.7]))
    xb = (xa[0] + 1.0, xa[1] - 1.0)
    assert np.allclose(ut(xa, 1), ut(xb, 1), atol=1e-12)


def test_adaptive_blast_refuses_what_it_cannot_do():
    with pytest.raises(ValueError, match="dead band"):
        adaptive_blast(P=3, refine_tol=1e-3, coarsen_tol=1e-3)
    with pytest.raises(ValueError, match="positive"):
        adaptive_blast(P=3, chunk=0.0)
    with pytest.raises(ValueError, match="P = 1"):
        adaptive_blast(P=1, E=2, roots=4, maxlevel_cap=1, refine_tol=0.01, coarsen_tol=0.001, chunk=0.05)
    f = wave_forest(np.float64, 2, 3, 2, roots=4)
    assert refinement_buffer(f, 2, 0.05) == 8
    with pytest.raises(ValueError, match="regrid more often"):
        refinement_buffer(f, 2, 0.1)


def test_blast_converges_and_keeps_its_energy():
    # test/blast_tests.jl:24-35: from 8 to 16 blocks per dimension at P = 3 the
    # L2 error falls by more than 2^3, the finer run's largest error is below
    # 0.05, and the energy lost is RK4's, small
    coarse, fine = oracle_uniform_run(3, 2, 8), oracle_uniform_run(3, 2, 16)
    assert coarse["l2"] / fine["l2"] > 2 ** 3
    assert fine["err"] < 0.05
    for r in (coarse, fine):
        assert 0 <= (r["energy0"] - r["energy"]) / r["energy0"] < 1e-6
