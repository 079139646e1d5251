"""Waveform extraction through libtwoldg (twoldg_gather) against the host's
reading of the same stencils and the oracle's element polynomials, on a
brick and on the seven-patch ball, with the modes' error bounded by the
values'. Marked gpu."""
import math

import numpy as np
import pytest

from ball_cases import ball_state
from cases import state_from
from oracle.oracle import oracle_point_values
from test_extraction import extraction_f, fill, gather

pytestmark = pytest.mark.gpu


def test_brick_sphere_values_and_modes(native):
    import torch
    import twoldg
    from twoldg.extraction import SphereExtraction, harmonic_modes, sphere_modes, sphere_values
    P = 3
    f = twoldg.wave_forest(np.float64, 3, P, 2, roots=4, L=4.0)
    p = twoldg.WaveProblem(f, twoldg.Element(np.float64, P))
    u = state_from(f, P, fill)
    ud = torch.from_numpy(u).cuda()
    ex = SphereExtraction(p, [0.5, 1.5], lmax=3, centre=(2.0, 2.0, 2.0))
    assert len(ex.points) == 2 * 2 * ex.ntheta ** 2
    idx = ex.index.cpu().numpy().reshape(ex.npoints, ex.nper)
    w = ex.weights.cpu().numpy().reshape(ex.npoints, ex.nper)
    for var in (1, 2):
        got = sphere_values(ex, p, ud, var)
        host = gather(idx, w, u, var, f.N ** 3)
        assert np.abs(got - host).max() < 1e-14 * np.abs(host).max()
    ref = oracle_point_values(f, P, u, ex.points[:200], var=1)
    assert np.abs(sphere_values(ex, p, ud)[:200] - ref).max() < 1e-13 * np.abs(ref).max()
    exact = extraction_f(ex.points.T)
    err = np.abs(sphere_values(ex, p, ud) - exact).max()
    m = sphere_modes(ex, p, ud) - sphere_modes(ex, exact)
    assert m.shape == (len(harmonic_modes(3)), 2)
    assert np.abs(m).max() <= math.sqrt(4 * math.pi) * err


@pytest.mark.parametrize("precision,refined", [("f64", False), ("f32c", False), ("f64", True)])
def test_ball_sphere_and_plane(native, precision, refined):
    import torch
    import twoldg
    from twoldg.ball import ball_tables
    from twoldg.extraction import PlaneExtraction, SphereExtraction, plane_values, sphere_modes, sphere_values
    P = 3
    T = np.float64 if precision == "f64" else np.float32
    # refined: the cube's (1, 3)^3 one level finer (test/extraction_tests.jl:95-200)
    f, geo = twoldg.sevenpatch_forest(T, P, 2, roots=(4, 2), refined=((1.0, 3.0),) * 3 if refined else False)
    p = twoldg.WaveProblem(f, twoldg.Element(T, P), geometry=geo, boundary=twoldg.RadiativeBoundary(),
                           precision=precision)
    u = ball_state(f, ball_tables(f, P), fill)
    ud = torch.from_numpy(u.astype(T)).cuda()
    ex = SphereExtraction(p, [0.3, 0.7, 1.3, 2.2], lmax=4)
    idx = ex.index.cpu().numpy().reshape(ex.npoints, ex.nper)
    w = ex.weights.cpu().numpy().astype(np.float64).reshape(ex.npoints, ex.nper)
    tol = 1e-14 if precision == "f64" else 2e-6
    for var in (1, 2):
        got = sphere_values(ex, p, ud, var)
        host = gather(idx, w, u.astype(T).astype(np.float64), var, f.N ** 3)
        assert np.abs(got - host).max() < tol * np.abs(host).max()
    modes = sphere_modes(ex, p, ud)
    assert modes.shape == (15, 4)
    exact = extraction_f(ex.points.T)
    assert np.abs(modes - sphere_modes(ex, exact)).max() <= math.sqrt(4 * math.pi) * \
        np.abs(sphere_values(ex, p, ud) - exact).max() + 1e-6
    pl = PlaneExtraction(p, (0.1, -0.2, 0.3), 2.9, 24)
    vals = plane_values(pl, p, ud)
    assert vals.shape == (24, 24)
    assert np.array_equal(np.isnan(vals.T.reshape(-1)), ~pl.inside)
    assert 0 < pl.inside.sum() < 24 * 24
    inside = pl.points[pl.inside]
    assert np.abs(vals.T.reshape(-1)[pl.inside] - extraction_f(inside.T)).max() < 1e-2
