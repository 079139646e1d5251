"""Parity at the benchmark sizes: the FP64 CUDA path against the oracle on
the very forests the benchmark times, not only on small ones of the same
block shape.

- the 256^3 periodic box (P = 3, E = 4, roots = 16: 4096 blocks of 16^3,
  16.8M nodes): one right-hand side and two RK4 steps at 1e-12, and the
  FP32 + compensated path's two steps against the oracle's FP64 run;
- the seven-patch ball at roots (4, 4) (P = 3, E = 2: 448 blocks, 229,376
  nodes) with the plane wave of |k| = 2 pi along (1.1, -0.7, 0.5) as its
  Dirichlet data: one right-hand side and one RK4 step at 1e-12;
- the 512-member 2D ensemble (P in 2..5, E in {2, 4}, roots in 4..16,
  12.9M nodes) stepped as one batch: three RK4 steps, every member against
  the oracle at 1e-12.

The oracle is the plain-C restatement, OpenMP over blocks; these runs take it
seconds to a minute. Marked gpu.
"""
import math

import numpy as np
import pytest

from cases import state_from
from oracle.oracle import Oracle
from twoldg.forest import wave_forest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a, dtype=np.float64) - b).max() / np.abs(b).max())


def box_data(x, var):
    # the benchmark's standing mode (1, 2, 3) in u, with a v of its own so
    # that both halves of the right-hand side carry data
    s = np.sin(2 * math.pi * x[0]) * np.sin(4 * math.pi * x[1]) * np.sin(6 * math.pi * x[2])
    if var == 1:
        return s
    return 0.5 * np.cos(2 * math.pi * (x[0] + x[2])) * np.sin(2 * math.pi * x[1]) + 0.1 * s


@pytest.fixture(scope="module")
def box():
    forest = wave_forest(np.float64, 3, 3, 4, roots=16)
    o = Oracle(forest, 3)
    u0 = o.truncate(state_from(forest, 3, box_data))
    return forest, o, u0


def test_box256_rhs_and_rk4_f64(native, box):
    import torch
    import twoldg
    forest, o, u0 = box
    assert len(forest.leaves) == 4096 and forest.N == 16
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, 3))
    ud = torch.from_numpy(u0).cuda()
    du = p.statevector()
    twoldg.wave_rhs(du, ud, p, 0.0)
    assert rel(du.cpu().numpy(), o.rhs(u0)) < 1e-12
    dt = 0.5 * forest.minimum_spacing() / 4
    integ = twoldg.wave_integrator(p, ud.clone(), 0.0, 2 * dt, dt)
    integ.solve()
    assert integ.nsteps == 2
    ref = o.rk4(u0, dt, 2)
    assert rel(integ.u.cpu().numpy(), ref) < 1e-12
    assert twoldg.wave_energy(p, integ.u) == pytest.approx(o.energy(ref), rel=1e-12)
    del p


def test_box256_f32c_against_the_oracle(native, box):
    """The benchmark's headline precision on its own forest: FP32 fields with
    the compensated accumulation, two steps, against the oracle's FP64 run.
    The bar is the FP32 right-hand side's, 2e-4 of the state's largest value:
    the Laplacian's 1/h^2 amplifies the fields' rounding, so at h = 1/256 a
    stage's v rate carries some 1e-4 of relative rounding where the small
    boxes' carry 64 times less (measured 6.6e-5 here)."""
    import torch
    import twoldg
    forest, o, u0 = box
    f32 = wave_forest(np.float32, 3, 3, 4, roots=16)
    p = twoldg.WaveProblem(f32, twoldg.Element(np.float32, 3), precision="f32c")
    dt = 0.5 * forest.minimum_spacing() / 4
    u = torch.from_numpy(u0.astype(np.float32)).cuda()
    integ = twoldg.wave_integrator(p, u, 0.0, 2 * dt, dt)
    integ.solve()
    ref = o.rk4(u0, dt, 2)
    assert rel(integ.u.cpu().numpy(), ref) < 2e-4
    del p


def test_sevenpatch_roots44_f64(native):
    import torch
    import twoldg
    from ball_cases import ball_setup, ball_state
    kdir = np.array([1.1, -0.7, 0.5])
    k = tuple(2 * math.pi * kdir / np.linalg.norm(kdir))
    forest, geo, wave, tables, o = ball_setup(3, 2, (4, 4), True, k=k, phi=0.3)
    assert forest.nleaves() == 448
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, 3), truncate=True, geometry=forest.geo,
                           boundary=wave)
    u0 = o.truncate(ball_state(forest, tables, lambda x, v: wave.state(x, 0.0, v)))
    ud = torch.from_numpy(u0).cuda()
    du = p.statevector()
    twoldg.wave_rhs(du, ud, p, 0.0)
    assert rel(du.cpu().numpy(), o.rhs(u0, 0.0)) < 1e-12
    dt = 0.5 * tables["hspeed"] / 4
    integ = twoldg.wave_integrator(p, ud.clone(), 0.0, dt, dt)
    integ.nsteps = 1
    integ.solve()
    assert rel(integ.u.cpu().numpy(), o.rk4(u0, dt, 1, 0.0)) < 1e-12


def test_ensemble512_every_member_f64(native):
    import torch  # noqa: F401
    import twoldg
    members = twoldg.sine_ensemble(512, seed=0, dtype=np.float64)
    roots = [len(f.leaves) for f, _, _ in members]
    assert min(roots) >= 16 and max(roots) <= 256            # roots 4..16 per dimension
    b = twoldg.Batch([(f, P) for f, P, _ in members], precision="f64")
    u0 = twoldg.fill_batch(b, members)
    dts = [0.5 * f.minimum_spacing() / (P + 1) for f, P, _ in members]
    u = u0.clone()
    b.rk4_step(u, dts, 3)
    b.synchronize()
    got, start = u.cpu().numpy(), u0.cpu().numpy()
    worst = 0.0
    for k, (forest, P, _) in enumerate(members):
        n = 2 * forest.N ** 2 * len(forest.leaves)
        a = b.offsets[k]
        ref = Oracle(forest, P).rk4(start[a:a + n], dts[k], 3)
        worst = max(worst, rel(got[a:a + n], ref))
    assert worst < 1e-12
