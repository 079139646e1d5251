"""The refined and batched configurations at their full sizes (GPU).

* The 3D reflecting box with three nested refinement levels (nested cubes of
  half-width 1/8, 1/4 and the box, P = 3, E = 2, roots = 8: 1408 blocks,
  720,896 nodes), Gaussian pulse u = exp(-r^2/0.05^2) at the centre: FP64 parity
  with the oracle over a few steps, the FP64 energy invariant over 100 steps
  (RK4's loss only), and the float32 paths against the FP64 run.
"""
import math

import numpy as np
import pytest

from cases import state_from
from oracle.oracle import Oracle
from twoldg.forest import nested_cubes, wave_forest

pytestmark = pytest.mark.gpu


def gaussian(x, var):
    r2 = sum((x[d] - 0.5) ** 2 for d in range(3))
    return np.exp(-r2 / 0.05 ** 2) if var == 1 else np.zeros_like(x[0])


def nested_box(dtype):
    return wave_forest(dtype, 3, 3, 2, roots=8, reflecting=True, refined=nested_cubes(3, 1 / 8, 3))



def test_nested_box_fp64_parity_with_oracle(native):
    import torch
    import twoldg
    forest = nested_box(np.float64)
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, 3))
    o = Oracle(forest, 3)
    u0 = o.truncate(state_from(forest, 3, gaussian))
    dt = 0.5 * forest.minimum_spacing() / 4
    integ = twoldg.wave_integrator(p, torch.from_numpy(u0).cuda(), 0.0, 3 * dt, dt)
    integ.solve()
    ref = o.rk4(u0, dt, 3)
    got = integ.u.cpu().numpy()
    assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max()
    assert twoldg.wave_energy(p, integ.u) == pytest.approx(o.energy(ref), rel=1e-12)


def test_nested_box_energy_invariant_and_float32(native):
    import twoldg
    runs = {}
    for prec, dtype in (("f64", np.float64), ("f32c", np.float32), ("f32", np.float32)):
        forest = nested_box(dtype)
        p = twoldg.WaveProblem(forest, twoldg.Element(dtype, 3), precision=prec)
        u0 = twoldg.initial_state(p, lambda x, var: gaussian(x, var).astype(dtype))
        dt = 0.5 * forest.minimum_spacing() / 4
        e0 = twoldg.wave_energy(p, u0)
        integ = twoldg.wave_integrator(p, u0, 0.0, 100 * dt, dt)
        integ.solve()
        runs[prec] = (p, integ.u, e0, twoldg.wave_energy(p, integ.u))
    p64, u64, e0, e1 = runs["f64"]
    # the semi-discrete energy is exact across the coarse-fine faces and the walls;
    # what a run loses is RK4's, (omega dt)^6-small for the pulse's wavenumbers
    assert e1 <= e0
    assert (e0 - e1) / e0 < 1e-9
    for prec in ("f32c", "f32"):
        p, u, f0, f1 = runs[prec]
        assert abs(f1 - e1) / e1 < 1e-5
        diff = twoldg.quadrature_norm(p64, u64, 2, ref=u.to(u64.dtype))
        scale = twoldg.quadrature_norm(p64, u64, 2)
        assert diff < 1e-5 * scale, prec
