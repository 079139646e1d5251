"""Parity of libtwoldg (CUDA, through the C ABI) with the CPU oracle, on the
same seeded inputs: FP64 to 1e-12 relative (the parity bar), float32
paths within stated tolerances. Marked gpu."""
import math

import numpy as np
import pytest

from cases import refined_forest, scrambled, smooth_data, state_from
from oracle.oracle import Oracle
from twoldg.forest import nested_cubes, wave_forest

pytestmark = pytest.mark.gpu

CASES = [
    # (D, P, E, roots, reflecting, refined)
    (1, 3, 2, 3, False, False),
    (1, 5, 4, 2, True, False),
    (2, 2, 2, 3, False, False),
    (2, 4, 2, 8, False, False),     # the 2D periodic P=4, E=2, roots=8 box (80x80 nodes)
    (2, 3, 4, 2, True, False),
    (3, 1, 2, 3, False, False),
    (3, 3, 4, 2, False, False),     # 3D P=3, E=4: the 16^3 blocks of the 256^3 box
    (3, 2, 2, 2, True, False),
    (2, 3, 2, 4, False, True),      # coarse-fine faces
    (2, 2, 2, 4, True, (( 0.0, 0.5), (0.0, 0.5))),
    (3, 2, 2, 3, False, True),
    (3, 3, 2, 2, True, ((0.0, 0.5), (0.0, 0.5), (0.0, 0.5))),
    (1, 3, 2, 4, False, True),
    (2, 2, 6, 2, False, False),     # E = 6: the run-time-shape kernel
    (3, 1, 6, 1, True, False),
    # orders above 6: the run-time-shape kernel (Element(T, P) is any P >= 1,
    # src/element.jl:129-170; the library builds P <= 8)
    (1, 7, 2, 3, False, False),
    (1, 8, 4, 2, True, False),
    (2, 7, 2, 2, False, False),
    (2, 8, 2, 2, True, False),
    (2, 7, 2, 4, False, True),
    (3, 7, 2, 1, False, False),
    (3, 8, 2, 1, True, False),
]


def ids(c):
    D, P, E, roots, refl, ref = c
    return "D%dP%dE%dr%d%s%s" % (D, P, E, roots, "-wall" if refl else "", "-refined" if ref else "")


def build(case, dtype=np.float64, precision=None, truncate=True, data=None):
    import twoldg
    D, P, E, roots, refl, ref = case
    forest = wave_forest(dtype, D, P, E, roots=roots, reflecting=refl, refined=ref)
    p = twoldg.WaveProblem(forest, twoldg.Element(dtype, P), truncate=truncate, precision=precision)
    o = Oracle(forest, P, truncate=truncate)
    u = state_from(forest, P, data or smooth_data(D))
    return forest, p, o, u


def dev(p, u):
    import torch
    return torch.from_numpy(np.ascontiguousarray(u).astype(p.dtype)).cuda()


def rel(a, b):
    return float(np.abs(np.asarray(a, dtype=np.float64) - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("case", CASES, ids=ids)
def test_rhs_parity_f64(native, case):
    forest, p, o, u = build(case)
    ud = dev(p, u)
    du = p.statevector()
    native.wave_rhs(du, ud, p, 0.0)
    ref = o.rhs(u)
    got = du.cpu().numpy()
    assert rel(got, ref) < 1e-12
    # the RHS never writes u
    assert np.array_equal(ud.cpu().numpy(), u)


@pytest.mark.parametrize("case", CASES[:8], ids=ids)
def test_truncate_parity_f64(native, case):
    forest, p, o, u = build(case)
    ud = dev(p, u)
    native.truncate_state(ud, p)
    ref = o.truncate(u)
    assert rel(ud.cpu().numpy(), ref) < 1e-13
    # idempotent, and u itself untouched
    again = ud.clone()
    native.truncate_state(again, p)
    assert rel(again.cpu().numpy(), ref) < 1e-14
    NN = forest.N ** forest.D
    assert np.array_equal(ud.cpu().numpy().reshape(-1, 2, NN)[:, 0], u.reshape(-1, 2, NN)[:, 0])


@pytest.mark.parametrize("case", CASES, ids=ids)
@pytest.mark.parametrize("truncate", [True, False])
def test_rk4_parity_f64(native, case, truncate):
    forest, p, o, u = build(case, truncate=truncate)
    u0 = o.truncate(u) if truncate else u
    dt = 0.5 * forest.minimum_spacing() / (case[1] + 1)
    ud = dev(p, u0)
    integ = native.wave_integrator(p, ud, 0.0, 5 * dt, dt)
    integ.solve()
    ref = o.rk4(u0, dt, 5)
    assert integ.nsteps == 5
    assert rel(integ.u.cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize("case", CASES, ids=ids)
def test_energy_and_norm_parity_f64(native, case):
    forest, p, o, u = build(case)
    ud = dev(p, u)
    e = native.wave_energy(p, ud)
    assert e == pytest.approx(o.energy(u), rel=1e-12)
    ref = state_from(forest, case[1], lambda x, v: 0.3 * np.cos(x[0]) * v)
    rd = dev(p, ref)
    for pn, po in ((2, 2), (1, 1), (3, 3), (math.inf, 0)):
        for vars, mask in (((1, 2), 3), ((1,), 1), ((2,), 2)):
            got = native.quadrature_norm(p, ud, pn, vars, ref=rd)
            assert got == pytest.approx(o.norm(u, po, mask, ref), rel=1e-12)


@pytest.mark.parametrize("case", [c for c in CASES if c[1] >= 2], ids=ids)
def test_modal_indicator_parity(native, case):
    forest, p, o, u = build(case)
    ud = dev(p, u)
    P = case[1]
    # A mode coefficient c = sum_j dual_j a_j cancels: |c| is far below the
    # data's scale A, so its rounding error is bounded by eps * A (amplitudes
    # are in units of A), not by eps * |c|: 1e-13 absolute on |c|/A.
    for var in (1, 2):
        tau = native.modal_indicator(p, ud, P - 1, var=var).cpu().numpy().reshape(-1)
        ref = o.modal_indicator(u, P - 1, var=var)
        assert np.abs(tau - ref).max() < 1e-12 * max(ref.max(), 1e-300) + 1e-13
        amp = native.mode_amplitude(p, ud, P, var=var).cpu().numpy().reshape(-1)
        ref = o.modes(u, var - 1, [P], [1.0], [1.0], 1.0)
        assert np.abs(amp - ref).max() < 1e-13


def test_indicator_vanishes_below_its_degree(native):
    # test/adaptive_tests.jl:46-110: zero on data of degree < mode along every line
    import twoldg
    forest = wave_forest(np.float64, 2, 4, 2, roots=2)
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, 4))
    u = state_from(forest, 4, lambda x, v: 1.0 + x[0] - 2 * x[1] + x[0] * x[1] + 0 * v)
    tau = native.mode_amplitude(p, dev(p, u), 2).cpu().numpy()
    # x0*x1 is degree 1 along each line: every mode >= 2 vanishes
    assert np.abs(tau).max() < 1e-12
    z = native.modal_indicator(p, dev(p, 0 * u), 3).cpu().numpy()
    assert np.all(z == 0)


@pytest.mark.parametrize("case", [CASES[3], CASES[6], CASES[10]], ids=ids)
def test_f32_paths_against_f64_oracle(native, case):
    # Float32 fields against the FP64 oracle started from the same
    # float32-rounded state, so what differs is the float32 arithmetic: the
    # stencil sums round at about eps32 |W|_1 |u| / h per derivative, which
    # two applications amplify to ~1e-5 of |Lap u| (4e-5 measured at h = 1/80
    # when the input rounding is included), and which a run accumulates
    # linearly: 1e-4 of the state's scale over 10 steps, for the plain and
    # the compensated path alike (compensation recovers the lost low bits of
    # the state update, not the stencil's rounding).
    forest, p, o, u = build(case, dtype=np.float32, precision="f32")
    u0 = o.truncate(u).astype(np.float32).astype(np.float64)
    du = p.statevector()
    native.wave_rhs(du, dev(p, u0), p, 0.0)
    ref = o.rhs(u0)
    assert rel(du.cpu().numpy(), ref) < 2e-4
    dt = float(np.float32(0.5 * forest.minimum_spacing() / (case[1] + 1)))
    ref = o.rk4(u0, dt, 10)
    for prec in ("f32", "f32c"):
        import twoldg
        q = twoldg.WaveProblem(forest, twoldg.Element(np.float32, case[1]), precision=prec)
        integ = native.wave_integrator(q, dev(q, u0), 0.0, 10 * np.float32(dt), np.float32(dt))
        assert integ.nsteps == 10
        integ.solve()
        assert rel(integ.u.cpu().numpy(), ref) < 1e-4, prec


@pytest.mark.parametrize("case", [CASES[3], CASES[6], CASES[10]], ids=ids)
@pytest.mark.parametrize("prec", ["f64", "f32c"])
def test_steps_in_one_call_equal_steps_one_by_one(native, case, prec):
    # 19 steps in one call run one graph of 16 steps and one of 3, the stage
    # kernels chained as programmatic dependent launches across the steps;
    # one step a call runs a graph of one. The same arithmetic: bitwise equal.
    # Except in FP32 on a refined forest: there a call's first stage reads
    # coarse-fine planes that a launch forms whole from the face exports,
    # where the later stages read them as the two sides' epilogues wrote them
    # (the other side's part plus this side's), which rounds differently
    dtype = np.float64 if prec == "f64" else np.float32
    forest, p, o, u = build(case, dtype=dtype, precision=prec)
    dt = 0.5 * forest.minimum_spacing() / (case[1] + 1)
    a = native.wave_integrator(p, dev(p, o.truncate(u)), 0.0, 19 * dt, dt)
    a.nsteps = 19
    a.solve()
    b = native.wave_integrator(p, dev(p, o.truncate(u)), 0.0, 19 * dt, dt)
    for _ in range(19):
        b.step()
    if case[5] and prec != "f64":
        assert rel(a.u.cpu().numpy(), b.u.cpu().numpy().astype(np.float64)) < 1e-5
    else:
        assert np.array_equal(a.u.cpu().numpy(), b.u.cpu().numpy())


def test_wave_errors_2d_p4_against_oracle_and_published(native):
    # the 2D periodic P=4, E=2, roots=8 standing mode to a quarter period at
    # cfl 0.25: the library's wave_errors equals the oracle's run to 1e-10,
    # and its u / v errors match the reference's published cfl-1/2 values
    # (CODE.md:4142: u 6.61e-6, v 6.38e-5) to the spatial error's 2 digits.
    from oracle_drivers import oracle_errors
    r = native.wave_errors(np.float64, 2, P=4, E=2, roots=8, cfl=0.25)
    ro = oracle_errors(2, 4, 2, 8, cfl=0.25)
    assert r["nsteps"] == ro["nsteps"]
    assert r["l2"] == pytest.approx(ro["l2"], rel=1e-9)
    assert r["linf"] == pytest.approx(ro["linf"], rel=1e-9)
    assert ro["eu"] == pytest.approx(6.61e-6, rel=0.05)
    assert ro["ev"] == pytest.approx(6.38e-5, rel=0.05)
    assert r["energy"] <= r["energy0"]


def test_float32_agrees_with_float64_at_coarse_resolution(native):
    # test/sinewave_tests.jl:49-59
    r32 = native.wave_errors(np.float32, 2, P=3, E=2, roots=2)
    r64 = native.wave_errors(np.float64, 2, P=3, E=2, roots=2)
    assert r32["nsteps"] == r64["nsteps"]
    assert r32["l2"] == pytest.approx(r64["l2"], rel=1e-3)


@pytest.mark.parametrize("D,P", [(1, 3), (2, 3), (3, 2)])
def test_refined_energy_rate_is_zero(native, D, P):
    # dE/dt = <v, Lap u>_w + <D u, D v>_w = 0 on a two-level forest
    # (test/refined_tests.jl:111-143), through the library's own RHS and energy
    import twoldg
    forest = refined_forest(D, P)
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, P), truncate=False)
    n = len(forest.leaves) * forest.N ** D
    u = np.stack([scrambled(n, 0.2).reshape(len(forest.leaves), -1),
                  scrambled(n, 0.6).reshape(len(forest.leaves), -1)], axis=1).reshape(-1)
    ud = dev(p, u)
    du = p.statevector()
    native.wave_rhs(du, ud, p)
    eps = 1e-6
    e1 = native.wave_energy(p, ud + eps * du)
    e0 = native.wave_energy(p, ud - eps * du)
    rate = (e1 - e0) / (2 * eps)
    scale = native.wave_energy(p, ud) * float(np.abs(du.cpu().numpy()).max())
    assert abs(rate) < 1e-8 * scale
