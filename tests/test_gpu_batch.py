"""The batched ensemble (twoldg_batch_*): independent 2D periodic problems
of uneven P, E and roots stepped together, one work list per shape and one
graph per step. Each member must equal the same problem stepped alone, bit
for bit (the same kernels and arithmetic; alone, a problem's stage kernels
run as programmatic dependent launches, in the batch as plain ones), and the
FP64 members the oracle."""
import ctypes
import math

import numpy as np
import pytest

from cases import state_from
from oracle.oracle import Oracle
from twoldg.forest import wave_forest

pytestmark = pytest.mark.gpu
NSTEPS = 19


def ensemble(n, seed, dtype=np.float64):
    """n members: P in 2..5, E in {2, 4}, roots in 2..5 (small for the test), a
    random-amplitude sum of 4 sine modes each (seeded)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        P = int(rng.integers(2, 6))
        E = int(rng.choice([2, 4]))
        roots = int(rng.integers(2, 6))
        a = rng.uniform(-1, 1, 4)
        m = rng.integers(1, 4, size=(4, 2))
        ph = rng.uniform(0, 2 * math.pi, 4)

        def f(x, var, a=a, m=m, ph=ph):
            s = np.zeros_like(x[0])
            if var == 1:
                for j in range(4):
                    s = s + a[j] * np.sin(2 * math.pi * (m[j, 0] * x[0] + m[j, 1] * x[1]) + ph[j])
            return s
        forest = wave_forest(dtype, 2, P, E, roots=roots)
        out.append((forest, P, f))
    return out


@pytest.mark.parametrize("prec", ["f64", "f32c"])
def test_batch_equals_members_alone(native, prec):
    import torch
    import twoldg
    from twoldg import _lib
    dtype = np.float64 if prec == "f64" else np.float32
    members = ensemble(12, 0, dtype)
    probs, descs, keep, states, dts = [], [], [], [], []
    for forest, P, f in members:
        p = twoldg.WaveProblem(forest, twoldg.Element(dtype, P), precision=prec)
        u0 = twoldg.initial_state(p, f)
        probs.append(p)
        d, k = twoldg.problem.make_desc(forest, twoldg.Element(dtype, P), True, p._desc.precision)
        descs.append(d)
        keep.append(k)
        states.append(u0)
        dts.append(0.5 * forest.minimum_spacing() / (P + 1))
    arr = (_lib.Desc * len(descs))(*descs)
    h = ctypes.c_void_p()
    _lib.check(_lib.lib().twoldg_batch_create(len(descs), arr, ctypes.byref(h)))
    try:
        offs = (ctypes.c_int64 * len(descs))()
        total = ctypes.c_int64()
        _lib.check(_lib.lib().twoldg_batch_offsets(h, offs, ctypes.byref(total)))
        big = torch.zeros(total.value, dtype=states[0].dtype, device="cuda")
        for k, u in enumerate(states):
            big[offs[k]:offs[k] + u.numel()] = u
        torch.cuda.synchronize()
        dtarr = (ctypes.c_double * len(dts))(*dts)
        # 19 steps: one launch of the batch's 16-step graph, whose groups run
        # their chains through the 16 steps unjoined, and one of a 3-step one
        _lib.check(_lib.lib().twoldg_batch_rk4_step(h, ctypes.c_void_p(big.data_ptr()), dtarr, NSTEPS))
        _lib.check(_lib.lib().twoldg_batch_synchronize(h))
        for k, (p, u0) in enumerate(zip(probs, states)):
            integ = twoldg.wave_integrator(p, u0, 0.0, NSTEPS * dts[k], dts[k])
            integ.nsteps = NSTEPS
            integ.solve()
            got = big[offs[k]:offs[k] + u0.numel()].cpu().numpy()
            assert np.array_equal(got, integ.u.cpu().numpy()), k
            if prec == "f64" and k < 4:
                forest, P, f = members[k]
                o = Oracle(forest, P)
                ref = o.rk4(u0.cpu().numpy(), dts[k], NSTEPS)
                assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max()
    finally:
        _lib.lib().twoldg_batch_destroy(h)
