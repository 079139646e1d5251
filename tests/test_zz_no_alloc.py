"""twoldg_rhs_static, the right-hand side for callers that cannot call
cudaMalloc (a host that lends the library only memory it manages itself),
against twoldg_rhs through the C ABI. It keeps its scratch in a static
device array shared by every call, so it is checked on two calls in a row,
with different inputs, on forests with and without coarse-fine faces. This
file sorts last so that a run stopping at the first failure has run every
other test first."""
import ctypes

import numpy as np
import pytest

from cases import scrambled, smooth_data, state_from
from twoldg.forest import wave_forest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("D,P,E,roots,refined,prec", [
    (1, 3, 4, 5, True, "f64"),
    (2, 4, 2, 8, False, "f64"),
    (3, 3, 2, 3, True, "f64"),
    (2, 3, 2, 4, True, "f32"),
])
def test_rhs_static_matches_rhs_on_two_calls(native, D, P, E, roots, refined, prec):
    import torch
    import twoldg
    from twoldg import _lib
    dtype = np.float64 if prec == "f64" else np.float32
    forest = wave_forest(dtype, D, P, E, roots=roots, refined=refined)
    p = twoldg.WaveProblem(forest, twoldg.Element(dtype, P), precision=prec)
    L = _lib.lib()
    n = p.state_words
    inputs = [state_from(forest, P, smooth_data(D)), scrambled(n, 0.3)]
    for u in inputs:
        ud = torch.from_numpy(np.ascontiguousarray(u, dtype=dtype)).cuda()
        ref = p.statevector()
        twoldg.wave_rhs(ref, ud, p)
        got = torch.full_like(ref, float("nan"))
        torch.cuda.synchronize()
        rc = L.twoldg_rhs_static(ctypes.byref(p._desc), ctypes.c_void_p(got.data_ptr()),
                                 ctypes.c_void_p(ud.data_ptr()), 0.0, None)
        _lib.check(rc)
        torch.cuda.synchronize()
        a, b = got.cpu().numpy().astype(np.float64), ref.cpu().numpy().astype(np.float64)
        tol = 1e-12 if prec == "f64" else 1e-6
        assert np.all(np.isfinite(a))
        assert np.abs(a - b).max() <= tol * np.abs(b).max()


def _static_against_rhs(native, forest, P, u, prec):
    import torch
    import twoldg
    from twoldg import _lib
    dtype = np.float64 if prec == "f64" else np.float32
    p = twoldg.WaveProblem(forest, twoldg.Element(dtype, P), precision=prec)
    ud = torch.from_numpy(np.ascontiguousarray(u, dtype=dtype)).cuda()
    ref = p.statevector()
    twoldg.wave_rhs(ref, ud, p)
    got = torch.full_like(ref, float("nan"))
    torch.cuda.synchronize()
    _lib.check(_lib.lib().twoldg_rhs_static(ctypes.byref(p._desc), ctypes.c_void_p(got.data_ptr()),
                                            ctypes.c_void_p(ud.data_ptr()), 0.0, None))
    torch.cuda.synchronize()
    a, b = got.cpu().numpy().astype(np.float64), ref.cpu().numpy().astype(np.float64)
    assert np.all(np.isfinite(a))
    assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()


def test_rhs_static_after_a_different_forest(native):
    """The static array keeps the last call's contents: a refined forest
    (coarse-fine faces, more blocks), then a smaller unrefined one with other
    slot counts, then the refined one again, each equal to twoldg_rhs."""
    refined = wave_forest(np.float64, 3, 3, 2, roots=3, refined=True)
    small = wave_forest(np.float64, 3, 2, 2, roots=2)
    for forest, P in ((refined, 3), (small, 2), (refined, 3)):
        u = scrambled(2 * forest.N ** 3 * len(forest.leaves), 0.7)
        _static_against_rhs(native, forest, P, u, "f64")


def test_rhs_static_rejects_a_forest_beyond_its_scratch(native):
    import torch
    import twoldg
    from twoldg import _lib
    forest = wave_forest(np.float64, 3, 3, 4, roots=10)  # 1000 blocks of 16^3: ~25 MB of face scratch
    desc, keep = twoldg.problem.make_desc(forest, twoldg.Element(np.float64, 3), True, _lib.F64)
    u = torch.zeros(2 * 16 ** 3 * 1000, dtype=torch.float64, device="cuda")
    du = torch.zeros_like(u)
    rc = _lib.lib().twoldg_rhs_static(ctypes.byref(desc), ctypes.c_void_p(du.data_ptr()),
                                      ctypes.c_void_p(u.data_ptr()), 0.0, None)
    assert rc == _lib.TWOLDG_EINVAL
    assert b"16 MiB" in _lib.lib().twoldg_last_error()
    del keep
