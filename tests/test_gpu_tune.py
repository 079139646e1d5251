"""The autotuner: it leaves the state alone, every launch layout it can pick
gives the oracle's result (FP64 to 1e-12 relative, with CTAs looping over
several blocks where the grid is persistent), and its JSON cache round-trips.
Marked gpu."""
import json

import numpy as np
import pytest

from cases import smooth_data, state_from
from oracle.oracle import Oracle
from twoldg.forest import wave_forest

pytestmark = pytest.mark.gpu

# (kernel, threads, waves): register-line 3D, fixed-shape, run-time-shape
LAYOUTS = ([(1, 0, w) for w in range(3)] + [(2, 0, w) for w in range(3)] +
           [(3, t, w) for t in (64, 128, 256) for w in range(2)])


def rel(a, b):
    return float(np.abs(np.asarray(a, dtype=np.float64) - b).max() / max(np.abs(b).max(), 1e-300))


def setup(D, P, E, roots):
    import torch
    import twoldg
    forest = wave_forest(np.float64, D, P, E, roots=roots)
    p = twoldg.WaveProblem(forest, twoldg.Element(np.float64, P))
    o = Oracle(forest, P)
    u0 = o.truncate(state_from(forest, P, smooth_data(D)))
    dt = 0.5 * forest.minimum_spacing() / (P + 1)
    return p, o, u0, dt, torch.from_numpy(u0).cuda()


def pin(path, key, layout):
    k, t, w = layout
    path.write_text('{\n  "%s": {"kernel": %d, "threads": %d, "waves": %d, "us": 0.00}\n}\n' % (key, k, t, w))


def test_autotune_keeps_state_and_steps_match_oracle(native):
    p, o, u0, dt, ud = setup(3, 3, 4, 2)
    rep = p.autotune(ud, dt)
    assert len(rep) == 1
    (key, choice), = rep.items()
    assert key.startswith("f64 d3 p3 e4 flat")
    assert choice["kernel"] in (1, 2, 3) and choice["us"] > 0
    assert np.array_equal(ud.cpu().numpy(), u0)
    integ = native.wave_integrator(p, ud, 0.0, 3 * dt, dt)
    integ.solve()
    assert rel(integ.u.cpu().numpy(), o.rk4(u0, dt, 3)) < 1e-12


# 13^3 blocks of 8^3 and 50^2 blocks of 6^2: more blocks than one wave of
# resident CTAs, so that a persistent grid loops
@pytest.mark.parametrize("shape", [(3, 3, 2, 13), (2, 2, 2, 50)], ids=["3D-13cube", "2D-50sq"])
def test_every_layout_matches_oracle(native, shape, tmp_path):
    p, o, u0, dt, ud = setup(*shape)
    ref = o.rk4(u0, dt, 2)
    key, = p.autotune(ud.clone(), dt).keys()
    for layout in LAYOUTS:
        cache = tmp_path / ("pin%d_%d_%d.json" % layout)
        pin(cache, key, layout)
        rep = p.autotune(ud, dt, cache=cache)
        assert (rep[key]["kernel"], rep[key]["threads"], rep[key]["waves"]) == layout
        integ = native.wave_integrator(p, ud.clone(), 0.0, 2 * dt, dt)
        integ.solve()
        assert rel(integ.u.cpu().numpy(), ref) < 1e-12, layout


def test_cache_roundtrip(native, tmp_path):
    cache = tmp_path / "tune.json"
    p, o, u0, dt, ud = setup(2, 3, 4, 3)
    rep = p.autotune(ud, dt, cache=cache)
    on_disk = json.loads(cache.read_text())
    assert on_disk == rep
    # a second problem of the same shape takes the cached choice without timing
    q, _, _, _, vd = setup(2, 3, 4, 3)
    assert q.autotune(vd, dt, cache=cache) == rep
    # a problem of another shape adds its entry and keeps the first
    r, _, _, _, wd = setup(2, 2, 2, 3)
    rep2 = r.autotune(wd, dt, cache=cache)
    merged = json.loads(cache.read_text())
    assert set(merged) == set(rep) | set(rep2) and len(merged) == 2


def test_batch_autotune(native):
    import twoldg
    members = twoldg.sine_ensemble(12, seed=3, dtype=np.float64, roots_range=(2, 4))
    b = twoldg.Batch([(f, P) for f, P, _ in members], precision="f64")
    u0 = twoldg.fill_batch(b, members)
    dts = [0.5 * f.minimum_spacing() / (P + 1) for f, P, _ in members]
    before = u0.clone()
    b.rk4_step(before, dts, 3)
    b.synchronize()
    rep = b.autotune(u0, dts)
    assert len(rep) == len({(P, f.N) for f, P, _ in members})
    after = u0.clone()
    b.rk4_step(after, dts, 3)
    b.synchronize()
    assert rel(after.cpu().numpy(), before.cpu().numpy()) < 1e-12
