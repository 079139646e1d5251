"""The regrid transfer through libtwoldg (twoldg_transfer) against the
oracle's restatement, the reference's regrid properties (sum w u kept,
coarsening brings v's top mode back and the truncation removes it,
refining keeps it out), and refine_flags on the device indicator. Marked
gpu."""
import numpy as np
import pytest

from cases import scrambled
from oracle.oracle import Oracle, oracle_transfer
from test_regrid import mass, same_mass
from twoldg.forest import wave_forest

pytestmark = pytest.mark.gpu


def middle_flags(forest):
    # refine the blocks whose centres lie in the middle half of the unit box
    from twoldg.regrid import KEEP, REFINE
    out = []
    for key in forest.leaves:
        ext = forest.block_extent(key)
        out.append(REFINE if all(0.25 < (e[0] + e[1]) / 2 < 0.75 for e in ext) else KEEP)
    return out


@pytest.mark.parametrize("D,P", [(1, 3), (2, 3), (3, 2)])
def test_regrid_transfer_keeps_mass_and_truncation(native, D, P):
    import torch
    import twoldg
    from twoldg.regrid import COARSEN, KEEP, regrid, transfer_state
    E = 2
    f = wave_forest(np.float64, D, P, E, roots=4, refined=True)
    el = twoldg.Element(np.float64, P)
    p = twoldg.WaveProblem(f, el)
    nb, N = f.nleaves(), E * (P + 1)
    u = torch.from_numpy(scrambled(nb * 2 * N ** D, 0.2)).cuda()
    twoldg.truncate_state(u, p)
    host = u.cpu().numpy()
    m0 = mass(f.leaves, host, D, P, E)
    # coarsen every refined block
    g = regrid(f, [COARSEN if lv > 0 else KEEP for lv, _ in f.leaves])
    assert max(lv for lv, _ in g.leaves) == 0
    q = twoldg.WaveProblem(g, el)
    ug = transfer_state(p, u, q)
    ref = oracle_transfer(f.leaves, host, g.leaves, D, P, E)
    got = ug.cpu().numpy()
    assert np.abs(got - ref).max() < 1e-13 * np.abs(ref).max()
    assert same_mass(g.leaves, got, m0, D, P, E)
    # coarsening brings v's top mode back; the truncation takes it out and keeps the mass
    assert twoldg.mode_amplitude(q, ug, P, var=2).max().item() > 1e-3
    twoldg.truncate_state(ug, q)
    assert twoldg.mode_amplitude(q, ug, P, var=2).max().item() < 1e-13
    assert same_mass(g.leaves, ug.cpu().numpy(), m0, D, P, E)
    # refine the middle: the coarse polynomial, v stays in Q_{P-1}
    h = regrid(g, middle_flags(g))
    assert max(lv for lv, _ in h.leaves) == 1
    r = twoldg.WaveProblem(h, el)
    uh = transfer_state(q, ug, r)
    ref = oracle_transfer(g.leaves, ug.cpu().numpy(), h.leaves, D, P, E)
    assert np.abs(uh.cpu().numpy() - ref).max() < 1e-13 * np.abs(ref).max()
    assert same_mass(h.leaves, uh.cpu().numpy(), m0, D, P, E)
    assert twoldg.mode_amplitude(r, uh, P, var=2).max().item() < 1e-13
    # the problem rebuilt on the new forest steps as the oracle does there
    dt = 0.5 * h.minimum_spacing() / (P + 1)
    integ = twoldg.wave_integrator(r, uh, 0.0, 3 * dt, dt)
    integ.solve()
    o = Oracle(h, P)
    want = o.rk4(uh.cpu().numpy(), dt, 3)
    assert np.abs(integ.u.cpu().numpy() - want).max() < 1e-12 * np.abs(want).max()


def test_refine_flags_and_a_regrid_cycle(native):
    # refine_flags is refine_mark of the device indicator per block; a
    # Gaussian in the middle of the box refines the blocks under it, the
    # state moves onto the new forest with its mass, and the quiet refined
    # blocks coarsen back once the data are gone
    import torch
    import twoldg
    from twoldg.regrid import COARSEN, KEEP, REFINE, refine_flags, refine_mark, regrid, transfer_state
    D, P, E = 2, 3, 2
    f = wave_forest(np.float64, D, P, E, roots=4)
    el = twoldg.Element(np.float64, P)
    p = twoldg.WaveProblem(f, el)
    bump = lambda x, v: np.exp(-((x[0] - 0.5) ** 2 + (x[1] - 0.5) ** 2) / 0.08 ** 2) if v == 1 else 0 * x[0]
    u = twoldg.initial_state(p, bump)
    tols = dict(refine_tol=3e-2, coarsen_tol=3e-5)
    flags = refine_flags(p, u, P - 1, maxlevel_cap=1, **tols)
    tau = twoldg.modal_indicator(p, u, P - 1).cpu().numpy()
    for b, (lv, _) in enumerate(f.leaves):
        assert flags[b] == refine_mark(tau[b].T, P, lv, maxlevel_cap=1, **tols)
    assert sum(1 for fl in flags if isinstance(fl, tuple) and fl[0] == REFINE) == 4
    g = regrid(f, flags, buffer=2)
    q = twoldg.WaveProblem(g, el)
    ug = transfer_state(p, u, q)
    m0 = mass(f.leaves, u.cpu().numpy(), D, P, E)
    assert same_mass(g.leaves, ug.cpu().numpy(), m0, D, P, E)
    assert sum(1 for lv, _ in g.leaves if lv == 1) >= 16
    back = [COARSEN if lv > 0 else KEEP for lv, _ in g.leaves]
    assert sorted(regrid(g, back).leaves) == sorted(f.leaves)


def test_float32_transfer(native):
    import torch
    import twoldg
    from twoldg.regrid import COARSEN, KEEP, regrid, transfer_state
    D, P, E = 3, 3, 2
    f = wave_forest(np.float32, D, P, E, roots=4, refined=True)
    el = twoldg.Element(np.float32, P)
    p = twoldg.WaveProblem(f, el, precision="f32c")
    N = E * (P + 1)
    host = scrambled(f.nleaves() * 2 * N ** D, 0.3).astype(np.float32)
    g = regrid(f, [COARSEN if lv > 0 else KEEP for lv, _ in f.leaves])
    q = twoldg.WaveProblem(g, el, precision="f32c")
    ug = transfer_state(p, torch.from_numpy(host).cuda(), q)
    ref = oracle_transfer(f.leaves, host.astype(np.float64), g.leaves, D, P, E)
    assert np.abs(ug.cpu().numpy() - ref).max() < 1e-5 * np.abs(ref).max()
