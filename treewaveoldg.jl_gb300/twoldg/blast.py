"""The 2D blast wave and its adaptive driver (src/blast.jl): a Gaussian peak
released at rest in the middle of a periodic box, its exact solution by
the inverse Hankel transform, the uniform run, and the adaptive run that
cycles the modal indicator, the regrid and the state transfer between
chunks of RK4 steps (TreeWave's track_blast for OLDG)."""
import math

import numpy as np

from .element import Element
from .forest import wave_forest
from .problem import (WaveProblem, chunk_count, initial_state, oldg_timestep, quadrature_norm, truncate_state,
                      wave_energy, wave_integrator)
from .regrid import check_thresholds, refine_flags, regrid, transfer_state


def supergaussian(x, sigma, n):
    return np.exp(-(x / sigma) ** (2 * n))


def wrap(x, L):
    """x reduced into [0, L) (src/precision.jl:61-68)."""
    return x - L * np.floor(x / L)


def blast_initial(L, x0, sigma):
    """u = exp(-(r/sigma)^2), v = 0, r the periodically wrapped distance from x0
    (src/blast.jl:15-34), as an f(x, var) callback."""
    def f(x, var):
        if var != 1:
            return np.zeros_like(x[0])
        r2 = np.zeros_like(x[0])
        for d in range(2):
            r2 = r2 + (wrap(x[d] - x0[d] + L / 2, L) - L / 2) ** 2
        return supergaussian(np.sqrt(r2), sigma, 1).astype(np.asarray(x[0]).dtype)
    return f


def blast_reference(L, x0, sigma, rmax, nr=2001, nk=2000):
    """The time-independent part of the exact solution (src/blast.jl:36-84):
    u(r,t) = int f^(k) J0(kr) cos(kt) k dk, f^(k) = (sigma^2/2) exp(-k^2 sigma^2/4),
    the k integral cut at 13/sigma and taken by the midpoint rule with nk
    points, J0 tabulated on nr radii in [0, rmax]."""
    from scipy.special import j0
    dk = (13.0 / sigma) / nk
    ks = (np.arange(1, nk + 1) - 0.5) * dk
    ws = (sigma ** 2 / 2) * np.exp(-(ks * sigma) ** 2 / 4) * ks * dk
    rs = np.linspace(0.0, rmax, nr)
    J = j0(np.outer(rs, ks))
    return dict(L=float(L), x0=tuple(float(v) for v in x0), sigma=float(sigma), rs=rs, dr=rs[1] - rs[0],
                rmax=float(rmax), ks=ks, ws=ws, J=J)


def blast_radial_table(ref, t):
    """The free-space radial profiles of u and du/dt at time t (src/blast.jl:86-110)."""
    wc = ref["ws"] * np.cos(ref["ks"] * t)
    wsn = ref["ws"] * np.sin(ref["ks"] * t) * ref["ks"]
    return ref["J"] @ wc, -(ref["J"] @ wsn)


def blast_exact(ref, t):
    """The exact solution at time t (src/blast.jl:112-143): the radial profile
    summed over the periodic images of the source within rmax, interpolated
    linearly in r; an f(x, var) callback."""
    us, vs = blast_radial_table(ref, t)
    L, rmax, dr = ref["L"], ref["rmax"], ref["dr"]
    x0 = ref["x0"]
    nimg = int(math.ceil(rmax / L))

    def f(x, var):
        X = [np.asarray(v, dtype=np.float64) for v in x]
        out = np.zeros_like(X[0])
        tab = us if var == 1 else vs
        for j1 in range(-nimg, nimg + 1):
            for j2 in range(-nimg, nimg + 1):
                r = np.hypot(X[0] - x0[0] - j1 * L, X[1] - x0[1] - j2 * L)
                inside = r < rmax
                q = np.where(inside, r / dr, 0.0)
                i = np.floor(q).astype(np.int64)
                s = q - i
                i1 = np.minimum(i + 1, len(tab) - 1)
                out = out + np.where(inside, (1 - s) * tab[i] + s * tab[i1], 0.0)
        return out.astype(np.asarray(x[0]).dtype)
    return f


def blast_errors(p, u, ref, t):
    """L-infinity and L2 errors of u and du/dt together against the exact state."""
    ue = p.to_device(p.fill_at_nodes(blast_exact(ref, t)))
    return quadrature_norm(p, u, math.inf, ref=ue), quadrature_norm(p, u, 2, ref=ue)


def uniform_blast(T=np.float64, P=3, E=2, roots=16, L=1.0, sigma=0.08, t_end=0.4, cfl=0.5, truncate=True,
                  precision=None):
    """uniform_blast (src/blast.jl:145-207): the blast wave on a uniform
    roots x roots box to t_end; L-infinity and L2 errors of u and v together,
    the spacing, the node count, the steps and the energies."""
    T = np.dtype(T)
    forest = wave_forest(T, 2, P, E, roots=roots, L=L)
    p = WaveProblem(forest, Element(T, P), truncate=truncate, precision=precision)
    x0 = (L / 2, L / 2)
    u0 = initial_state(p, blast_initial(L, x0, sigma))
    ref = blast_reference(L, x0, sigma, rmax=t_end + 6 * sigma)
    nsteps = int(math.ceil(T.type(t_end) / oldg_timestep(p, cfl)))
    dt = float(T.type(T.type(t_end) / T.type(nsteps)))
    integ = wave_integrator(p, u0, 0.0, t_end, dt)
    integ.nsteps = nsteps
    integ.solve()
    err, l2 = blast_errors(p, integ.u, ref, t_end)
    return dict(err=err, l2=l2, h=forest.minimum_spacing(), nodes=forest.nleaves() * forest.N ** 2,
                nsteps=nsteps, energy0=wave_energy(p, u0), energy=wave_energy(p, integ.u))


def refinement_buffer(forest, maxlevel_cap, travel):
    """The regrid buffer in points for a feature travelling `travel` between
    regrids, at the spacing of level maxlevel_cap: ceil(travel/h) + 1, at most
    the block width N (src/refinement.jl:288-315)."""
    h = (forest.hi[0] - forest.lo[0]) / forest.roots[0] / (1 << maxlevel_cap) / forest.N
    points = int(math.ceil(travel / h)) + 1
    if points > forest.N:
        raise ValueError("a feature travelling %r between regrids needs a %d-point margin at level %d (h = %r), "
                         "which exceeds the block width N = %d: the travel must stay under one finest-level "
                         "block width, %r; regrid more often" % (travel, points, maxlevel_cap, h, forest.N,
                                                                  forest.N * h))
    return points


def adaptive_blast(T=np.float64, P=3, E=2, roots=4, maxlevel_cap=2, refine_tol=1e-2, coarsen_tol=1e-5, chunk=0.05,
                   buffer=None, L=1.0, sigma=0.08, t_end=0.4, cfl=0.5, truncate=True, maxpasses=8, precision=None):
    """adaptive_blast (src/blast.jl:209-360): adapt the mesh to the initial
    Gaussian (refill, flag, regrid until the mesh stands), then in chunks of
    `chunk` step the problem, flag by the modal indicator of u up to mode
    P - truncate, regrid, move the state onto the new mesh and truncate it.
    Each chunk's steps share one dt, the chunk's span over ceil(span /
    (cfl h_min / (P+1))) steps, so that every chunk ends on its bound. Returns
    the errors at t_end against the exact solution and the run's record."""
    check_thresholds(refine_tol, coarsen_tol)
    if not chunk > 0:
        raise ValueError("chunk = %r: the time between regrids must be positive" % (chunk,))
    mode = P - (1 if truncate else 0)
    if not 1 <= mode <= P:
        raise ValueError("mode = %d is not a Legendre mode an element of order P = %d can be refined by: the "
                         "truncated scheme at P = 1 has no mode to refine by" % (mode, P))
    T = np.dtype(T)
    forest = wave_forest(T, 2, P, E, roots=roots, L=L)
    el = Element(T, P)
    x0 = (L / 2, L / 2)
    initial = blast_initial(L, x0, sigma)
    ref = blast_reference(L, x0, sigma, rmax=t_end + 6 * sigma)
    if buffer is None:
        buffer = refinement_buffer(forest, maxlevel_cap, chunk)

    def flags(p, u):
        return refine_flags(p, u, mode, refine_tol, coarsen_tol, maxlevel_cap)

    converged, passes = False, 0
    for passes in range(1, maxpasses + 1):
        p = WaveProblem(forest, el, truncate=truncate, precision=precision)
        u = initial_state(p, initial)
        new = regrid(forest, flags(p, u), buffer)
        if sorted(new.leaves) == sorted(forest.leaves):
            converged = True
            break
        forest = new
    p = WaveProblem(forest, el, truncate=truncate, precision=precision)
    u = initial_state(p, initial)
    energy0 = wave_energy(p, u)
    nodes = lambda f: f.nleaves() * f.N ** 2
    nodes_max, node_steps, nsteps_total, nregrids = nodes(forest), 0, 0, 0
    chunks = []
    nchunks = chunk_count(T, t_end, chunk)
    for c in range(1, nchunks + 1):
        tstart = min((c - 1) * chunk, t_end)
        t = t_end if c == nchunks else min(c * chunk, t_end)
        if not t > tstart:
            break
        e_start = wave_energy(p, u, t=tstart)
        nsteps = int(math.ceil((t - tstart) / oldg_timestep(p, cfl) - 1e-12))
        integ = wave_integrator(p, u, tstart, t, (t - tstart) / nsteps, alias_u0=True)
        integ.nsteps = nsteps
        integ.solve()
        e_end = wave_energy(p, u, t=t)
        nsteps_total += nsteps
        node_steps += nsteps * nodes(forest)
        record = dict(tstart=tstart, t=t, nsteps=nsteps, nblocks=forest.nleaves(),
                      maxlevel=max(lv for lv, _ in forest.leaves), energy_start=e_start, energy_end=e_end,
                      regridded=False)
        if c < nchunks:
            new = regrid(forest, flags(p, u), buffer)
            if sorted(new.leaves) != sorted(forest.leaves):
                q = WaveProblem(new, el, truncate=truncate, precision=precision)
                u = transfer_state(p, u, q)
                if truncate:
                    truncate_state(u, q)
                p, forest = q, new
                nregrids += 1
                nodes_max = max(nodes_max, nodes(forest))
                record["regridded"] = True
        chunks.append(record)
    err, l2 = blast_errors(p, u, ref, t_end)
    return dict(err=err, l2=l2, h=forest.minimum_spacing(), nodes=nodes(forest), nodes_max=nodes_max,
                node_steps=node_steps, nsteps=nsteps_total, nregrids=nregrids,
                maxlevel=max(lv for lv, _ in forest.leaves), forest=forest, passes=passes, converged=converged,
                energy0=energy0, energy=wave_energy(p, u), chunks=chunks)
