"""The particle-grid transfer (src/transfer.jl): the projection of a source
onto the nodes, (P S)_n = (1/w_n) int_{element(n)} S phi_n, through the
library's plan and kernels, and the reconstruction of a state at a point.

project_source(du, p, S, particles; ball, rnear, factor, var) mirrors
project_source! (src/transfer.jl:918-944): the far rule beyond rfar h_e, the
graded bands within it, and the nested rule split at the nearest particle's
support within rnear h_e. S is either "density" (the particles' own density,
evaluated in the kernels) or a callable that takes the points as a (D, n)
tensor on the problem's device and returns their values: the role of the
closure the reference's launch_points! hook runs (ext/TreeWaveOLDGCUDAExt.jl:
23-30). The transfer runs in the particles' frame (ParticleFrame, src/
transfer.jl:705-766): a brick's own coordinates, or the affine cube patch of
the seven- and thirteen-patch balls.

The other direction, from the field to the particles: TransferPlan.pairing
is pairing(p, t, u, K, s; var, continuous) (src/transfer.jl:1779-1797) for
each particle's density kernel K = (grad rho, rho), particle_forces the grid's
part of the force (src/inspiral.jl:474-504), and source_pairing the pairing of
a source's own projection (src/transfer.jl:1799-1825). reconstruct and
reconstruct_gradient read a state's element polynomial and its gradient at a
point.
"""
import ctypes
import math

import numpy as np

from . import _lib
from .problem import _check_state, _dptr, _sync_torch

RFAR = 9.0
GRADED = ((1, 14), (2, 10), (3, 8), (4, 7))
NSINH, NMID, NINNER = 48, 16, 24


def transfer_table(P, dtype, name, q=None):
    """A transfer table of order P in float64 or float32: "bary" (P+1), and of
    the q-point Gauss rule "gauss_nodes", "gauss_weights" (q), "lagrange"
    (q, P+1) and "contract" (P+1, q) (TransferTables, src/transfer.jl:107-170)."""
    dtype = np.dtype(dtype)
    prec = {np.dtype(np.float64): 0, np.dtype(np.float32): 1}.get(dtype)
    if prec is None:
        raise ValueError("transfer tables exist in float64 and float32, not %s" % dtype)
    P1 = P + 1
    q = P + 3 if q is None else int(q)
    shape = {"bary": (P1,), "gauss_nodes": (q,), "gauss_weights": (q,), "lagrange": (q, P1),
             "contract": (P1, q)}.get(name)
    if shape is None:
        raise ValueError("unknown transfer table %r" % (name,))
    out = np.zeros(shape, dtype=dtype)
    _lib.check(_lib.lib().twoldg_transfer_table(int(P), prec, name.encode(), q,
                                                out.ctypes.data_as(ctypes.c_void_p)))
    return out


class ParticleSupport:
    """ParticleSupport(z, v, ell) (src/transfer.jl:264-290): where a particle
    is, its velocity and its size; its support is |L(v)(x - z)| <= ell.
    `charge` is the Q of the built-in density source."""

    def __init__(self, z, v=None, ell=1e-3, charge=0.0):
        self.z = tuple(float(x) for x in z)
        self.v = tuple(float(x) for x in (v if v is not None else [0.0] * len(self.z)))
        self.ell = float(ell)
        self.charge = float(charge)
        if not self.ell > 0:
            raise ValueError("the particle size ell must be positive, got %r" % (ell,))
        if not sum(x * x for x in self.v) < 1:
            raise ValueError("the particle's speed |v| must be below 1, got %r" % (self.v,))

    def _c(self):
        c = _lib.Particle()
        for d in range(3):
            c.z[d] = self.z[d] if d < len(self.z) else 0.0
            c.v[d] = self.v[d] if d < len(self.v) else 0.0
        c.ell = self.ell
        c.charge = self.charge
        return c


def particle_frame(p):
    """The particles' frame of problem p (src/transfer.jl:705-800): per block
    its origin and node spacing in physical coordinates, whether it is in the
    frame's patch, its level, the finest element width h_e and the frame's
    domain ((lo, hi) per dimension)."""
    from .ball import BallForest
    forest = p.forest
    D, N, P1 = p.D, p.N, p.P + 1
    if isinstance(forest, BallForest):
        geo = forest.geo
        if not geo.affine_patch(0):
            raise ValueError("the particles run in the ball's affine cube patch")
        n = geo.patch_roots(0)[0]
        scale = 2 * geo.Lc / n
        bs = np.array([forest.block_scale(b) for b in range(forest.nleaves())])
        origins = np.array([[-geo.Lc + scale * s * c[d] for d in range(3)] for s, (_, c) in zip(bs, forest.blocks)])
        spacings = scale * bs / N
        mask = np.array([1 if patch == 0 else 0 for patch, _ in forest.blocks], dtype=np.uint8)
        levels = np.array(forest.levels, dtype=np.int32)
        he = scale * bs.min() / N * P1
        dom = tuple((-geo.Lc, geo.Lc) for _ in range(3))
        return origins, spacings, mask, levels, he, dom
    if getattr(p, "geometry", None) is not None or getattr(p, "metric", None) is not None:
        raise ValueError("the particles run on a brick in flat space or in the affine patch of a ball; this "
                         "problem has a diagonal metric whose patches are not affine")
    origins = np.array([[forest.block_extent(k)[d][0] for d in range(D)] for k in forest.leaves])
    spacings = np.array([forest.spacing(k) for k in forest.leaves])
    mask = np.ones(forest.nleaves(), dtype=np.uint8)
    levels = np.array([k[0] for k in forest.leaves], dtype=np.int32)
    he = forest.minimum_spacing() * P1
    dom = tuple((forest.lo[d], forest.hi[d]) for d in range(D))
    return origins, spacings, mask, levels, he, dom


class TransferPlan:
    """projection_plan(p, t, particles, ball, rnear) (src/transfer.jl:984-1022)
    in the library: the elements by rule and the nested rule's points, for one
    set of particle positions. Reuse it for several sources; rebuild it when
    the particles move."""

    def __init__(self, p, particles, ball, rnear=1.0, q=None, graded=None, rfar=None, nsinh=None, nmid=None,
                 ninner=None):
        self.p = p
        self.particles = tuple(particles)
        D = p.D
        origins, spacings, mask, levels, he, dom = particle_frame(p)
        centre = tuple(float(x) for x in ball[0])
        R = float(ball[1])
        if len(centre) != D:
            raise ValueError("the ball's centre has %d coordinates in %d dimensions" % (len(centre), D))
        from .ball import BallForest
        self.frame_domain = dom if isinstance(p.forest, BallForest) else None
        if self.frame_domain is not None:
            self._check_in_patch([("the source's ball of radius %r about %r" % (R, centre),
                                   [c - R for c in centre], [c + R for c in centre])])
        self._arrays = [np.ascontiguousarray(origins.reshape(-1), dtype=np.float64),
                        np.ascontiguousarray(spacings, dtype=np.float64), np.ascontiguousarray(levels),
                        np.ascontiguousarray(mask)]
        d = _lib.TransferDesc()
        dp = ctypes.POINTER(ctypes.c_double)
        d.origins = self._arrays[0].ctypes.data_as(dp)
        d.spacings = self._arrays[1].ctypes.data_as(dp)
        d.levels = self._arrays[2].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        d.mask = self._arrays[3].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
        d.h_e = he
        for k in range(D):
            d.ball_centre[k] = centre[k]
        d.ball_radius = R
        parts = (_lib.Particle * max(1, len(self.particles)))(*[s._c() for s in self.particles])
        self._parts = parts
        d.particles = ctypes.cast(parts, ctypes.POINTER(_lib.Particle))
        d.nparticles = len(self.particles)
        d.rnear = float(rnear)
        d.q = int(q or 0)
        d.nsinh, d.nmid, d.ninner = int(nsinh or 0), int(nmid or 0), int(ninner or 0)
        if graded is not None:
            bf = np.array([float(a) for a, _ in graded], dtype=np.float64)
            bp = np.array([int(b) for _, b in graded], dtype=np.int32)
            self._arrays += [bf, bp]
            d.nbands = len(graded)
            d.band_from = bf.ctypes.data_as(dp)
            d.band_points = bp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        d.rfar = float(rfar or 0.0)
        self.h_e = he
        self.ball = (centre, R)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().twoldg_transfer_plan_create(p.handle, ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self._read_counts()

    def _read_counts(self):
        c = (ctypes.c_int64 * 8)()
        _lib.check(_lib.lib().twoldg_transfer_plan_counts(self._h, c))
        keys = ("far_elements", "far_points", "graded_elements", "graded_points", "near_elements", "near_points",
                "near_chunks", "points")
        self.counts = dict(zip(keys, [int(x) for x in c]))

    def update(self, particles):
        """The plan for the particles at new positions: the ball, the frame
        and the quadrature stay (the reference's SourceBall), the elements by
        rule and the nested rule's points are redone."""
        self.particles = tuple(particles)
        if self.frame_domain is not None:
            self._check_in_patch([])
        parts = (_lib.Particle * max(1, len(self.particles)))(*[s._c() for s in self.particles])
        _lib.check(_lib.lib().twoldg_transfer_plan_update(self._h, ctypes.cast(parts, ctypes.POINTER(_lib.Particle)),
                                                          len(self.particles)))
        self._parts = parts
        self._read_counts()
        return self

    def _check_in_patch(self, extra):
        """The transfer works in the cube alone (check_in_patch, src/transfer.jl:802-812)."""
        dom = self.frame_domain
        D = self.p.D
        for what, lo, hi in extra + [("the support of radius %r about z = %r" % (s.ell, s.z),
                                      [z - s.ell for z in s.z], [z + s.ell for z in s.z]) for s in self.particles]:
            if not all(dom[d][0] <= lo[d] and hi[d] <= dom[d][1] for d in range(D)):
                raise ValueError("the transfer needs %s inside the ball's cube patch, %r, where the particles run"
                                 % (what, dom))

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().twoldg_transfer_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def points(self):
        """Every point S is evaluated at, as a (D, n) tensor on the device:
        the far and graded elements' Gauss points, then the nested rule's."""
        torch = _torch()
        xs = torch.empty((self.p.D, max(1, self.counts["points"])), dtype=self.p.torch_dtype(),
                         device=self.p.device)
        _lib.check(_lib.lib().twoldg_transfer_points(self._h, _dptr(xs)))
        self.p.synchronize()
        return xs[:, :self.counts["points"]]

    def project(self, du, S, factor=-1.0, var=2):
        """du[var] += factor P S: S is "density" or a callable of the (D, n)
        points tensor returning n values. Returns du."""
        _check_state(self.p, du)
        if isinstance(S, str):
            if S != "density":
                raise ValueError("the built-in source is 'density', got %r" % (S,))
            _sync_torch()
            _lib.check(_lib.lib().twoldg_project_density(self._h, _dptr(du), float(factor), int(var)))
        else:
            vals = S(self.points())
            torch = _torch()
            vals = torch.as_tensor(vals, dtype=self.p.torch_dtype(), device=self.p.device).contiguous()
            if vals.numel() != self.counts["points"]:
                raise ValueError("the source returned %d values for %d points" % (vals.numel(),
                                                                                 self.counts["points"]))
            _sync_torch()
            _lib.check(_lib.lib().twoldg_project_values(self._h, _dptr(vals), _dptr(du), float(factor), int(var)))
        self.p.synchronize()
        return du


    def average_shared(self, u, var=2):
        """average_shared!(ua, sn, var) (src/transfer.jl:1616-1714): variable
        var of u, in the blocks the plan's ball meets, with every node that
        elements share replaced by the mean over them. Returns u."""
        _check_state(self.p, u)
        _sync_torch()
        _lib.check(_lib.lib().twoldg_average_shared(self._h, _dptr(u), int(var)))
        self.p.synchronize()
        return u

    def pairing(self, u, var=1, continuous=False):
        """pairing(p, t, u, K, s; var, continuous) (src/transfer.jl:1779-1797)
        of every particle's density kernel K = (grad rho, rho) (density_kernel,
        src/dynamic.jl:124-135) with variable var of the state u, as a
        (nparticles, 4) float64 array: row k is int (grad rho_k) g_h, then
        int rho_k g_h, over the elements that meet particle k's support. With
        continuous=True g_h is first averaged over the elements that share each
        node (continuous_values, :1449-1500)."""
        _check_state(self.p, u)
        out = np.zeros((len(self.particles), 4), dtype=np.float64)
        _sync_torch()
        _lib.check(_lib.lib().twoldg_pairing(self._h, _dptr(u), int(var), 1 if continuous else 0,
                                             out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def support_elements(self, k=0):
        """support_elements(p, s) (src/transfer.jl:1726-1758) of particle k:
        the (block, (e0, e1, e2)) pairs that hold a corner of its support's box,
        block and element indices from 0."""
        out = np.zeros((8, 4), dtype=np.int32)
        n = ctypes.c_int32()
        _lib.check(_lib.lib().twoldg_support_elements(self._h, int(k), out.ctypes.data_as(ctypes.c_void_p),
                                                      ctypes.byref(n)))
        return [(int(r[0]), (int(r[1]), int(r[2]), int(r[3]))) for r in out[:n.value]]


def source_pairing(plan, S, continuous=True):
    """source_pairing(p, t, S, K, s; continuous) (src/transfer.jl:1799-1825)
    for the plan's particles' kernels (grad rho, rho): <K, A P S> without a
    field, as the pairing of S's projection (S as TransferPlan.project takes
    it), averaged over shared nodes with continuous=True. The plan's ball must
    hold the supports' elements and every element sharing a node with them,
    where the reference projects. Returns (nparticles, 4) float64."""
    du = plan.p.statevector()
    plan.project(du, S, factor=1.0, var=1)
    return plan.pairing(du, var=1, continuous=continuous)


def particle_forces(plan, u, continuous=True):
    """The grid's part of each particle's force, particle_forces
    (src/inspiral.jl:474-504): F_k = int (grad rho_k) Phi - v_k int rho_k Pi,
    Phi and Pi variables 1 and 2 of the field state u, read through the
    pairing (continuous by default, as the averaging writes the source).
    Returns (nparticles, 3) float64."""
    phi = plan.pairing(u, var=1, continuous=continuous)
    pi = plan.pairing(u, var=2, continuous=continuous)
    v = np.array([s.v for s in plan.particles], dtype=np.float64).reshape(len(plan.particles), -1)
    return phi[:, :3] - v[:, :3] * pi[:, 3:4]


def source_rhs(du, u, p, plan, S, t=0.0, factor=-1.0, average=True):
    """The field part of the reference's inspiral_rhs! (src/inspiral.jl):
    wave_rhs! of u, then factor times the projection of S onto v's rate, then
    (average=True) the averaging over shared nodes of that rate, as the
    reference writes the source. `plan` is the TransferPlan of the particles'
    current positions. Returns du."""
    from .problem import wave_rhs
    wave_rhs(du, u, p, t)
    plan.project(du, S, factor=factor, var=2)
    if average:
        plan.average_shared(du, var=2)
    return du


def _torch():
    import torch
    return torch


def project_source(du, p, S, particles, ball, rnear=1.0, factor=-1.0, var=2, plan=None, **quadrature):
    """project_source!(du, p, t, S, particles; ball, rnear, factor, var)
    (src/transfer.jl:918-944): du[var] += factor (P S). `plan` reuses a
    TransferPlan made for the same particles and ball."""
    if plan is None:
        plan = TransferPlan(p, particles, ball, rnear, **quadrature)
        try:
            return plan.project(du, S, factor, var)
        finally:
            plan.close()
    return plan.project(du, S, factor, var)


def reconstruct(p, u, x, var=1):
    """reconstruct(p, t, u, x; var) (src/transfer.jl:1990-2009): the element's
    polynomial of variable var at the point x (the upper element on a face)."""
    from .extraction import element_stencils
    from .problem import _dptr as dptr
    torch = _torch()
    index, weights = element_stencils(p.forest, p.P, np.asarray([x], dtype=np.float64))
    idx = torch.as_tensor(index, device=p.device)
    w = torch.as_tensor(weights, dtype=p.torch_dtype(), device=p.device)
    out = torch.empty(1, dtype=p.torch_dtype(), device=p.device)
    _check_state(p, u)
    _sync_torch()
    _lib.check(_lib.lib().twoldg_gather(p.handle, dptr(u), int(var), 1, index.shape[1], dptr(idx), dptr(w),
                                        dptr(out)))
    p.synchronize()
    return float(out.item())


def reconstruct_gradient(p, u, x, var=1):
    """reconstruct_gradient(p, t, u, x; var) (src/transfer.jl:2011-2030): the
    gradient of reconstruct's polynomial at the point x of a brick, as a (D,)
    array: one gather of D rows of derivative weights."""
    from .extraction import element_stencils
    from .problem import _dptr as dptr
    torch = _torch()
    rows = [element_stencils(p.forest, p.P, np.asarray([x], dtype=np.float64), deriv=d) for d in range(p.D)]
    index = np.concatenate([r[0] for r in rows])
    weights = np.concatenate([r[1] for r in rows])
    idx = torch.as_tensor(index, device=p.device)
    w = torch.as_tensor(weights, dtype=p.torch_dtype(), device=p.device)
    out = torch.empty(p.D, dtype=p.torch_dtype(), device=p.device)
    _check_state(p, u)
    _sync_torch()
    _lib.check(_lib.lib().twoldg_gather(p.handle, dptr(u), int(var), p.D, index.shape[1], dptr(idx), dptr(w),
                                        dptr(out)))
    p.synchronize()
    return out.double().cpu().numpy()


def self_inertia(Q, ell):
    """delta m = 693 Q^2 / (4199 pi ell), the self-inertia of the particle's own
    near field (src/particle_forms.jl:2070-2074)."""
    return 693 * Q * Q / (4199 * math.pi * ell)
