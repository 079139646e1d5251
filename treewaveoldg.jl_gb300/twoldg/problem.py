"""WaveProblem and its operations, over libtwoldg.

Mirrors the reference's evolution and stepping API (src/evolution.jl,
src/stepping.jl): WaveProblem, initial_state, wave_rhs, truncate_state,
truncate_stage, wave_energy, wave_norm, quadrature_norm, oldg_timestep,
wave_integrator. State vectors are CUDA tensors (torch is the device
memory allocator only) in the reference's state layout (N^D, 2, nblocks),
column-major, u then v per block; every operation runs in libtwoldg.
"""
import ctypes
import math

import numpy as np

from . import _lib
from .element import Element

_PREC = {"f64": _lib.F64, "f32": _lib.F32, "f32c": _lib.F32C}


def _torch():
    import torch
    return torch


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def check_layout(forest, el):
    """check_layout (src/layout.jl:31-47)."""
    P1 = el.P + 1
    if forest.N % P1:
        raise ValueError("the block size N = %d is not a whole number of elements of order P = %d, which hold "
                         "%d nodes each: choose N = E*%d for some even number of elements E per block"
                         % (forest.N, el.P, P1, P1))
    E = forest.N // P1
    if E % 2:
        raise ValueError("the block size N = %d holds E = %d elements of order P = %d, and E must be even: a "
                         "block of a refined forest covers half of its parent, and has to cover whole "
                         "elements of it, so N must be a multiple of 2(P+1) = %d" % (forest.N, E, el.P, 2 * P1))


def make_desc(forest, el, truncate, precision, metric=None):
    """The twoldg_desc of a forest (and of a diagonal metric's tables, from
    geometry.metric_tables); returns (desc, keepalive arrays)."""
    D = forest.D
    levels = np.array([lv for lv, _ in forest.leaves], dtype=np.int32)
    corners = np.array([c for _, c in forest.leaves], dtype=np.int64).reshape(-1)
    d = _lib.Desc()
    d.dim = D
    d.order = el.P
    d.elems = forest.N // (el.P + 1)
    d.precision = precision
    d.truncate = 1 if truncate else 0
    d.nblocks = len(forest.leaves)
    for k in range(3):
        d.roots[k] = forest.roots[k] if k < D else 1
        d.periodic[k] = int(forest.periodic[k]) if k < D else 1
        d.reflecting[k] = int(forest.reflecting[k]) if k < D else 0
        d.lo[k] = forest.lo[k] if k < D else 0.0
        d.hi[k] = forest.hi[k] if k < D else 1.0
    d.level = levels.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    d.corner = corners.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    keep = [levels, corners]
    if metric is not None:
        coef, modes, duals = metric[:3]
        dp = ctypes.POINTER(ctypes.c_double)
        d.coef = coef.ctypes.data_as(dp)
        d.trunc_modes = modes.ctypes.data_as(dp)
        d.trunc_duals = duals.ctypes.data_as(dp)
        keep += [coef, modes, duals]
    return d, tuple(keep)


class WaveProblem:
    """WaveProblem(forest, el; truncate=true) (src/evolution.jl:1043-1108).

    `precision` selects the device arithmetic: "f64" (the element's type must
    be float64), "f32" or "f32c" (float32 element; "f32c" adds the compensated
    RK4 accumulation). By default it follows the element's type.
    """

    def __init__(self, forest, el, truncate=True, precision=None, device="cuda", geometry=None, boundary=None):
        check_layout(forest, el)
        if precision is None:
            precision = "f64" if el.T == np.float64 else "f32"
        if precision not in _PREC:
            raise ValueError("precision must be one of %s" % sorted(_PREC))
        want = np.float64 if precision == "f64" else np.float32
        if el.T != want:
            raise ValueError("precision %s runs on a %s element, got %s" % (precision, np.dtype(want).name, el.T))
        self.forest = forest
        self.element = el
        self.truncate = bool(truncate)
        self.precision = precision
        self.D = forest.D
        self.P = el.P
        self.N = forest.N
        self.E = forest.N // (el.P + 1)
        self.nblocks = forest.nleaves()
        self.NN = self.N ** self.D
        self.dtype = el.T
        self.device = device
        self.geometry = geometry
        self.boundary = boundary
        self.metric = None
        self.hspeed = None
        self.full = False
        from .ball import BallForest
        if isinstance(forest, BallForest):
            # a full-metric geometry with glue (the seven-patch ball): Dirichlet data required
            from .ball import ball_desc, ball_tables
            if boundary is None:
                raise ValueError("the geometry has outer faces, and no data were given for them: pass "
                                 "boundary = PlaneWave(k, phi), the Dirichlet data on the sphere, or a "
                                 "RadiativeBoundary")
            self.full = True
            self.metric = ball_tables(forest, el.P, boundary)
            self.hspeed = self.metric["hspeed"]
            self._desc, self._keep = ball_desc(forest, el.P, truncate, _PREC[precision], self.metric, boundary)
        else:
            if boundary is not None:
                raise ValueError("Dirichlet data (boundary) are taken by a full geometry only")
            if geometry is not None:
                from .geometry import metric_tables
                self.metric = metric_tables(forest, Element(np.float64, el.P), geometry)
                self.hspeed = self.metric[3]
            self._desc, self._keep = make_desc(forest, el, truncate, _PREC[precision], self.metric)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().twoldg_problem_create(ctypes.byref(self._desc), ctypes.byref(h)))
        self._h = h
        w = ctypes.c_int64()
        _lib.check(_lib.lib().twoldg_state_words(h, ctypes.byref(w)))
        self.state_words = w.value
        self._bnd = None
        from .ball import DirichletData
        if self.full and isinstance(boundary, DirichletData):
            n = ctypes.c_int32()
            _lib.check(_lib.lib().twoldg_boundary_faces(h, None, ctypes.byref(n)))
            slots = np.zeros(max(1, n.value), dtype=np.int32)
            _lib.check(_lib.lib().twoldg_boundary_faces(h, slots.ctypes.data_as(ctypes.c_void_p), ctypes.byref(n)))
            F = self.N ** 2
            X = np.asarray(self.metric["bnd_x"]).reshape(-1, 3, F)[slots[:n.value]]
            # the boundary face nodes' positions, (3, nbf F): face by face
            self._bnd = np.ascontiguousarray(X.transpose(1, 0, 2).reshape(3, -1))
            self._bnd_table = None

    # the most levels one table holds: a longer run is stepped in chunks
    BOUNDARY_CHUNK_STEPS = 256

    def boundary_window(self, t0, dt, nlevels):
        """Boundary kind 2: the caller's Dirichlet data at the boundary face
        nodes for the times t0 + k dt/2, k < nlevels, as the device table the
        library reads (u and the three gradient components per face)."""
        torch = _torch()
        if self._bnd is None:
            return
        F = self.N ** 2
        nbf = self._bnd.shape[1] // F
        table = np.empty((nlevels, 4, nbf, F))
        for k in range(nlevels):
            u, g = self.boundary.data(self._bnd, t0 + k * (0.5 * dt))
            table[k, 0] = np.asarray(u).reshape(nbf, F)
            table[k, 1:] = np.asarray(g).reshape(3, nbf, F)
        dev = torch.from_numpy(np.ascontiguousarray(table.transpose(0, 2, 1, 3))).to(self.device)
        self.synchronize()            # the table it replaces is read no more
        self._bnd_table = dev
        _lib.check(_lib.lib().twoldg_set_boundary_values(self.handle, _dptr(dev), int(nlevels), float(t0),
                                                         float(dt)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().twoldg_problem_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def torch_dtype(self):
        torch = _torch()
        return torch.float64 if self.dtype == np.float64 else torch.float32

    def statevector(self):
        torch = _torch()
        return torch.zeros(self.state_words, dtype=self.torch_dtype(), device=self.device)

    def statearray(self, u):
        """The (nblocks, 2, N^D) view of a state vector (row-major view of the
        column-major (N^D, 2, nblocks) layout)."""
        return u.view(self.nblocks, 2, self.NN)

    def node_coordinates(self):
        """Positions of every owned node, shape (nblocks, D, N^D), in the
        element's type: lo + h (B N + q(P+1) + offsets[i]) per dimension
        (src/layout.jl:59-76), with B the block's integer corner; on the ball,
        the physical positions of the patches' nodes."""
        T = self.dtype.type
        if self.full:
            xl = self.metric["xl"]
            out = np.empty(xl.shape, dtype=self.dtype)
            for b, (p, c) in enumerate(self.forest.blocks):
                x = self.forest.geo.position(tuple(xl[b, k] for k in range(3)), p)
                for k in range(3):
                    out[b, k] = np.asarray(x[k])
            return out
        P1 = self.P + 1
        n = np.arange(self.N)
        local = (n // P1) * P1  # element start, integer
        offs = self.element.offsets[n % P1]
        out = np.empty((self.nblocks, self.D, self.NN), dtype=self.dtype)
        grids = np.indices([self.N] * self.D).reshape(self.D, -1)[::-1]  # dim 0 fastest
        for b, (lv, c) in enumerate(self.forest.leaves):
            h = T(self.forest.spacing((lv, c)))
            for k in range(self.D):
                ints = (c[k] * self.N + local).astype(self.dtype)
                x1 = T(self.forest.lo[k]) + h * (ints + offs)
                out[b, k] = x1[grids[k]]
        return out

    def fill_at_nodes(self, f):
        """Host array (nblocks, 2, N^D) of f(x, var) at the nodes; f takes a
        tuple of D coordinate arrays and var in (1, 2)."""
        x = self.node_coordinates()
        out = np.empty((self.nblocks, 2, self.NN), dtype=self.dtype)
        xs = tuple(x[:, k, :] for k in range(self.D))
        out[:, 0, :] = f(xs, 1)
        out[:, 1, :] = f(xs, 2)
        return out

    def to_device(self, host):
        torch = _torch()
        return torch.from_numpy(np.ascontiguousarray(host).reshape(-1)).to(self.device)

    def synchronize(self):
        _lib.check(_lib.lib().twoldg_synchronize(self._h))

    def autotune(self, u, dt, cache=None):
        """Time the stage kernel's launch layouts (kernel, threads per CTA,
        grid) of every (dim, P, E) group on u, which is not changed, with step
        dt, and keep the fastest for later steps; cache: a JSON file of
        earlier choices, read and extended. Returns {group key: choice}."""
        _check_state(self, u)
        _torch().cuda.synchronize()
        buf = ctypes.create_string_buffer(1 << 16)
        _lib.check(_lib.lib().twoldg_autotune(self._h, ctypes.c_void_p(u.data_ptr()), float(dt),
                                              None if cache is None else str(cache).encode(), buf, len(buf)))
        return _lib.tune_report(buf.value.decode())


def _check_state(p, u):
    torch = _torch()
    if not isinstance(u, torch.Tensor) or not u.is_cuda:
        raise ValueError("state vectors are CUDA tensors")
    if u.dtype != p.torch_dtype() or u.numel() != p.state_words or not u.is_contiguous():
        raise ValueError("the state vector has %d entries of %s but the problem's blocks hold %d of %s"
                         % (u.numel(), u.dtype, p.state_words, p.torch_dtype()))


def _sync_torch():
    _torch().cuda.synchronize()


def initial_state(p, f):
    """initial_state(p, f) (src/evolution.jl:1440-1445): f at the nodes, v truncated."""
    u = p.to_device(p.fill_at_nodes(f))
    return truncate_state(u, p)


def wave_rhs(du, u, p, t=0.0):
    """wave_rhs!(du, u, p, t) (src/evolution.jl:1367-1371)."""
    _check_state(p, u)
    _check_state(p, du)
    if p._bnd is not None:
        p.boundary_window(float(t), 1.0, 1)
    _sync_torch()
    _lib.check(_lib.lib().twoldg_rhs(p.handle, _dptr(du), _dptr(u), float(t)))
    p.synchronize()
    return du


def truncate_state(u, p):
    """truncate_state!(u, p) (src/evolution.jl:1383-1395)."""
    _check_state(p, u)
    _sync_torch()
    _lib.check(_lib.lib().twoldg_truncate(p.handle, _dptr(u)))
    p.synchronize()
    return u


def truncate_stage(u, integrator, p, t):
    """truncate_stage!(u, integrator, p, t) (src/evolution.jl:1427-1430)."""
    truncate_state(u, p)


def wave_energy(p, u, t=None):
    """wave_energy(p, u) (src/evolution.jl:1472-1489), accumulated in FP64."""
    _check_state(p, u)
    if p._bnd is not None:
        p.boundary_window(0.0 if t is None else float(t), 1.0, 1)
    _sync_torch()
    e = ctypes.c_double()
    _lib.check(_lib.lib().twoldg_energy(p.handle, _dptr(u), 0.0 if t is None else float(t), ctypes.byref(e)))
    return e.value


def _vars_mask(vars):
    mask = 0
    for v in vars:
        if v not in (1, 2):
            raise ValueError("vars selects 1 (u) and/or 2 (v), got %r" % (vars,))
        mask |= 1 << (v - 1)
    return mask


def quadrature_norm(p, u, pnorm=2, vars=(1, 2), ref=None):
    """quadrature_norm(fs, el, u; p, vars) (src/layout.jl:223-235); of u - ref
    when ref is given. pnorm is an integer >= 1 or math.inf."""
    _check_state(p, u)
    if ref is not None:
        _check_state(p, ref)
    if math.isinf(pnorm):
        pi = 0
    else:
        if pnorm != int(pnorm) or pnorm < 1:
            raise ValueError("quadrature_norm takes an integer p >= 1 or Inf, got p = %r" % (pnorm,))
        pi = int(pnorm)
    _sync_torch()
    out = ctypes.c_double()
    _lib.check(_lib.lib().twoldg_norm(p.handle, _dptr(u), _dptr(ref) if ref is not None else None, pi,
                                      _vars_mask(vars), ctypes.byref(out)))
    return out.value


def wave_norm(p, u, pnorm=2, vars=(1, 2)):
    """wave_norm(p, u; p, vars) (src/evolution.jl:1498-1512), flat problems."""
    return quadrature_norm(p, u, pnorm, vars)


def oldg_timestep(p, cfl):
    """oldg_timestep(p; cfl) = cfl h_min / (P+1) (src/evolution.jl:1528-1531),
    in T; on a geometry h_min is the smallest block spacing over the block's
    largest logical wave speed."""
    T = p.dtype.type
    h = p.forest.minimum_spacing() if p.hspeed is None else p.hspeed
    return T(cfl) * T(h) / T(p.P + 1)


def chunk_count(T, span, chunk):
    """ceil(span / chunk), except that a quotient within a few ulp of an
    integer m gives m (src/precision.jl:30-49, chunk_count), in type T."""
    T = np.dtype(T).type
    r = T(T(span) / T(chunk))
    m = np.round(r)
    tol = 4 * (np.spacing(r) + np.spacing(T(span)) / T(chunk))
    if m >= 1 and abs(r - m) <= tol:
        return int(m)
    return int(math.ceil(r))


class WaveIntegrator:
    """The RK4 integrator of wave_integrator (src/stepping.jl:72-78):
    truncation as stage and step limiter, fixed dt, ceil((t1-t0)/dt) steps.
    step() advances one step and solve() to t1, each as fused CUDA-graph
    steps in libtwoldg."""

    def __init__(self, p, u0, t0, t1, dt, alias_u0=False):
        _check_state(p, u0)
        self.p = p
        self.u = u0 if alias_u0 else u0.clone()
        self.t0 = float(t0)
        self.t = float(t0)
        self.t1 = float(t1)
        self.dt = float(dt)
        self.nsteps = chunk_count(p.dtype.type, float(t1) - float(t0), float(dt))
        self.nstep = 0

    def _advance(self, n):
        if n <= 0:
            return
        if self.p._bnd is not None:
            # the caller's Dirichlet data, chunk by chunk of steps
            while n > 0:
                m = min(n, self.p.BOUNDARY_CHUNK_STEPS)
                self.p.boundary_window(self.t, self.dt, 2 * m + 1)
                self._steps(m)
                n -= m
            return
        self._steps(n)

    def _steps(self, n):
        _sync_torch()
        _lib.check(_lib.lib().twoldg_rk4_step(self.p.handle, _dptr(self.u), self.t, self.dt, int(n)))
        self.p.synchronize()
        self.nstep += n
        self.t = self.t0 + self.nstep * self.dt

    def step(self):
        self._advance(1)
        return self

    def solve(self):
        self._advance(self.nsteps - self.nstep)
        return self


def wave_integrator(p, u0, t0, t1, dt, alias_u0=False):
    """wave_integrator(p, u0, t0, t1; dt) (src/stepping.jl:72-78)."""
    return WaveIntegrator(p, u0, t0, t1, dt, alias_u0=alias_u0)


def solve(integ):
    return integ.solve()


__all__ = ["WaveProblem", "Element", "initial_state", "wave_rhs", "truncate_state", "truncate_stage",
           "wave_energy", "wave_norm", "quadrature_norm", "oldg_timestep", "wave_integrator", "solve",
           "check_layout"]
