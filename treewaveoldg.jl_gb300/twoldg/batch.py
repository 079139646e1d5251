"""The batched ensemble over libtwoldg's twoldg_batch_* entry points: many
independent problems of uneven (P, E, roots) stepped together, one work list
per shape and up to 16 RK4 steps per CUDA graph launch. No reference counterpart:
the reference runs one forest per WaveProblem."""
import ctypes
import math

import numpy as np

from . import _lib
from .element import Element
from .forest import wave_forest
from .problem import WaveProblem, _PREC, make_desc


class Batch:
    """n problems (forests + orders) in one state buffer, FP64 or float32."""

    def __init__(self, members, precision="f64", truncate=True):
        """members: list of (forest, P)."""
        self.precision = precision
        self.dtype = np.float64 if precision == "f64" else np.float32
        self.members = members
        descs, self._keep = [], []
        for forest, P in members:
            d, k = make_desc(forest, Element(self.dtype, P), truncate, _PREC[precision])
            descs.append(d)
            self._keep.append(k)
        self._descs = (_lib.Desc * len(descs))(*descs)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().twoldg_batch_create(len(descs), self._descs, ctypes.byref(h)))
        self._h = h
        offs = (ctypes.c_int64 * len(descs))()
        total = ctypes.c_int64()
        _lib.check(_lib.lib().twoldg_batch_offsets(h, offs, ctypes.byref(total)))
        self.offsets = list(offs)
        self.total_words = total.value
        self.nodes = self.total_words // 2

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().twoldg_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def statevector(self):
        import torch
        return torch.zeros(self.total_words, dtype=torch.float64 if self.dtype == np.float64 else torch.float32,
                           device="cuda")

    def rk4_step(self, u, dts, nsteps):
        import torch
        torch.cuda.synchronize()
        arr = (ctypes.c_double * len(dts))(*[float(x) for x in dts])
        _lib.check(_lib.lib().twoldg_batch_rk4_step(self._h, ctypes.c_void_p(u.data_ptr()), arr, int(nsteps)))

    def synchronize(self):
        _lib.check(_lib.lib().twoldg_batch_synchronize(self._h))

    def stream(self):
        """The batch's CUDA stream as a torch ExternalStream (for events)."""
        import torch
        return torch.cuda.ExternalStream(_lib.lib().twoldg_batch_stream(self._h))

    def autotune(self, u, dts, cache=None):
        """Time the stage kernel's launch layouts of every shape group on u
        (unchanged) with steps dts and keep the fastest; cache: a JSON file of
        earlier choices, read and extended. Returns {group key: choice}."""
        import torch
        torch.cuda.synchronize()
        arr = (ctypes.c_double * len(dts))(*[float(x) for x in dts])
        buf = ctypes.create_string_buffer(1 << 16)
        _lib.check(_lib.lib().twoldg_batch_autotune(self._h, ctypes.c_void_p(u.data_ptr()), arr,
                                                    None if cache is None else str(cache).encode(), buf,
                                                    len(buf)))
        return _lib.tune_report(buf.value.decode())


def sine_ensemble(n, seed=0, dtype=np.float64, P_range=(2, 5), E_choices=(2, 4), roots_range=(4, 16)):
    """n 2D periodic problems: P uniform in P_range, E in E_choices, roots
    uniform in roots_range, each u = sum_j a_j sin(2 pi (m_j . x) + phi_j) over
    4 modes with a_j ~ U(-1, 1), m_j in {1..3}^2, phi_j ~ U(0, 2 pi), v = 0
    (numpy PCG64 with the given seed). Returns [(forest, P, f)]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        P = int(rng.integers(P_range[0], P_range[1] + 1))
        E = int(rng.choice(list(E_choices)))
        roots = int(rng.integers(roots_range[0], roots_range[1] + 1))
        a = rng.uniform(-1, 1, 4)
        m = rng.integers(1, 4, size=(4, 2))
        ph = rng.uniform(0, 2 * math.pi, 4)

        def f(x, var, a=a, m=m, ph=ph):
            s = np.zeros_like(x[0])
            if var == 1:
                for j in range(4):
                    s = s + a[j] * np.sin(2 * math.pi * (m[j, 0] * x[0] + m[j, 1] * x[1]) + ph[j])
            return s
        out.append((wave_forest(dtype, 2, P, E, roots=roots), P, f))
    return out


def fill_batch(batch, members):
    """The batch's state vector with every member's initial data (v truncated
    through each member's own problem)."""
    from .problem import initial_state
    u = batch.statevector()
    for k, (forest, P, f) in enumerate(members):
        p = WaveProblem(forest, Element(batch.dtype, P), precision=batch.precision)
        u0 = initial_state(p, f)
        u[batch.offsets[k]:batch.offsets[k] + u0.numel()] = u0
    return u
