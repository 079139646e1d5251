"""The modal refinement indicator (src/refinement.jl:56-179), over libtwoldg."""
import ctypes

from . import _lib
from .problem import _check_state, _dptr, _sync_torch


def _tau(p):
    torch = __import__("torch")
    return torch.empty((p.nblocks,) + (p.E,) * p.D, dtype=p.torch_dtype(), device=p.device)


def modal_indicator(p, u, mode, var=1):
    """modal_indicator(fs, el; mode, var) (src/refinement.jl:147-155): tau per
    element, shape (nblocks, E, ..., E) with the last axis the first
    dimension (the element index e1 fastest in memory)."""
    _check_state(p, u)
    if mode < 1 or mode > p.P:
        raise ValueError("mode = %r must be one of 1 .. P = %d: mode 0, an element's mean, says nothing "
                         "about resolution" % (mode, p.P))
    if p.truncate and p.P == 1:
        raise ValueError("the truncated scheme at P = 1 has no mode that moves with the solution")
    tau = _tau(p)
    _sync_torch()
    _lib.check(_lib.lib().twoldg_modal_indicator(p.handle, _dptr(u), int(var), int(mode), _dptr(tau)))
    p.synchronize()
    return tau


def mode_amplitude(p, u, mode, var=1):
    """mode_amplitude(fs, el; mode, var) (src/refinement.jl:169-175)."""
    _check_state(p, u)
    tau = _tau(p)
    _sync_torch()
    _lib.check(_lib.lib().twoldg_mode_amplitude(p.handle, _dptr(u), int(var), int(mode), _dptr(tau)))
    p.synchronize()
    return tau
