"""The reference element: Element(T, P) of src/element.jl:58-170.

The tables are built by libtwoldg's double-double builder and rounded once
to T, as the reference rounds its BigFloat tables once
(test/element_tests.jl:122-137).
"""
import ctypes

import numpy as np

from . import _lib

_SIZES = {
    "nodes": lambda P: (P + 1,),
    "weights": lambda P: (P + 1,),
    "offsets": lambda P: (P + 1,),
    "stencil": lambda P: (P + 1, P + 3),
    "truncate": lambda P: (P + 1, P + 1),
    "topmode": lambda P: (P + 1,),
    "topdual": lambda P: (P + 1,),
    "duals": lambda P: (P + 1, P + 1),
    "prolong": lambda P: (2 * (P + 1), P + 1),
    "restrict": lambda P: (P + 1, 2 * (P + 1)),
}


def element_table(P, dtype, name):
    """One table of order P in dtype (float64 or float32), as a numpy array."""
    dtype = np.dtype(dtype)
    if dtype not in (np.dtype(np.float64), np.dtype(np.float32)):
        raise ValueError("element tables exist in float64 and float32, not %s" % dtype)
    if not isinstance(P, (int, np.integer)) or P < 1:
        raise ValueError("the element order P must be at least 1, got %r" % (P,))
    out = np.zeros(_SIZES[name](P), dtype=dtype)
    prec = 0 if dtype == np.float64 else 1
    _lib.check(_lib.lib().twoldg_element_tables(int(P), prec, name.encode(),
                                                out.ctypes.data_as(ctypes.c_void_p)))
    return out


class Element:
    """Element(T, P): nodes, weights, offsets, stencil, truncate, topmode,
    topdual, duals (src/element.jl:58-67), as numpy arrays of dtype T."""

    def __init__(self, T, P):
        self.T = np.dtype(T)
        self.P = int(P)
        for name in _SIZES:
            setattr(self, name if name != "restrict" else "restrict_", element_table(self.P, self.T, name))

    @property
    def order(self):
        return self.P

    def __repr__(self):
        return "Element(%s, %d)" % (self.T.name, self.P)
