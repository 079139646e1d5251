"""Generate tests/golden/element_tables.json: the OLDG reference-element tables.

This is a restatement, in mpmath at 512 bits, of the reference's `Element(T, P)`
and `gll_nodes_weights(P)` (src/element.jl:95-114 and :129-170), and of the
coarse-fine tangential operators `I` and `R = M_c^-1 I^T M_f` that TreeAMR's
element-local ghost operators use (documented in the reference's CODE.md,
"The coupling"). Every table is built in 512-bit arithmetic and rounded ONCE to
the target type (float64, and float32 with correct rounding), which is the
precision rule the reference's tests pin ("The tables are built once in
BigFloat and rounded once", test/element_tests.jl:122-137).

The fixture is the parity anchor for the native library's double-double table
builder (tests/test_tables.py asserts bit equality) and the source of tables
for the CPU oracle. Run from the repository root:

    python tests/golden/make_tables.py
"""
import json
import os
import struct

import mpmath
from mpmath import mp, mpf

PREC = 512
P_MAX = 8


def legendre_all(P, x):
    """L_0 .. L_P at x by the three-term recurrence (src/element.jl:72-80)."""
    L = [mpf(1)]
    if P >= 1:
        L.append(x)
    for k in range(2, P + 1):
        L.append(((2 * k - 1) * x * L[k - 1] - (k - 1) * L[k - 2]) / k)
    return L


def gll_nodes_weights(P):
    """Newton on (1-x^2) L_P' from Chebyshev-Gauss-Lobatto points, then
    symmetrised; endpoints exactly +-1 (src/element.jl:95-114)."""
    x = [-mpmath.cospi(mpf(i) / P) for i in range(P + 1)]
    tol = mpmath.ldexp(mpf(1), 8 - PREC)
    for _ in range(200):
        delta = []
        for xi in x:
            L = legendre_all(P, xi)
            delta.append((xi * L[P] - L[P - 1]) / ((P + 1) * L[P]))
        x = [xi - di for xi, di in zip(x, delta)]
        if max(abs(d) for d in delta) <= tol:
            break
    x = [(x[i] - x[P - i]) / 2 for i in range(P + 1)]
    x[0], x[P] = mpf(-1), mpf(1)
    w = [2 / (P * (P + 1) * legendre_all(P, xi)[P] ** 2) for xi in x]
    return x, w


def element_tables(P):
    """All tables of `Element(T, P)` in 512-bit precision (src/element.jl:129-170)."""
    xi, wh = gll_nodes_weights(P)
    P1 = P + 1
    Lall = [legendre_all(P, x) for x in xi]
    LP = [L[P] for L in Lall]
    d = [[mpf(0)] * P1 for _ in range(P1)]
    for i in range(P1):
        for j in range(P1):
            if i != j:
                d[i][j] = LP[i] / (LP[j] * (xi[i] - xi[j]))
    d[0][0] = -mpf(P) * (P + 1) / 4
    d[P][P] = mpf(P) * (P + 1) / 4
    # columns 0 .. P+2 are nodes -1 .. P+1
    W = [[mpf(0)] * (P1 + 2) for _ in range(P1)]
    for i in range(P1):
        for j in range(P1):
            W[i][j + 1] = 2 * d[i][j] / (P + 1)
    face = mpf(P) / 2
    W[0][1] += face
    W[0][0] -= face
    W[P][P1] -= face
    W[P][P1 + 1] += face
    gamma = sum(wh[i] * LP[i] ** 2 for i in range(P1))
    Pi = [[(mpf(1) if i == j else mpf(0)) - LP[i] * wh[j] * LP[j] / gamma
           for j in range(P1)] for i in range(P1)]
    duals = []
    for k in range(P1):
        g = sum(wh[i] * Lall[i][k] ** 2 for i in range(P1))
        duals.append([wh[j] * Lall[j][k] / g for j in range(P1)])
    topdual = [wh[j] * LP[j] / gamma for j in range(P1)]
    duals[P] = list(topdual)
    offsets = [(P + 1) * (1 + x) / 2 for x in xi]
    offsets[0], offsets[P] = mpf(0), mpf(P1)
    return dict(nodes=xi, weights=wh, offsets=offsets, stencil=W, truncate=Pi,
                topmode=LP, topdual=topdual, duals=duals)


def lagrange(xi, j, x):
    r = mpf(1)
    for k in range(len(xi)):
        if k != j:
            r *= (x - xi[k]) / (xi[j] - xi[k])
    return r


def coarse_fine(P):
    """Tangential coarse->fine prolongation I (2(P+1) x (P+1)): the coarse
    element's degree-P polynomial at the nodes of the two fine elements that
    cover it; and the restriction R = M_c^-1 I^T M_f ((P+1) x 2(P+1)), its
    adjoint in the face quadrature (reference CODE.md, "The coupling")."""
    xi, wh = gll_nodes_weights(P)
    P1 = P + 1
    I = [[mpf(0)] * P1 for _ in range(2 * P1)]
    for half in range(2):
        for i in range(P1):
            xc = (xi[i] - 1) / 2 if half == 0 else (xi[i] + 1) / 2
            for j in range(P1):
                I[half * P1 + i][j] = lagrange(xi, j, xc)
    # fine weights are h_f(P+1)/2 w, coarse h_c(P+1)/2 w with h_c = 2 h_f
    R = [[I[r][j] * wh[r % P1] / (2 * wh[j]) for r in range(2 * P1)]
         for j in range(P1)]
    return dict(prolong=I, restrict=R)


def f64_bits(x):
    return struct.unpack("<Q", struct.pack("<d", float(x)))[0]


def f32_bits(x):
    with mp.workprec(24):
        y = +x          # correctly rounded to 24 significant bits
    return struct.unpack("<I", struct.pack("<f", float(y)))[0]


def rounded(tabs, fn):
    out = {}
    for k, v in tabs.items():
        if isinstance(v[0], list):
            out[k] = [[fn(x) for x in row] for row in v]
        else:
            out[k] = [fn(x) for x in v]
    return out


def main():
    mp.prec = PREC
    doc = {"generator": "tests/golden/make_tables.py", "precision_bits": PREC,
           "follows": "src/element.jl:72-170 (Element, gll_nodes_weights, legendre_all)",
           "orders": {}}
    for P in range(1, P_MAX + 1):
        tabs = element_tables(P)
        tabs.update(coarse_fine(P))
        doc["orders"][str(P)] = {"f64": rounded(tabs, f64_bits),
                                 "f32": rounded(tabs, f32_bits)}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "element_tables.json")
    with open(path, "w") as f:
        json.dump(doc, f, separators=(",", ":"))
    print("wrote", path)


if __name__ == "__main__":
    main()
