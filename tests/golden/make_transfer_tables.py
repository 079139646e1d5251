"""Generate tests/golden/transfer_tables.json: the particle-grid transfer's tables.

A restatement, in mpmath at 512 bits, of the reference's `gauss_nodes_weights(n)`
and `TransferTables(T, P)` (src/transfer.jl:44-62 and :139-170): Gauss-Legendre
nodes by Newton's iteration on L_n from the Chebyshev points
-cos(pi (4i - 1) / (4n + 2)), symmetrised, weights 2 / ((1 - x^2) L_n'(x)^2);
the barycentric weights of the Gauss-Lobatto nodes; the Lagrange table at a
rule's points and its contraction w_k phi_i(x_k) / w^_i. Every entry is rounded
once to float64 and float32, which is what the reference's test "The tables are
the BigFloat ones, rounded once" (test/transfer_tests.jl:78-106) pins.

The fixture anchors the native library's double-double builder (bit equality in
tests/test_transfer.py) and feeds the transfer oracle (oracle/transfer.py). Run
from the repository root:

    python tests/golden/make_transfer_tables.py
"""
import json
import os
import struct
import sys

import mpmath
from mpmath import mp, mpf

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from make_tables import PREC, f32_bits as bits32, gll_nodes_weights, legendre_all  # noqa: E402

# every rule size the tests and the oracle use: the far rule q = P + 3 for
# P = 1..6, the graded bands (14, 10, 8, 7), the nested rule's lines (48, 16,
# 24), the exactness pins (1, 2, 5, 12) and a reference rule (32)
RULES = sorted({1, 2, 5, 12, 4, 6, 7, 8, 9, 10, 14, 16, 24, 32, 48, 40, 56, 80})
ORDERS = (1, 2, 3, 4, 5, 6)


def gauss_nodes_weights(n):
    x = [-mpmath.cos(mp.pi * (4 * i - 1) / (4 * n + 2)) for i in range(1, n + 1)]
    tol = mpmath.ldexp(mpf(1), 8 - PREC)

    def value_and_slope(t):
        L = legendre_all(n, t)
        return L[n], n * (t * L[n] - L[n - 1]) / (t * t - 1)

    for _ in range(200):
        delta = []
        for t in x:
            L, dL = value_and_slope(t)
            delta.append(L / dL)
        x = [t - d for t, d in zip(x, delta)]
        if max(abs(d) for d in delta) <= tol:
            break
    x = [(x[i] - x[n - 1 - i]) / 2 for i in range(n)]
    w = [2 / ((1 - t * t) * value_and_slope(t)[1] ** 2) for t in x]
    return x, w


def bits64(v):
    return struct.unpack("<Q", struct.pack("<d", float(v)))[0]


def main():
    mp.prec = PREC
    rules = {}
    for n in RULES:
        x, w = gauss_nodes_weights(n)
        rules[str(n)] = {"nodes": {"f64": [bits64(v) for v in x], "f32": [bits32(v) for v in x]},
                         "weights": {"f64": [bits64(v) for v in w], "f32": [bits32(v) for v in w]}}
    orders = {}
    for P in ORDERS:
        xi, wh = gll_nodes_weights(P)
        P1 = P + 1
        bary = []
        for i in range(P1):
            p = mpf(1)
            for j in range(P1):
                if j != i:
                    p *= xi[i] - xi[j]
            bary.append(1 / p)
        tabs = {"bary": {"f64": [bits64(v) for v in bary], "f32": [bits32(v) for v in bary]}}
        for q in sorted({P + 3, 14, 10, 8, 7}):
            xg, wg = gauss_nodes_weights(q)
            lag = [[bary[i] * mpmath.fprod(xg[k] - xi[j] for j in range(P1) if j != i) for i in range(P1)]
                   for k in range(q)]
            con = [[wg[k] * lag[k][i] / wh[i] for k in range(q)] for i in range(P1)]
            tabs["lagrange_%d" % q] = {"f64": [[bits64(v) for v in row] for row in lag],
                                       "f32": [[bits32(v) for v in row] for row in lag]}
            tabs["contract_%d" % q] = {"f64": [[bits64(v) for v in row] for row in con],
                                       "f32": [[bits32(v) for v in row] for row in con]}
        orders[str(P)] = tabs
    out = {"generator": "tests/golden/make_transfer_tables.py", "precision_bits": PREC,
           "follows": "src/transfer.jl:44-62, 139-170", "rules": rules, "orders": orders}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "transfer_tables.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", path)


if __name__ == "__main__":
    main()
