"""Dense global operators on a periodic line, a numpy restatement of the
reference's test/reference.jl:9-54 (global_operators, along, global_array).
Test infrastructure: the reference the oracle's per-point loops are checked
against, built from the element's tables by a loop that shares nothing with
either implementation."""
import numpy as np


def global_operators(stencil, projector, weights, P, K, h):
    """The wide derivative Dm, projector Pim and quadrature weights w on a
    periodic line of K elements of spacing h."""
    P1 = P + 1
    n = K * P1
    Dm = np.zeros((n, n))
    Pim = np.zeros((n, n))
    w = np.zeros(n)
    for e in range(K):
        for i in range(P1):
            r = e * P1 + i
            w[r] = h * P1 / 2 * weights[i]
            for j in range(-1, P1 + 1):
                Dm[r, (e * P1 + j) % n] += stencil[i, j + 1] / h
            for j in range(P1):
                Pim[r, e * P1 + j] = projector[i, j]
    return Dm, Pim, w


def along(A, d, D):
    """A acting along dimension d of a D-dim array flattened with dim 0 fastest."""
    n = A.shape[0]
    I = np.eye(n)
    out = np.ones((1, 1))
    for e in range(D - 1, -1, -1):
        out = np.kron(out, A if e == d else I)
    return out


def global_array(forest, u, var):
    """Variable var (0 = u, 1 = v) of a state vector as one global array
    (flattened, dim 0 fastest) over a uniform box."""
    D, N = forest.D, forest.N
    n = forest.roots[0] * N
    nb = len(forest.leaves)
    ua = np.asarray(u).reshape(nb, 2, N ** D)
    A = np.zeros([n] * D)
    for b, (lv, c) in enumerate(forest.leaves):
        blk = ua[b, var].reshape([N] * D, order="F")
        sl = tuple(slice(c[k] * N, (c[k] + 1) * N) for k in range(D))
        A[sl] = blk
    return A.reshape(-1, order="F")


def from_global(forest, A, out, var):
    D, N = forest.D, forest.N
    n = forest.roots[0] * N
    Ag = np.asarray(A).reshape([n] * D, order="F")
    nb = len(forest.leaves)
    ua = out.reshape(nb, 2, N ** D)
    for b, (lv, c) in enumerate(forest.leaves):
        sl = tuple(slice(c[k] * N, (c[k] + 1) * N) for k in range(D))
        ua[b, var] = Ag[sl].reshape(-1, order="F")
    return out
