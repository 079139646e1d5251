"""The transfer plan's host logic on the CPU: csrc/transfer.cpp built into a
library of its own over a host stand-in for the CUDA runtime
(tests/host_stub/cuda_stub.cpp), whose "device" buffers are host memory and
whose copies are logged. Against the oracle: the classification of the
ball's elements (host_elements, src/transfer.jl:1380-1415), every point and
weight of the nested rule as the plan lays them out in innermost lines
(:1302-1328), the pairing's support elements, compact points and node
gathers (:1449-1500, :1726-1797), and the refusals, with the reference's
first-run counts."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import transfer as T

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "treewaveoldg.jl_gb300", "csrc")


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "include", "cuda_runtime_api.h")):
            return os.path.join(base, "include")
    return None


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    gxx, inc = shutil.which("g++"), _cuda_include()
    if not gxx or not inc:
        pytest.skip("needs g++ and the CUDA runtime headers")
    out = str(tmp_path_factory.mktemp("transfer_host") / "libtransfer_host.so")
    subprocess.run([gxx, "-O1", "-std=c++17", "-shared", "-fPIC", "-pthread", "-I" + inc,
                    os.path.join(ROOT, "tests", "host_stub", "cuda_stub.cpp"), os.path.join(CSRC, "transfer.cpp"),
                    os.path.join(CSRC, "tables.cpp"), "-o", out], check=True, capture_output=True, timeout=600)
    lib = ctypes.CDLL(out)
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    for name, res, args in (("twoldg_transfer_plan_create", ctypes.c_int, [vp, vp, vp]),
                            ("twoldg_transfer_plan_update", ctypes.c_int, [vp, vp, i32]),
                            ("twoldg_transfer_plan_destroy", ctypes.c_int, [vp]),
                            ("twoldg_transfer_plan_counts", ctypes.c_int, [vp, vp]),
                            ("twoldg_support_elements", ctypes.c_int, [vp, i32, vp, vp]),
                            ("stub_set_shape", None, [ctypes.c_int] * 5),
                            ("stub_last_error", ctypes.c_char_p, []),
                            ("stub_reset_uploads", None, []),
                            ("stub_nuploads", i64, []),
                            ("stub_upload_size", i64, [i64]),
                            ("stub_upload_data", vp, [i64])):
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args
    return lib


class Plan:
    """A plan of the host-only library over the oracle's brick mesh."""

    def __init__(self, lib, mesh, supports, ball, he, rnear=1.0, prec=0):
        from twoldg import _lib
        self.lib = lib
        lib.stub_set_shape(mesh.D, mesh.P, mesh.E, prec, mesh.nblocks)
        self._keep = [np.ascontiguousarray(mesh.origins.reshape(-1), dtype=np.float64),
                      np.ascontiguousarray(mesh.spacings, dtype=np.float64)]
        d = _lib.TransferDesc()
        dp = ctypes.POINTER(ctypes.c_double)
        d.origins = self._keep[0].ctypes.data_as(dp)
        d.spacings = self._keep[1].ctypes.data_as(dp)
        d.h_e = he
        for k in range(mesh.D):
            d.ball_centre[k] = ball[0][k]
        d.ball_radius = ball[1]
        self.parts = self._particles(supports)
        d.particles = ctypes.cast(self.parts, ctypes.POINTER(_lib.Particle))
        d.nparticles = len(supports)
        d.rnear = rnear
        self.desc = d
        self.h = ctypes.c_void_p()
        self.rc = lib.twoldg_transfer_plan_create(ctypes.c_void_p(1), ctypes.byref(d), ctypes.byref(self.h))

    @staticmethod
    def _particles(supports):
        from twoldg import _lib
        arr = (_lib.Particle * max(1, len(supports)))()
        for i, s in enumerate(supports):
            for d in range(3):
                arr[i].z[d] = s.z[d] if d < len(s.z) else 0.0
                arr[i].v[d] = s.v[d] if d < len(s.v) else 0.0
            arr[i].ell = s.ell
            arr[i].charge = 1.0
        return arr

    def update(self, supports):
        self.parts = self._particles(supports)
        return self.lib.twoldg_transfer_plan_update(self.h, self.parts, len(supports))

    def counts(self):
        c = (ctypes.c_int64 * 8)()
        assert self.lib.twoldg_transfer_plan_counts(self.h, c) == 0
        return list(c)

    def close(self):
        self.lib.twoldg_transfer_plan_destroy(self.h)


def _uploads(lib):
    out = []
    for i in range(lib.stub_nuploads()):
        n = lib.stub_upload_size(i)
        out.append(ctypes.string_at(lib.stub_upload_data(i), n))
    return out


def _same_rule(X, W, RX, RW):
    """The plan's points and weights against the oracle's. The two restate
    the support's breakpoints with their own roundings, and where a line only
    grazes the support (the discriminant nearly zero) the square root carries
    that into the breakpoint: coordinates agree to 1e-13, and the weights of
    the segments that rounding cuts to a sliver (down to 1e-27 here) agree to
    1e-13 of the largest weight, not of their own."""
    assert X.shape == RX.shape
    assert np.abs(X - RX).max() <= 1e-13
    assert np.abs(W - RW).max() <= 1e-13 * np.abs(RW).max()


def _lines_points(lx, lw, vals, lines):
    """Every point (prefix0, prefix1, x) and weight of a plan's innermost lines."""
    X, W = [], []
    for l in range(len(lines)):
        p0, p1 = lines[l]
        pre0, pre1, wl = vals[3 * l:3 * l + 3]
        X.append(np.stack([np.full(p1 - p0, pre0), np.full(p1 - p0, pre1), lx[p0:p1]], axis=1))
        W.append(wl * lw[p0:p1])
    return np.concatenate(X), np.concatenate(W)


def _two_particles():
    return [T.Support(np.array([0.41, 0.52, 0.47]), np.array([0.1, 0.0, 0.0]), 0.02),
            T.Support(np.array([0.7, 0.33, 0.61]), np.array([0.0, -0.2, 0.05]), 0.015)]


def test_plan_classifies_and_lists_the_nested_rule_as_the_oracle(host):
    mesh = T.brick_mesh(3, 3, 2, 2)
    t = T.Tables(3)
    he, ball = 0.25, ((0.5, 0.5, 0.5), 0.6)
    supports = _two_particles()
    plan = Plan(host, mesh, supports, ball, he)
    assert plan.rc == 0, host.stub_last_error()
    far, graded, near = T.classify(mesh, t, supports, ball, 1.0, he)
    c = plan.counts()
    assert c[0] == len(far) and c[1] == len(far) * 6 ** 3
    assert c[2] == sum(len(g) for g in graded)
    assert c[3] == sum(len(g) * len(r[0]) ** 3 for g, r in zip(graded, t.graded))
    assert c[4] == len(near)
    # the update's uploads: the rule elements, then the points' last
    # coordinates and weights, the lines' values and the lines
    host.stub_reset_uploads()
    assert plan.update(supports) == 0
    ups = _uploads(host)
    npts = c[5]
    i = next(k for k in range(len(ups) - 1) if len(ups[k]) == len(ups[k + 1]) == 8 * npts)
    lx, lw = np.frombuffer(ups[i], np.float64), np.frombuffer(ups[i + 1], np.float64)
    vals = np.frombuffer(ups[i + 2], np.float64)
    lines = np.frombuffer(ups[i + 3], np.int32).reshape(-1, 2)
    assert len(vals) == 3 * len(lines)
    X, W = _lines_points(lx, lw, vals, lines)
    RX, RW = [], []
    for b, e, k in near:
        lo, hi = mesh.element_box(b, e)
        x, w = T.nested_points(supports[k], t, lo, hi, 3)
        RX.append(x)
        RW.append(w)
    _same_rule(X, W, np.concatenate(RX), np.concatenate(RW))
    plan.close()


def test_plan_has_the_reference_first_run_counts(host):
    # the first run's window (bin/projection.jl): 31 102 far elements, the
    # reference's own count at h_e = d/8 (CODE.md "Quadrature")
    import math
    he = 0.125
    mesh = T.brick_mesh(3, 3, 4, 10, L=5.0)
    c = np.array([2.5, 2.5, 2.5])
    off = np.array([0.31, 0.17, 0.43]) * he
    supports = [T.Support(c + np.array([0.5, 0, 0]) + off, np.array([0.0, 0.2, 0.0]), 1e-3),
                T.Support(c - np.array([0.5, 0, 0]) + off, np.array([0.0, -0.2, 0.0]), 1e-3)]
    plan = Plan(host, mesh, supports, (c, 2.5), he)
    assert plan.rc == 0, host.stub_last_error()
    counts = plan.counts()
    assert counts[0] == 31102 and counts[1] == 31102 * 216
    assert counts[2] == 134 + 266 + 438 + 5240 and counts[4] == 44
    assert counts[3] == 134 * 14 ** 3 + 266 * 10 ** 3 + 438 * 8 ** 3 + 5240 * 7 ** 3
    assert math.isclose(counts[7], counts[1] + counts[3] + counts[5])
    plan.close()


def test_pairing_supports_points_and_gathers_are_the_oracle(host):
    mesh = T.brick_mesh(3, 3, 2, 4)
    t = T.Tables(3)
    he = 0.125
    ell = 0.05 * he
    supports = [T.Support(np.array([0.5 + 0.3 * ell, 0.5 - 0.2 * ell, 0.5 + 0.1 * ell]), np.array([0.2, -0.1, 0.05]),
                          ell),
                T.Support(np.array([0.3, 0.375 - 0.4 * ell, 0.7]), np.array([-0.2, 0.1, -0.05]), ell)]
    plan = Plan(host, mesh, supports, ((0.5, 0.5, 0.5), 0.6), he)
    assert plan.rc == 0, host.stub_last_error()
    host.stub_reset_uploads()
    elems = []
    for k, s in enumerate(supports):
        out = (ctypes.c_int32 * 32)()
        n = ctypes.c_int32()
        assert host.twoldg_support_elements(plan.h, k, out, ctypes.byref(n)) == 0
        got = [(out[4 * i], (out[4 * i + 1], out[4 * i + 2], out[4 * i + 3])) for i in range(n.value)]
        assert got == T.support_elements(mesh, s, he)
        elems += [(b, e, k) for b, e in got]
    # the build's uploads: barycentric weights, nodes, the elements, the
    # points' last coordinates and weights, the lines' values, the lines,
    # the chunks, the plain gather and the continuous one
    ups = _uploads(host)
    lx, lw = np.frombuffer(ups[3], np.float64), np.frombuffer(ups[4], np.float64)
    vals = np.frombuffer(ups[5], np.float64)
    lines = np.frombuffer(ups[6], np.int32).reshape(-1, 2)
    X, W = _lines_points(lx, lw, vals, lines)
    RX, RW = [], []
    for b, e, k in elems:
        lo, hi = mesh.element_box(b, e)
        x, w = T.nested_points(supports[k], t, lo, hi, 3, compact=True)
        RX.append(x)
        RW.append(w)
    _same_rule(X, W, np.concatenate(RX), np.concatenate(RW))
    M = 64
    plain = np.frombuffer(ups[8], np.int64).reshape(len(elems), M, 8)
    cont = np.frombuffer(ups[9], np.int64).reshape(len(elems), M, 8)
    u = np.sin(np.arange(mesh.nblocks * 2 * mesh.NN) * 0.37)
    for i, (b, e, _) in enumerate(elems):
        assert np.array_equal(plain[i, :, 0], mesh.node_index(b, e, 1)) and np.all(plain[i, :, 1:] == -1)
        avg = np.array([sum(u[o] for o in row if o >= 0) / sum(1 for o in row if o >= 0) for row in cont[i]])
        assert np.array_equal(avg, T.continuous_values(u, mesh, b, e, 1))
    plan.close()


def test_plan_refusals_on_the_host(host):
    mesh = T.brick_mesh(3, 3, 2, 1)
    he = 0.5
    a = T.Support(np.array([0.26, 0.26, 0.26]), np.zeros(3), 0.02)
    b = T.Support(np.array([0.27, 0.27, 0.27]), np.zeros(3), 0.02)
    plan = Plan(host, mesh, [a, b], ((0.5, 0.5, 0.5), 1.0), he)
    assert plan.rc == 1 and b"two particles" in host.stub_last_error()
    plan = Plan(host, mesh, [T.Support(np.array([0.3, 0.3, 0.3]), np.zeros(3), 0.3)], ((0.3, 0.3, 0.3), 0.5), he)
    assert plan.rc == 0
    out = (ctypes.c_int32 * 32)()
    n = ctypes.c_int32()
    assert host.twoldg_support_elements(plan.h, 0, out, ctypes.byref(n)) == 1
    assert b"not smaller than an element" in host.stub_last_error()
    assert plan.update([T.Support(np.array([0.01, 0.3, 0.3]), np.zeros(3), 0.02)]) == 0
    assert host.twoldg_support_elements(plan.h, 0, out, ctypes.byref(n)) == 1
    assert b"periodic images" in host.stub_last_error()
    plan.close()
