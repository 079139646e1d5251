"""Host-side logic without a GPU: the C ABI's exports, forests, descriptors
and the library's argument checks (which run before any CUDA call)."""
import ctypes
import os
import re

import numpy as np
import pytest

import twoldg
from twoldg import _lib
from twoldg.forest import nested_cubes, wave_forest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "twoldg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(twoldg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_function():
    twoldg.build()
    L = ctypes.CDLL(twoldg.lib_path())
    declared = header_functions()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(_lib.EXPORTS) == declared


def test_nested_cubes_forest():
    # the 3D reflecting box with three nested levels: 448 + 448 + 512 blocks
    f = wave_forest(np.float64, 3, 3, 2, roots=8, reflecting=True, refined=nested_cubes(3, 1 / 8, 3))
    levels = [lv for lv, _ in f.leaves]
    assert [levels.count(k) for k in range(3)] == [448, 448, 512]
    assert f.minimum_spacing() == pytest.approx(1 / 256)


def test_refined_middle_and_balance():
    f = wave_forest(np.float64, 2, 3, 2, roots=4, refined=True)
    assert len(f.leaves) == 16 - 4 + 16
    # a region refining one corner block twice forces its neighbours (2:1)
    g = wave_forest(np.float64, 2, 1, 2, roots=4, refined=[((0.0, 0.25), (0.0, 0.25)), ((0.0, 0.125), (0.0, 0.125))])
    lv = {k: 0 for k in range(3)}
    for level, _ in g.leaves:
        lv[level] += 1
    assert lv[2] == 4
    with pytest.raises(ValueError):
        wave_forest(np.float64, 2, 3, 3, roots=4)         # odd E
    with pytest.raises(ValueError):
        wave_forest(np.float64, 2, 3, 2, roots=2, refined=True)  # no block centre in the middle half


def _create(desc):
    h = ctypes.c_void_p()
    return _lib.lib().twoldg_problem_create(ctypes.byref(desc), ctypes.byref(h))


def test_descriptor_errors_are_rejected_on_the_host():
    f = wave_forest(np.float64, 2, 3, 2, roots=2)
    d, keep = twoldg.problem.make_desc(f, twoldg.Element(np.float64, 3), True, _lib.F64)
    d.elems = 3
    assert _create(d) == _lib.TWOLDG_EINVAL
    assert b"even" in _lib.lib().twoldg_last_error()
    d.elems = 2
    d.periodic[0] = 0
    assert _create(d) == _lib.TWOLDG_EINVAL
    d.periodic[0] = 1
    d.dim = 4
    assert _create(d) == _lib.TWOLDG_EINVAL
    d.dim = 2
    d.precision = 7
    # precision is checked after the mesh, still before any device work
    assert _create(d) in (_lib.TWOLDG_EINVAL, _lib.TWOLDG_ECUDA)
    del keep


def test_unbalanced_forest_is_rejected():
    # a level-2 block beside a level-0 block
    d = _lib.Desc()
    d.dim, d.order, d.elems, d.precision, d.truncate = 1, 2, 2, _lib.F64, 1
    levels = np.array([0, 2, 2, 1, 0], dtype=np.int32)
    corners = np.array([0, 4, 5, 3, 2], dtype=np.int64)
    d.nblocks = 5
    d.roots[0], d.periodic[0] = 3, 1
    d.hi[0] = 1.0
    d.level = levels.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    d.corner = corners.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    assert _create(d) == _lib.TWOLDG_EINVAL
    assert b"balanced" in _lib.lib().twoldg_last_error()


def test_element_tables_reject_bad_orders():
    with pytest.raises(ValueError):
        twoldg.element_table(0, np.float64, "nodes")
    with pytest.raises(ValueError):
        twoldg.element_table(9, np.float64, "nodes")


def test_chunk_count():
    from twoldg.problem import chunk_count
    dt = 0.5 / 256 / 4
    assert chunk_count(np.float64, 5 * dt, dt) == 5
    assert chunk_count(np.float64, 0.33, 0.03) == 11
    assert chunk_count(np.float64, 1.0, 0.3) == 4


def test_sine_ensemble_is_seeded():
    a = twoldg.sine_ensemble(8, seed=0)
    b = twoldg.sine_ensemble(8, seed=0)
    assert [(f.N, P, len(f.leaves)) for f, P, _ in a] == [(f.N, P, len(f.leaves)) for f, P, _ in b]
    assert all(2 <= P <= 5 for _, P, _ in a)


def test_flat_kernels_refuse_a_face_table_or_a_bare_metric_kind():
    """The flat and diagonal kernels read a neighbour's face plane as it lies:
    a descriptor with an explicit face table (glued patches, boundary faces)
    but no full metric, or a metric kind without its coefficients, is refused
    before any device work, by the problem and by the static right-hand side."""
    f = wave_forest(np.float64, 3, 3, 4, roots=1)
    d, keep = twoldg.problem.make_desc(f, twoldg.Element(np.float64, 3), True, _lib.F64)
    nb = np.full(6, -1, dtype=np.int32)
    code = np.zeros(6, dtype=np.int32)
    d.face_nb = nb.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    d.face_code = code.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    assert _create(d) == _lib.TWOLDG_EUNSUP
    assert b"face table" in _lib.lib().twoldg_last_error()
    buf = (ctypes.c_double * 16)()
    du, u = ctypes.cast(buf, ctypes.c_void_p), ctypes.c_void_p(ctypes.addressof(buf) + 64)
    assert _lib.lib().twoldg_rhs_static(ctypes.byref(d), du, u, 0.0, None) == _lib.TWOLDG_EUNSUP
    assert b"face table" in _lib.lib().twoldg_last_error()
    d.face_nb = None
    d.face_code = None
    d.metric = 1
    assert _create(d) == _lib.TWOLDG_EINVAL
    assert b"needs coef" in _lib.lib().twoldg_last_error()
    assert _lib.lib().twoldg_rhs_static(ctypes.byref(d), du, u, 0.0, None) == _lib.TWOLDG_EUNSUP
    d.metric = 5
    assert _create(d) == _lib.TWOLDG_EINVAL
    d.metric = 0
    # a forest past the static array's 16 MiB is refused on the host too:
    # 1000 blocks of 16^3 in FP64 need two face arrays of 1000 * 6 * 16^2
    # words, 23.4 MiB
    g = wave_forest(np.float64, 3, 3, 4, roots=10)
    d2, keep2 = twoldg.problem.make_desc(g, twoldg.Element(np.float64, 3), True, _lib.F64)
    assert _lib.lib().twoldg_rhs_static(ctypes.byref(d2), du, u, 0.0, None) == _lib.TWOLDG_EINVAL
    assert b"16 MiB" in _lib.lib().twoldg_last_error()
    del keep, keep2
