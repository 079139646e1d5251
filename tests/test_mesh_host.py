"""The mesh compiler (csrc/mesh.cpp) on the CPU, built into a library of its
own (tests/host_stub/mesh_shim.cpp): every block face's neighbour, wall and
coarse-fine face against a geometric search of the leaves' extents, which
finds them by position where the compiler finds them by integer keys, on
uniform, reflecting, refined and nested forests in 1D to 3D."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "treewaveoldg.jl_gb300", "csrc")


@pytest.fixture(scope="module")
def mesh_lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("needs g++")
    out = str(tmp_path_factory.mktemp("mesh_host") / "libmesh_host.so")
    subprocess.run([gxx, "-O1", "-std=c++17", "-shared", "-fPIC",
                    os.path.join(ROOT, "tests", "host_stub", "mesh_shim.cpp"), os.path.join(CSRC, "mesh.cpp"), "-o", out],
                   check=True, capture_output=True, timeout=300)
    lib = ctypes.CDLL(out)
    vp = ctypes.c_void_p
    lib.mesh_tables.restype = ctypes.c_int
    lib.mesh_tables.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int32, ctypes.c_char_p, ctypes.c_int32]
    return lib


def compiled(lib, forest):
    """The compiler's neighbour slots, flags and coarse-fine faces (by slot);
    the forests here have E = 2 elements per block."""
    import twoldg
    from twoldg import _lib
    P = forest.N // 2 - 1
    d, keep = twoldg.problem.make_desc(forest, twoldg.Element(np.float64, P), True, _lib.F64)
    n = len(forest.leaves)
    nb = np.zeros((n, 6), dtype=np.int32)
    flags = np.zeros(n, dtype=np.uint32)
    ncf = ctypes.c_int32()
    cap = 12 * n
    cf = np.zeros((cap, 8), dtype=np.int32)
    err = ctypes.create_string_buffer(512)
    rc = lib.mesh_tables(ctypes.addressof(d), nb.ctypes.data, flags.ctypes.data, ctypes.addressof(ncf),
                         cf.ctypes.data, cap, err, 512)
    del keep
    return rc, err.value, nb, flags, {int(r[0]): r for r in cf[:ncf.value]}


def geometric(forest):
    """The same tables from the leaves' extents: a probe point just across the
    middle of each face (wrapped where the box is periodic, a wall where it
    reflects) names the leaf there; its level against the block's tells a
    same-level face, the fine side of a coarse-fine face or its coarse side,
    whose 2^(D-1) fine neighbours are probed at the quarter points."""
    D = forest.D
    ext = np.array([forest.block_extent(k) for k in forest.leaves])      # (n, D, 2)
    lo, hi = ext[..., 0], ext[..., 1]
    levels = np.array([lv for lv, _ in forest.leaves])
    dlo, dhi = np.array(forest.lo, dtype=float), np.array(forest.hi, dtype=float)

    def find(x):
        x = np.array(x, dtype=float)
        for k in range(D):
            if x[k] < dlo[k] or x[k] >= dhi[k]:
                if not forest.periodic[k]:
                    return None
                x[k] = dlo[k] + (x[k] - dlo[k]) % (dhi[k] - dlo[k])
        hit = np.nonzero(np.all((lo <= x) & (x < hi), axis=1))[0]
        assert len(hit) == 1, x
        return int(hit[0])

    n = len(forest.leaves)
    nb = np.full((n, 6), -1, dtype=np.int32)
    flags = np.zeros(n, dtype=np.uint32)
    cf = {}
    for b in range(n):
        w = hi[b, 0] - lo[b, 0]
        mid = (lo[b] + hi[b]) / 2
        for f in range(2 * D):
            d, side = f // 2, f % 2
            face = hi[b, d] if side else lo[b, d]
            across = 1 if side else -1
            x = mid.copy()
            x[d] = face + across * w / 4
            m = find(x)
            slot = b * 2 * D + f
            if m is None:
                nb[b, f] = slot
                flags[b] |= 1 << (8 + f)
            elif levels[m] == levels[b]:
                nb[b, f] = m * 2 * D + (f ^ 1)
            elif levels[m] == levels[b] - 1:
                sub, bit = 0, 0
                for k in range(D):
                    if k == d:
                        continue
                    sub |= int(lo[b, k] > lo[m, k] + 1e-12 * w) << bit
                    bit += 1
                cf[slot] = (0, [m * 2 * D + (f ^ 1)], sub, side)
                flags[b] |= 1 << f
            else:
                assert levels[m] == levels[b] + 1
                tang = [k for k in range(D) if k != d]
                src = []
                for q in range(1 << (D - 1)):
                    y = mid.copy()
                    y[d] = face + across * w / 8
                    for bit, k in enumerate(tang):
                        y[k] = lo[b, k] + w / 4 + ((q >> bit) & 1) * w / 2
                    src.append(find(y) * 2 * D + (f ^ 1))
                cf[slot] = (1, src, None, side)
                flags[b] |= 1 << f
    return nb, flags, cf


def _forests():
    from cases import refined_forest
    from twoldg.forest import nested_cubes, wave_forest
    return [("1D periodic", wave_forest(np.float64, 1, 3, 2, roots=5)),
            ("2D periodic", wave_forest(np.float64, 2, 3, 2, roots=3)),
            ("3D reflecting", wave_forest(np.float64, 3, 2, 2, roots=2, reflecting=True)),
            ("1D refined", refined_forest(1, 3)),
            ("2D refined", refined_forest(2, 3)),
            ("2D refined corner, walls", refined_forest(2, 2, reflecting=True)),
            ("3D refined", refined_forest(3, 2)),
            ("3D refined corner, walls", refined_forest(3, 2, reflecting=True)),
            ("nested cubes", wave_forest(np.float64, 3, 3, 2, roots=8, reflecting=True,
                                         refined=nested_cubes(3, 1 / 8, 3)))]


@pytest.mark.parametrize("case", range(9), ids=[n for n, _ in _forests()])
def test_mesh_tables_are_the_geometric_ones(mesh_lib, case):
    _, forest = _forests()[case]
    rc, err, nb, flags, cf = compiled(mesh_lib, forest)
    assert rc == 0, err
    gnb, gflags, gcf = geometric(forest)
    D = forest.D
    assert np.array_equal(nb[:, :2 * D], gnb[:, :2 * D])
    assert np.array_equal(flags, gflags)
    assert set(cf) == set(gcf)
    for slot, (kind, src, sub, side) in gcf.items():
        row = cf[slot]
        assert row[1] == kind and row[7] == side
        assert list(row[2:2 + len(src)]) == src
        if kind == 0:
            assert row[6] == sub


def test_mesh_refuses_odd_elements_and_unbalanced_forests(mesh_lib):
    from twoldg.forest import wave_forest
    f = wave_forest(np.float64, 2, 3, 2, roots=2)
    f.refine([f.leaves[0]])
    f.refine([k for k in f.leaves if k[0] == 1][:1])      # two levels apart across a face
    rc, err, *_ = compiled(mesh_lib, f)
    assert rc == 1 and b"balanced" in err
