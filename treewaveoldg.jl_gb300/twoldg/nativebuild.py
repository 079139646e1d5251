"""Build libtwoldg.so in-tree from csrc/ for sm_103a.

Compiles every translation unit in parallel (nvcc for .cu, g++ for the host
.cpp files) and links a shared library into twoldg/_lib/. The CUDA runtime is
linked statically so the library has no run-time path dependency beyond the
driver. Host code is compiled with -ffp-contract=off: the double-double table
builder needs separately rounded products, and the same flags give identical
tables on x86 and Arm hosts.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
CSRC = os.path.join(PKG_ROOT, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIBNAME = "libtwoldg.so"
OBJDIR = os.path.join(PKG_ROOT, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cand, "bin", "nvcc")
    return p if os.path.exists(p) else shutil.which("nvcc")


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _sources():
    srcs = sorted(os.listdir(CSRC))
    return [s for s in srcs if s.endswith(".cu") or s.endswith(".cpp")]


def _deps():
    return [os.path.join(CSRC, s) for s in os.listdir(CSRC)] + [
        os.path.join(os.path.dirname(PKG_ROOT), "include", "twoldg.h")]


def up_to_date():
    lib = lib_path()
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _cost(src):
    import re
    m = re.match(r"kernels_d(\d)(?:_p(\d))?", src)
    if m:
        return 100 * int(m.group(1)) + (int(m.group(2)) if m.group(2) else 0) * 10 + ("_cf" not in src)
    return 50 if src.endswith(".cu") else 0


def _compile(src, nvcc, verbose):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJDIR, src + ".o")
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "-c", path, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-pthread",
               "-I" + cuda_inc, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, (r.stdout + r.stderr)


def build(force=False, verbose=False):
    """Compile and link libtwoldg.so; returns its path."""
    if not force and up_to_date():
        return lib_path()
    nvcc = _nvcc()
    if nvcc is None:
        raise RuntimeError("nvcc not found: set CUDA_HOME")
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    # the longest compiles first (the 3D kernels, the higher orders first),
    # so that the build's wall time is close to its longest unit's
    srcs = sorted(_sources(), key=_cost, reverse=True)
    workers = min(len(srcs), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(workers) as ex:
        results = list(ex.map(lambda s: _compile(s, nvcc, verbose), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for o, log in results:
            if log.strip():
                print(o, "\n", log, file=sys.stderr)
    tmp = lib_path() + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static", "-Xcompiler", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, lib_path())
    return lib_path()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
