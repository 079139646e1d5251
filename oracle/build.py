"""Build recipe for the CPU oracle and the CPU baseline (test infrastructure
only): compiles oracle/oracle.c into oracle/_build/liboracle.so and
oracle/refcpu.c into oracle/_build/librefcpu.so, both with OpenMP.

The reference is Julia (no C/C++ sources), so there is no oracle/_ref build:
the oracle and the baseline are these plain-C restatements.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "liboracle.so")
OUT_REF = os.path.join(HERE, "_build", "librefcpu.so")


def _compile(src, out, opt, force):
    src = os.path.join(HERE, src)
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = ["gcc", opt, "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-Wall",
           src, "-o", out + ".tmp", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(out + ".tmp", out)
    return out


def build(force=False):
    """The oracle's library (and the CPU baseline's beside it)."""
    build_refcpu(force)
    return _compile("oracle.c", OUT, "-O2", force)


def build_refcpu(force=False):
    """The CPU baseline: the reference's threaded CPU data flow at -O3 (no
    -march flags, so x86 and Arm hosts compile the same source the same way)."""
    return _compile("refcpu.c", OUT_REF, "-O3", force)


if __name__ == "__main__":
    print(build(force=True))
