"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/pir_oracle.cpp and oracle/pc_oracle.cpp into
oracle/_build/liboracle.so with the host C++ compiler.  Portable flags only (the same source builds on x86_64 and
aarch64 hosts).  The reference itself (lala-pc) cannot be compiled here: it
includes lala-core and cuda-battery headers that its CMake fetches over the
network, so the oracle is this restatement, not a build of the reference.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "pir_oracle.cpp"), os.path.join(HERE, "pc_oracle.cpp")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = SOURCES + [os.path.join(HERE, "pir_oracle.h"), os.path.join(HERE, "pc_oracle.h")]
    return any(os.path.getmtime(s) > t for s in deps)


def build(force=False, verbose=False):
    """Compile liboracle.so if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread",
           "-Wall", "-Wno-unused-function", "-o", tmp] + SOURCES
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
