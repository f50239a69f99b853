"""Build recipe for libpirgpu.so (the C-ABI engine) for sm_103a.

Each .cu translation unit is compiled in parallel with one -gencode
(compute_103a / sm_103a), then linked into lala-pc_gb300/_build/libpirgpu.so
against the CUDA runtime.  No torch, no cmake: nvcc only, so the same recipe
runs on the x86_64 build host and on the aarch64 GPU host.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpirgpu.so")
SOURCES = ["pir_engine.cu", "pir_batch.cu", "pir_sched.cu", "pir_static.cu", "pir_events.cu", "pir_search.cu",
           "pir_pc.cu", "pir_install.cu"]
HEADERS = ["pir_device.cuh", "pir_kernels.cuh", "pir_engine.h", "pir_csr.h", "pir_sort.h", "pir_segments.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I" + os.path.join(ROOT, "include"), "-Xptxas", "-warn-spills"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    """Compile and link libpirgpu.so when missing or older than its sources."""
    os.makedirs(OUT_DIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "pirgpu.h")]
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc()] + _flags() + list(extra) + ["-c", s, "-o", o])
    if jobs:
        def run(cmd):
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            p = subprocess.run(cmd, capture_output=True, text=True)
            if p.returncode != 0:
                raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), p.stderr))
            return p.stderr
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for err in ex.map(run, jobs):
                if err and verbose:
                    print(err, file=sys.stderr)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp.%d" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.check_call(cmd)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else []))
