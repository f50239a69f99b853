"""The C++ facade lala_gpu::PIR (include/pirgpu.hpp): it compiles and links
against libpirgpu.so on any host; on a GPU its known-answer program passes."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_test.cpp")


def _build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("pirgpu_build", os.path.join(ROOT, "lala-pc_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    lib = b.build()
    libdir = os.path.dirname(lib)
    exe = os.path.join(libdir, "facade_test")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I" + os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L" + libdir, "-lpirgpu", "-Wl,-rpath," + libdir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_facade_compiles_and_links():
    assert os.path.exists(_build())


@pytest.mark.gpu
def test_facade_known_answers_on_gpu():
    exe = _build()
    p = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "0 failures" in p.stdout
