"""The C-ABI library: it builds, loads and exports every entry point that
include/pirgpu.h declares (no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pir_[a-z_0-9]+)\s*\(", src)))


def _lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "pirgpu_build", os.path.join(ROOT, "lala-pc_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return ctypes.CDLL(b.build())


def test_header_declares_entry_points():
    names = _declared("pirgpu.h")
    for n in ("pir_ctx_create", "pir_tell", "pir_fixpoint", "pir_ask_all", "pir_snapshot",
              "pir_restore", "pir_fixpoint_nodes", "pir_fixpoint_instances", "pir_deduce_batch"):
        assert n in names


def test_library_exports_every_declared_symbol():
    L = _lib()
    missing = [n for n in _declared("pirgpu.h") if not hasattr(L, n)]
    assert missing == []


def test_python_binding_covers_header():
    import pirgpu
    bound = {n for n, _, _ in pirgpu.SIGNATURES}
    assert set(_declared("pirgpu.h")) <= bound
    pirgpu.lib()  # loads and sets every signature


def test_context_create_fails_cleanly_without_gpu():
    import pirgpu
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    # no device: creation must return an error code, not crash
    h = ctypes.c_void_p()
    rc = pirgpu.lib().pir_ctx_create(ctypes.byref(h), 0)
    assert rc == pirgpu.ECUDA and not h.value


def test_python_constants_match_header():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "lala-pc_gb300"))
    import pirgpu
    src = open(os.path.join(ROOT, "include", "pirgpu.h")).read()
    assert int(re.search(r"#define PIR_PERSISTENT_VARIANTS (\d+)", src).group(1)) == pirgpu.PERSISTENT_VARIANTS
    assert int(re.search(r"#define PIR_NODE_VARIANTS (\d+)", src).group(1)) == pirgpu.NODE_VARIANTS


def test_pc_kinds_match_header_builder_and_oracle():
    """The tape node kinds of include/pirgpu.h (enum pc_kind) are the ones the
    Python builder (pc.py) and the oracle (oracle/pc_oracle.h) use."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "lala-pc_gb300"))
    import pc as P
    src = open(os.path.join(ROOT, "include", "pirgpu.h")).read()
    orc = open(os.path.join(ROOT, "oracle", "pc_oracle.h")).read()
    enum = src[src.index("enum pc_kind"):]
    enum = enum[:enum.index("};")]
    kinds = dict((m.group(1), int(m.group(2))) for m in re.finditer(r"PC_([A-Z_]+) = (\d+)", enum))
    assert len(kinds) == 38 and kinds["NUM_KINDS"] == P.NUM_KINDS == 37
    for name, v in kinds.items():
        if name != "NUM_KINDS":
            assert getattr(P, name) == v, name
        assert int(re.search(r"ORC_PC_%s = (\d+)" % name, orc).group(1)) == v, name
    assert int(re.search(r"#define PC_MAX_DEPTH (\d+)", src).group(1)) == P.MAX_DEPTH


def _struct_fields(header, name):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if decl:
            m = re.match(r"[A-Za-z_0-9 ]+?\s+([a-z_0-9]+)(?:\[(\d+)\])?$", decl)
            fields.append(m.group(1))
    return fields


def test_python_structs_match_header_layout(tmp_path):
    """The ctypes mirrors of the C structs: same fields, offsets and sizes as
    the C compiler lays them out from include/pirgpu.h."""
    import shutil
    import subprocess
    import pirgpu
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    pairs = [("pir_opts", pirgpu.Opts), ("pir_stats", pirgpu.Stats), ("pir_search_opts", pirgpu.SearchOpts),
             ("pir_search_stats", pirgpu.SearchStats)]
    lines = ['#include <stdio.h>', '#include "pirgpu.h"', "int main(void) {"]
    for cname, _ in pairs:
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in _struct_fields("pirgpu.h", cname):
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("  return 0;\n}")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    for cname, py in pairs:
        assert [f for f, _ in py._fields_] == _struct_fields("pirgpu.h", cname), cname
        assert ctypes.sizeof(py) == got[(cname, "sizeof")], cname
        for f, _ in py._fields_:
            assert getattr(py, f).offset == got[(cname, f)], (cname, f)
