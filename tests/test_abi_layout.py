"""Struct layouts across the ctypes bindings: every structure that
imd_gb300/api.py mirrors from include/imdgpu.h, and that oracle/oracle.py
mirrors from oracle/imd_oracle.h, has the C compiler's size and the C
compiler's offset for every field.  A field added on one side only, or
declared in another order, fails here on the CPU instead of corrupting
memory at run time."""
import ctypes as C
import os
import subprocess

import pytest

from conftest import ROOT


def _c_layout(tmp_path, header_dir, header, structs):
    """sizeof and offsetof of each (C type, ctypes class) as the compiler
    lays them out."""
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "%s"' % header,
             "int main(void) {"]
    for ctype, cls in structs:
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (ctype, ctype))
        for name, _ in cls._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));'
                         % (ctype, name, ctype, name))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    r = subprocess.run(["gcc", "-std=gnu11", "-I", header_dir, str(src), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    got = {}
    for line in out.splitlines():
        t, f, v = line.split()
        got[(t, f)] = int(v)
    return got


def _check(got, structs):
    for ctype, cls in structs:
        assert got[(ctype, "sizeof")] == C.sizeof(cls), ctype
        for name, _ in cls._fields_:
            assert got[(ctype, name)] == getattr(cls, name).offset, (ctype, name)


def test_api_structs_match_header(tmp_path):
    from imd_gb300 import api
    structs = [("imdgpu_scalars", api.Scalars), ("imdgpu_timing", api.Timing),
               ("imdgpu_glok_params", api.GlokParams), ("imdgpu_glok_state", api.GlokState),
               ("imdgpu_npt_params", api.NptParams), ("imdgpu_npt_state", api.NptState),
               ("imdgpu_npt_axial_params", api.NptAxialParams),
               ("imdgpu_npt_axial_state", api.NptAxialState)]
    got = _c_layout(tmp_path, os.path.join(ROOT, "include"), "imdgpu.h", structs)
    _check(got, structs)


def test_oracle_structs_match_header(tmp_path):
    oracle = pytest.importorskip("oracle")
    structs = [("orc_table_t", oracle.Table), ("orc_sys_t", oracle.Sys),
               ("orc_glok_t", oracle.Glok), ("orc_npt_t", oracle.Npt),
               ("orc_npt_axial_t", oracle.NptAxial)]
    got = _c_layout(tmp_path, os.path.join(ROOT, "oracle"), "imd_oracle.h", structs)
    _check(got, structs)
