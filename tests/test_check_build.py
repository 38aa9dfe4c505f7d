"""The bounds-checked variant (-DIMDGPU_CHECK, python -m imd_gb300.build
--check) builds without a GPU, exports every entry point include/imdgpu.h
declares and says what it is; the default library has no checks.  Its GPU
run is tests/test_gpu_check_build.py."""
import ctypes
import re
import subprocess

from test_abi import declared


def test_checked_variant_builds_and_exports_every_symbol():
    from imd_gb300 import build
    lib = build.build(check=True)
    L = ctypes.CDLL(lib)
    L.imdgpu_version.restype = ctypes.c_char_p
    assert b"bounds-checked" in L.imdgpu_version()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r"\sT\s(imdgpu_\w+)", out))
    assert set(declared()) <= exported


def test_default_library_has_no_checks():
    from imd_gb300 import api
    assert b"bounds-checked" not in api.lib().imdgpu_version()
