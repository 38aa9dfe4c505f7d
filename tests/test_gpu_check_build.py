"""The bounds-checked build on the GPU.  Built with -DIMDGPU_CHECK, the
kernels check every index they take from device data (list partners, ghost
owners, table rows and columns, cell bins, permutation slots) before using
it, and a failed check makes the API call that reads the status word fail.
So the parity tests against the reference's goldens and the oracle, the
deterministic mode and the batch tests against the oracle and with
per-system rebuilds run again here against that library, in a child process
with IMDGPU_LIB naming it: passing means no check failed on any of them and
the checked kernels give the results those tests demand."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT, golden

pytestmark = pytest.mark.gpu

TESTS = os.path.join(ROOT, "tests")
BATCH = os.path.join(TESTS, "test_gpu_batch.py")
RUN = [
    os.path.join(TESTS, "test_gpu_check_build.py") + "::test_loaded_library_is_the_checked_one",
    os.path.join(TESTS, "test_gpu_parity.py"),
    os.path.join(TESTS, "test_gpu_deterministic.py"),
    BATCH + "::test_batch_matches_oracle_per_cell",
    BATCH + "::test_partial_rebuilds_relax_like_full_ones",
]


@pytest.mark.late
def test_parity_and_batch_tests_pass_in_the_checked_build():
    from imd_gb300 import build
    lib = build.build(check=True)
    env = dict(os.environ, IMDGPU_LIB=lib)
    cmd = [sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider"]
    r = subprocess.run(cmd + RUN, env=env, cwd=ROOT, capture_output=True, text=True,
                       timeout=3600)
    print(r.stdout[-1500:])
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]


def test_loaded_library_is_the_checked_one():
    """Runs inside the child process only: the library loaded is the
    checked build, and a force call on a golden case leaves no failed check."""
    if not os.environ.get("IMDGPU_LIB"):
        pytest.skip("part of the checked-build run")
    from imd_gb300 import api
    from test_gpu_parity import gpu_system, rel_rms
    assert b"bounds-checked" in api.lib().imdgpu_version()
    g = golden("cu_pert")
    s = gpu_system(g, "cu", 1, 1, 0.4)
    s.calc_forces(0)
    checked, sites = s.check_sites()
    assert checked and sites == 0
    assert rel_rms(s.get_atoms()["f"], g["f"]) < 1e-11
    s.close()
