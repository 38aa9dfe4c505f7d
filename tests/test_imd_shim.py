"""IMD's `cuda` make target, compiled and linked from the reference sources.

integration/imd_forces_cuda.c is the reference-side binding: it takes the
place of src/imd_forces_nbl.c (calc_forces, make_nblist, check_nblist,
deallocate_nblist, estimate_nblist_size) and of move_atoms_nve, which the
target renames in src/imd_integrate.c at compile time; every other IMD
source compiles unchanged.  oracle/Makefile (`make imd-cuda`) builds, from
the reference sources where they lie:

* IMD's own serial NBL EAM2 NVE program (imd_nve_nbl_eam);
* the same program as the `cuda` target, linked with libimdgpu.so;
* the `cuda` target linked with the oracle behind the same C-ABI
  (oracle/imdgpu_standin.c), which runs without a GPU.

The test runs IMD's own program and the stand-in build on one parameter
file (Sutton-Chen Cu, IMD's _fcc generator 8^3, 300 K, 60 NVE steps, energy
output every 10 steps, a checkpoint every 25) and requires the .eng file to
be identical and every checkpoint to be identical apart from the header
lines naming the program and the time.  That covers the shim's data
movement: cell arrays to the library and back by NUMMER, the globals it
sets, the steps where main_loop reads the cell arrays.  The build linked
with libimdgpu.so must start, read its inputs and, where no GPU is present,
stop with IMD's error() carrying the library's message.

Skipped where the reference sources are absent (the GPU host has none);
IMD_REFERENCE_SRC names them elsewhere.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")


def _refsrc():
    r = subprocess.run(["make", "-s", "-C", ORACLE, "refsrc"], capture_output=True, text=True)
    return r.stdout.strip()


pytestmark = pytest.mark.skipif(not os.path.isdir(_refsrc() or "/nonexistent"),
                                reason="reference sources not present")


@pytest.fixture(scope="module")
def programs():
    from imd_gb300 import build
    build.build()   # libimdgpu.so, when stale or absent
    subprocess.run(["make", "-s", "-C", ORACLE, "imd-cuda"], check=True,
                   capture_output=True)
    ref = os.path.join(ORACLE, "_ref")
    return {"imd": os.path.join(ref, "imd_nve_nbl_eam", "imd"),
            "cuda": os.path.join(ref, "imd_cuda_nve_nbl_eam", "imd"),
            "standin": os.path.join(ref, "imd_cuda_nve_nbl_eam", "imd_standin")}


def _param(d, tabs, **kw):
    from imd_gb300 import workloads as wl
    tok = dict(simulation=1, coordname="_fcc", outfiles=os.path.join(d, "out"), ensemble="nve",
               ntypes=1, masses=63.546, pbc_dirs=[1, 1, 1], timestep=0.0982266, maxsteps=60,
               starttemp=0.0258520, seed=2, core_potential_file=tabs[0],
               **{"atomic_e-density_file": tabs[1]}, embedding_energy_file=tabs[2],
               nbl_margin=0.4, eng_int=10, checkpt_int=25, box_param=[8, 8, 8], box_unit=3.615)
    tok.update(kw)
    path = os.path.join(d, "cu.param")
    wl.write_param(path, **tok)
    return path


def _run(prog, d, param):
    return subprocess.run([prog, "-p", param], cwd=d, capture_output=True, text=True,
                          timeout=300)


def _body(path):
    """A checkpoint without the lines naming the program and the time."""
    with open(path) as f:
        return [ln for ln in f if not ln.startswith(("## Generated", "## by"))]


def test_cuda_target_output_equals_imd(programs, tmp_path):
    from imd_gb300 import workloads as wl
    tabs = wl.sutton_chen_tables(str(tmp_path / "cu"), [wl.CU])
    runs = {}
    for name in ("imd", "standin"):
        d = tmp_path / name
        d.mkdir()
        r = _run(programs[name], str(d), _param(str(d), tabs))
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        runs[name] = d
    a, b = runs["imd"], runs["standin"]
    eng_a = (a / "out.eng").read_text().splitlines()
    eng_b = (b / "out.eng").read_text().splitlines()
    assert len(eng_a) == 8   # header, steps 0, 10, ..., 60
    assert eng_a == eng_b
    chk = sorted(f for f in os.listdir(a) if f.endswith(".chkpt"))
    assert chk == ["out.00000.chkpt", "out.00001.chkpt", "out.00002.chkpt"]
    assert chk == sorted(f for f in os.listdir(b) if f.endswith(".chkpt"))
    for f in chk:
        body = _body(a / f)
        assert len(body) > 2048
        assert body == _body(b / f), f


def test_cuda_target_links_libimdgpu_and_reports_its_errors(programs, tmp_path):
    """The build linked with libimdgpu.so reads the parameter file, the
    tables and generates the crystal like IMD; its first calc_forces creates
    the device system.  Without a GPU that fails, and the shim hands the
    library's message to IMD's error()."""
    from imd_gb300 import workloads as wl
    out = subprocess.run(["ldd", programs["cuda"]], capture_output=True, text=True).stdout
    assert "libimdgpu.so" in out
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present: the error path is not reached")
    tabs = wl.sutton_chen_tables(str(tmp_path / "cu"), [wl.CU])
    r = _run(programs["cuda"], str(tmp_path), _param(str(tmp_path), tabs, maxsteps=5))
    assert r.returncode != 0
    text = r.stdout + r.stderr
    assert "Global cell array dimensions" in text or "maximal cell occupancy" in text
    assert "Error: imdgpu_create" in text
