"""IMD's `cuda` make target, compiled and linked from the reference sources.

integration/imd_forces_cuda.c is the reference-side binding: it takes the
place of src/imd_forces_nbl.c (calc_forces, make_nblist, check_nblist,
deallocate_nblist, estimate_nblist_size), of src/imd_cg.c in CG builds
(reset_cg, cg_step) and of move_atoms_nve / _mik / _nvt, which the target
renames in src/imd_integrate.c at compile time; every other IMD source
compiles unchanged.  oracle/Makefile (`make imd-cuda`) builds, from the
reference sources where they lie:

* IMD's own serial NBL EAM2 program of each target;
* the same program as the `cuda` target, linked with libimdgpu.so;
* the `cuda` target linked with the oracle behind the same C-ABI
  (oracle/imdgpu_standin.c), which runs without a GPU.

Four targets are built: nve, cg, mik and nvt (serial NBL EAM2).  For each,
the test runs IMD's own program and the stand-in build on the same parameter
file and requires every output file (.eng, checkpoints, the relaxed
configuration that check_relaxed writes, .itr) to be identical apart from
the header lines naming the program and the time.  That covers the shim's data
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


VARIANTS = ("nve_nbl_eam", "cg_nbl_eam", "mik_nbl_eam", "nvt_nbl_eam")


@pytest.fixture(scope="module")
def programs():
    from imd_gb300 import build
    build.build()   # libimdgpu.so, when stale or absent
    subprocess.run(["make", "-s", "-C", ORACLE, "imd-cuda"], check=True,
                   capture_output=True)
    ref = os.path.join(ORACLE, "_ref")
    return {v: {"imd": os.path.join(ref, "imd", v, "imd"),
                "cuda": os.path.join(ref, "cuda", v, "imd"),
                "standin": os.path.join(ref, "cuda", v, "imd_standin")} for v in VARIANTS}


@pytest.fixture(scope="module")
def inputs(tmp_path_factory):
    """Tables and a configuration: Cu 6^3 fcc with one vacancy and 0.08 A
    noise (seed 4), for the relaxations."""
    import numpy as np
    from imd_gb300 import workloads as wl
    d = tmp_path_factory.mktemp("imdin")
    tabs = wl.sutton_chen_tables(str(d / "cu"), [wl.CU])
    s = wl.eam_fcc_system(6)
    keep = np.ones(s.n, bool)
    keep[37] = False
    x = s.x + 0.08 * np.random.default_rng(4).standard_normal(s.x.shape)
    cfg = str(d / "vac.cfg")
    wl.write_config(cfg, s.box, s.number[keep], s.types[keep], s.mass[keep], x[keep])
    return tabs, cfg


# per variant: the run's parameters and the output files it must write
CASES = {
    # 60 NVE steps from IMD's generator at 300 K; energies every 10 steps,
    # checkpoints at 0, 25, 50 and the end of the phase
    "nve_nbl_eam": (dict(coordname="_fcc", box_param=[8, 8, 8], box_unit=3.615, ensemble="nve",
                         maxsteps=60, starttemp=0.0258520, eng_int=10, checkpt_int=25),
                    ["out.00000.chkpt", "out.00001.chkpt", "out.00002.chkpt"]),
    # CG until IMD's force-norm criterion stops it (check_relaxed writes the
    # relaxed configuration, out.00000.ss)
    "cg_nbl_eam": (dict(coordname="VAC", box_from_header=1, ensemble="cg", maxsteps=400,
                        starttemp=0.0, eng_int=1, checkpt_int=1000, fnorm_threshold=2e-4),
                   ["out.00000.chkpt", "out.00000.ss"]),
    "mik_nbl_eam": (dict(coordname="VAC", box_from_header=1, ensemble="mik", maxsteps=2000,
                         starttemp=0.0, eng_int=5, checkpt_int=10000, fnorm_threshold=2e-3),
                    ["out.00000.chkpt", "out.00000.ss"]),
    "nvt_nbl_eam": (dict(coordname="_fcc", box_param=[6, 6, 6], box_unit=3.615, ensemble="nvt",
                         maxsteps=60, starttemp=0.0258520, tau_eta=10.0, eng_int=10,
                         checkpt_int=30),
                    ["out.00000.chkpt", "out.00001.chkpt", "out.00002.chkpt"]),
}


def _param(d, tabs, cfg, **kw):
    from imd_gb300 import workloads as wl
    tok = dict(simulation=1, outfiles=os.path.join(d, "out"), ntypes=1, masses=63.546,
               pbc_dirs=[1, 1, 1], timestep=0.0982266, seed=2, core_potential_file=tabs[0],
               **{"atomic_e-density_file": tabs[1]}, embedding_energy_file=tabs[2],
               nbl_margin=0.4)
    tok.update(kw)
    if tok.get("coordname") == "VAC":
        tok["coordname"] = cfg
    path = os.path.join(d, "a.param")
    wl.write_param(path, **tok)
    return path


def _run(prog, d, param):
    return subprocess.run([prog, "-p", param], cwd=d, capture_output=True, text=True,
                          timeout=300)


def _body(path):
    """An output file without the lines naming the program and the time."""
    with open(path) as f:
        return [ln for ln in f if not ln.startswith(("## Generated", "## by"))]


@pytest.mark.parametrize("variant", VARIANTS)
def test_cuda_target_output_equals_imd(programs, inputs, tmp_path, variant):
    tabs, cfg = inputs
    tok, expect = CASES[variant]
    runs = {}
    for name in ("imd", "standin"):
        d = tmp_path / name
        d.mkdir()
        r = _run(programs[variant][name], str(d), _param(str(d), tabs, cfg, **tok))
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        runs[name] = d
    a, b = runs["imd"], runs["standin"]
    files = sorted(f for f in os.listdir(a) if f.startswith("out"))
    assert files == sorted(f for f in os.listdir(b) if f.startswith("out"))
    for f in expect + ["out.eng"]:
        assert f in files, (f, files)
    assert len(_body(a / "out.eng")) > 5
    for f in files:
        assert _body(a / f) == _body(b / f), f


def test_cuda_target_links_libimdgpu_and_reports_its_errors(programs, inputs, tmp_path):
    """The build linked with libimdgpu.so reads the parameter file, the
    tables and generates the crystal like IMD; its first calc_forces creates
    the device system.  Without a GPU that fails, and the shim hands the
    library's message to IMD's error()."""
    tabs, cfg = inputs
    for v in VARIANTS:
        out = subprocess.run(["ldd", programs[v]["cuda"]], capture_output=True, text=True).stdout
        assert "libimdgpu.so" in out, v
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present: the error path is not reached")
    tok = dict(CASES["nve_nbl_eam"][0], maxsteps=5)
    r = _run(programs["nve_nbl_eam"]["cuda"], str(tmp_path), _param(str(tmp_path), tabs, cfg,
                                                                      **tok))
    assert r.returncode != 0
    text = r.stdout + r.stderr
    assert "maximal cell occupancy" in text
    assert "Error: imdgpu_create" in text
