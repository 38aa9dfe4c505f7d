"""Generate the golden vectors under tests/golden/ from the reference itself.

Runs in the build container only (it needs the reference sources): builds
the unmodified reference with oracle/Makefile (`make ref`), writes
potential tables, parameter and configuration files in IMD's formats, runs
oracle/_ref/<variant>/ref_harness on them and stores the outputs as small
.npz fixtures next to this script, together with the table files the runs
read.  Re-run with `python tests/golden/make_golden.py`.

Fixtures (all sorted by atom number):
  lj_pert     LJ fcc 10^3 (4000 atoms), positions perturbed, table format 2
  lj_pert_f1  same system, table format 1
  lj_nve      LJ fcc 10^3 from IMD's own _fcc generator + maxwell (seed 1,
              T*=0.72), 200 NVE steps, dt 0.005, skin 0.3
  cu_pert     Sutton-Chen Cu fcc 8^3 (2048 atoms), perturbed
  cu_nve      Sutton-Chen Cu _fcc 8^3, 300 K, 100 NVE steps of 1 fs, skin 0.4
  alloy_pert  binary Sutton-Chen Cu/Ni fcc 6^3 a0=3.57 (864 atoms)
  tri_cg      strained (triclinic) Cu cell 3x4x3 with a vacancy and noise:
              forces and a CG relaxation to max |F| <= 1e-4 eV/A
  cu_pert_spline, cu_pert_4point   cu_pert with IMD's spline / 4-point
              table interpolation (targets with `spline`, `4point`)
  defect_cg_spline  a defect cell of the batched-relaxation generator
              (1005 atoms), CG to max |F| <= 1e-4 eV/A with spline tables
  cu_pert_stress, alloy_pert_stress, lj_pert_stress   the perturbed Cu,
              Cu/Ni and LJ cases run by the `stress` build (STRESS_TENS):
              per-atom PRESSTENS and calc_tot_presstens

  lj_nve1000  the LJ set-up of lj_nve run for the full 1000 steps:
              energies of every step; every 250 steps the positions and
              momenta before the step and the forces of its calc_forces
  cu_nvt      Sutton-Chen Cu _fcc 8^3, 300 K, 100 Nose-Hoover NVT steps
              (tau_eta 10 time units): energies and eta per step
  cu_mik      cu_pert's configuration quenched by 200 MIK steps: energies,
              force norms per step, final positions
  cu_fire, cu_glok, cu_mixglok   a perturbed Cu crystal with two vacancies
              relaxed by the glok ensemble of the `fire` build (300 steps,
              adaptive time step and mixing), of the `glok` build and of the
              `mix glok` build (200 steps each)
  cu_npt      Cu _fcc 8^3 at 300 K, 200 steps of ensemble npt_iso with the
              external pressure ramped from 0.01 to 0.005 eV/A^3
  cu_npt_axial  the same set-up, 200 steps of ensemble npt_axial with a
              stress per axis and the z axis held

`python tests/golden/make_golden.py stress` writes the stress fixtures only,
`... ensembles` the NVT / MIK ones, `... lj1000` the 1000-step LJ run,
`... glok` the glok ones, `... npt` the NPT ones.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from imd_gb300 import workloads as wl  # noqa: E402

ORACLE = os.path.join(ROOT, "oracle")


def harness(variant: str) -> str:
    return os.path.join(ORACLE, "_ref", variant, "ref_harness")


def load_state(path: str) -> dict:
    a = np.loadtxt(path, ndmin=2)
    order = np.argsort(a[:, 0], kind="stable")
    a = a[order]
    return {"number": a[:, 0].astype(np.int32), "type": a[:, 1].astype(np.int32),
            "mass": a[:, 2], "x": a[:, 3:6], "p": a[:, 6:9], "f": a[:, 9:12],
            "epot": a[:, 12], "rho": a[:, 13], "df": a[:, 14]}


def load_box(path: str):
    lines = open(path).read().split("\n")
    box = np.array([[float(v) for v in lines[i].split()] for i in range(3)])
    gdim = np.array([int(v) for v in lines[3].split()], np.int32)
    cellsz = float(lines[4])
    return box, gdim, cellsz


def canonical_pairs(path: str):
    """Canonical unordered pair set: (lo, hi, shift of hi's image rel. lo, r2).
    r2 is kept as computed by the reference (orientation does not change it
    bitwise for the reference's own orientation; the key is the set)."""
    a = np.loadtxt(path, ndmin=2)
    ni, nj = a[:, 0].astype(np.int64), a[:, 1].astype(np.int64)
    s = a[:, 2:5].astype(np.int64)
    r2 = a[:, 5]
    flip = (ni > nj) | ((ni == nj) & (
        (s[:, 0] < 0) | ((s[:, 0] == 0) & ((s[:, 1] < 0) | ((s[:, 1] == 0) & (s[:, 2] < 0))))))
    lo = np.where(flip, nj, ni)
    hi = np.where(flip, ni, nj)
    s = np.where(flip[:, None], -s, s)
    key = ((lo * (1 << 24) + hi) * 27 + (s[:, 0] + 1) * 9 + (s[:, 1] + 1) * 3 + (s[:, 2] + 1))
    order = np.argsort(key, kind="stable")
    return key[order], r2[order]


def pair_digest(key: np.ndarray, r2: np.ndarray) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(key, np.int64).tobytes())
    h.update(np.ascontiguousarray(r2, np.float64).tobytes())
    return h.hexdigest()


def run(variant: str, param: str, mode: str, pre: str, *extra) -> None:
    cmd = [harness(variant), param, mode, pre] + [str(e) for e in extra]
    r = subprocess.run(cmd, cwd=os.path.dirname(param), capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s failed:\n%s\n%s" % (cmd, r.stdout[-2000:], r.stderr[-2000:]))


def perturbed_config(sysobj, sigma: float, seed: int, path: str, remove=None,
                     strain=None) -> None:
    rng = np.random.default_rng(seed)
    x = sysobj.x.copy()
    box = sysobj.box.copy()
    keep = np.ones(len(x), bool)
    if remove is not None:
        keep[remove] = False
    if strain is not None:
        m = np.eye(3) + strain
        x = x @ m.T
        box = box @ m.T
    x = x + sigma * rng.standard_normal(x.shape)
    wl.write_config(path, box, sysobj.number[keep], sysobj.types[keep],
                    sysobj.mass[keep], x[keep])


def main() -> None:
    subprocess.run(["make", "-s", "-C", ORACLE, "ref"], check=True)
    tmp = tempfile.mkdtemp(prefix="imdgold")
    out = {}
    # ---- tables (kept as fixtures: the runs read exactly these files) ----
    lj2 = os.path.join(HERE, "lj.pt")
    lj1 = os.path.join(HERE, "lj_f1.pt")
    wl.lj_table(lj2, fmt=2)
    wl.lj_table(lj1, npts=300, fmt=1)
    cu = wl.sutton_chen_tables(os.path.join(HERE, "cu"), [wl.CU])
    alloy = wl.sutton_chen_tables(os.path.join(HERE, "cuni"), [wl.CU, wl.NI])

    def lj_param(path, coord, potfile, **kw):
        tok = dict(coordname=coord, outfiles=os.path.join(tmp, "o"), ensemble="nve",
                   ntypes=1, masses=1.0, pbc_dirs=[1, 1, 1], timestep=0.005,
                   maxsteps=0, starttemp=0.0, seed=1, potfile=potfile,
                   nbl_margin=0.3, eng_int=0, checkpt_int=100000000)
        tok.update(kw)
        wl.write_param(path, **tok)

    def eam_param(path, coord, tabs, ntypes, masses, **kw):
        tok = dict(coordname=coord, outfiles=os.path.join(tmp, "o"), ensemble="nve",
                   ntypes=ntypes, masses=masses, pbc_dirs=[1, 1, 1],
                   timestep=0.0982266, maxsteps=0, starttemp=0.0, seed=2,
                   core_potential_file=tabs[0], **{"atomic_e-density_file": tabs[1]},
                   embedding_energy_file=tabs[2], nbl_margin=0.4, eng_int=0,
                   checkpt_int=100000000)
        tok.update(kw)
        wl.write_param(path, **tok)

    def forces_case(name, variant, param):
        pre = os.path.join(tmp, name)
        run(variant, param, "forces", pre)
        st = load_state(pre + ".forces")
        box, gdim, cellsz = load_box(pre + ".box")
        key, r2 = canonical_pairs(pre + ".pairs")
        tot = np.loadtxt(pre + ".totals")
        d = dict(box=box, gdim=gdim, cellsz=cellsz, epot_total=tot[0], virial=tot[1],
                 npairs=len(key), pair_digest=pair_digest(key, r2), **st)
        return d, key, r2

    # ---- LJ perturbed, format 2 and format 1 ----
    lj = wl.lj_fcc_system(10)
    cfg = os.path.join(tmp, "lj_pert.cfg")
    perturbed_config(lj, 0.05, 11, cfg)
    p = os.path.join(tmp, "lj_pert.param")
    lj_param(p, cfg, lj2, box_from_header=1)
    out["lj_pert"], _, _ = forces_case("lj_pert", "nve_nbl", p)
    p = os.path.join(tmp, "lj_pert_f1.param")
    lj_param(p, cfg, lj1, box_from_header=1)
    out["lj_pert_f1"], _, _ = forces_case("lj_pert_f1", "nve_nbl", p)

    # ---- LJ NVE from IMD's own generator (config-1 set-up, shortened) ----
    p = os.path.join(tmp, "lj_nve.param")
    lj_param(p, "_fcc", lj2, box_param=[10, 10, 10], box_unit=lj.meta["a0"],
             starttemp=0.72, seed=1)
    pre = os.path.join(tmp, "lj_nve")
    run("nve_nbl", p, "nve", pre, 200)
    st0 = load_state(pre + ".state0")
    stf = load_state(pre + ".final")
    steps = np.loadtxt(pre + ".steps")
    box, gdim, cellsz = load_box(pre + ".box")
    out["lj_nve"] = dict(box=box, gdim=gdim, cellsz=cellsz, number=st0["number"],
                         type=st0["type"], mass=st0["mass"], x0=st0["x"], p0=st0["p"],
                         epot=steps[:, 1], ekin=steps[:, 2], nbl_count=steps[:, 3],
                         x_final=stf["x"], p_final=stf["p"], dt=0.005, skin=0.3)

    # ---- Cu perturbed ----
    cus = wl.eam_fcc_system(8)
    cfg = os.path.join(tmp, "cu_pert.cfg")
    perturbed_config(cus, 0.1, 12, cfg)
    p = os.path.join(tmp, "cu_pert.param")
    eam_param(p, cfg, cu, 1, 63.546, box_from_header=1)
    out["cu_pert"], _, _ = forces_case("cu_pert", "nve_nbl_eam", p)

    # ---- Cu NVE (config-2 set-up at 8^3 cells, shortened) ----
    p = os.path.join(tmp, "cu_nve.param")
    eam_param(p, "_fcc", cu, 1, 63.546, box_param=[8, 8, 8], box_unit=3.615,
              starttemp=0.0258520, seed=2)
    pre = os.path.join(tmp, "cu_nve")
    run("nve_nbl_eam", p, "nve", pre, 100)
    st0 = load_state(pre + ".state0")
    stf = load_state(pre + ".final")
    steps = np.loadtxt(pre + ".steps")
    box, gdim, cellsz = load_box(pre + ".box")
    out["cu_nve"] = dict(box=box, gdim=gdim, cellsz=cellsz, number=st0["number"],
                         type=st0["type"], mass=st0["mass"], x0=st0["x"], p0=st0["p"],
                         epot=steps[:, 1], ekin=steps[:, 2], nbl_count=steps[:, 3],
                         x_final=stf["x"], p_final=stf["p"], dt=0.0982266, skin=0.4)

    # ---- binary alloy ----
    als = wl.eam_fcc_system(6, a0=3.57, species=(wl.CU, wl.NI), type_seed=3)
    cfg = os.path.join(tmp, "alloy.cfg")
    perturbed_config(als, 0.08, 13, cfg)
    p = os.path.join(tmp, "alloy.param")
    eam_param(p, cfg, alloy, 2, [63.546, 58.69], box_from_header=1)
    out["alloy_pert"], _, _ = forces_case("alloy_pert", "nve_nbl_eam", p)

    # ---- small triclinic defect cell: forces + CG ----
    x, box = wl.fcc(3, 4, 3, 3.615)
    n = len(x)
    tri = wl.System(box, x, np.zeros_like(x), np.zeros(n, np.int32),
                    np.full(n, 63.546), np.arange(n, dtype=np.int32))
    strain = np.array([[0.015, 0.01, -0.005], [0.0, -0.012, 0.008], [0.0, 0.0, 0.018]])
    cfg = os.path.join(tmp, "tri.cfg")
    perturbed_config(tri, 0.05, 14, cfg, remove=[17], strain=strain)
    p = os.path.join(tmp, "tri.param")
    eam_param(p, cfg, cu, 1, 63.546, box_from_header=1, ensemble="cg")
    d, key, r2 = forces_case("tri", "cg_nbl_eam", p)
    d["pair_key"] = key
    d["pair_r2"] = r2
    pre = os.path.join(tmp, "tri")
    run("cg_nbl_eam", p, "cg", pre, 5000, 1e-4)
    cg = np.loadtxt(pre + ".cg")
    stf = load_state(pre + ".final")
    d.update(cg_steps=int(cg[0]), cg_nfc=int(cg[1]), cg_epot=cg[2], cg_fmax=cg[3],
             cg_x=stf["x"])
    out["tri_cg"] = d

    # ---- spline and 4-point interpolation ----
    cfg = os.path.join(tmp, "cu_pert.cfg")
    p = os.path.join(tmp, "cu_pert.param")
    out["cu_pert_spline"], _, _ = forces_case("cu_pert_spline", "nve_nbl_eam_spline", p)
    out["cu_pert_4point"], _, _ = forces_case("cu_pert_4point", "nve_nbl_eam_4point", p)
    rng = np.random.default_rng(4)
    cells = [wl.defect_cell(rng) for _ in range(3)]
    dc = cells[2]
    cfg = os.path.join(tmp, "defect.cfg")
    wl.write_config(cfg, dc.box, dc.number, dc.types, dc.mass, dc.x)
    p = os.path.join(tmp, "defect.param")
    eam_param(p, cfg, cu, 1, 63.546, box_from_header=1, ensemble="cg")
    d, _, _ = forces_case("defect", "cg_nbl_eam_spline", p)
    pre = os.path.join(tmp, "defect")
    run("cg_nbl_eam_spline", p, "cg", pre, 20000, 1e-4)
    cg = np.loadtxt(pre + ".cg")
    stf = load_state(pre + ".final")
    d.update(cg_steps=int(cg[0]), cg_nfc=int(cg[1]), cg_epot=cg[2], cg_fmax=cg[3],
             cg_x=stf["x"], cg_seconds=cg[4])
    out["defect_cg_spline"] = d

    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, {k: (v.shape if hasattr(v, "shape") and v.shape else v)
                     for k, v in d.items() if k in ("npairs", "epot_total", "cg_steps",
                                                    "cg_epot", "cg_nfc")})


def load_stress(pre: str):
    a = np.loadtxt(pre + ".stress", ndmin=2)
    a = a[np.argsort(a[:, 0], kind="stable")]
    return a[:, 1:7], np.loadtxt(pre + ".totstress")


def stress_cases() -> None:
    """The STRESS_TENS fixtures, on the same inputs as cu_pert, alloy_pert and
    lj_pert (same generators and seeds)."""
    subprocess.run(["make", "-s", "-C", ORACLE, "ref"], check=True)
    tmp = tempfile.mkdtemp(prefix="imdgold_stress")
    cu = tuple(os.path.join(HERE, "cu" + e) for e in (".pt", ".rho", ".emb"))
    alloy = tuple(os.path.join(HERE, "cuni" + e) for e in (".pt", ".rho", ".emb"))
    lj2 = os.path.join(HERE, "lj.pt")
    cases = []
    cus = wl.eam_fcc_system(8)
    cfg = os.path.join(tmp, "cu_pert.cfg")
    perturbed_config(cus, 0.1, 12, cfg)
    cases.append(("cu_pert_stress", "nve_nbl_eam_stress", cfg,
                  dict(core_potential_file=cu[0], **{"atomic_e-density_file": cu[1]},
                       embedding_energy_file=cu[2], ntypes=1, masses=63.546,
                       timestep=0.0982266, nbl_margin=0.4, seed=2)))
    als = wl.eam_fcc_system(6, a0=3.57, species=(wl.CU, wl.NI), type_seed=3)
    cfg = os.path.join(tmp, "alloy.cfg")
    perturbed_config(als, 0.08, 13, cfg)
    cases.append(("alloy_pert_stress", "nve_nbl_eam_stress", cfg,
                  dict(core_potential_file=alloy[0], **{"atomic_e-density_file": alloy[1]},
                       embedding_energy_file=alloy[2], ntypes=2, masses=[63.546, 58.69],
                       timestep=0.0982266, nbl_margin=0.4, seed=2)))
    lj = wl.lj_fcc_system(10)
    cfg = os.path.join(tmp, "lj_pert.cfg")
    perturbed_config(lj, 0.05, 11, cfg)
    cases.append(("lj_pert_stress", "nve_nbl_stress", cfg,
                  dict(potfile=lj2, ntypes=1, masses=1.0, timestep=0.005, nbl_margin=0.3,
                       seed=1)))
    for name, variant, cfg, kw in cases:
        p = os.path.join(tmp, name + ".param")
        tok = dict(coordname=cfg, outfiles=os.path.join(tmp, "o"), ensemble="nve",
                   pbc_dirs=[1, 1, 1], maxsteps=0, starttemp=0.0, eng_int=0,
                   checkpt_int=100000000, box_from_header=1)
        tok.update(kw)
        wl.write_param(p, **tok)
        pre = os.path.join(tmp, name)
        run(variant, p, "forces", pre)
        st = load_state(pre + ".forces")
        box, gdim, cellsz = load_box(pre + ".box")
        tot = np.loadtxt(pre + ".totals")
        stress, tot_stress = load_stress(pre)
        d = dict(box=box, gdim=gdim, cellsz=cellsz, epot_total=tot[0], virial=tot[1],
                 stress=stress, tot_stress=tot_stress, **st)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, "atoms", len(st["x"]), "tot_stress", tot_stress)


def ensemble_cases() -> None:
    """move_atoms_nvt and move_atoms_mik (src/imd_integrate.c:891, :675) run by
    the reference's `nvt` and `mik` builds through the same main_loop steps."""
    subprocess.run(["make", "-s", "-C", ORACLE, "ref"], check=True)
    tmp = tempfile.mkdtemp(prefix="imdgold_ens")
    cu = tuple(os.path.join(HERE, "cu" + e) for e in (".pt", ".rho", ".emb"))
    base = dict(outfiles=os.path.join(tmp, "o"), ntypes=1, masses=63.546,
                pbc_dirs=[1, 1, 1], timestep=0.0982266, maxsteps=0, seed=2,
                core_potential_file=cu[0], **{"atomic_e-density_file": cu[1]},
                embedding_energy_file=cu[2], nbl_margin=0.4, eng_int=0,
                checkpt_int=100000000)
    # NVT from IMD's own generator and maxwell at 300 K
    p = os.path.join(tmp, "cu_nvt.param")
    wl.write_param(p, coordname="_fcc", box_param=[8, 8, 8], box_unit=3.615,
                   ensemble="nvt", starttemp=0.0258520, tau_eta=10.0, **base)
    pre = os.path.join(tmp, "cu_nvt")
    run("nvt_nbl_eam", p, "nve", pre, 100)
    st0 = load_state(pre + ".state0")
    stf = load_state(pre + ".final")
    steps = np.loadtxt(pre + ".steps")
    box, gdim, cellsz = load_box(pre + ".box")
    d = dict(box=box, gdim=gdim, cellsz=cellsz, number=st0["number"], type=st0["type"],
             mass=st0["mass"], x0=st0["x"], p0=st0["p"], epot=steps[:, 1], ekin=steps[:, 2],
             nbl_count=steps[:, 3], eta=steps[:, 4], x_final=stf["x"], p_final=stf["p"],
             dt=0.0982266, skin=0.4, temperature=0.0258520, isq_tau_eta=1.0 / 100.0)
    np.savez_compressed(os.path.join(HERE, "cu_nvt.npz"), **d)
    print("cu_nvt eta", steps[[0, -1], 4], "ekin", steps[[0, -1], 2])
    # MIK quench of cu_pert's configuration
    cus = wl.eam_fcc_system(8)
    cfg = os.path.join(tmp, "cu_pert.cfg")
    perturbed_config(cus, 0.1, 12, cfg)
    p = os.path.join(tmp, "cu_mik.param")
    wl.write_param(p, coordname=cfg, box_from_header=1, ensemble="mik", starttemp=0.0, **base)
    pre = os.path.join(tmp, "cu_mik")
    run("mik_nbl_eam", p, "nve", pre, 200)
    st0 = load_state(pre + ".state0")
    stf = load_state(pre + ".final")
    steps = np.loadtxt(pre + ".steps")
    box, gdim, cellsz = load_box(pre + ".box")
    d = dict(box=box, gdim=gdim, cellsz=cellsz, number=st0["number"], type=st0["type"],
             mass=st0["mass"], x0=st0["x"], p0=st0["p"], epot=steps[:, 1], ekin=steps[:, 2],
             nbl_count=steps[:, 3], fnorm=steps[:, 4], f_max2=steps[:, 5],
             x_final=stf["x"], p_final=stf["p"], dt=0.0982266, skin=0.4)
    np.savez_compressed(os.path.join(HERE, "cu_mik.npz"), **d)
    print("cu_mik epot", steps[[0, -1], 1], "fnorm", steps[[0, -1], 4])


GLOK_CASES = {
    # name: (reference build, steps, parameters beyond the ensemble)
    "cu_fire": ("fire_nbl_eam", 300,
                dict(glok_mix=0.1, glok_mixdec=0.99, glok_incfac=1.1, glok_decfac=0.5,
                     glok_maxtimestep=0.5, glok_minsteps=5)),
    "cu_glok": ("glok_nbl_eam", 200, {}),
    "cu_mixglok": ("mix_glok_nbl_eam", 200, dict(glok_mix=0.05, glok_ekin_threshold=0.004)),
}


def glok_cases() -> None:
    """The glok ensemble (update_glok, src/imd_main_3d.c:972-1055, before
    move_atoms_nve) of the reference's `fire` and `glok` builds on a
    perturbed Cu crystal with a vacancy pair: per step the energies, the
    force norms, the adaptive time step, the mixing factor, P.F and
    glok_start, and the final state."""
    subprocess.run(["make", "-s", "-C", ORACLE, "ref"], check=True)
    tmp = tempfile.mkdtemp(prefix="imdgold_glok")
    cu = tuple(os.path.join(HERE, "cu" + e) for e in (".pt", ".rho", ".emb"))
    cus = wl.eam_fcc_system(8)
    cfg = os.path.join(tmp, "cu_glok.cfg")
    perturbed_config(cus, 0.15, 21, cfg, remove=[5, 900])
    for name, (variant, nsteps, extra) in GLOK_CASES.items():
        p = os.path.join(tmp, name + ".param")
        extra = dict(extra)
        dt = extra.pop("timestep", 0.0982266)
        wl.write_param(p, coordname=cfg, box_from_header=1, ensemble="glok", starttemp=0.0,
                       outfiles=os.path.join(tmp, "o"), ntypes=1, masses=63.546,
                       pbc_dirs=[1, 1, 1], timestep=dt, maxsteps=0, seed=2,
                       core_potential_file=cu[0], **{"atomic_e-density_file": cu[1]},
                       embedding_energy_file=cu[2], nbl_margin=0.4, eng_int=0,
                       checkpt_int=100000000, **extra)
        pre = os.path.join(tmp, name)
        run(variant, p, "glok", pre, nsteps)
        st0 = load_state(pre + ".state0")
        stf = load_state(pre + ".final")
        steps = np.loadtxt(pre + ".steps")
        box, gdim, cellsz = load_box(pre + ".box")
        prm = dict(GLOK_PARAM_DEFAULTS)
        prm.update(extra)
        d = dict(box=box, gdim=gdim, cellsz=cellsz, number=st0["number"], type=st0["type"],
                 mass=st0["mass"], x0=st0["x"], p0=st0["p"], step=steps[:, 0],
                 epot=steps[:, 1], ekin=steps[:, 2], nbl_count=steps[:, 3],
                 fnorm=steps[:, 4], f_max2=steps[:, 5], timestep=steps[:, 6], mix=steps[:, 7],
                 pxf=steps[:, 8], glok_start=steps[:, 9], npxf=steps[:, 10],
                 x_final=stf["x"], p_final=stf["p"], dt=dt, skin=0.4,
                 mix_on=int(variant.startswith(("fire", "mix"))),
                 adapt=int(variant.startswith("fire")),
                 **{"param_" + k: v for k, v in prm.items()})
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, "epot", steps[[0, -1], 1], "dt", steps[[0, -1], 6],
              "restarts", len(np.unique(steps[:, 9])), "nPxF", steps[-1, 10])


def npt_case() -> None:
    """ensemble npt_iso (move_atoms_npt_iso, src/imd_integrate.c:1475-1728)
    of the reference's `npt_iso` build: Cu _fcc 8^3 at 300 K from IMD's
    generator and maxwell, external pressure ramped from 0.01 to 0.005
    eV/A^3 over 200 steps; per step the energies, xi, eta, the pressure,
    the volume and the box."""
    subprocess.run(["make", "-s", "-C", ORACLE, "ref"], check=True)
    tmp = tempfile.mkdtemp(prefix="imdgold_npt")
    cu = tuple(os.path.join(HERE, "cu" + e) for e in (".pt", ".rho", ".emb"))
    nsteps = 200
    prm = dict(temperature=0.0258520, tau_eta=10.0, tau_xi=20.0, pressure_start=0.01,
               pressure_end=0.005)
    p = os.path.join(tmp, "cu_npt.param")
    wl.write_param(p, coordname="_fcc", box_param=[8, 8, 8], box_unit=3.615,
                   ensemble="npt_iso", starttemp=prm["temperature"], tau_eta=prm["tau_eta"],
                   tau_xi=prm["tau_xi"], pressure_start=prm["pressure_start"],
                   pressure_end=prm["pressure_end"], outfiles=os.path.join(tmp, "o"),
                   ntypes=1, masses=63.546, pbc_dirs=[1, 1, 1], timestep=0.0982266,
                   maxsteps=nsteps - 1, seed=2, core_potential_file=cu[0],
                   **{"atomic_e-density_file": cu[1]}, embedding_energy_file=cu[2],
                   nbl_margin=0.4, eng_int=0, checkpt_int=100000000)
    pre = os.path.join(tmp, "cu_npt")
    run("npt_iso_nbl_eam", p, "npt", pre, nsteps)
    st0 = load_state(pre + ".state0")
    stf = load_state(pre + ".final")
    steps = np.loadtxt(pre + ".steps")
    box, gdim, cellsz = load_box(pre + ".box")
    boxf, gdimf, _ = load_box(pre + ".finalbox")
    d = dict(box=box, gdim=gdim, cellsz=cellsz, number=st0["number"], type=st0["type"],
             mass=st0["mass"], x0=st0["x"], p0=st0["p"], epot=steps[:, 1], ekin=steps[:, 2],
             nbl_count=steps[:, 3], xi=steps[:, 4], eta=steps[:, 5], pressure=steps[:, 6],
             volume=steps[:, 7], box_xx=steps[:, 8], pressure_ext=steps[:, 9],
             x_final=stf["x"], p_final=stf["p"], box_final=boxf, gdim_final=gdimf,
             dt=0.0982266, skin=0.4, temperature=prm["temperature"],
             isq_tau_eta=1.0 / prm["tau_eta"] ** 2, isq_tau_xi=1.0 / prm["tau_xi"] ** 2,
             pressure_start=prm["pressure_start"], pressure_end=prm["pressure_end"],
             steps_max=nsteps - 1)
    np.savez_compressed(os.path.join(HERE, "cu_npt.npz"), **d)
    print("cu_npt volume", steps[[0, -1], 7], "pressure", steps[[0, -1], 6], "gdim", gdim,
          gdimf, "rebuilds", steps[-1, 3])


def npt_axial_case() -> None:
    """ensemble npt_axial (move_atoms_npt_axial, src/imd_integrate.c:1747-1960)
    of the reference's `npt_axial` build: the Cu set-up of cu_npt with a
    different external stress per axis and the z axis held (relax_dirs
    1 1 0); per step the energies, xi, eta, the axial stresses and the box
    diagonal."""
    subprocess.run(["make", "-s", "-C", ORACLE, "ref"], check=True)
    tmp = tempfile.mkdtemp(prefix="imdgold_npta")
    cu = tuple(os.path.join(HERE, "cu" + e) for e in (".pt", ".rho", ".emb"))
    nsteps = 200
    prm = dict(temperature=0.0258520, tau_eta=10.0, tau_xi=20.0,
               pressure_start=[0.01, 0.0, -0.005], pressure_end=[0.005, 0.0, -0.005],
               relax_dirs=[1, 1, 0])
    p = os.path.join(tmp, "cu_npt_axial.param")
    wl.write_param(p, coordname="_fcc", box_param=[8, 8, 8], box_unit=3.615,
                   ensemble="npt_axial", starttemp=prm["temperature"], tau_eta=prm["tau_eta"],
                   tau_xi=prm["tau_xi"], pressure_start=prm["pressure_start"],
                   pressure_end=prm["pressure_end"], relax_dirs=prm["relax_dirs"],
                   outfiles=os.path.join(tmp, "o"), ntypes=1, masses=63.546,
                   pbc_dirs=[1, 1, 1], timestep=0.0982266, maxsteps=nsteps - 1, seed=2,
                   core_potential_file=cu[0], **{"atomic_e-density_file": cu[1]},
                   embedding_energy_file=cu[2], nbl_margin=0.4, eng_int=0,
                   checkpt_int=100000000)
    pre = os.path.join(tmp, "cu_npt_axial")
    run("npt_axial_nbl_eam", p, "npt", pre, nsteps)
    st0 = load_state(pre + ".state0")
    stf = load_state(pre + ".final")
    steps = np.loadtxt(pre + ".steps")
    box, gdim, cellsz = load_box(pre + ".box")
    boxf, gdimf, _ = load_box(pre + ".finalbox")
    d = dict(box=box, gdim=gdim, cellsz=cellsz, number=st0["number"], type=st0["type"],
             mass=st0["mass"], x0=st0["x"], p0=st0["p"], epot=steps[:, 1], ekin=steps[:, 2],
             nbl_count=steps[:, 3], xi=steps[:, 4:7], eta=steps[:, 7], stress=steps[:, 8:11],
             box_diag=steps[:, 11:14], x_final=stf["x"], p_final=stf["p"], box_final=boxf,
             gdim_final=gdimf, dt=0.0982266, skin=0.4, temperature=prm["temperature"],
             isq_tau_eta=1.0 / prm["tau_eta"] ** 2, isq_tau_xi=1.0 / prm["tau_xi"] ** 2,
             pressure_start=np.array(prm["pressure_start"]),
             pressure_end=np.array(prm["pressure_end"]),
             relax_dirs=np.array(prm["relax_dirs"], np.int32), steps_max=nsteps - 1)
    np.savez_compressed(os.path.join(HERE, "cu_npt_axial.npz"), **d)
    print("cu_npt_axial box", steps[[0, -1], 11:14], "stress", steps[[0, -1], 8:11])


# IMD's INIT values of the glok parameters (src/globals.h:580-600)
GLOK_PARAM_DEFAULTS = dict(glok_ekin_threshold=100.0, glok_fmaxcrit=10000.0, glok_mix=0.0,
                           glok_mixdec=1.0, glok_incfac=1.02, glok_decfac=0.5,
                           glok_maxtimestep=0.0, glok_minsteps=5, min_nPxF=0)


def lj1000_case() -> None:
    """The plain-method LJ workload (4000 atoms, T* 0.72, dt 0.005, skin 0.3)
    for all of its 1000 steps, with snapshots every 250 steps."""
    subprocess.run(["make", "-s", "-C", ORACLE, "ref"], check=True)
    tmp = tempfile.mkdtemp(prefix="imdgold_lj")
    lj2 = os.path.join(HERE, "lj.pt")
    lj = wl.lj_fcc_system(10)
    p = os.path.join(tmp, "lj.param")
    wl.write_param(p, coordname="_fcc", outfiles=os.path.join(tmp, "o"), ensemble="nve",
                   ntypes=1, masses=1.0, pbc_dirs=[1, 1, 1], timestep=0.005, maxsteps=0,
                   starttemp=0.72, seed=1, potfile=lj2, nbl_margin=0.3, eng_int=0,
                   checkpt_int=100000000, box_param=[10, 10, 10], box_unit=lj.meta["a0"])
    pre = os.path.join(tmp, "lj")
    every = 250
    run("nve_nbl", p, "snap", pre, 1000, every)
    steps = np.loadtxt(pre + ".steps")
    box, gdim, cellsz = load_box(pre + ".box")
    snaps = list(range(0, 1001, every))
    x, pp, f, ep = [], [], [], []
    for k in snaps:
        a = load_state(pre + ".pre%05d" % k)
        b = load_state(pre + ".snap%05d" % k)
        x.append(a["x"])
        pp.append(a["p"])
        f.append(b["f"])
    st0 = load_state(pre + ".pre00000")
    d = dict(box=box, gdim=gdim, cellsz=cellsz, number=st0["number"], type=st0["type"],
             mass=st0["mass"], snap_steps=np.array(snaps), snap_x=np.array(x),
             snap_p=np.array(pp), snap_f=np.array(f), epot=steps[:, 1], ekin=steps[:-1, 2],
             nbl_count=steps[:, 3], dt=0.005, skin=0.3)
    np.savez_compressed(os.path.join(HERE, "lj_nve1000.npz"), **d)
    print("lj_nve1000 steps", len(steps), "rebuilds", steps[-1, 3])


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "stress":
        stress_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == "ensembles":
        ensemble_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == "lj1000":
        lj1000_case()
    elif len(sys.argv) > 1 and sys.argv[1] == "glok":
        glok_cases()
    elif len(sys.argv) > 1 and sys.argv[1] == "npt":
        npt_case()
        npt_axial_case()
    else:
        main()
        stress_cases()
        ensemble_cases()
        lj1000_case()
        glok_cases()
        npt_case()
        npt_axial_case()
