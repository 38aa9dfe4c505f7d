"""Pins the C oracle (restatement of IMD's hot path) to outputs of the
unmodified reference built here (tests/golden/, made by make_golden.py).

CPU only.  Bars: pair sets identical (keys and r^2 bits), forces within
1e-11 relative RMS, per-atom energies / rho / dF within 1e-11, totals within
1e-12 relative.
"""
import numpy as np
import pytest

import oracle
from conftest import golden, tables
from oracle import OracleSystem, OracleTable, canonical  # noqa: F401

Q, F4, SP = oracle.QUADRATIC, oracle.FOURPOINT, oracle.SPLINE
# name -> (tables, eam, ntypes, skin, interpolation)
CASES = {
    "lj_pert": ("lj", False, 1, 0.3, Q),
    "lj_pert_f1": ("lj_f1", False, 1, 0.3, Q),
    "cu_pert": ("cu", True, 1, 0.4, Q),
    "alloy_pert": ("cuni", True, 2, 0.4, Q),
    "tri_cg": ("cu", True, 1, 0.4, Q),
    "cu_pert_spline": ("cu", True, 1, 0.4, SP),
    "cu_pert_4point": ("cu", True, 1, 0.4, F4),
    "defect_cg_spline": ("cu", True, 1, 0.4, SP),
}


def rel_rms(a, b):
    return np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2))


def make(name):
    g = golden(name)
    tab, eam, nt, skin, mode = CASES[name]
    oracle.set_interpolation(mode)
    try:
        s = OracleSystem(g["box"], g["x"], g["type"], g["mass"], g["number"], nt,
                         tables(tab), eam, skin)
    finally:
        oracle.set_interpolation(Q)
    return g, s


@pytest.mark.parametrize("name", list(CASES))
def test_forces_match_reference(name):
    g, s = make(name)
    assert tuple(s.s.gdim) == tuple(g["gdim"])
    assert s.s.cellsz == g["cellsz"]
    s.calc_forces()
    # order: fixtures are sorted by number, oracle keeps input order (= same)
    assert rel_rms(s.f, g["f"]) < 1e-11
    assert np.max(np.abs(s.epot - g["epot"])) <= 1e-11 * np.max(np.abs(g["epot"]))
    assert abs(s.epot_total - g["epot_total"]) <= 1e-12 * abs(g["epot_total"])
    assert abs(s.virial - g["virial"]) <= 1e-12 * abs(g["virial"])
    # the compensated totals sum the same terms
    assert abs(s.epot_total_exact - g["epot_total"]) <= 1e-12 * abs(g["epot_total"])
    assert abs(s.virial_exact - g["virial"]) <= 1e-12 * abs(g["virial"])
    if CASES[name][1]:
        assert np.max(np.abs(s.rho - g["rho"])) <= 1e-11 * np.max(g["rho"])
        assert np.max(np.abs(s.df - g["df"])) <= 1e-11 * np.max(np.abs(g["df"]))


@pytest.mark.parametrize("name", list(CASES))
def test_pair_set_identical(name):
    import hashlib
    g, s = make(name)
    s.calc_forces()
    key, r2 = s.pairs()
    assert len(key) == int(g["npairs"])
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(key, np.int64).tobytes())
    h.update(np.ascontiguousarray(r2, np.float64).tobytes())
    assert h.hexdigest() == str(g["pair_digest"])
    if "pair_key" in g:
        np.testing.assert_array_equal(key, g["pair_key"])
        np.testing.assert_array_equal(r2, g["pair_r2"])


def test_order_independent_pair_digest():
    """pair_digest (used where a pair set is too large to sort) is the same
    for the reference's canonical pair set and for the oracle's list in list
    order, and changes with one bit of one r^2."""
    from oracle import decode_keys, pair_digest
    g, s = make("tri_cg")
    s.calc_forces()
    ni, nj, sh, r2 = s.raw_pairs()
    lo, hi, gsh = decode_keys(g["pair_key"])
    ref = pair_digest(lo, hi, gsh, g["pair_r2"])
    assert pair_digest(ni, nj, sh, r2) == ref
    perm = np.random.default_rng(3).permutation(len(ni))
    assert pair_digest(nj[perm], ni[perm], -sh[perm], r2[perm], chunk=1000) == ref
    r2b = r2.copy()
    r2b[17] = np.nextafter(r2b[17], np.inf)
    assert pair_digest(ni, nj, sh, r2b) != ref


@pytest.mark.parametrize("name,tab,eam,skin", [("lj_nve", "lj", False, 0.3),
                                               ("cu_nve", "cu", True, 0.4)])
def test_nve_trajectory_matches_reference(name, tab, eam, skin):
    """Same start state (IMD's own generator + maxwell), same steps.  The
    summation order of forces differs from the reference, so trajectories
    separate by rounding; energies agree to 1e-9 relative over the run and
    the list is rebuilt on the same steps."""
    g = golden(name)
    s = OracleSystem(g["box"], g["x0"], g["type"], g["mass"], g["number"], 1, tables(tab),
                     eam, skin, timestep=float(g["dt"]), p=g["p0"])
    nsteps = len(g["epot"])
    ep, ek = s.nve(nsteps)
    np.testing.assert_allclose(ep, g["epot"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(ek, g["ekin"], rtol=1e-8, atol=0)
    assert s.nbl_count == int(g["nbl_count"][-1])


@pytest.mark.parametrize("name", ["tri_cg", "defect_cg_spline"])
def test_cg_relaxation_matches_reference(name):
    g, s = make(name)
    steps, fm = s.cg_relax(1e-4)
    assert fm <= 1e-4
    # final energy equal to the reference's to 1e-6 eV/atom; CG path length
    # may differ by a few steps through rounding
    assert abs(s.epot_total - float(g["cg_epot"])) / s.n <= 1e-6
    assert 0.5 * int(g["cg_steps"]) <= steps <= 2 * int(g["cg_steps"]) + 3


def test_interpolation_modes_differ_from_quadratic():
    """The three interpolations give different forces on the same atoms:
    the spline / 4-point fixtures test something the quadratic ones do not."""
    q, sp, f4 = golden("cu_pert"), golden("cu_pert_spline"), golden("cu_pert_4point")
    assert np.array_equal(q["x"], sp["x"]) and np.array_equal(q["x"], f4["x"])
    assert rel_rms(sp["f"], q["f"]) > 1e-9 and rel_rms(f4["f"], q["f"]) > 1e-9
    assert rel_rms(sp["f"], f4["f"]) > 1e-9


def test_table_reader_quirks():
    """format 1: end = r2 of the last nonzero value; threepoint rows."""
    t2 = OracleTable(tables("lj")[0], 1, True)
    t1 = OracleTable(tables("lj_f1")[0], 1, True)
    assert t2.t.len[0] == 1000 and t2.t.maxsteps == 1000
    assert abs(t2.cellsz.value - 6.25) < 1e-12
    assert t1.t.len[0] == 300
    assert t1.t.end[0] == 6.25
    # values continue the quadratic through the extra rows
    r2 = np.linspace(0.5, 7.0, 1001)
    pot, grad = t2.pair_int2(0, 1, r2)
    assert np.all(np.isfinite(pot)) and np.all(np.isfinite(grad))
    assert abs(pot[-1]) < 1e-12 * abs(pot[0])


STRESS = {"cu_pert_stress": ("cu", True, 1, 0.4), "alloy_pert_stress": ("cuni", True, 2, 0.4),
          "lj_pert_stress": ("lj", False, 1, 0.3)}


@pytest.mark.parametrize("name", list(STRESS))
def test_stress_matches_reference(name):
    """STRESS_TENS: per-atom PRESSTENS within 1e-11 of the largest component,
    the total tensor (calc_tot_presstens) within 1e-12 relative; its trace is
    the virial."""
    g = golden(name)
    tab, eam, nt, skin = STRESS[name]
    s = OracleSystem(g["box"], g["x"], g["type"], g["mass"], g["number"], nt, tables(tab),
                     eam, skin)
    s.set_stress(True)
    s.calc_forces()
    scale = np.max(np.abs(g["stress"]))
    assert np.max(np.abs(s.stress - g["stress"])) <= 1e-11 * scale
    tot = s.tot_stress
    assert np.all(np.abs(tot - g["tot_stress"]) <= 1e-12 * np.max(np.abs(g["tot_stress"])))
    assert abs(tot[:3].sum() - g["virial"]) <= 1e-11 * abs(g["virial"])
    assert rel_rms(s.f, g["f"]) < 1e-11


def test_nvt_trajectory_matches_reference():
    """move_atoms_nvt (Nose-Hoover): same start, 100 steps; energies to 1e-9
    relative, the thermostat variable eta to 1e-8 relative (1e-12 absolute),
    the same list rebuilds."""
    g = golden("cu_nvt")
    s = OracleSystem(g["box"], g["x0"], g["type"], g["mass"], g["number"], 1, tables("cu"),
                     True, float(g["skin"]), timestep=float(g["dt"]), p=g["p0"])
    s.set_nvt(float(g["temperature"]), float(g["isq_tau_eta"]))
    ep, ek, eta = s.md(len(g["epot"]), "nvt")
    np.testing.assert_allclose(ep, g["epot"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(ek, g["ekin"], rtol=1e-8, atol=0)
    np.testing.assert_allclose(eta, g["eta"], rtol=1e-8, atol=1e-12)
    assert s.nbl_count == int(g["nbl_count"][-1])


def test_mik_quench_matches_reference():
    """move_atoms_mik: 200 quench steps from a perturbed lattice; energies to
    1e-9 relative, force norms to 1e-6 relative (a momentum zeroed one step
    apart would show far above that), final positions to 1e-8 A."""
    g = golden("cu_mik")
    s = OracleSystem(g["box"], g["x0"], g["type"], g["mass"], g["number"], 1, tables("cu"),
                     True, float(g["skin"]), timestep=float(g["dt"]), p=g["p0"])
    ep, ek, fn = s.md(len(g["epot"]), "mik")
    np.testing.assert_allclose(ep, g["epot"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(ek, g["ekin"], rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(fn, g["fnorm"], rtol=1e-6, atol=0)
    d = s.x - g["x_final"]
    d -= np.round(d @ np.linalg.inv(g["box"])) @ g["box"]
    assert np.abs(d).max() < 1e-8


def glok_params(g) -> dict:
    """The glok parameters a golden run used (IMD's names)."""
    out = {"mix_on": int(g["mix_on"]), "adapt": int(g["adapt"])}
    for k in g:
        if k.startswith("param_"):
            name = k[len("param_"):]
            out[name] = int(g[k]) if name in ("glok_minsteps", "min_nPxF") else float(g[k])
    return out


@pytest.mark.parametrize("name", ["cu_fire", "cu_glok", "cu_mixglok"])
def test_glok_matches_reference(name):
    """update_glok + move_atoms_nve of the `fire`, `glok` and `mix glok`
    builds (the last restarting on glok_ekin_threshold): the
    decisions of every step (time step, mixing factor, restarts) identical,
    energies to 1e-12, P.F to 1e-8 relative, final positions to 1e-12 A."""
    g = golden(name)
    s = OracleSystem(g["box"], g["x0"], g["type"], g["mass"], g["number"], 1, tables("cu"),
                     True, float(g["skin"]), timestep=float(g["dt"]), p=g["p0"])
    out, st = s.glok(len(g["epot"]), 0, **glok_params(g))
    np.testing.assert_array_equal(out[:, 4], g["timestep"])
    np.testing.assert_array_equal(out[:, 5], g["mix"])
    np.testing.assert_array_equal(out[:, 7], g["glok_start"])
    assert st.nPxF == int(g["npxf"][-1])
    np.testing.assert_allclose(out[:, 0], g["epot"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(out[:, 1], g["ekin"], rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose(out[:, 2], g["fnorm"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(out[:, 6], g["pxf"], rtol=1e-8, atol=1e-12)
    d = s.x - g["x_final"]
    d -= np.round(d @ np.linalg.inv(g["box"])) @ g["box"]
    assert np.abs(d).max() < 1e-12
    # the runs exercise the restarts (and, for fire, the adaptive step)
    assert len(np.unique(g["glok_start"])) > 3
    if g["adapt"]:
        assert g["timestep"].max() > g["timestep"][0] and int(g["npxf"][-1]) > 0


def npt_params(g) -> dict:
    """The npt_iso parameters of a golden run (IMD's names)."""
    return dict(temperature=float(g["temperature"]), isq_tau_eta=float(g["isq_tau_eta"]),
                isq_tau_xi=float(g["isq_tau_xi"]), pressure_ext=float(g["pressure_start"]),
                pressure_end=float(g["pressure_end"]), steps_min=0,
                steps_max=int(g["steps_max"]))


def test_npt_iso_matches_reference():
    """move_atoms_npt_iso with the box scaled every step, 200 steps against
    the reference's `npt_iso` build: energies, xi, eta, the pressure and the
    box to 1e-12 relative, final positions to 1e-10 A."""
    g = golden("cu_npt")
    s = OracleSystem(g["box"], g["x0"], g["type"], g["mass"], g["number"], 1, tables("cu"),
                     True, float(g["skin"]), timestep=float(g["dt"]), p=g["p0"])
    out, st = s.npt(len(g["epot"]), 0, **npt_params(g))
    for j, k in enumerate(["epot", "ekin", "xi", "eta", "pressure", "volume", "box_xx",
                           "pressure_ext"]):
        np.testing.assert_allclose(out[:, j], g[k], rtol=1e-12, atol=1e-15, err_msg=k)
    box = np.array(s.s.box)
    np.testing.assert_allclose(box, g["box_final"], rtol=1e-12, atol=0)
    d = s.x - g["x_final"]
    d -= np.round(d @ np.linalg.inv(box)) @ box
    assert np.abs(d).max() < 1e-10
    # the run changes the volume by far more than the tolerance of the bars
    assert g["volume"][-1] / g["volume"][0] - 1.0 > 5e-3


def test_npt_axial_matches_reference():
    """move_atoms_npt_axial (P_AXIAL virial components, a barostat per
    axis, z held by relax_dirs) against the reference's `npt_axial` build
    over 200 steps: energies, xi, eta, the axial stresses and the box to
    1e-12 relative, final positions to 1e-10 A."""
    g = golden("cu_npt_axial")
    s = OracleSystem(g["box"], g["x0"], g["type"], g["mass"], g["number"], 1, tables("cu"),
                     True, float(g["skin"]), timestep=float(g["dt"]), p=g["p0"])
    out, st = s.npt_axial(len(g["epot"]), 0, temperature=float(g["temperature"]),
                          isq_tau_eta=float(g["isq_tau_eta"]), isq_tau_xi=float(g["isq_tau_xi"]),
                          pressure_ext=list(g["pressure_start"]),
                          pressure_end=list(g["pressure_end"]),
                          relax_dirs=[int(v) for v in g["relax_dirs"]], steps_min=0,
                          steps_max=int(g["steps_max"]))
    np.testing.assert_allclose(out[:, 0], g["epot"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(out[:, 1], g["ekin"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(out[:, 2:5], g["xi"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(out[:, 5], g["eta"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(out[:, 6:9], g["stress"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(out[:, 9:12], g["box_diag"], rtol=1e-12, atol=0)
    box = np.array(s.s.box)
    np.testing.assert_allclose(box, g["box_final"], rtol=1e-12, atol=0)
    d = s.x - g["x_final"]
    d -= np.round(d @ np.linalg.inv(box)) @ box
    assert np.abs(d).max() < 1e-10
    # the axes move apart, the held one stays
    assert g["box_diag"][-1, 2] == g["box_diag"][0, 2]
    assert abs(g["box_diag"][-1, 1] / g["box_diag"][0, 1] - 1.0) > 5e-3


@pytest.mark.parametrize("name", ["cu_pert", "alloy_pert", "lj_pert"])
def test_p_axial_virial_is_the_stress_diagonal(name):
    """IMD's P_AXIAL sums (vir_xx -= d_x f_x over pairs) equal the diagonal
    of calc_tot_presstens (every pair puts -d_a f_b / 2 on both atoms'
    PRESSTENS): the identity the device uses for npt_axial.  Their sum is
    the virial."""
    g, s = make(name)
    s.set_stress(True)
    s.calc_forces()
    va = np.array(s.s.vir_axial[:])
    np.testing.assert_allclose(va, s.tot_stress[:3], rtol=1e-12, atol=0)
    assert abs(va.sum() - s.virial) <= 1e-12 * abs(s.virial)


def test_npt_iso_new_cell_grid():
    """A box that shrinks out of its height bounds gets a new cell grid
    (make_box calling init_cells, src/imd_geom_3d.c:82-86) and a new list;
    the forces on the new grid equal those of a fresh system on that box."""
    g = golden("cu_npt")
    # a crystal stretched by 9.5 %, pulled further by a negative pressure: its
    # box grows past the largest height of the 3x3x3 grid within 20 steps
    s = OracleSystem(g["box"] * 1.095, g["x0"] * 1.095, g["type"], g["mass"], g["number"], 1,
                     tables("cu"), True, float(g["skin"]), timestep=float(g["dt"]), p=g["p0"])
    prm = npt_params(g)
    prm.update(pressure_ext=-0.2, pressure_end=-0.2, isq_tau_xi=1.0 / 25.0, steps_max=19)
    out, st = s.npt(20, 0, **prm)
    assert list(s.s.gdim) == [4, 4, 4]               # 3x3x3 at the start
    s.calc_forces()
    box = np.array(s.s.box)
    t = OracleSystem(box, s.x.copy(), g["type"], g["mass"], g["number"], 1, tables("cu"),
                     True, float(g["skin"]), timestep=float(g["dt"]), p=s.p.copy())
    t.calc_forces()
    assert rel_rms(s.f, t.f) < 1e-12
    assert abs(s.epot_total - t.epot_total) <= 1e-12 * abs(t.epot_total)


def test_lj_1000_steps_segmentwise():
    """The plain-method LJ run over all 1000 steps, step by step: from each
    of the reference's snapshots (every 250 steps) the oracle reproduces the
    forces of that step (1e-11 relative RMS) and the energies of the next
    250 steps (1e-9 relative)."""
    g = golden("lj_nve1000")
    snaps = list(g["snap_steps"])
    for k, st in enumerate(snaps):
        s = OracleSystem(g["box"], g["snap_x"][k], g["type"], g["mass"], g["number"], 1,
                         tables("lj"), False, float(g["skin"]), timestep=float(g["dt"]),
                         p=g["snap_p"][k])
        s.calc_forces()
        assert rel_rms(s.f, g["snap_f"][k]) < 1e-11
        assert abs(s.epot_total - g["epot"][st]) <= 1e-12 * abs(g["epot"][st])
        if st == snaps[-1]:
            continue
        s = OracleSystem(g["box"], g["snap_x"][k], g["type"], g["mass"], g["number"], 1,
                         tables("lj"), False, float(g["skin"]), timestep=float(g["dt"]),
                         p=g["snap_p"][k])
        n = snaps[k + 1] - st
        ep, ek = s.nve(n)
        np.testing.assert_allclose(ep, g["epot"][st:st + n], rtol=1e-9, atol=0)
        np.testing.assert_allclose(ek, g["ekin"][st:st + n], rtol=1e-8, atol=0)
