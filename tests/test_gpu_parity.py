"""GPU parity: libimdgpu (through its C-ABI) against the oracle and against
the golden vectors of the reference.

Bars (from the benchmark spec of this path): neighbour pair sets identical
(pair keys and r^2 bits), per-atom forces within 1e-11 relative RMS, energy
and virial within 1e-12 relative.
"""
import hashlib

import numpy as np
import pytest

from conftest import golden, tables

pytestmark = pytest.mark.gpu

CASES = {
    "lj_pert": ("lj", 0, 1, 0.3),
    "lj_pert_f1": ("lj_f1", 0, 1, 0.3),
    "cu_pert": ("cu", 1, 1, 0.4),
    "alloy_pert": ("cuni", 1, 2, 0.4),
    "tri_cg": ("cu", 1, 1, 0.4),
}


def rel_rms(a, b):
    return np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2))


def gpu_system(g, tab, eam, nt, skin, x=None, p=None, precision=0, interpolation=0):
    from imd_gb300 import api
    s = api.GpuSystem(nt, api.EAM2 if eam else api.PAIR, precision, interpolation)
    s.read_tables(tables(tab), default_format=2 if eam else 1)
    s.set_box(g["box"], (1, 1, 1), skin)
    s.set_atoms(g["number"], g["type"], g["mass"], g["x"] if x is None else x, p)
    return s


def digest(key, r2):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(key, np.int64).tobytes())
    h.update(np.ascontiguousarray(r2, np.float64).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", list(CASES))
def test_forces_match_reference(name):
    g = golden(name)
    tab, eam, nt, skin = CASES[name]
    s = gpu_system(g, tab, eam, nt, skin)
    rc = s.calc_forces(0)
    assert rc == 0
    a = s.get_atoms()
    sc = s.scalars()
    assert tuple(sc.gdim) == tuple(g["gdim"])
    assert rel_rms(a["f"], g["f"]) < 1e-11
    assert np.max(np.abs(a["epot"] - g["epot"])) <= 1e-11 * np.max(np.abs(g["epot"]))
    assert abs(sc.tot_pot_energy - g["epot_total"]) <= 1e-12 * abs(g["epot_total"])
    assert abs(sc.virial - g["virial"]) <= 1e-12 * abs(g["virial"])
    if eam:
        assert np.max(np.abs(a["rho"] - g["rho"])) <= 1e-11 * np.max(g["rho"])
        assert np.max(np.abs(a["df"] - g["df"])) <= 1e-11 * np.max(np.abs(g["df"]))


@pytest.mark.parametrize("name", list(CASES))
def test_pair_set_identical_to_reference(name):
    from oracle import canonical
    g = golden(name)
    tab, eam, nt, skin = CASES[name]
    s = gpu_system(g, tab, eam, nt, skin)
    s.calc_forces(0)
    ni, nj, sh, r2 = s.pairs()
    key, r2s = canonical(ni, nj, sh, r2)
    assert len(key) == int(g["npairs"])
    assert digest(key, r2s) == str(g["pair_digest"])
    if "pair_key" in g:
        np.testing.assert_array_equal(key, g["pair_key"])
        np.testing.assert_array_equal(r2s, g["pair_r2"])


@pytest.mark.parametrize("name", ["cu_pert", "alloy_pert", "lj_pert"])
def test_forces_match_oracle_bitwise_tables(name):
    """Against the oracle on the same inputs: per-atom energies and forces
    agree to rounding of the summation order only."""
    from oracle import OracleSystem
    g = golden(name)
    tab, eam, nt, skin = CASES[name]
    rng = np.random.default_rng(5)
    x = g["x"] + 0.02 * rng.standard_normal(g["x"].shape)
    o = OracleSystem(g["box"], x, g["type"], g["mass"], g["number"], nt, tables(tab),
                     bool(eam), skin)
    o.calc_forces()
    s = gpu_system(g, tab, eam, nt, skin, x=x)
    s.calc_forces(0)
    a = s.get_atoms()
    assert rel_rms(a["f"], o.f) < 1e-12
    assert abs(s.scalars().tot_pot_energy - o.epot_total) <= 1e-12 * abs(o.epot_total)


@pytest.mark.parametrize("name,tab,eam,skin", [("lj_nve", "lj", 0, 0.3),
                                               ("cu_nve", "cu", 1, 0.4)])
def test_nve_run_matches_reference(name, tab, eam, skin):
    """main_loop NVE steps on the device against the reference's own run
    (same start state from IMD's generator and maxwell)."""
    g = golden(name)
    gg = dict(g)
    gg["x"] = g["x0"]
    s = gpu_system(gg, tab, eam, 1, skin, p=g["p0"])
    nsteps = len(g["epot"])
    ep, ek = s.nve_run(nsteps, float(g["dt"]))
    np.testing.assert_allclose(ep, g["epot"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(ek, g["ekin"], rtol=1e-8, atol=0)
    assert s.scalars().nbl_count == int(g["nbl_count"][-1])


def test_stepwise_api_matches_fused_run():
    """calc_forces / move_atoms_nve / check_nblist one call at a time (the
    order of main_loop) gives the same trajectory as nve_run."""
    g = golden("cu_nve")
    gg = dict(g)
    gg["x"] = g["x0"]
    a = gpu_system(gg, "cu", 1, 1, 0.4, p=g["p0"])
    b = gpu_system(gg, "cu", 1, 1, 0.4, p=g["p0"])
    dt = float(g["dt"])
    ep_a, _ = a.nve_run(30, dt)
    ep_b = []
    for st in range(30):
        b.calc_forces(st)
        ep_b.append(b.scalars().tot_pot_energy)
        b.move_atoms_nve(dt)
        b.check_nblist()
    np.testing.assert_allclose(ep_a, ep_b, rtol=1e-11)


def test_cg_relaxation_matches_reference():
    g = golden("tri_cg")
    s = gpu_system(g, "cu", 1, 1, 0.4)
    steps, fm = s.cg_relax(1e-4)
    assert fm <= 1e-4
    e = s.scalars().tot_pot_energy
    # the final energy is the bar (1e-6 eV/atom); the number of line
    # searches depends on rounding of the force sums and may differ
    assert abs(e - float(g["cg_epot"])) / len(g["x"]) <= 1e-6
    assert 0.5 * int(g["cg_steps"]) <= steps <= 2 * int(g["cg_steps"])


def test_list_regrow_keeps_parity():
    """A crowded region makes the first capacity estimate too small; the
    library grows the list and the result still matches the oracle."""
    from oracle import OracleSystem
    g = golden("cu_pert")
    x = g["x"].copy()
    L = g["box"][0, 0]
    sel = x[:, 0] < 0.25 * L
    x[sel, 0] *= 0.8   # compress a slab: +25 % density there
    o = OracleSystem(g["box"], x, g["type"], g["mass"], g["number"], 1, tables("cu"), True, 0.4)
    o.calc_forces()
    s = gpu_system(g, "cu", 1, 1, 0.4, x=x)
    s.calc_forces(0)
    a = s.get_atoms()
    assert rel_rms(a["f"], o.f) < 1e-12


def test_short_distance_is_reported():
    g = golden("cu_pert")
    x = g["x"].copy()
    x[1] = x[0] + np.array([1.0, 0.0, 0.0])   # below the table begin (1.5 A)
    s = gpu_system(g, "cu", 1, 1, 0.4, x=x)
    assert s.calc_forces(0) == 1
    assert s.scalars().short_distance == 1


def test_bad_inputs_are_errors():
    from imd_gb300 import api
    g = golden("cu_pert")
    s = api.GpuSystem(1, api.EAM2)
    with pytest.raises(api.IMDGPUError):
        s.calc_forces(0)            # no tables / atoms yet
    s.read_tables(tables("cu"))
    s.set_box(np.diag([6.0, 6.0, 6.0]), (1, 1, 1), 0.4)   # smaller than one list radius
    s.set_atoms(g["number"][:10], g["type"][:10], g["mass"][:10], g["x"][:10] * 0.2)
    with pytest.raises(api.IMDGPUError):
        s.calc_forces(0)
    with pytest.raises(api.IMDGPUError):
        s.set_atoms(g["number"][:10], g["type"][:10] + 3, g["mass"][:10], g["x"][:10])
    # a NaN in a host buffer (IMD's arrays after a blow-up) is refused before upload
    x = g["x"][:10].copy()
    x[3, 1] = np.nan
    with pytest.raises(api.IMDGPUError):
        s.set_atoms(g["number"][:10], g["type"][:10], g["mass"][:10], x)
    with pytest.raises(api.IMDGPUError):
        s.set_atoms(g["number"][:10], g["type"][:10], np.zeros(10), g["x"][:10])


def test_put_state_refuses_non_finite():
    """put_state checks the uploaded values on the device: a NaN or an inf
    momentum is an error naming the lowest bad atom, and the state on the
    device stays the one before the call."""
    from imd_gb300 import api
    g = golden("cu_pert")
    tab, eam, nt, skin = CASES["cu_pert"]
    p0 = np.random.default_rng(3).normal(0.0, 0.5, g["x"].shape)
    s = gpu_system(g, tab, eam, nt, skin, p=p0)
    s.calc_forces(0)
    e0 = s.scalars()
    a0 = s.get_atoms()
    x, p = g["x"].copy(), p0.copy()
    p[17, 2] = np.nan
    p[40, 0] = np.inf
    with pytest.raises(api.IMDGPUError, match="atom 17"):
        s.put_state(x, p)
    x[5, 0] = -np.inf
    with pytest.raises(api.IMDGPUError, match="atom 5"):
        s.put_state(x, None)
    s.calc_forces(1)
    e1 = s.scalars()
    # forces are summed with atomics: equal to rounding of the order
    assert abs(e1.tot_pot_energy - e0.tot_pot_energy) <= 1e-13 * abs(e0.tot_pot_energy)
    a = s.get_atoms()
    assert np.array_equal(a["x"], a0["x"]) and np.array_equal(a["p"], a0["p"])
    assert rel_rms(a["f"], a0["f"]) < 1e-13


@pytest.mark.parametrize("name", ["cu_pert", "alloy_pert", "lj_pert"])
def test_exact_mode_matches_reference(name):
    """IMD's unfused table arithmetic (parity mode) also meets the bars."""
    g = golden(name)
    tab, eam, nt, skin = CASES[name]
    s = gpu_system(g, tab, eam, nt, skin)
    s.set_exact(True)
    s.calc_forces(0)
    a = s.get_atoms()
    assert rel_rms(a["f"], g["f"]) < 1e-11
    assert abs(s.scalars().tot_pot_energy - g["epot_total"]) <= 1e-12 * abs(g["epot_total"])


@pytest.mark.parametrize("name", ["cu_pert", "alloy_pert", "lj_pert", "tri_cg"])
def test_mixed_precision_force_error(name):
    """FP32 pair/EAM arithmetic, FP64 accumulation: force RMS error within
    1e-5 of the FP64 reference, energy within 1e-6 relative."""
    from imd_gb300 import api
    g = golden(name)
    tab, eam, nt, skin = CASES[name]
    s = gpu_system(g, tab, eam, nt, skin, precision=api.MIXED)
    s.calc_forces(0)
    a = s.get_atoms()
    err = rel_rms(a["f"], g["f"])
    assert err < 1e-5, err
    de = abs(s.scalars().tot_pot_energy - g["epot_total"]) / abs(g["epot_total"])
    assert de < 1e-6, de
    np.testing.assert_allclose(a["epot"], g["epot"], rtol=0, atol=1e-5 * np.max(np.abs(g["epot"])))


def test_mixed_fused_rows_match_per_table_lookups(tmp_path):
    """One species whose pair and density tables are quadratic on one grid
    (the Sutton-Chen Cu tables) takes the fused-row force pass, with the rows
    staged in shared memory or read from global memory (the same bits); the
    same physics written as two identical species takes the per-table
    lookups.  All agree to FP32 rounding and are within the mixed bar of
    FP64."""
    from imd_gb300 import api
    from imd_gb300 import workloads as wl
    st = wl.eam_fcc_system(12, a0=3.615, T=300.0, seed=5)
    x = st.x + 0.05 * np.random.default_rng(6).standard_normal(st.x.shape)
    one = wl.sutton_chen_tables(str(tmp_path / "one"), [wl.CU])
    two = wl.sutton_chen_tables(str(tmp_path / "two"), [wl.CU, wl.CU])
    res = {}
    for key, tabs, nt, prec in (("fused", one, 1, api.MIXED), ("global", one, 1, api.MIXED),
                                ("split", two, 2, api.MIXED), ("fp64", one, 1, api.FP64)):
        s = api.GpuSystem(nt, api.EAM2, prec)
        s.set_table_staging(key != "global")
        s.read_tables(tabs)
        s.set_box(st.box, (1, 1, 1), 0.4)
        s.set_atoms(st.number, st.types, st.mass, x, st.p)
        assert s.calc_forces(0) == 0
        res[key] = (s.get_atoms()["f"], s.scalars().tot_pot_energy)
        s.close()
    f64, e64 = res["fp64"]
    np.testing.assert_array_equal(res["fused"][0], res["global"][0])
    assert abs(res["fused"][1] - res["global"][1]) <= 1e-12 * abs(e64)
    assert rel_rms(res["fused"][0], res["split"][0]) < 1e-6
    assert abs(res["fused"][1] - res["split"][1]) <= 1e-7 * abs(e64)
    for key in ("fused", "split"):
        assert rel_rms(res[key][0], f64) < 1e-5, key
        assert abs(res[key][1] - e64) <= 1e-6 * abs(e64), key


def test_pair_cache_matches_recomputed_terms(tmp_path):
    """FP64 Sutton-Chen Cu (one species, pair and density tables on one
    grid): the force pass reading the density pass's cached pair terms gives
    the forces of the pass that computes them again (FP64 atomics change the
    last bits from run to run, hence 1e-14), the same energies and, over 30
    NVE steps with rebuilds, the same trajectory."""
    from imd_gb300 import api
    from imd_gb300 import workloads as wl
    st = wl.eam_fcc_system(12, a0=3.615, T=300.0, seed=7)
    x = st.x + 0.05 * np.random.default_rng(8).standard_normal(st.x.shape)
    tabs = wl.sutton_chen_tables(str(tmp_path / "cu"), [wl.CU])
    res = {}
    for cache in (True, False):
        s = api.GpuSystem(1, api.EAM2, api.FP64)
        s.set_pair_cache(cache)
        s.read_tables(tabs)
        s.set_box(st.box, (1, 1, 1), 0.4)
        s.set_atoms(st.number, st.types, st.mass, x, st.p)
        assert s.calc_forces(0) == 0
        a = s.get_atoms()
        sc = s.scalars()
        ep, ek = s.nve_run(30, wl.FS)
        res[cache] = (a, sc.tot_pot_energy, sc.virial, ep, ek, s.get_atoms()["x"],
                      s.scalars().nbl_count)
        s.close()
    (a1, e1, w1, ep1, ek1, x1, n1), (a0, e0, w0, ep0, ek0, x0, n0) = res[True], res[False]
    assert rel_rms(a1["f"], a0["f"]) < 1e-14
    np.testing.assert_allclose(a1["epot"], a0["epot"], rtol=1e-13, atol=0)
    assert abs(e1 - e0) <= 1e-13 * abs(e0) and abs(w1 - w0) <= 1e-13 * abs(w0)
    np.testing.assert_allclose(ep1, ep0, rtol=1e-12)
    np.testing.assert_allclose(ek1, ek0, rtol=1e-12)
    np.testing.assert_allclose(x1, x0, rtol=0, atol=1e-11)
    assert n1 == n0 and n1 > 1


def test_mixed_nve_conserves_energy():
    from imd_gb300 import api
    g = golden("cu_nve")
    gg = dict(g)
    gg["x"] = g["x0"]
    s = gpu_system(gg, "cu", 1, 1, 0.4, p=g["p0"], precision=api.MIXED)
    ep, ek = s.nve_run(len(g["epot"]), float(g["dt"]))
    et = ep + ek
    n = len(g["x0"])
    # same trajectory as the reference to the FP32 force error, and the total
    # energy fluctuates like the FP64 run's
    np.testing.assert_allclose(ep, g["epot"], rtol=1e-6)
    ref = g["epot"] + g["ekin"]
    assert np.max(np.abs(et - et[0])) / n < 2 * np.max(np.abs(ref - ref[0])) / n + 1e-7


def test_precision_switch_keeps_state():
    """Switching FP64 -> mixed -> FP64 rebuilds the matching list and gives
    the FP64 forces again."""
    from imd_gb300 import api
    g = golden("cu_pert")
    s = gpu_system(g, "cu", 1, 1, 0.4)
    s.calc_forces(0)
    f0 = s.get_atoms()["f"]
    s.set_precision(api.MIXED)
    s.calc_forces(0)
    f1 = s.get_atoms()["f"]
    s.set_precision(api.FP64)
    s.calc_forces(0)
    f2 = s.get_atoms()["f"]
    assert rel_rms(f1, f0) < 1e-5
    assert rel_rms(f2, f0) < 1e-13


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_replay_matches_direct_launches(precision):
    """nve_run with chunks replayed from a captured CUDA graph follows the
    same trajectory as with every launch issued from the host."""
    g = golden("cu_nve")
    gg = dict(g)
    gg["x"] = g["x0"]
    a = gpu_system(gg, "cu", 1, 1, 0.4, p=g["p0"], precision=precision)
    b = gpu_system(gg, "cu", 1, 1, 0.4, p=g["p0"], precision=precision)
    b.set_graphs(False)
    dt = float(g["dt"])
    ea, ka = a.nve_run(80, dt)
    eb, kb = b.nve_run(80, dt)
    np.testing.assert_allclose(ea, eb, rtol=1e-10)
    np.testing.assert_allclose(ka, kb, rtol=1e-9)
    assert a.scalars().nbl_count == b.scalars().nbl_count


# IMD's `spline` and `4point` table interpolations (reference built with
# -DSPLINE / -DFOURPOINT): interpolation mode 2 / 1
CUBIC = {"cu_pert_spline": 2, "cu_pert_4point": 1, "defect_cg_spline": 2}


@pytest.mark.parametrize("name", list(CUBIC))
def test_cubic_interpolation_forces_match_reference(name):
    g = golden(name)
    s = gpu_system(g, "cu", 1, 1, 0.4, interpolation=CUBIC[name])
    assert s.calc_forces(0) == 0
    a = s.get_atoms()
    sc = s.scalars()
    assert rel_rms(a["f"], g["f"]) < 1e-11
    assert np.max(np.abs(a["epot"] - g["epot"])) <= 1e-11 * np.max(np.abs(g["epot"]))
    assert abs(sc.tot_pot_energy - g["epot_total"]) <= 1e-12 * abs(g["epot_total"])
    assert abs(sc.virial - g["virial"]) <= 1e-12 * abs(g["virial"])
    assert np.max(np.abs(a["rho"] - g["rho"])) <= 1e-11 * np.max(g["rho"])
    assert np.max(np.abs(a["df"] - g["df"])) <= 1e-11 * np.max(np.abs(g["df"]))


@pytest.mark.parametrize("name", ["cu_pert_spline", "cu_pert_4point"])
def test_cubic_interpolation_mixed_force_error(name):
    from imd_gb300 import api
    g = golden(name)
    s = gpu_system(g, "cu", 1, 1, 0.4, precision=api.MIXED, interpolation=CUBIC[name])
    s.calc_forces(0)
    err = rel_rms(s.get_atoms()["f"], g["f"])
    assert err < 1e-5, err
    de = abs(s.scalars().tot_pot_energy - g["epot_total"]) / abs(g["epot_total"])
    assert de < 1e-6, de


def test_spline_cg_relaxation_matches_reference():
    """With spline tables the forces are smooth and IMD's CG reaches
    1e-4 eV/A on a defect cell; the device run ends at the reference's
    energy."""
    g = golden("defect_cg_spline")
    s = gpu_system(g, "cu", 1, 1, 0.4, interpolation=2)
    steps, fm = s.cg_relax(1e-4)
    assert fm <= 1e-4
    e = s.scalars().tot_pot_energy
    assert abs(e - float(g["cg_epot"])) / len(g["x"]) <= 1e-6
    assert 0.5 * int(g["cg_steps"]) <= steps <= 2 * int(g["cg_steps"]) + 3


STRESS = {"cu_pert_stress": ("cu", True, 1, 0.4), "alloy_pert_stress": ("cuni", True, 2, 0.4),
          "lj_pert_stress": ("lj", False, 1, 0.3)}


@pytest.mark.parametrize("name", list(STRESS))
def test_stress_matches_reference(name):
    """STRESS_TENS on the device against the reference's `stress` build:
    per-atom PRESSTENS within 1e-11 of the largest component, the total
    tensor within 1e-12 relative, forces unchanged."""
    g = golden(name)
    tab, eam, nt, skin = STRESS[name]
    s = gpu_system(g, tab, eam, nt, skin)
    st, tot = s.calc_stress()
    scale = np.max(np.abs(g["stress"]))
    assert np.max(np.abs(st - g["stress"])) <= 1e-11 * scale
    assert np.all(np.abs(tot - g["tot_stress"]) <= 1e-12 * np.max(np.abs(g["tot_stress"])))
    assert rel_rms(s.get_atoms()["f"], g["f"]) < 1e-11


def _stepwise(name, move):
    g = golden(name)
    gg = dict(g)
    gg["x"] = g["x0"]
    s = gpu_system(gg, "cu", 1, 1, float(g["skin"]), p=g["p0"])
    dt = float(g["dt"])
    ep, ek, extra = [], [], []
    for st in range(len(g["epot"])):
        s.calc_forces(st)
        ep.append(s.scalars().tot_pot_energy)
        extra.append(move(s, dt))
        ek.append(s.scalars().tot_kin_energy)
        s.check_nblist()
    return g, s, np.array(ep), np.array(ek), np.array(extra)


def test_nvt_matches_reference():
    """move_atoms_nvt on the device, 100 main_loop steps against the
    reference's `nvt` build: energies to 1e-9, eta to 1e-8 relative."""
    g0 = golden("cu_nvt")

    def move(s, dt):
        if not hasattr(s, "_nvt"):
            s.set_nvt(float(g0["temperature"]), float(g0["isq_tau_eta"]))
            s._nvt = True
        return s.move_atoms_nvt(dt)

    g, s, ep, ek, eta = _stepwise("cu_nvt", move)
    np.testing.assert_allclose(ep, g["epot"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(ek, g["ekin"], rtol=1e-8, atol=0)
    np.testing.assert_allclose(eta, g["eta"], rtol=1e-8, atol=1e-12)
    assert s.scalars().nbl_count == int(g["nbl_count"][-1])


def test_mik_matches_reference():
    """move_atoms_mik on the device, 200 quench steps against the reference's
    `mik` build: energies to 1e-9, force norms to 1e-6 relative, final
    positions to 1e-8 A."""
    def move(s, dt):
        s.move_atoms_mik(dt)
        return s.scalars().fnorm

    g, s, ep, ek, fn = _stepwise("cu_mik", move)
    np.testing.assert_allclose(ep, g["epot"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(ek, g["ekin"], rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(fn, g["fnorm"], rtol=1e-6, atol=0)
    x = s.get_atoms()["x"]
    d = x - g["x_final"]
    d -= np.round(d @ np.linalg.inv(g["box"])) @ g["box"]
    assert np.abs(d).max() < 1e-8


@pytest.mark.parametrize("name", ["cu_fire", "cu_glok", "cu_mixglok"])
def test_glok_matches_reference(name):
    """The glok ensemble (IMD's FIRE) on the device against the reference's
    `fire` (adaptive step, mixing), `glok` and `mix glok` (mixing, fixed
    step, 28 restarts on glok_ekin_threshold) builds, main_loop step by step:
    every decision identical (time step, mixing factor, restarts, nPxF),
    energies to 1e-9, P.F to 1e-6 relative, final positions to 1e-8 A."""
    g = golden(name)
    gg = dict(g)
    gg["x"] = g["x0"]
    s = gpu_system(gg, "cu", 1, 1, float(g["skin"]), p=g["p0"])
    prm = {"mix": int(g["mix_on"]), "adapt": int(g["adapt"])}
    for k in g:
        if k.startswith("param_"):
            n = k[len("param_"):]
            prm[n] = int(g[k]) if n in ("glok_minsteps", "min_nPxF") else float(g[k])
    s.set_glok(float(g["dt"]), **prm)
    rows = []
    for st in range(len(g["epot"])):
        s.calc_forces(st)
        ep = s.scalars().tot_pot_energy
        gs = s.move_atoms_glok(st)
        sc = s.scalars()
        rows.append((ep, sc.tot_kin_energy, sc.fnorm, gs.timestep, gs.mix, gs.PxF,
                     gs.glok_start))
        s.check_nblist()
    r = np.array(rows)
    np.testing.assert_array_equal(r[:, 3], g["timestep"])
    np.testing.assert_array_equal(r[:, 4], g["mix"])
    np.testing.assert_array_equal(r[:, 6], g["glok_start"])
    assert s.glok_state().nPxF == int(g["npxf"][-1])
    np.testing.assert_allclose(r[:, 0], g["epot"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(r[:, 1], g["ekin"], rtol=1e-7, atol=1e-12)
    np.testing.assert_allclose(r[:, 2], g["fnorm"], rtol=1e-6, atol=0)
    np.testing.assert_allclose(r[:, 5], g["pxf"], rtol=1e-6, atol=1e-9)
    x = s.get_atoms()["x"]
    d = x - g["x_final"]
    d -= np.round(d @ np.linalg.inv(g["box"])) @ g["box"]
    assert np.abs(d).max() < 1e-8


def test_glok_relax_stops_where_reference_does():
    """main_loop of `ensemble glok` with check_relaxed: the run stops at the
    first step whose sqrt(fnorm/nactive) is below fnorm_threshold, the step
    the reference's per-step force norms give."""
    g = golden("cu_fire")
    gg = dict(g)
    gg["x"] = g["x0"]
    n = len(g["x0"])
    f2 = np.sqrt(g["fnorm"] / (3.0 * n))
    thr = f2[150] * 1.0001
    expect = int(np.flatnonzero(f2 < thr)[0]) + 1
    assert np.all(np.abs(f2[:expect] / thr - 1.0) > 1e-6)   # no decision on a knife edge
    prm = {"mix": 1, "adapt": 1}
    for k in g:
        if k.startswith("param_"):
            nm = k[len("param_"):]
            prm[nm] = int(g[k]) if nm in ("glok_minsteps", "min_nPxF") else float(g[k])
    s = gpu_system(gg, "cu", 1, 1, float(g["skin"]), p=g["p0"])
    nsteps, relaxed = s.relax_glok(float(g["dt"]), len(g["epot"]), fnorm_threshold=thr, **prm)
    assert relaxed and nsteps == expect
    assert s.glok_state().timestep == g["timestep"][expect - 1]


def test_npt_iso_matches_reference():
    """ensemble npt_iso on the device, 200 main_loop steps against the
    reference's `npt_iso` build (the box scaled every step): energies to
    1e-9, xi, eta, the pressure and the volume to 1e-8 relative, final box
    to 1e-10 and positions to 1e-8 A."""
    g = golden("cu_npt")
    gg = dict(g)
    gg["x"] = g["x0"]
    s = gpu_system(gg, "cu", 1, 1, float(g["skin"]), p=g["p0"])
    s.set_npt(temperature=float(g["temperature"]), isq_tau_eta=float(g["isq_tau_eta"]),
              isq_tau_xi=float(g["isq_tau_xi"]), pressure_ext=float(g["pressure_start"]),
              pressure_end=float(g["pressure_end"]), steps_min=0, steps_max=int(g["steps_max"]))
    dt = float(g["dt"])
    rows = []
    for st in range(len(g["epot"])):
        s.calc_forces(st)
        ep = s.scalars().tot_pot_energy
        ns = s.move_atoms_npt_iso(st, dt)
        rows.append((ep, s.scalars().tot_kin_energy, ns.xi, ns.eta, ns.pressure, ns.volume,
                     ns.box[0], ns.pressure_ext))
        s.check_nblist()
    r = np.array(rows)
    np.testing.assert_allclose(r[:, 0], g["epot"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(r[:, 1], g["ekin"], rtol=1e-8, atol=0)
    for j, k in ((2, "xi"), (3, "eta"), (4, "pressure")):
        np.testing.assert_allclose(r[:, j], g[k], rtol=1e-8, atol=1e-12, err_msg=k)
    np.testing.assert_allclose(r[:, 5], g["volume"], rtol=1e-10, atol=0)
    np.testing.assert_allclose(r[:, 6], g["box_xx"], rtol=1e-10, atol=0)
    np.testing.assert_allclose(r[:, 7], g["pressure_ext"], rtol=1e-12, atol=0)
    box = np.array(s.npt_state().box).reshape(3, 3)
    np.testing.assert_allclose(box, g["box_final"], rtol=1e-10, atol=1e-12)
    x = s.get_atoms()["x"]
    d = x - g["x_final"]
    d -= np.round(d @ np.linalg.inv(box)) @ box
    assert np.abs(d).max() < 1e-8


def test_npt_axial_matches_reference():
    """ensemble npt_axial on the device (P_AXIAL virial, a barostat per
    axis, z held by relax_dirs), 200 main_loop steps against the reference's
    `npt_axial` build: energies to 1e-9, xi, eta and the axial stresses to
    1e-8 relative, the box diagonal every step and the final box to 1e-10,
    positions to 1e-8 A."""
    g = golden("cu_npt_axial")
    gg = dict(g)
    gg["x"] = g["x0"]
    s = gpu_system(gg, "cu", 1, 1, float(g["skin"]), p=g["p0"])
    s.set_npt_axial(temperature=float(g["temperature"]), isq_tau_eta=float(g["isq_tau_eta"]),
                    isq_tau_xi=float(g["isq_tau_xi"]), pressure_ext=list(g["pressure_start"]),
                    pressure_end=list(g["pressure_end"]),
                    relax_dirs=[int(v) for v in g["relax_dirs"]], steps_min=0,
                    steps_max=int(g["steps_max"]))
    dt = float(g["dt"])
    rows = []
    for st in range(len(g["epot"])):
        s.calc_forces(st)
        ep = s.scalars().tot_pot_energy
        ns = s.move_atoms_npt_axial(st, dt)
        rows.append([ep, s.scalars().tot_kin_energy] + list(ns.xi) + [ns.eta]
                    + list(ns.stress) + [ns.box[0], ns.box[4], ns.box[8]])
        s.check_nblist()
    r = np.array(rows)
    np.testing.assert_allclose(r[:, 0], g["epot"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(r[:, 1], g["ekin"], rtol=1e-8, atol=0)
    np.testing.assert_allclose(r[:, 2:5], g["xi"], rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(r[:, 5], g["eta"], rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(r[:, 6:9], g["stress"], rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(r[:, 9:12], g["box_diag"], rtol=1e-10, atol=0)
    assert np.all(r[:, 4] == 0.0)   # the held axis never moves
    box = np.array(s.npt_axial_state().box).reshape(3, 3)
    np.testing.assert_allclose(box, g["box_final"], rtol=1e-10, atol=1e-12)
    x = s.get_atoms()["x"]
    d = x - g["x_final"]
    d -= np.round(d @ np.linalg.inv(box)) @ box
    assert np.abs(d).max() < 1e-8


def test_npt_axial_virial_is_the_oracle_p_axial():
    """The P_AXIAL components of one calc_forces on the perturbed Cu and
    Cu/Ni cases: the device's vir_xx, vir_yy, vir_zz against the oracle's
    running sums (IMD's order) to 1e-11 relative."""
    from oracle import OracleSystem
    for name in ("cu_pert", "alloy_pert"):
        g = golden(name)
        tab, eam, nt, skin = CASES[name]
        s = gpu_system(g, tab, eam, nt, skin)
        s.set_npt_axial(temperature=0.0258520, steps_min=0, steps_max=10)
        s.calc_forces(0)
        va = np.array(s.npt_axial_state().vir_axial)
        o = OracleSystem(g["box"], g["x"], g["type"], g["mass"], g["number"], nt, tables(tab),
                         bool(eam), skin)
        o.calc_forces()
        ref = np.array(o.s.vir_axial[:])
        np.testing.assert_allclose(va, ref, rtol=1e-11, atol=0, err_msg=name)
        assert abs(va.sum() - o.virial) <= 1e-11 * abs(o.virial)


def test_npt_iso_new_cell_grid_matches_oracle():
    """A stretched crystal pulled by a negative pressure: its box grows out
    of the 3x3x3 grid's height bounds, the device sets up a 4x4x4 grid and a
    new list, and energies and positions follow the oracle (1e-9)."""
    from oracle import OracleSystem
    g = golden("cu_npt")
    box0, x0 = g["box"] * 1.095, g["x0"] * 1.095
    prm = dict(temperature=float(g["temperature"]), isq_tau_eta=float(g["isq_tau_eta"]),
               isq_tau_xi=1.0 / 25.0, pressure_ext=-0.2, pressure_end=-0.2, steps_min=0,
               steps_max=19)
    o = OracleSystem(box0, x0, g["type"], g["mass"], g["number"], 1, tables("cu"), True,
                     float(g["skin"]), timestep=float(g["dt"]), p=g["p0"])
    out, _ = o.npt(20, 0, **prm)
    assert list(o.s.gdim) == [4, 4, 4]
    gg = dict(g)
    gg["box"], gg["x"] = box0, x0
    s = gpu_system(gg, "cu", 1, 1, float(g["skin"]), p=g["p0"])
    s.set_npt(**prm)
    ep = []
    for st in range(20):
        s.calc_forces(st)
        ep.append(s.scalars().tot_pot_energy)
        s.move_atoms_npt_iso(st, float(g["dt"]))
        s.check_nblist()
    assert list(s.scalars().gdim) == [4, 4, 4]
    np.testing.assert_allclose(ep, out[:, 0], rtol=1e-9, atol=0)
    box = np.array(s.npt_state().box).reshape(3, 3)
    np.testing.assert_allclose(box, np.array(o.s.box), rtol=1e-10, atol=1e-12)
    d = s.get_atoms()["x"] - o.x
    d -= np.round(d @ np.linalg.inv(box)) @ box
    assert np.abs(d).max() < 1e-8


def test_glok_parameters_checked():
    from imd_gb300 import api
    g = golden("cu_fire")
    gg = dict(g)
    gg["x"] = g["x0"]
    s = gpu_system(gg, "cu", 1, 1, float(g["skin"]), p=g["p0"])
    with pytest.raises(api.IMDGPUError):
        s.move_atoms_glok(0)                       # no set_glok yet
    with pytest.raises(api.IMDGPUError):
        s.set_glok(0.1, mix=0, adapt=1, glok_maxtimestep=0.5)   # ADAPTGLOK needs MIX
    with pytest.raises(api.IMDGPUError):
        s.set_glok(0.1, mix=1, adapt=1)            # adaptive step without a maximum
    with pytest.raises(TypeError):
        s.set_glok(0.1, glok_mixx=0.1)


def test_lj_1000_steps_segmentwise():
    """The plain-method LJ workload (4000 atoms, 1000 steps) against the
    reference step by step: from each reference snapshot (every 250 steps)
    the device reproduces that step's forces (1e-11 relative RMS) and the
    energies of the next 250 steps (1e-9 relative); the device's own
    1000-step run from step 0 conserves energy as the reference's does."""
    g = golden("lj_nve1000")
    snaps = list(g["snap_steps"])
    dt = float(g["dt"])
    for k, st in enumerate(snaps):
        gg = dict(g)
        gg["x"] = g["snap_x"][k]
        s = gpu_system(gg, "lj", False, 1, float(g["skin"]), p=g["snap_p"][k])
        s.calc_forces(st)
        # step 0 is the perfect lattice, whose forces are rounding noise: the
        # bar is relative to a force scale of at least 1
        f, gf = s.get_atoms()["f"], g["snap_f"][k]
        assert np.sqrt(np.mean((f - gf) ** 2)) < 1e-11 * max(1.0, np.sqrt(np.mean(gf ** 2)))
        assert abs(s.scalars().tot_pot_energy - g["epot"][st]) <= 1e-12 * abs(g["epot"][st])
        if st == snaps[-1]:
            continue
        s = gpu_system(gg, "lj", False, 1, float(g["skin"]), p=g["snap_p"][k])
        n = snaps[k + 1] - st
        ep, ek = s.nve_run(n, dt)
        np.testing.assert_allclose(ep, g["epot"][st:st + n], rtol=1e-9, atol=0)
        np.testing.assert_allclose(ek, g["ekin"][st:st + n], rtol=1e-8, atol=0)
    gg = dict(g)
    gg["x"] = g["snap_x"][0]
    s = gpu_system(gg, "lj", False, 1, float(g["skin"]), p=g["snap_p"][0])
    ep, ek = s.nve_run(1000, dt)
    # past a few hundred steps the two trajectories separate (rounding grows
    # in a chaotic system); energy conservation stays alike
    etot, eref = ep + ek, g["epot"][:1000] + g["ekin"]
    n = len(g["number"])
    np.testing.assert_allclose(ep[:250], g["epot"][:250], rtol=1e-9, atol=0)
    assert abs((etot[-1] - etot[0]) - (eref[-1] - eref[0])) / n < 1e-3
    assert (etot.max() - etot.min()) <= 2.0 * (eref.max() - eref.min())
