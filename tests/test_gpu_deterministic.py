"""Deterministic reduction mode (imdgpu_set_deterministic) on the device.

The default FP64 half-list passes add each pair's reaction with FP64
atomics, so the order of the per-atom sums, and their last bits, vary from
run to run.  In the deterministic mode the density and force passes run on
the full list, each atom's sums formed by one quad of lanes in list order
and a fixed shuffle tree.  Checked here:

* two independent 100-step NVE runs of a 32,000-atom Cu crystal (fcc 20^3,
  300 K, positions displaced by 0.05 A) give bitwise equal positions,
  momenta and per-step energies;
* the mode meets the same parity bars against the reference as the default
  path: forces 1e-11 relative RMS, per-atom energies, rho and 2F' 1e-11,
  energy and virial 1e-12 (perturbed Cu, Cu/Ni alloy and LJ), the 100-step
  Cu NVE run to 1e-9;
* the entry points that need IMD's half list refuse the mode.
"""
import numpy as np
import pytest

from conftest import golden, tables

pytestmark = pytest.mark.gpu


def rel_rms(a, b):
    return np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2))


def _system(g, tab, eam, nt, skin, x=None, p=None):
    from imd_gb300 import api
    s = api.GpuSystem(nt, api.EAM2 if eam else api.PAIR, api.FP64)
    s.read_tables(tables(tab), default_format=2 if eam else 1)
    s.set_box(g["box"], (1, 1, 1), skin)
    s.set_deterministic(True)
    s.set_atoms(g["number"], g["type"], g["mass"], g["x"] if x is None else x, p)
    return s


def test_deterministic_runs_are_bitwise_equal(tmp_path):
    from imd_gb300 import api
    from imd_gb300 import workloads as wl
    tabs = wl.sutton_chen_tables(str(tmp_path / "cu"), [wl.CU])
    st = wl.eam_fcc_system(20, a0=3.615, T=300.0, seed=2)
    x = st.x + 0.05 * np.random.default_rng(21).standard_normal(st.x.shape)
    out = []
    for run in range(2):
        s = api.GpuSystem(1, api.EAM2, api.FP64)
        s.read_tables(tabs)
        s.set_box(st.box, (1, 1, 1), 0.4)
        s.set_deterministic(True)
        s.set_atoms(st.number, st.types, st.mass, x, st.p)
        ep, ek = s.nve_run(100, wl.FS)
        a = s.get_atoms()
        out.append((ep.copy(), ek.copy(), a["x"].copy(), a["p"].copy(), a["f"].copy()))
        s.close()
    for u, w in zip(out[0], out[1]):
        np.testing.assert_array_equal(u, w)
    assert out[0][4].any()


@pytest.mark.parametrize("name,tab,eam,nt,skin", [("cu_pert", "cu", 1, 1, 0.4),
                                                  ("alloy_pert", "cuni", 1, 2, 0.4),
                                                  ("lj_pert", "lj", 0, 1, 0.3)])
def test_deterministic_forces_match_reference(name, tab, eam, nt, skin):
    g = golden(name)
    s = _system(g, tab, eam, nt, skin)
    assert s.calc_forces(0) == 0
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


def test_deterministic_nve_matches_reference():
    g = golden("cu_nve")
    gg = dict(g)
    gg["x"] = g["x0"]
    s = _system(gg, "cu", 1, 1, 0.4, p=g["p0"])
    ep, ek = s.nve_run(len(g["epot"]), float(g["dt"]))
    np.testing.assert_allclose(ep, g["epot"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(ek, g["ekin"], rtol=1e-8, atol=0)
    assert s.scalars().nbl_count == int(g["nbl_count"][-1])


def test_half_list_entry_points_refuse_the_mode():
    from imd_gb300 import api
    g = golden("cu_pert")
    s = _system(g, "cu", 1, 1, 0.4)
    s.calc_forces(0)
    with pytest.raises(api.IMDGPUError):
        s.calc_stress()
    with pytest.raises(api.IMDGPUError):
        s.pairs()
    s.set_deterministic(False)   # back to the half list: both work again
    s.calc_forces(0)
    assert len(s.pairs()[0]) == int(g["npairs"])
