"""imdgpu_move_atoms_nve_noalloc against imdgpu_move_atoms_nve.

The no-allocation entry point serves host programs that cannot let a library
call cudaMalloc: all their device memory comes from their own pool, or a
cudaMalloc/cudaFree (which may synchronise the device) must not happen inside
their time step.  It takes the caller's device arrays and keeps its partial
sums in a fixed file-scope device array.  This test calls it through the
C-ABI on device arrays that the test owns, twice in a row, and compares every
output with the regular entry point on the same state: positions and momenta
bit for bit (same per-atom arithmetic), the summed scalars within 1e-12
relative (different summation order), the maxima exactly, and the largest
displacement since the list build against the same quantity computed on the
host from the device arrays.  A two-species case with a restriction vector
that fixes one component per species checks the per-type restriction rows.
It also checks that a size beyond the fixed scratch is refused with an
error, and so is an atom type outside the tables, which the kernel checks on
the device (the atom is left unmoved; no out-of-range read happens).

Named test_zz_* so that pytest collects it after every other test file.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden, tables

pytestmark = pytest.mark.gpu


def _sig(L):
    f = L.imdgpu_move_atoms_nve_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_nve_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    from imd_gb300 import api
    g = golden("cu_nve")
    s = api.GpuSystem(1, api.EAM2, api.FP64)
    s.read_tables(tables("cu"))
    s.set_box(g["box"], (1, 1, 1), 0.4)
    s.set_atoms(g["number"], g["type"], g["mass"], g["x0"], g["p0"])
    s.calc_forces(0)
    a0 = s.get_atoms()  # caller order; x as wrapped by the list build
    n = len(a0["x"])
    dev = torch.device("cuda:0")
    x = torch.tensor(a0["x"].reshape(-1), dtype=torch.float64, device=dev)
    p = torch.tensor(a0["p"].reshape(-1), dtype=torch.float64, device=dev)
    f = torch.tensor(a0["f"].reshape(-1), dtype=torch.float64, device=dev)
    m = torch.tensor(np.asarray(g["mass"], np.float64), device=dev)
    t = torch.tensor(np.asarray(g["type"], np.int32), device=dev)
    xref = x.clone()
    dt = float(g["dt"])
    fn = _sig(api.lib())
    out = np.zeros(4)
    for call in range(2):
        s.move_atoms_nve(dt)
        ref = s.get_atoms()
        sc = s.scalars()
        torch.cuda.synchronize()
        rc = fn(n, 1, x.data_ptr(), p.data_ptr(), f.data_ptr(), m.data_ptr(), t.data_ptr(),
                None, dt, xref.data_ptr(), out.ctypes.data, None)
        assert rc == 0, api.lib().imdgpu_last_error().decode()
        torch.cuda.synchronize()
        xd = x.cpu().numpy().reshape(n, 3)
        np.testing.assert_array_equal(xd, ref["x"])
        np.testing.assert_array_equal(p.cpu().numpy().reshape(n, 3), ref["p"])
        assert abs(out[0] - sc.tot_kin_energy) <= 1e-12 * abs(sc.tot_kin_energy), call
        assert abs(out[1] - sc.fnorm) <= 1e-12 * abs(sc.fnorm), call
        assert out[2] == sc.f_max2, call
        d = xd - xref.cpu().numpy().reshape(n, 3)
        dmax = np.max((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
        assert out[3] == dmax and dmax > 0.0, call


def test_noalloc_nve_two_species_restrictions_bitwise():
    """ntypes = 2 with a restriction vector that fixes x for type 0 and z for
    type 1: positions, momenta and masked forces equal the regular entry
    point's (after imdgpu_set_restrictions) bit for bit."""
    torch = pytest.importorskip("torch")
    from imd_gb300 import api
    g = golden("alloy_pert")
    restr = np.array([0.0, 1.0, 1.0, 1.0, 1.0, 0.0])
    n = len(g["x"])
    rng = np.random.default_rng(11)
    p0 = 0.05 * rng.standard_normal((n, 3)) * np.sqrt(np.asarray(g["mass"]))[:, None]
    s = api.GpuSystem(2, api.EAM2, api.FP64)
    s.read_tables(tables("cuni"))
    s.set_box(g["box"], (1, 1, 1), 0.4)
    s.set_restrictions(restr)
    s.set_atoms(g["number"], g["type"], g["mass"], g["x"], p0)
    s.calc_forces(0)
    a0 = s.get_atoms()
    dev = torch.device("cuda:0")
    x = torch.tensor(a0["x"].reshape(-1), dtype=torch.float64, device=dev)
    p = torch.tensor(a0["p"].reshape(-1), dtype=torch.float64, device=dev)
    f = torch.tensor(a0["f"].reshape(-1), dtype=torch.float64, device=dev)
    m = torch.tensor(np.asarray(g["mass"], np.float64), device=dev)
    t = torch.tensor(np.asarray(g["type"], np.int32), device=dev)
    dt = 0.0982266
    fn = _sig(api.lib())
    out = np.zeros(4)
    s.move_atoms_nve(dt)
    ref = s.get_atoms()
    sc = s.scalars()
    torch.cuda.synchronize()
    rc = fn(n, 2, x.data_ptr(), p.data_ptr(), f.data_ptr(), m.data_ptr(), t.data_ptr(),
            restr.ctypes.data, dt, None, out.ctypes.data, None)
    assert rc == 0, api.lib().imdgpu_last_error().decode()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(x.cpu().numpy().reshape(n, 3), ref["x"])
    np.testing.assert_array_equal(p.cpu().numpy().reshape(n, 3), ref["p"])
    fd = f.cpu().numpy().reshape(n, 3)
    ty = np.asarray(g["type"])
    assert np.all(fd[ty == 0, 0] == 0.0) and np.all(fd[ty == 1, 2] == 0.0)
    assert np.any(fd[ty == 0, 1] != 0.0)
    assert abs(out[0] - sc.tot_kin_energy) <= 1e-12 * abs(sc.tot_kin_energy)
    assert abs(out[1] - sc.fnorm) <= 1e-12 * abs(sc.fnorm)
    assert out[2] == sc.f_max2
    assert out[3] == 0.0   # no x_ref given


def test_noalloc_refuses_a_type_outside_the_tables():
    """The types live in the caller's device memory, so the kernel checks
    them: atom 5 with type 7 of ntypes = 1 stays where it is, the others
    move, and the call names atom 5."""
    torch = pytest.importorskip("torch")
    from imd_gb300 import api
    fn = _sig(api.lib())
    n = 64
    dev = torch.device("cuda:0")
    x = torch.zeros(3 * n, dtype=torch.float64, device=dev)
    p = torch.ones(3 * n, dtype=torch.float64, device=dev)
    f = torch.zeros(3 * n, dtype=torch.float64, device=dev)
    m = torch.ones(n, dtype=torch.float64, device=dev)
    ty = np.zeros(n, np.int32)
    ty[5] = 7
    ty[40] = -1
    t = torch.tensor(ty, device=dev)
    out = np.zeros(4)
    rc = fn(n, 1, x.data_ptr(), p.data_ptr(), f.data_ptr(), m.data_ptr(), t.data_ptr(),
            None, 0.5, None, out.ctypes.data, None)
    assert rc == -1
    assert "atom 5 " in api.lib().imdgpu_last_error().decode()
    xd = x.cpu().numpy().reshape(n, 3)
    assert np.all(xd[5] == 0.0) and np.all(xd[40] == 0.0)
    assert np.all(xd[0] == 0.5)


def test_noalloc_refuses_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from imd_gb300 import api
    fn = _sig(api.lib())
    buf = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    ti = torch.zeros(8, dtype=torch.int32, device="cuda:0")
    out = np.zeros(4)
    rc = fn((1 << 24) + 1, 1, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
            ti.data_ptr(), None, 1.0, None, out.ctypes.data, None)
    assert rc == -1
    assert "16777216" in api.lib().imdgpu_last_error().decode()
