"""imdgpu_nve_step_host: one NVE step of main_loop with the state on the host.

The fused call must leave exactly what the separate C-ABI calls leave
(put_state, calc_forces, move_atoms_nve, check_nblist, get_atoms): the same
positions and momenta bit for bit and the same energies, over 40 steps of the
Cu NVE golden run (rebuilds included), in place or into separate buffers.
Bit for bit needs the deterministic mode: the default FP64 passes add the
partner's reaction with atomics, so two runs of one code path differ in the
last bits.  The default mode is held to 1e-12 against the separate calls.  A
non-finite input is an error and moves no atom.
"""
import numpy as np
import pytest

from conftest import golden, tables

pytestmark = pytest.mark.gpu


def _system(deterministic=False):
    from imd_gb300 import api
    g = golden("cu_nve")
    s = api.GpuSystem(1, api.EAM2, api.FP64)
    s.set_deterministic(deterministic)
    s.read_tables(tables("cu"))
    s.set_box(g["box"], (1, 1, 1), 0.4)
    s.set_atoms(g["number"], g["type"], g["mass"], g["x0"], g["p0"])
    return s, g


def _buffers(shape, pinned):
    """Host arrays, page-locked when asked (the captured-graph path of the
    call needs pinned buffers; pageable ones take the direct launches)."""
    if not pinned:
        return np.empty(shape)
    torch = pytest.importorskip("torch")
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


@pytest.mark.parametrize("deterministic,pinned", [(True, False), (True, True), (False, True)])
def test_fused_step_equals_separate_calls(deterministic, pinned):
    a, g = _system(deterministic)
    b, _ = _system(deterministic)
    same = np.testing.assert_array_equal if deterministic else \
        (lambda u, w: np.testing.assert_allclose(u, w, rtol=1e-12, atol=1e-13))
    dt = float(g["dt"])
    xa = np.ascontiguousarray(g["x0"], np.float64).copy()
    pa = np.ascontiguousarray(g["p0"], np.float64).copy()
    xb, pb = _buffers(xa.shape, pinned), _buffers(pa.shape, pinned)
    xb[:], pb[:] = xa, pa
    xo, po = _buffers(xb.shape, pinned), _buffers(pb.shape, pinned)
    rebuilds = set()
    for k in range(40):
        a.put_state(xa, pa)
        a.calc_forces(k)
        a.move_atoms_nve(dt)
        a.check_nblist()
        a.get_state(xa, pa)
        sa = a.scalars()
        if k % 2:
            sb = b.nve_step_host(xb, pb, dt, xb, pb)          # in place
        else:
            sb = b.nve_step_host(xb, pb, dt, xo, po)
            xb[:], pb[:] = xo, po
        same(xb, xa)
        same(pb, pa)
        same(np.array([sb.tot_pot_energy, sb.tot_kin_energy]),
             np.array([sa.tot_pot_energy, sa.tot_kin_energy]))
        assert sb.nbl_count == sa.nbl_count
        rebuilds.add(sb.nbl_count)
    assert len(rebuilds) > 1   # the run crossed at least one list rebuild


def test_fused_step_refuses_non_finite_input():
    from imd_gb300 import api
    s, g = _system()
    dt = float(g["dt"])
    x = np.ascontiguousarray(g["x0"], np.float64).copy()
    p = np.ascontiguousarray(g["p0"], np.float64).copy()
    s.nve_step_host(x, p, dt, x, p)
    before = s.get_atoms()
    bad = x.copy()
    bad[7, 1] = np.nan
    with pytest.raises(api.IMDGPUError, match="atom 7"):
        s.nve_step_host(bad, p, dt, None, None)
    after = s.get_atoms()
    np.testing.assert_array_equal(after["x"], before["x"])
    np.testing.assert_array_equal(after["p"], before["p"])
    # and the next good step goes on from where the system was
    s.nve_step_host(x, p, dt, x, p)
