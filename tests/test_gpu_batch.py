"""Batched CG (imdgpu_batch_*): every cell relaxed by IMD's CG on the device,
checked against the reference (golden triclinic cell) and the oracle's CG on
small defect cells of the batched workload's generator.  Bar: final energy
within 1e-6 eV/atom, max |F| <= 1e-4 eV/A."""
import numpy as np
import pytest

from conftest import golden, tables

pytestmark = pytest.mark.gpu


def _cell_from_golden(g):
    from imd_gb300 import workloads as wl
    n = len(g["x"])
    return wl.System(g["box"], g["x"], np.zeros((n, 3)), g["type"].astype(np.int32),
                     g["mass"], g["number"].astype(np.int32))


def test_batch_of_one_matches_reference_cg():
    from imd_gb300 import api
    g = golden("tri_cg")
    b = api.GpuBatch(1, api.EAM2)
    b.read_tables(tables("cu"))
    b.set_cells([_cell_from_golden(g)])
    b.relax(1e-4)
    r = b.results()
    assert r["status"][0] == 0
    assert r["fmax"][0] <= 1e-4
    assert abs(r["epot"][0] - float(g["cg_epot"])) / len(g["x"]) <= 1e-6


def test_batch_matches_oracle_per_cell():
    from imd_gb300 import api
    from imd_gb300 import workloads as wl
    from oracle import OracleSystem
    rng = np.random.default_rng(11)
    cells = [wl.defect_cell(rng, nmin=300, nmax=900, nlim=(3, 6)) for _ in range(5)]
    b = api.GpuBatch(1, api.EAM2)
    b.read_tables(tables("cu"))
    b.set_cells(cells)
    b.relax(1e-4)
    r = b.results()
    xs = b.positions()
    for k, c in enumerate(cells):
        o = OracleSystem(c.box, c.x, c.types, c.mass, c.number, 1, tables("cu"), True, 0.4)
        steps, fm = o.cg_relax(1e-4)
        assert fm <= 1e-4
        assert r["status"][k] == 0, r
        assert r["fmax"][k] <= 1e-4
        assert abs(r["epot"][k] - o.epot_total) / c.n <= 1e-6, (k, r["epot"][k], o.epot_total)
        # final positions: the energy check above is the bar; positions of a
        # relaxed cell agree closely too (same minimum, up to its soft modes)
        assert xs[k].shape == c.x.shape


def test_engine_rounds_equal_four_kernel_rounds():
    """The persistent CG engine (one launch per round, cells taken largest
    first) and the four-kernel round (control, vector, flag, reduction) do
    the same arithmetic: the cells converge in both, to the same energy
    (1e-8 eV/atom; the force passes' FP64 atomics make two runs of either
    differ in the last bits, which CG carries along), with compaction on."""
    from imd_gb300 import api
    from imd_gb300 import workloads as wl
    rng = np.random.default_rng(11)
    cells = [wl.defect_cell(rng, nmin=300, nmax=900, nlim=(3, 6)) for _ in range(5)]
    out = []
    for engine in (True, False):
        b = api.GpuBatch(1, api.EAM2)
        b.read_tables(tables("cu"))
        b.set_cells(cells)
        b.set_engine(engine)
        b.set_compaction(50)
        b.relax(1e-4, max_rounds=100_000)
        out.append((b.results(), b.positions()))
        b.close()
    (ra, xa), (rb, xb) = out
    n = np.array([c.n for c in cells])
    both = (ra["status"] == 0) & (rb["status"] == 0)
    assert both.sum() >= len(cells) - 1, (ra["status"], rb["status"])
    assert (ra["fmax"][both] <= 1e-4).all() and (rb["fmax"][both] <= 1e-4).all()
    assert np.max(np.abs(ra["epot"] - rb["epot"])[both] / n[both]) <= 1e-8
    for a, b in zip(xa, xb):
        assert a.shape == b.shape


@pytest.mark.parametrize("engine", [True, False])
def test_partial_rebuilds_relax_like_full_ones(engine):
    """Per-system rebuilds (fixed ghost ranges, only the cells that moved
    past skin/2 rebuilt) relax every cell to the energy of whole-batch
    rebuilds (1e-8 eV/atom, the bar of the compaction test: the force
    passes' FP64 atomics let two runs' CG paths part in the last bits); the
    lists they keep stay valid because a cell's ghosts and slots do not
    move.  The final positions' energies are checked against the oracle."""
    from imd_gb300 import api
    from imd_gb300 import workloads as wl
    rng = np.random.default_rng(11)
    cells = [wl.defect_cell(rng, nmin=300, nmax=900, nlim=(3, 6)) for _ in range(5)]
    from oracle import OracleSystem
    out = []
    for partial in (True, False):
        b = api.GpuBatch(1, api.EAM2)
        b.read_tables(tables("cu"))
        b.set_cells(cells)
        b.set_engine(engine)
        b.set_partial_rebuild(partial)
        b.relax(1e-4, max_rounds=100_000)
        out.append(b.results())
        if partial:
            xs = b.positions()
        b.close()
    ra, rb = out
    for k, c in enumerate(cells):  # the reported energy is the final positions' energy
        o = OracleSystem(c.box, xs[k], c.types, c.mass, c.number, 1, tables("cu"), True, 0.4)
        o.calc_forces()
        assert abs(o.epot_total - ra["epot"][k]) <= 1e-10 * abs(o.epot_total), k
    # IMD's CG on these cells is chaotic: identical runs take 5 000 to 13 000
    # rounds, and now and then one cell wanders for long; the cells both runs
    # finished are compared
    n = np.array([c.n for c in cells])
    both = (ra["status"] == 0) & (rb["status"] == 0)
    assert both.sum() >= len(cells) - 1, (ra["status"], rb["status"])
    assert (ra["fmax"][both] <= 1e-4).all()
    assert np.max(np.abs(ra["epot"] - rb["epot"])[both] / n[both]) <= 1e-8


def test_overflow_replays_keep_the_relaxation():
    """A list with the least head-room (a capacity of the largest count
    plus 8 at every build) may overflow as the cells relax; each overflow
    replays its chunk of rounds from the snapshot with a grown list, and the
    replayed rounds must continue the same relaxation (the last forces, which
    the next round's CG sums and directions read, move with the atoms to
    their new slots).  Every cell ends at the energy of a run with the
    default head-room (1e-8 eV/atom) and no atom ends far from where it
    started.  Whether a replay happens depends on how the cells relax; the
    count is printed."""
    from imd_gb300 import api, learned
    from imd_gb300 import workloads as wl
    rng = np.random.default_rng(17)
    cells = [wl.defect_cell(rng, nmin=300, nmax=1200, nlim=(3, 7)) for _ in range(8)]
    out = []
    for headroom in (1.0, 1.3):
        b = api.GpuBatch(1, api.EAM2)
        b.read_tables(tables("cu"))
        b.set_cells(cells)
        b.set_list_headroom(headroom)
        b.relax(1e-4, max_rounds=100_000)
        out.append((b.results(), b.positions(), b.replays()))
        b.close()
    (ra, xa, na), (rb, xb, nb) = out
    print("replays with the least head-room: %d, with the default: %d" % (na, nb))
    n = np.array([c.n for c in cells])
    both = (ra["status"] == 0) & (rb["status"] == 0)
    assert both.sum() >= len(cells) - 1, (ra["status"], rb["status"])
    assert np.max(np.abs(ra["epot"] - rb["epot"])[both] / n[both]) <= 1e-8
    for c, x in zip(cells, xa):
        d = learned.min_image(x - c.x, np.asarray(c.box))
        assert np.max(np.sqrt(np.sum(d * d, axis=1))) < 6.0


@pytest.mark.late
@pytest.mark.parametrize("partial", [True, False])
def test_injected_replays_keep_atoms_in_step(partial):
    """Chunks of rounds replayed from their snapshot (forced from the host
    every fourth chunk, eight times) continue every relaxation with each
    atom's CG vectors in step with the atom.  The energies cannot show a
    fault here: atoms that take other atoms' line-search origins still relax
    to the same crystal, with the atoms exchanged.  So every cell's returned
    positions are checked against its start: for every relaxed cell a mean
    squared displacement below 1 A^2 and no atom beyond 5 A (20 000 relaxed
    cells of this workload stay below 0.012 A^2 on average and 4.3 A at
    most; cells with exchanged atoms reach 1-50 A^2).  The batch is large
    enough (about a million atoms) that the snapshot restore takes tens of
    microseconds, long enough to overlap the rebuild that follows it if the
    two were not ordered on one stream."""
    from imd_gb300 import api, learned
    from imd_gb300 import workloads as wl
    cells = wl.defect_batch(256, seed=5)
    b = api.GpuBatch(1, api.EAM2)
    b.read_tables(tables("cu"))
    b.set_cells(cells)
    b.set_partial_rebuild(partial)
    b.begin(1e-4)
    b.inject_replays(4, 8)
    nd, rounds = 0, 0
    while nd < len(cells) and rounds < 100_000:
        nd, rounds = b.advance(256)
    r = b.results()
    xs = b.positions()
    nrep = b.replays()
    b.close()
    assert nrep >= 8, nrep
    # about 0.6% of this workload's cells stop with status 4 (a pair below a
    # table's first point); the relaxed ones are checked
    ok = r["status"] == 0
    assert ok.sum() >= 0.97 * len(cells), r["status"]
    bad = []
    for k, (c, x) in enumerate(zip(cells, xs)):
        if not ok[k]:
            continue
        d = learned.min_image(x - c.x, np.asarray(c.box))
        d2 = np.sum(d * d, axis=1)
        if np.mean(d2) >= 1.0 or np.max(d2) >= 25.0:
            bad.append((k, round(float(np.mean(d2)), 3), round(float(np.sqrt(np.max(d2))), 2)))
    assert not bad, bad


def test_batch_mixed_precision_relaxes():
    from imd_gb300 import api
    from imd_gb300 import workloads as wl
    rng = np.random.default_rng(12)
    cells = [wl.defect_cell(rng, nmin=300, nmax=900, nlim=(3, 6)) for _ in range(4)]
    b64 = api.GpuBatch(1, api.EAM2, api.FP64)
    b64.read_tables(tables("cu"))
    b64.set_cells(cells)
    b64.relax(1e-4)
    bm = api.GpuBatch(1, api.EAM2, api.MIXED)
    bm.read_tables(tables("cu"))
    bm.set_cells(cells)
    bm.relax(1e-4)
    r64, rm = b64.results(), bm.results()
    n = np.array([c.n for c in cells])
    assert np.all(r64["status"] == 0)
    assert np.all(np.abs(rm["epot"] - r64["epot"]) / n <= 1e-6), (rm, r64)


def test_compaction_keeps_every_cell_result():
    """Finished cells leave the device batch (compaction at every chance with
    pct = 100); every cell still ends at the energy of the uncompacted run,
    positions() returns each cell's final positions (the oracle's energy of
    them is the reported one) and bringing all cells back restores them."""
    import oracle
    from imd_gb300 import api, learned
    from imd_gb300 import workloads as wl
    from oracle import OracleSystem
    rng = np.random.default_rng(13)
    cells = [wl.defect_cell(rng, nmin=200, nmax=700, nlim=(3, 6)) for _ in range(6)]
    out = {}
    for pct in (0, 100):
        b = api.GpuBatch(1, api.EAM2, api.FP64, api.SPLINE)
        b.read_tables(tables("cu"))
        b.set_cells(cells)
        b.set_compaction(pct)
        b.relax(1e-4)
        out[pct] = (b.results(), b.positions(), b)
    r0, _, _ = out[0]
    r1, x1, b1 = out[100]
    n = np.array([c.n for c in cells])
    assert np.all(r0["status"] == 0) and np.all(r1["status"] == 0)
    assert np.all(r1["fmax"] <= 1e-4)
    assert np.all(np.abs(r1["epot"] - r0["epot"]) / n <= 1e-8), (r1["epot"] - r0["epot"]) / n
    oracle.set_interpolation(oracle.SPLINE)
    try:
        for k, c in enumerate(cells):
            o = OracleSystem(c.box, x1[k], c.types, c.mass, c.number, 1, tables("cu"), True, 0.4)
            o.calc_forces()
            assert abs(o.epot_total - r1["epot"][k]) <= 1e-10 * abs(o.epot_total)
    finally:
        oracle.set_interpolation(oracle.QUADRATIC)
    # all cells back on the device: their energies at the final positions
    b1.ml_set_weights(np.zeros(learned.NPARAM, np.float32))
    used, e0, e1 = b1.ml_start()
    assert np.allclose(e0, r1["epot"], rtol=1e-11, atol=0)


def test_autotune_keeps_results():
    """The autotuner picks one of its block shapes; forces and energies with
    the tuned shape equal those of the default shape (only the order of the
    block sums changes), and a hand-set shape is kept."""
    from imd_gb300 import api
    from conftest import golden
    g = golden("cu_pert")
    out = {}
    for mode in ("default", "tuned", "32"):
        s = api.GpuSystem(1, api.EAM2, api.FP64)
        s.read_tables(tables("cu"))
        s.set_box(g["box"], (1, 1, 1), 0.4)
        s.set_atoms(g["number"], g["type"], g["mass"], g["x"])
        if mode == "tuned":
            bd, bf = s.autotune()
            assert bd in (32, 64, 96, 128) and bf in (32, 64, 96, 128)
        elif mode == "32":
            s.set_blocks(32, 64)
        s.calc_forces(0)
        out[mode] = (s.get_atoms()["f"], s.scalars().tot_pot_energy)
        s.close()
    f0, e0 = out["default"]
    for mode in ("tuned", "32"):
        f, e = out[mode]
        assert np.abs(f - f0).max() <= 1e-12 * np.abs(f0).max()
        assert abs(e - e0) <= 1e-13 * abs(e0)


def _overlap_cell():
    """A noisy 4x4x4 Cu cell with one atom pushed to 0.9 A from a neighbour,
    inside the tables' first point (1.5 A), where the tables clamp."""
    from imd_gb300 import workloads as wl
    x, box = wl.fcc(4, 4, 4, 3.615)
    x = x + 0.02 * np.random.default_rng(1).standard_normal(x.shape)
    d = x[1] - x[0]
    x[0] = x[1] - 0.9 * d / np.linalg.norm(d)
    n = len(x)
    return wl.System(box, x, np.zeros((n, 3)), np.zeros(n, np.int32), np.full(n, wl.CU.mass),
                     np.arange(n, dtype=np.int32))


def test_short_distance_cell_stops_others_relax():
    """IMD's CG cannot leave a pair inside the tables' first point (the
    oracle restatement stays at the same max force, energy creeping up, for
    as long as it runs); the batch stops that cell with status 4 after five
    such line searches and relaxes the other cell normally."""
    import ctypes as C
    import oracle
    from imd_gb300 import api
    from imd_gb300 import workloads as wl
    from oracle import OracleSystem
    bad = _overlap_cell()
    good = wl.defect_cell(np.random.default_rng(14), nmin=300, nmax=600, nlim=(3, 6))
    b = api.GpuBatch(1, api.EAM2, api.FP64, api.SPLINE)
    b.read_tables(tables("cu"))
    b.set_cells([bad, good])
    b.relax(1e-4, maxsteps=2000)
    r = b.results()
    assert r["status"][0] == 4 and r["steps"][0] <= 8, r
    assert r["status"][1] == 0 and r["fmax"][1] <= 1e-4, r
    o = OracleSystem(bad.box, bad.x, bad.types, bad.mass, bad.number, 1, tables("cu"), True, 0.4)
    L = oracle.lib()
    L.orc_reset_cg(C.byref(o.s))
    f0 = L.orc_max_atom_force(C.byref(o.s))
    for k in range(1, 11):
        L.orc_cg_step(C.byref(o.s), k)
    assert L.orc_max_atom_force(C.byref(o.s)) > 10.0 and f0 > 10.0
