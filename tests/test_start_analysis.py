"""Where a CG start saves force calls, measured with the oracle's CG (IMD's
algorithm, spline tables) on a cell of the held-out relaxation batch.

A start that puts every atom displaced by less than 0.2 A (the elastic
field) at its relaxed position saves almost nothing; a start that puts
only the few defect-core atoms there saves more than half of the force
calls.  The learned start's per-pair model mostly predicts the elastic
field, which is why its gain is small."""
import os

import numpy as np
import pytest

oracle = pytest.importorskip("oracle")


def test_defect_cores_set_the_cg_cost(tmp_path):
    from imd_gb300 import workloads as wl
    tabs = wl.sutton_chen_tables(str(tmp_path / "cu"), [wl.CU])
    cells = wl.defect_batch(512, seed=6)
    c = cells[np.argsort([k.n for k in cells], kind="stable")[5]]   # 575 atoms, a vacancy pair
    n = c.n
    oracle.set_interpolation(oracle.SPLINE)
    try:
        def relax(x):
            o = oracle.OracleSystem(c.box, x, np.zeros(n, np.int32), c.mass,
                                    np.arange(n, dtype=np.int32), 1, tabs, True, 0.4)
            steps, fm = o.cg_relax(1e-4, 3000)
            assert steps >= 0 and fm <= 1e-4
            return int(o.nfc), o.x.copy()

        nfc_plain, xs = relax(c.x)
        d = xs - c.x
        d -= np.round(d @ np.linalg.inv(c.box)) @ c.box
        core = (np.sqrt((d ** 2).sum(1)) >= 0.2)[:, None]
        assert 0 < int(core.sum()) < 0.05 * n
        nfc_elastic, _ = relax(c.x + np.where(core, 0.0, d))
        nfc_core, _ = relax(c.x + np.where(core, d, 0.0))
    finally:
        oracle.set_interpolation(oracle.QUADRATIC)
    assert nfc_elastic > 0.85 * nfc_plain
    assert nfc_core < 0.5 * nfc_plain
