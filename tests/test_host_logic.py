"""CPU checks of the host-side logic around the kernels: the learned
start's parameter layout against the oracle's, the minimum-image
displacements that make its training targets, and the workload
generator's rules (atom counts, overlap-free defect sites)."""
import numpy as np

import mlp_oracle as M
from imd_gb300 import learned
from imd_gb300 import workloads as wl


def test_mlp_layout_matches_oracle():
    assert learned.NPARAM == M.NPARAM
    for name in ("OFF_W1", "OFF_B1", "OFF_W2", "OFF_B2", "OFF_W3", "OFF_B3"):
        assert getattr(learned, name) == getattr(M, name)
    w = learned.init_weights(1)
    assert w.dtype == np.float32 and w.shape == (M.NPARAM,)
    W1 = w[learned.OFF_W1:learned.OFF_B1].reshape(learned.H, learned.K1)
    assert np.all(W1[:, learned.NIN:] == 0.0)       # padding inputs stay zero
    assert np.all(w[learned.OFF_B1:learned.OFF_W2] == 0.0)


def test_min_image_triclinic():
    rng = np.random.default_rng(2)
    box = np.array([[10.0, 0.5, 0.0], [0.3, 11.0, 0.2], [0.0, -0.4, 9.5]])
    d = rng.uniform(-0.3, 0.3, size=(50, 3))
    shifts = rng.integers(-2, 3, size=(50, 3))
    wrapped = d + shifts @ box
    np.testing.assert_allclose(learned.min_image(wrapped, box), d, atol=1e-12)


def test_defect_cells_follow_the_generator_rules():
    rng = np.random.default_rng(7)
    for _ in range(20):
        c = wl.defect_cell(rng, nmin=300, nmax=3000, nlim=(3, 8))
        n1, n2, n3 = c.meta["dims"]
        assert 3 <= min(n1, n2, n3) and max(n1, n2, n3) <= 8
        assert 1 <= c.meta["defects"] <= 4
        # every defect removes or adds one atom
        assert abs(c.n - 4 * n1 * n2 * n3) <= c.meta["defects"]
        # no two atoms closer than the overlap bar minus strain and noise
        x, box = c.x, np.asarray(c.box)
        tb = np.linalg.inv(box)
        for i in range(c.n):
            dd = x - x[i]
            s = dd @ tb
            s -= np.round(s)
            r = np.sqrt(np.einsum("ij,ij->i", s @ box, s @ box))
            r[i] = 9.0
            assert r.min() > 1.4


def test_defect_batch_is_reproducible():
    a = wl.defect_batch(6, seed=4)
    b = wl.defect_batch(6, seed=4)
    for ca, cb in zip(a, b):
        np.testing.assert_array_equal(ca.x, cb.x)
        np.testing.assert_array_equal(ca.box, cb.box)
