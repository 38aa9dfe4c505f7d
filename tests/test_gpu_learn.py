"""Learned start: the hand-written BF16 tensor-core forward and backward
kernels of the per-pair MLP against the numpy oracle (same BF16 rounding
points), and Adam training on the GPU reducing the loss."""
import numpy as np
import pytest

from conftest import golden, tables

pytestmark = pytest.mark.gpu


def _system(g, x=None):
    from imd_gb300 import api
    s = api.GpuSystem(1, api.EAM2, api.FP64)
    s.read_tables(tables("cu"))
    s.set_box(g["box"], (1, 1, 1), 0.4)
    s.set_atoms(g["number"], g["type"], g["mass"], g["x"] if x is None else x)
    return s


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def test_mlp_forward_and_gradients_match_oracle():
    import mlp_oracle as M
    g = golden("cu_pert")
    n = len(g["x"])
    s = _system(g)
    w = M.init_weights(3)
    s.ml_set_weights(w)
    rng = np.random.default_rng(4)
    target = 0.05 * rng.standard_normal((n, 3))
    loss_g, grad_g = s.ml_train_step(target, lr=0.0, want_grad=True)
    dx_g = s.ml_predict()
    pi, d = M.pairs_min_image(g["x"], g["box"])
    loss_o, grad_o, dx_o = M.loss_and_grad(w, pi, d, g["rho"], target)
    assert rel(dx_g, dx_o) < 2e-3
    assert abs(loss_g - loss_o) / loss_o < 1e-3
    assert rel(grad_g, grad_o) < 1e-2
    for lo, hi in ((M.OFF_W1, M.OFF_B1), (M.OFF_W2, M.OFF_B2), (M.OFF_W3, M.OFF_B3)):
        assert rel(grad_g[lo:hi], grad_o[lo:hi]) < 2e-2


def test_training_reduces_loss():
    """Fit a pair-additive target (a scaled force field): Adam steps on the
    device lower the loss."""
    import mlp_oracle as M
    g = golden("cu_pert")
    s = _system(g)
    s.calc_forces(0)
    target = 0.02 * s.get_atoms()["f"]
    s.ml_set_weights(M.init_weights(5))
    l0 = s.ml_train_step(target, lr=0.0)
    for _ in range(60):
        s.ml_train_step(target, lr=3e-3)
    l1 = s.ml_train_step(target, lr=0.0)
    assert l1 < 0.5 * l0, (l0, l1)


def _small_cells(seed, k, nmin=300, nmax=900):
    from imd_gb300 import workloads as wl
    rng = np.random.default_rng(seed)
    return [wl.defect_cell(rng, nmin=nmin, nmax=nmax, nlim=(3, 6)) for _ in range(k)]


def test_batch_ml_start_energies_and_gate():
    """imdgpu_batch_ml_start: e_start of every cell is the oracle's energy of
    the cell, e_pred is the energy at start + predicted displacement, and
    exactly the cells with e_pred < e_start keep the prediction."""
    from imd_gb300 import api, learned
    from oracle import OracleSystem
    cells = _small_cells(21, 4)
    w = learned.init_weights(7)
    w[learned.OFF_W3:learned.OFF_B3] *= 30.0  # displacements large enough to matter
    b = learned.make_batch(tables("cu"), cells)
    b.ml_set_weights(w)
    # prediction at the start positions, cell by cell through single systems
    pred = []
    for c in cells:
        s = api.system_from_tables(tables("cu"), c.box, c.number, c.types, c.mass, c.x)
        s.ml_set_weights(w)
        pred.append(s.ml_predict())
        s.close()
    used, e0, e1 = b.ml_start()
    xs = b.positions()
    for k, c in enumerate(cells):
        o = OracleSystem(c.box, c.x, c.types, c.mass, c.number, 1, tables("cu"), True, 0.4)
        o.calc_forces()
        assert abs(e0[k] - o.epot_total) <= 1e-12 * abs(o.epot_total)
        o2 = OracleSystem(c.box, c.x + pred[k], c.types, c.mass, c.number, 1, tables("cu"),
                          True, 0.4)
        o2.calc_forces()
        assert abs(e1[k] - o2.epot_total) <= 1e-9 * abs(o2.epot_total)
        assert used[k] == (e1[k] < e0[k])
        expect = c.x + pred[k] if used[k] else c.x
        d = learned.min_image(xs[k] - expect, np.asarray(c.box))
        assert np.abs(d).max() < 1e-6, (k, used[k], np.abs(d).max())


def test_learned_start_beats_plain_cg():
    """Train on displacements that the plain batched CG produced for small
    defect cells, then relax held-out cells from the learned start: the
    start lowers the energy of every held-out cell, CG needs fewer force
    calls in total (the learned start's two included), and the final
    energies equal plain CG's within 1e-6 eV/atom."""
    from imd_gb300 import learned
    train = _small_cells(31, 24)
    held = _small_cells(32, 8)
    plain_train = learned.relax(tables("cu"), train, keep_positions=True)
    assert np.all(plain_train.status == 0)
    disp = learned.targets(train, plain_train.positions)
    tr = learned.Trainer(tables("cu"), train, disp, batch_cells=8, seed=3)
    l0 = tr.loss()
    for _ in range(60):
        tr.epoch(lr=3e-3)
    l1 = tr.loss()
    w = tr.w.copy()
    tr.close()
    assert l1 < 0.5 * l0, (l0, l1)
    plain = learned.relax(tables("cu"), held)
    ml = learned.relax(tables("cu"), held, weights=w)
    n = np.array([c.n for c in held])
    assert np.all(plain.status == 0) and np.all(ml.status == 0)
    assert np.all(ml.used == 1), (ml.e_start, ml.e_pred)
    assert ml.nfc.sum() < plain.nfc.sum(), (ml.nfc, plain.nfc)
    assert np.all(np.abs(ml.epot - plain.epot) / n <= 1e-6), (ml.epot - plain.epot) / n
