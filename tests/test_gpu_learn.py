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
