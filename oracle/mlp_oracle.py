"""CPU oracle of the learned-start MLP (test infrastructure only).

Restates the network of imd_gb300/csrc/learn.cu in numpy, in float64 with
the same BF16 rounding points as the tensor-core kernels: inputs, W1, W2, W3,
the hidden activations fed to the second layer and the backward signals fed
to the weight-gradient products are rounded to BF16; everything else is
exact.  Used to check the GPU forward pass and gradients.

Network: x_ij = [16 Gaussian RBF of r_ij (centres 2.0-5.5 A, width 0.25 A),
rho_i / 100] -> 64 -> 64 -> 1 (SiLU); dx_i = sum_j w_ij unit(r_ij).
Parameters (flat, float32): W1[64][32] (inputs >= 17 zero), b1[64],
W2[64][64], b2[64], W3[64], b3.
"""
from __future__ import annotations

import numpy as np

H, K1, NIN = 64, 32, 17
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * K1
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NPARAM = OFF_B3 + 1
CENTRES = 2.0 + np.arange(16) * (3.5 / 15.0)


def bf16(a) -> np.ndarray:
    """Round to bfloat16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(a, np.float32))
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16 << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w):
    w = np.asarray(w, np.float64)
    W1 = w[OFF_W1:OFF_B1].reshape(H, K1)
    return (W1, w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(H, H), w[OFF_B2:OFF_W3],
            w[OFF_W3:OFF_B3], w[OFF_B3])


def init_weights(seed: int = 0, scale: float = 1.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    w = np.zeros(NPARAM, np.float32)
    w[OFF_W1:OFF_B1] = (rng.standard_normal((H, K1)) * scale / np.sqrt(NIN)).ravel()
    w[OFF_W1:OFF_B1].reshape(H, K1)[:, NIN:] = 0.0
    w[OFF_W2:OFF_B2] = (rng.standard_normal((H, H)) * scale / np.sqrt(H)).ravel()
    w[OFF_W3:OFF_B3] = rng.standard_normal(H) * 0.01 * scale
    return w


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def pairs_min_image(x, box, rc: float = 5.5):
    """Directed pairs (i, j) with r_ij < rc by minimum image (box > 2 rc)."""
    x = np.asarray(x, np.float64)
    tb = np.linalg.inv(np.asarray(box, np.float64))
    I, D = [], []
    for i in range(len(x)):
        d = x - x[i]
        s = d @ tb
        s -= np.round(s)
        d = s @ box
        r2 = np.einsum("ij,ij->i", d, d)
        m = (r2 < rc * rc) & (np.arange(len(x)) != i)
        I.append(np.full(m.sum(), i))
        D.append(d[m])
    return np.concatenate(I), np.concatenate(D)


def features(d, rho_i):
    r = np.sqrt(np.einsum("ij,ij->i", d, d))
    X = np.zeros((len(d), K1))
    X[:, :16] = np.exp(-0.5 * ((r[:, None] - CENTRES[None, :]) / 0.25) ** 2)
    X[:, 16] = rho_i * 0.01
    return X, d / r[:, None]


def forward(w, pi, d, rho, n):
    W1, b1, W2, b2, W3, b3 = unpack(w)
    X, u = features(d, rho[pi])
    Xb = bf16(X)
    z1 = Xb @ bf16(W1).T + b1
    h1b = bf16(silu(z1))
    z2 = h1b @ bf16(W2).T + b2
    h2 = silu(z2)
    wv = h2 @ bf16(W3) + b3
    dx = np.zeros((n, 3))
    np.add.at(dx, pi, wv[:, None] * u)
    return dx, dict(Xb=Xb, z1=z1, h1b=h1b, z2=z2, h2=h2, u=u, wv=wv)


def loss_and_grad(w, pi, d, rho, target):
    n = len(target)
    W1, b1, W2, b2, W3, b3 = unpack(w)
    dx, c = forward(w, pi, d, rho, n)
    e = dx - target
    loss = float(np.sum(e * e) / n)
    dldx = 2.0 * e / n
    g = np.einsum("ij,ij->i", dldx[pi], c["u"])
    grad = np.zeros(NPARAM)
    grad[OFF_W3:OFF_B3] = g @ c["h2"]
    grad[OFF_B3] = g.sum()
    dz2 = g[:, None] * bf16(W3)[None, :] * dsilu(c["z2"])
    grad[OFF_B2:OFF_W3] = dz2.sum(0)
    dz2b = bf16(dz2)
    grad[OFF_W2:OFF_B2] = (dz2b.T @ c["h1b"]).ravel()
    dh1 = dz2b @ bf16(W2)
    dz1 = dh1 * dsilu(c["z1"])
    grad[OFF_B1:OFF_W2] = dz1.sum(0)
    gW1 = bf16(dz1).T @ c["Xb"]
    gW1[:, NIN:] = 0.0
    grad[OFF_W1:OFF_B1] = gW1.ravel()
    return loss, grad, dx
