"""FP64 numpy statement of the learned step-size controller's network -- test infrastructure
(the checker of the CUDA training and inference kernels, never used by the product path).

Network: 16 -> 64 -> 64 -> 1 with SiLU, z = W x + b; weights packed W1[64][16], b1[64],
W2[64][64], b2[64], W3[64], b3 (5313 values); inputs normalised (x - mean) / std, targets
(y - y_mean) / y_std; loss = mean over samples of (out - y_n)^2.  Gradients by hand-written
reverse mode, checked here against central finite differences.
"""
from __future__ import annotations

import numpy as np

NI, NH = 16, 64
NW = NH * NI + NH + NH * NH + NH + NH + 1


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    assert w.size == NW
    o = 0
    W1 = w[o:o + NH * NI].reshape(NH, NI); o += NH * NI
    b1 = w[o:o + NH]; o += NH
    W2 = w[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = w[o:o + NH]; o += NH
    W3 = w[o:o + NH]; o += NH
    b3 = w[o]
    return W1, b1, W2, b2, W3, b3


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def forward(w, X, norm):
    """Network output in target units; norm = [mean(16), std(16), y_mean, y_std]."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    norm = np.asarray(norm, dtype=np.float64)
    x = (np.asarray(X, dtype=np.float64) - norm[:NI]) / norm[NI:2 * NI]
    z1 = x @ W1.T + b1
    h1 = z1 * _sig(z1)
    z2 = h1 @ W2.T + b2
    h2 = z2 * _sig(z2)
    out = h2 @ W3 + b3
    return norm[2 * NI] + norm[2 * NI + 1] * out


def loss_grad(w, X, y, norm):
    """(loss, gradient) of the mean squared error in normalised units."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    norm = np.asarray(norm, dtype=np.float64)
    x = (np.asarray(X, dtype=np.float64) - norm[:NI]) / norm[NI:2 * NI]
    yn = (np.asarray(y, dtype=np.float64) - norm[2 * NI]) / norm[2 * NI + 1]
    n = len(yn)
    z1 = x @ W1.T + b1
    s1 = _sig(z1)
    h1 = z1 * s1
    z2 = h1 @ W2.T + b2
    s2 = _sig(z2)
    h2 = z2 * s2
    out = h2 @ W3 + b3
    r = out - yn
    loss = float(np.mean(r * r))
    d3 = 2.0 * r / n
    d2 = d3[:, None] * W3[None, :] * (s2 * (1 + z2 * (1 - s2)))
    d1 = (d2 @ W2) * (s1 * (1 + z1 * (1 - s1)))
    g = np.concatenate([(d1.T @ x).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), d3 @ h2, [d3.sum()]])
    return loss, g
