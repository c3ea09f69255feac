"""CPU ORACLE of the culling network — test infrastructure only.

float64 numpy forward and backward of the per-shape network the GPU trains
(``sand_atlas_dem_gb300/csrc/culler.cu``): h0 = sin(W0 p + b0),
h1 = relu(W1 h0 + b1), y = w2 . h1 + b2, loss = mean(w (y - phi/scale)^2)
with w = ``over`` where the target is inside (phi <= 0) and y exceeds it, else 1.
Used to check the GPU gradients (there is no reference counterpart).
"""

import numpy as np

H = 64
W0, B0, W1, B1, W2, B2 = 0, 192, 256, 256 + 4096, 256 + 4096 + 64, 256 + 4096 + 128


def forward_backward(params, points, scale, over=1.0):
    """Loss and gradient (same flat layout as ``params``) for one batch."""
    p = np.asarray(params, np.float64)
    x = np.asarray(points[:, :3], np.float64)
    t = np.asarray(points[:, 3], np.float64) / scale
    w0 = p[W0:B0].reshape(H, 3)
    b0 = p[B0:W1]
    w1 = p[W1:B1].reshape(H, H)
    b1 = p[B1:W2]
    w2 = p[W2:B2]
    b2 = p[B2]
    z0 = x @ w0.T + b0
    h0 = np.sin(z0)
    a1 = h0 @ w1.T + b1
    h1 = np.maximum(a1, 0)
    y = h1 @ w2 + b2
    n = len(x)
    err = y - t
    weight = np.where((t <= 0) & (err > 0), over, 1.0)
    loss = np.mean(weight * err**2)
    dy = 2 * weight * err / n
    grad = np.zeros_like(p)
    grad[W2:B2] = dy @ h1
    grad[B2] = dy.sum()
    da1 = np.outer(dy, w2) * (a1 > 0)
    grad[W1:B1] = (da1.T @ h0).ravel()
    grad[B1:W2] = da1.sum(0)
    dz0 = (da1 @ w1) * np.cos(z0)
    grad[W0:B0] = (dz0.T @ x).ravel()
    grad[B0:W1] = dz0.sum(0)
    return loss, grad
