"""numpy reference of the guess network (xcape_gb300/csrc/guess_mlp.cuh), for
the gradient and inference checks.

forward(..., bf16_hidden=True) reproduces the GPU training/inference
forward pass: the 64x64 hidden layer multiplies BF16-rounded activations by
BF16-rounded weights (exact products, accumulated here in FP64); everything
else is FP64.  loss_and_grad() follows guess_train_kernel, whose two
backward products run on the tensor cores too: dW2 = dZ2^T H1 and
dH1 = dZ2 W2 take BF16-rounded operands (exact products, FP64 sums here).
"""
import numpy as np

from xcape_gb300.guess import H, OFF_B1, OFF_B2, OFF_B3, OFF_W1, OFF_W2, OFF_W3, bf16_round


def unpack(w):
    w = np.asarray(w, np.float64)
    return (w[OFF_W1:OFF_B1].reshape(H, 3), w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(H, H),
            w[OFF_B2:OFF_W3], w[OFF_W3:OFF_B3], w[OFF_B3])


def forward(w, x, bf16_hidden=True):
    W1, b1, W2, b2, w3, b3 = unpack(w)
    x = np.asarray(x, np.float64)
    h1 = np.maximum(x @ W1.T + b1, 0.0)
    if bf16_hidden:
        h1q = bf16_round(h1.astype(np.float32)).astype(np.float64)
        W2q = bf16_round(W2.astype(np.float32)).astype(np.float64)
        z2 = h1q @ W2q.T + b2
    else:
        z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0.0)
    y = h2 @ w3 + b3
    return y, (x, h1, z2, h2)


def loss_and_grad(w, x, t):
    W1, b1, W2, b2, w3, b3 = unpack(w)
    y, (x, h1, z2, h2) = forward(w, x)
    n = len(t)
    err = y - np.asarray(t, np.float64)
    loss = np.mean(err ** 2)
    dy = 2.0 * err / n
    g = np.zeros(len(w))
    g[OFF_W3:OFF_B3] = h2.T @ dy
    g[OFF_B3] = dy.sum()
    dz2 = (dy[:, None] * w3[None, :]) * (z2 > 0)
    q = lambda a: bf16_round(np.asarray(a, np.float32)).astype(np.float64)
    g[OFF_W2:OFF_B2] = (q(dz2).T @ q(h1)).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz1 = (q(dz2) @ q(W2)) * (h1 > 0)
    g[OFF_W1:OFF_B1] = (dz1.T @ x).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return loss, g
