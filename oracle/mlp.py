"""CPU oracle of the Strassen scheduler's MLP (test infrastructure only).

The same parameter layout as strassen_gb300/csrc/bsg_sched.cu -- W1 [64 x 29],
b1 [64], W2 [64 x 64], b2 [64], W3 [64], b3 [1], float32 on the device -- and
the forward pass y = W3 relu(W2 relu(W1 x + b1) + b2) + b3 with the mean
squared error loss and its gradient, here in float64 numpy.
"""
import numpy as np

IN, H = 29, 64  # 25 node features + 4 option one-hot inputs
N_PARAMS = H * IN + H + H * H + H + H + 1


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + H * IN].reshape(H, IN); o += H * IN
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, np.float64)
    h1 = np.maximum(X @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return h2 @ W3 + b3, (h1, h2)


def loss_grad(p, X, T):
    """mean squared error and its gradient (flattened like the parameters)"""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    y, (h1, h2) = forward(p, X)
    n = len(X)
    dy = 2.0 * (y - T) / n
    gW3 = dy @ h2
    gb3 = dy.sum()
    dh2 = dy[:, None] * W3[None, :] * (h2 > 0)
    gW2 = dh2.T @ h1
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    gW1 = dh1.T @ X
    gb1 = dh1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return float(np.mean((y - T) ** 2)), g
