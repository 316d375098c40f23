"""float64 restatement of the scheduler's MLP (in -> 64 -> 64 -> 1, ReLU, mean
squared error) for checking the library's CUDA training kernels."""
import numpy as np

H = 64


def unpack(p, n_in):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + H * n_in].reshape(H, n_in); o += H * n_in
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def forward(p, X):
    W1, b1, W2, b2, w3, b3 = unpack(p, X.shape[1])
    z1 = X @ W1.T + b1
    a1 = np.maximum(z1, 0.0)
    z2 = a1 @ W2.T + b2
    a2 = np.maximum(z2, 0.0)
    return a2 @ w3 + b3, (z1, a1, z2, a2)


def loss_grad(p, X, y):
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    W1, b1, W2, b2, w3, b3 = unpack(p, X.shape[1])
    out, (z1, a1, z2, a2) = forward(p, X)
    n = X.shape[0]
    e = out - y
    loss = float((e * e).mean())
    dout = 2.0 * e / n
    dw3 = a2.T @ dout
    db3 = dout.sum()
    dz2 = np.outer(dout, w3) * (z2 > 0)
    dW2 = dz2.T @ a1
    db2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * (z1 > 0)
    dW1 = dz1.T @ X
    db1 = dz1.sum(0)
    return loss, np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dw3, [db3]])
