"""Float64 CPU restatement of the plan-selection MLP -- TEST INFRASTRUCTURE ONLY.

Forward and backward of NFEAT -> 128 -> 128 -> 128 -> 1 with ReLU and an MSE
loss, in numpy float64, with the parameter layout of the engine (W1 [128][F],
b1, W2 [128][128], b2, W3, b3, W4 [1][128], b4; row-major [out][in]).  Tests
compare the engine's CUDA forward/backward kernels and its host inference
against it.
"""
import numpy as np

H = 128


def unpack(params, nfeat):
    p = np.asarray(params, dtype=np.float64)
    sizes = [H * nfeat, H, H * H, H, H * H, H, H, 1]
    out, o = [], 0
    for s in sizes:
        out.append(p[o:o + s])
        o += s
    W1, b1, W2, b2, W3, b3, W4, b4 = out
    return W1.reshape(H, nfeat), b1, W2.reshape(H, H), b2, W3.reshape(H, H), b3, W4.reshape(1, H), b4


def forward(params, X):
    X = np.asarray(X, dtype=np.float64)
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(params, X.shape[1])
    A1 = np.maximum(X @ W1.T + b1, 0.0)
    A2 = np.maximum(A1 @ W2.T + b2, 0.0)
    A3 = np.maximum(A2 @ W3.T + b3, 0.0)
    out = (A3 @ W4.T + b4)[:, 0]
    return out, (A1, A2, A3)


def mse_gradients(params, X, y):
    """Loss and the gradient of mean((out - y)^2) w.r.t. every parameter."""
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(params, X.shape[1])
    out, (A1, A2, A3) = forward(params, X)
    n = X.shape[0]
    d = out - y
    loss = float(np.mean(d * d))
    dout = (2.0 * d / n)[:, None]
    gW4 = dout.T @ A3
    gb4 = dout.sum(0)
    dZ3 = (dout @ W4) * (A3 > 0)
    gW3 = dZ3.T @ A2
    gb3 = dZ3.sum(0)
    dZ2 = (dZ3 @ W3) * (A2 > 0)
    gW2 = dZ2.T @ A1
    gb2 = dZ2.sum(0)
    dZ1 = (dZ2 @ W2) * (A1 > 0)
    gW1 = dZ1.T @ X
    gb1 = dZ1.sum(0)
    grads = np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3, gW4, gb4)])
    return loss, grads
