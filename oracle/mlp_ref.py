"""CPU model of the lossy proposer's network (TEST INFRASTRUCTURE: the tests
check the GPU forward/backward kernels of csrc/mlp.cu against it; the product
never calls it).  512 -> 256 -> 256 -> 64 with ReLU; parameters
W1[512x256], b1, W2[256x256], b2, W3[256x64], b3 concatenated; siamese loss
mean((|f(a) - f(b)|^2 - t)^2), in float64."""
import numpy as np

SHAPES = [(512, 256), (256,), (256, 256), (256,), (256, 64), (64,)]


def unpack(w):
    out, o = [], 0
    for s in SHAPES:
        n = int(np.prod(s))
        out.append(np.asarray(w[o:o + n], np.float64).reshape(s))
        o += n
    return out


def forward(w, x):
    W1, b1, W2, b2, W3, b3 = unpack(w)
    h1 = np.maximum(x @ W1 + b1, 0.0)
    h2 = np.maximum(h1 @ W2 + b2, 0.0)
    return h1, h2, h2 @ W3 + b3


def loss_grad(w, xa, xb, t):
    W1, b1, W2, b2, W3, b3 = unpack(w)
    n = xa.shape[0]
    x = np.concatenate([xa, xb]).astype(np.float64)
    h1, h2, e = forward(w, x)
    d = e[:n] - e[n:]
    r = (d * d).sum(1) - np.asarray(t, np.float64)
    loss = float((r * r).mean())
    g = (2.0 * r / n)[:, None] * 2.0 * d
    de = np.concatenate([g, -g])
    dW3 = h2.T @ de
    db3 = de.sum(0)
    dh2 = (de @ W3.T) * (h2 > 0)
    dW2 = h1.T @ dh2
    db2 = dh2.sum(0)
    dh1 = (dh2 @ W2.T) * (h1 > 0)
    dW1 = x.T @ dh1
    db1 = dh1.sum(0)
    return loss, np.concatenate([a.ravel() for a in (dW1, db1, dW2, db2, dW3, db3)])
