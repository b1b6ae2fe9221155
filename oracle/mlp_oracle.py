"""ORACLE — test infrastructure only.  FP64 numpy restatement of the
16 -> 64 -> 64 -> 3 selector MLP (ReLU, softmax cross-entropy, mean over the
batch) used to check the GPU forward and gradient kernels
(elemental_gb300/csrc/mlp.cu).  Parameter layout: W1[16][64] b1[64]
W2[64][64] b2[64] W3[64][3] b3[3], row-major (input x output)."""
import numpy as np

IN, H, OUT = 16, 64, 3
SHAPES = [("W1", (IN, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, OUT)),
          ("b3", (OUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(theta):
    theta = np.asarray(theta, dtype=np.float64)
    out, o = {}, 0
    for name, shp in SHAPES:
        k = int(np.prod(shp))
        out[name] = theta[o:o + k].reshape(shp)
        o += k
    return out


def forward(theta, X):
    p = unpack(theta)
    X = np.asarray(X, dtype=np.float64)
    z1 = X @ p["W1"] + p["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ p["W2"] + p["b2"]
    h2 = np.maximum(z2, 0)
    lg = h2 @ p["W3"] + p["b3"]
    lg = lg - lg.max(axis=1, keepdims=True)
    e = np.exp(lg)
    P = e / e.sum(axis=1, keepdims=True)
    return dict(z1=z1, h1=h1, z2=z2, h2=h2, logits=lg, probs=P)


def loss_and_grad(theta, X, y):
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y)
    B = X.shape[0]
    f = forward(theta, X)
    p = unpack(theta)
    loss = -np.mean(np.log(f["probs"][np.arange(B), y]))
    d3 = f["probs"].copy()
    d3[np.arange(B), y] -= 1.0
    d3 /= B
    gW3 = f["h2"].T @ d3
    gb3 = d3.sum(0)
    d2 = (d3 @ p["W3"].T) * (f["z2"] > 0)
    gW2 = f["h1"].T @ d2
    gb2 = d2.sum(0)
    d1 = (d2 @ p["W2"].T) * (f["z1"] > 0)
    gW1 = X.T @ d1
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
