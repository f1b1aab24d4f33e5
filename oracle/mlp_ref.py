"""FP64 restatement of the policy network's loss and gradient (numpy).

TEST INFRASTRUCTURE ONLY: the checker for the device training kernels in
byo_gb300/csrc/mlp.cu.  Parameter layout (1765 floats): W1[32][16], b1[32],
W2[32][32], b2[32], W3[5][32], b3[5]; y = W3 relu(W2 relu(W1 x + b1) + b2) + b3;
loss = mean over the targets marked in `mask` of (y - t)^2.
"""
import numpy as np

NIN, NH, NOUT = 16, 32, 5
SIZES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NOUT, NH)),
         ("b3", (NOUT,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    p = np.asarray(p, np.float64)
    out, o = {}, 0
    for name, shape in SIZES:
        k = int(np.prod(shape))
        out[name] = p[o:o + k].reshape(shape)
        o += k
    return out


def pack(d):
    return np.concatenate([d[name].reshape(-1) for name, _ in SIZES])


def forward(p, X):
    w = unpack(p)
    a1 = X @ w["W1"].T + w["b1"]
    h1 = np.maximum(a1, 0)
    a2 = h1 @ w["W2"].T + w["b2"]
    h2 = np.maximum(a2, 0)
    return h2 @ w["W3"].T + w["b3"], (a1, h1, a2, h2)


def loss_grad(p, X, Y, mask):
    X = np.asarray(X, np.float64)
    Y = np.asarray(Y, np.float64)
    M = ((np.asarray(mask, np.uint8)[:, None] >> np.arange(NOUT)) & 1).astype(np.float64)
    w = unpack(p)
    y, (a1, h1, a2, h2) = forward(p, X)
    cnt = M.sum()
    d = (y - Y) * M
    loss = (d ** 2).sum() / cnt
    dy = 2 * d / cnt
    g = {"W3": dy.T @ h2, "b3": dy.sum(0)}
    dh2 = (dy @ w["W3"]) * (a2 > 0)
    g["W2"] = dh2.T @ h1
    g["b2"] = dh2.sum(0)
    dh1 = (dh2 @ w["W2"]) * (a1 > 0)
    g["W1"] = dh1.T @ X
    g["b1"] = dh1.sum(0)
    return loss, pack(g)
