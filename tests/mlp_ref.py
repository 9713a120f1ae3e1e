"""CPU restatement (numpy) of the proposal network's forward and backward
passes, used to check the tensor-core kernels.  It rounds to bfloat16 exactly
where the kernels feed the tensor cores (inputs, weights, hidden activations,
back-propagated signals) and accumulates in float64, so the only remaining
difference is the GPU's FP32 accumulation order."""
import numpy as np

IN, HID = 10, 64
# master layout: W1[64][10], b1[64], W2[64][64], b2[64], w3[64], b3
OFF = dict(W1=0, b1=640, W2=704, b2=4800, w3=4864, b3=4928)


def bf16(x):
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).reshape(x.shape)


def unpack(m):
    m = np.asarray(m, np.float32)
    return dict(W1=m[0:640].reshape(HID, IN), b1=m[640:704], W2=m[704:4800].reshape(HID, HID), b2=m[4800:4864],
                w3=m[4864:4928], b3=m[4928])


def forward(m, X):
    p = unpack(m)
    Xb = bf16(X).astype(np.float64)
    z1 = Xb @ bf16(p["W1"]).astype(np.float64).T + p["b1"]
    h1 = bf16(np.maximum(z1, 0)).astype(np.float64)
    z2 = h1 @ bf16(p["W2"]).astype(np.float64).T + p["b2"]
    h2 = np.maximum(z2, 0)
    out = h2 @ p["w3"].astype(np.float64) + float(p["b3"])
    return out, dict(Xb=Xb, z1=z1, h1=h1, z2=z2, h2=h2)


def grad(m, X, t):
    """Gradient of mean((out - t)^2) with respect to the master parameters."""
    p = unpack(m)
    n = len(t)
    out, c = forward(m, X)
    e = out - t
    dout = 2.0 * e / n
    g = np.zeros(4929)
    g[OFF["w3"]:OFF["w3"] + HID] = dout @ c["h2"]
    g[OFF["b3"]] = dout.sum()
    g2 = np.where(c["z2"] > 0, dout[:, None] * p["w3"][None, :].astype(np.float64), 0.0)
    g[OFF["b2"]:OFF["b2"] + HID] = g2.sum(0)
    G2 = bf16(g2).astype(np.float64)
    dh1 = G2 @ bf16(p["W2"]).astype(np.float64)
    g[OFF["W2"]:OFF["W2"] + HID * HID] = (G2.T @ c["h1"]).reshape(-1)
    g1 = np.where(c["z1"] > 0, dh1, 0.0)
    g[OFF["b1"]:OFF["b1"] + HID] = g1.sum(0)
    G1 = bf16(g1).astype(np.float64)
    g[OFF["W1"]:OFF["W1"] + HID * IN] = (G1.T @ c["Xb"]).reshape(-1)
    return g, float((e * e).sum())
