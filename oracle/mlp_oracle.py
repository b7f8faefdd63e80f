"""mlp_oracle.py -- numpy restatement of the learned wall-stress network
(3 -> 64 -> 64 -> 1, tanh) with the arithmetic of the CUDA kernels: the
64 x 64 layer (the tensor-core layer) with BF16 weights and BF16 inputs,
layers 1 and 3 in FP32, FP32 accumulation, mean-squared error on the
normalised log of the stress over its laminar value, Adam.  TEST INFRASTRUCTURE ONLY: the checker of
the device forward, backward and update kernels.

Parameter vector layout (FP32, 4481 values), shared with the device:
W1[64][3], b1[64], W2[64][64] (row = output unit), b2[64], W3[64], b3.
"""
import numpy as np

H = 64
O_W1, O_B1, O_W2, O_B2, O_W3, O_B3, NPARAM = 0, 192, 256, 4352, 4416, 4480, 4481


def bf16(a):
    """Round float32 values to bfloat16 (round to nearest even), as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    out = (((b + r) >> 16) << 16).astype(np.uint32)
    nan = np.isnan(a)
    out[nan] = 0x7FC00000
    return out.view(np.float32).reshape(a.shape)


def unpack(p):
    p = np.asarray(p, dtype=np.float32)
    return (p[O_W1:O_B1].reshape(H, 3), p[O_B1:O_W2], p[O_W2:O_B2].reshape(H, H), p[O_B2:O_W3], p[O_W3:O_B3],
            p[O_B3])


def logs32(u, h, nu):
    """The FP32 logs of the inputs the kernels take."""
    return (np.log(np.asarray(u, dtype=np.float32)), np.log(np.asarray(h, dtype=np.float32)),
            np.log(np.asarray(nu, dtype=np.float32)))


def features(u, h, nu, norm):
    """Normalised log inputs: norm = (mean, std) of log u, log h, log nu and the
    target log(tau h / (nu u))."""
    m, s = norm[:4], norm[4:]
    lu, lh, ln = logs32(u, h, nu)
    x = np.stack([(lu - m[0]) / s[0], (lh - m[1]) / s[1], (ln - m[2]) / s[2]], axis=1)
    return x.astype(np.float32)


def target(u, h, nu, tau, norm):
    lu, lh, ln = logs32(u, h, nu)
    lt = np.log(np.asarray(tau, dtype=np.float32))
    return ((lt - (ln + lu - lh) - norm[3]) / norm[7]).astype(np.float32)


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    W1b, W2b, W3b = W1, bf16(W2), W3  # BF16: the tensor-core layer's operands only
    z1 = (x @ W1b.T + b1).astype(np.float32)
    h1 = np.tanh(z1).astype(np.float32)
    h1b = bf16(h1)
    z2 = (h1b @ W2b.T + b2).astype(np.float32)
    h2 = np.tanh(z2).astype(np.float32)
    y = (h2 @ W3b + b3).astype(np.float32)
    return dict(x=x, h1=h1, h1b=h1b, h2=h2, y=y, W2b=W2b, W3b=W3b)


def gradient(p, x, t, delta_bf16=False):
    """Gradient of mean((y - t)^2) over the batch with respect to the FP32
    parameters (the rounding to BF16 passes gradients straight through).
    delta_bf16: layer 2's output gradient enters the input- and
    weight-gradient products rounded to BF16 (their operands on the tensor
    cores); its bias gradient keeps the FP32 values."""
    f = forward(p, x)
    B = x.shape[0]
    dy = (2.0 * (f["y"] - t) / B).astype(np.float32)
    g = np.zeros(NPARAM, dtype=np.float64)
    g[O_W3:O_B3] = dy @ f["h2"]
    g[O_B3] = dy.sum()
    dz2 = (dy[:, None] * f["W3b"][None, :] * (1.0 - f["h2"] ** 2)).astype(np.float32)
    dz2m = bf16(dz2) if delta_bf16 else dz2
    g[O_W2:O_B2] = (dz2m.astype(np.float64).T @ f["h1b"].astype(np.float64)).ravel()
    g[O_B2:O_W3] = dz2.sum(axis=0)
    dh1 = dz2m @ f["W2b"]
    dz1 = dh1 * (1.0 - f["h1"] ** 2)
    g[O_W1:O_B1] = (dz1.T @ x).ravel()
    g[O_B1:O_W2] = dz1.sum(axis=0)
    return g, float(np.mean((f["y"] - t) ** 2))


def predict_tau(p, norm, u, h, nu):
    y = forward(p, features(u, h, nu, norm))["y"].astype(np.float64)
    lu, lh, ln = logs32(u, h, nu)
    return np.exp(y * norm[7] + norm[3] + (ln + lu - lh).astype(np.float64))
