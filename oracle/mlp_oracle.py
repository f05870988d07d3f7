"""FP64 oracle of the screen proposer's MLP (16 -> 256 -> 256 -> 3).  TEST INFRASTRUCTURE ONLY.

Forward and backward in float64 with the same BF16 roundings the CUDA kernels apply
(auto_gb300/csrc/mlp.cu): inputs, weights and stored activations are rounded to bfloat16
(round to nearest even); every sum is exact in float64.  The loss is the mean binary
cross-entropy with logits over the batch and the 3 labels.  The reference has no learned
component, so this oracle has no reference counterpart; it checks the kernels' gradients.
"""
import numpy as np

IN, HID, OUT = 16, 256, 3
P_W1 = 0
P_B1 = P_W1 + HID * IN
P_W2 = P_B1 + HID
P_B2 = P_W2 + HID * HID
P_W3 = P_B2 + HID
P_B3 = P_W3 + OUT * HID
NPARAM = P_B3 + OUT


_ROUND = [True]


def bf16(a):
    """Round float values to bfloat16 (nearest, ties to even), returned as float64; identity when
    rounding is switched off (the finite-difference self-check runs the plain float64 network)."""
    if not _ROUND[0]:
        return np.asarray(a, np.float64)
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[P_W1:P_B1].reshape(HID, IN), p[P_B1:P_W2], p[P_W2:P_B2].reshape(HID, HID), p[P_B2:P_W3],
            p[P_W3:P_B3].reshape(OUT, HID), p[P_B3:NPARAM])


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    xb = bf16(x)
    h1 = bf16(np.maximum(xb @ bf16(W1).T + b1, 0.0))
    h2 = bf16(np.maximum(h1 @ bf16(W2).T + b2, 0.0))
    z = h2 @ bf16(W3).T + b3
    return xb, h1, h2, z


def loss_and_grads(p, x, y, bf16_rounding=True):
    _ROUND[0] = bf16_rounding
    try:
        return _loss_and_grads(p, x, y)
    finally:
        _ROUND[0] = True


def _loss_and_grads(p, x, y):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    y = np.asarray(y, np.float64)
    xb, h1, h2, z = forward(p, x)
    B = x.shape[0]
    loss = np.mean(np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))
    dz = (1.0 / (1.0 + np.exp(-z)) - y) / (B * OUT)
    dzb = bf16(dz)
    g = np.zeros(NPARAM)
    g[P_W3:P_B3] = (dzb.T @ h2).ravel()
    g[P_B3:NPARAM] = dz.sum(0)
    dh2 = (dzb @ bf16(W3)) * (h2 > 0)
    dh2b = bf16(dh2)
    g[P_W2:P_B2] = (dh2b.T @ h1).ravel()
    g[P_B2:P_W3] = dh2.sum(0)
    dh1 = (dh2b @ bf16(W2)) * (h1 > 0)
    dh1b = bf16(dh1)
    g[P_W1:P_B1] = (dh1b.T @ xb).ravel()
    g[P_B1:P_W2] = dh1.sum(0)
    return loss, g


def predict(p, x):
    return 1.0 / (1.0 + np.exp(-forward(p, x)[3]))
