"""CPU oracle of the warm-start network (csrc/fl_mlp.cu): forward pass, loss and gradients in
FP64 numpy with the same BF16 rounding of every GEMM operand (round to nearest even), so the GPU
kernels' FP32 accumulation is the only difference. TEST INFRASTRUCTURE ONLY (tests/)."""
import numpy as np
from scipy.special import erf

SIZES = [(3, 256), (256,), (256, 256), (256,), (256, 64), (64,)]


def _bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(x, np.float32)  # values already in float32 range
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    out, off = [], 0
    for s in SIZES:
        k = int(np.prod(s))
        out.append(np.asarray(params[off:off + k], np.float64).reshape(s))
        off += k
    return out


def gelu(z):
    return 0.5 * z * (1 + erf(z / np.sqrt(2)))


def gelu_d(z):
    return 0.5 * (1 + erf(z / np.sqrt(2))) + z * np.exp(-0.5 * z * z) / np.sqrt(2 * np.pi)


def forward(params, x, rounding=True):
    """rounding=False: the exact FP64 network (for finite-difference checks of the oracle)."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    bf16 = _bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W1b, W2b, W3b = bf16(W1), bf16(W2), bf16(W3)
    xb = bf16(x)
    z1 = xb @ W1b + b1
    h1 = bf16(gelu(z1))
    z2 = h1 @ W2b + b2
    h2 = bf16(gelu(z2))
    y = h2 @ W3b + b3
    return dict(xb=xb, z1=z1, h1=h1, z2=z2, h2=h2, y=y, W1b=W1b, W2b=W2b, W3b=W3b)


def gradients(params, x, t, rounding=True):
    f = forward(params, x, rounding)
    bf16 = _bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    B = x.shape[0]
    scale = 1.0 / (B * 64)
    d = f["y"] - t
    loss = 0.5 * scale * np.sum(d * d)
    dy = bf16(d * scale)
    dW3 = f["h2"].T @ dy
    db3 = dy.sum(0)
    dz2 = bf16((dy @ f["W3b"].T) * gelu_d(f["z2"]))
    dW2 = f["h1"].T @ dz2
    db2 = dz2.sum(0)
    dz1 = bf16((dz2 @ f["W2b"].T) * gelu_d(f["z1"]))
    dW1 = f["xb"].T @ dz1
    db1 = dz1.sum(0)
    g = np.concatenate([a.ravel() for a in (dW1, db1, dW2, db2, dW3, db3)])
    return g, loss, f["y"]
