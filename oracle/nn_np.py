"""NumPy reference of the learned warm start's kernels (test infrastructure:
only tests import it).  NHWC float32 arithmetic on bfloat16-rounded operands,
the same conventions as include/glgpu_nn.h; no counterpart in the reference."""
import numpy as np


def bf16_round(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(f.shape)


def bf16_bits(x):
    """bfloat16 bit patterns (uint16) of float32 values rounded to bfloat16."""
    return (bf16_round(x).view(np.uint32) >> 16).astype(np.uint16)


def from_bf16_bits(u):
    return (np.asarray(u, dtype=np.uint32) << 16).view(np.float32)


def _pad(x):
    return np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))


def conv3x3(x, w, b, relu):
    """y[n,i,j,co] = b[co] + sum_{ky,kx,ci} x[n,i+ky-1,j+kx-1,ci] w[co,ky,kx,ci]."""
    n, h, wd, _ = x.shape
    xp = _pad(x.astype(np.float64))
    y = np.zeros((n, h, wd, w.shape[0]))
    for ky in range(3):
        for kx in range(3):
            y += np.einsum("nhwc,oc->nhwo", xp[:, ky:ky + h, kx:kx + wd, :], w[:, ky, kx, :].astype(np.float64))
    y += b[None, None, None, :]
    return np.maximum(y, 0.0) if relu else y


def conv3x3_bwd(x, w, y, dy, relu):
    """(dx, dw, db) of conv3x3 given the output y (for the ReLU derivative)."""
    n, h, wd, _ = x.shape
    d = dy.astype(np.float64) * ((y > 0) if relu else 1.0)
    xp = _pad(x.astype(np.float64))
    dxp = np.zeros_like(xp)
    dw = np.zeros(w.shape)
    for ky in range(3):
        for kx in range(3):
            dxp[:, ky:ky + h, kx:kx + wd, :] += np.einsum("nhwo,oc->nhwc", d, w[:, ky, kx, :].astype(np.float64))
            dw[:, ky, kx, :] = np.einsum("nhwo,nhwc->oc", d, xp[:, ky:ky + h, kx:kx + wd, :])
    return dxp[:, 1:-1, 1:-1, :], dw, d.sum(axis=(0, 1, 2))


def pool2(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def up2(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def adam(w, g, m, v, lr, b1, b2, eps, wd, step):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return w - lr * (mh / (np.sqrt(vh) + eps) + wd * w), m, v
