"""FP64 CPU reference of the learned start's MLP (test infrastructure only).

8 -> 64 -> 64 -> 1 with SiLU; parameters in the flat layout of
pbf_gb300.h (W1[k][n] 8x64, b1, W2[k][n] 64x64, b2, w3, b3).  `emulate=True`
rounds to bfloat16 where the GPU kernels do (inputs, weights of layers 1-2,
h1, h2, dZ2 and dZ1 before the tensor-core products), so the GPU's FP32
accumulation is the only remaining difference.
"""
import numpy as np

OFF_W1, OFF_B1, OFF_W2, OFF_B2, OFF_W3, OFF_B3 = 0, 512, 576, 4672, 4736, 4800


def bf16(x):
    """Round float64/float32 values to the nearest bfloat16 (ties to even), as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(8, 64), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(64, 64), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3], p[OFF_B3])


def sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def forward(p, mean, inv_std, lam_scale, feat, emulate=True):
    q = (lambda x: bf16(x)) if emulate else (lambda x: np.asarray(x, np.float64))
    W1, b1, W2, b2, w3, b3 = unpack(p)
    x = (np.asarray(feat, np.float64) - np.asarray(mean, np.float32)) * np.asarray(inv_std, np.float32)
    if emulate:
        x = x.astype(np.float32)
    xq = q(x)
    z1 = xq @ q(W1) + b1
    h1 = q(z1 * sig(z1))
    z2 = h1 @ q(W2) + b2
    h2 = q(z2 * sig(z2))
    y = h2 @ w3 + b3
    return dict(x=xq, z1=z1, h1=h1, z2=z2, h2=h2, y=y, lam=y * lam_scale)


def gradient(p, mean, inv_std, lam_scale, feat, target, emulate=True):
    q = (lambda x: bf16(x)) if emulate else (lambda x: np.asarray(x, np.float64))
    W1, b1, W2, b2, w3, b3 = unpack(p)
    f = forward(p, mean, inv_std, lam_scale, feat, emulate)
    n = f["y"].shape[0]
    t = np.asarray(target, np.float64) / lam_scale
    e = f["y"] - t
    dy = 2.0 * e / n
    ds = lambda z: sig(z) * (1.0 + z * (1.0 - sig(z)))
    dz2 = np.outer(dy, w3) * ds(f["z2"])
    dh1 = q(dz2) @ q(W2).T
    dz1 = dh1 * ds(f["z1"])
    g = np.zeros(len(p))
    g[OFF_W1:OFF_B1] = (f["x"].T @ q(dz1)).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W2:OFF_B2] = (f["h1"].T @ q(dz2)).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    g[OFF_W3:OFF_B3] = f["h2"].T @ dy
    g[OFF_B3] = dy.sum()
    return g, float(np.mean(e * e))
