"""CPU restatement of the radiance cache (hash-grid encoding + MLP), forward
and backward, in numpy.

TEST INFRASTRUCTURE ONLY: the checker of the GPU cache kernels
(hala-pathtracer_gb300/csrc/pt_cache.cu). There is no reference
counterpart: the reference integrator has no radiance cache.

The restatement rounds to BF16 at the points where the tensor-core kernels
hold BF16 operands (the encoded input, every hidden activation, every
output gradient before it is multiplied) and accumulates in float64, so it
differs from the GPU only by accumulation order and the rare BF16 rounding
flip that order causes. With `exact=True` nothing is rounded: that variant
is the one the finite-difference check uses.
"""
import math

import numpy as np

LEVELS = 16
IN = 64
LAYERS = 6
OUT = 16
P1, P2 = 2654435761, 805459861


def layer_shape(l):
    return 64, (OUT if l == LAYERS - 1 else 64)


def layer_off(l):
    return l * 64 * 64


def n_params():
    return 5 * 64 * 64 + 64 * OUT


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even)."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def resolutions(min_res=16, max_res=2048):
    b = math.exp((math.log(max_res) - math.log(min_res)) / (LEVELS - 1))
    return [max(2, int(math.floor(min_res * math.pow(b, l)))) for l in range(LEVELS)]


def weights(mlp):
    """Flat master vector -> list of (64, N) matrices [in][out] (float32,
    or float64 when the vector is float64)."""
    mlp = np.asarray(mlp)
    dt = np.float64 if mlp.dtype == np.float64 else np.float32
    out = []
    for l in range(LAYERS):
        k, n = layer_shape(l)
        out.append(np.asarray(mlp[layer_off(l):layer_off(l) + k * n], dt).reshape(k, n))
    return out


def corners(pos01, N, log2_table):
    """(rows, 8) global-in-level indices and weights of one level."""
    T = 1 << log2_table
    x = (pos01 * np.float32(N)).astype(np.float32)
    x0 = np.minimum(x.astype(np.uint64), N - 1)
    f = (x - x0.astype(np.float32)).astype(np.float32)
    side = N + 1
    dense = side ** 3 <= T
    idx = np.empty((len(pos01), 8), np.uint64)
    w = np.empty((len(pos01), 8), np.float32)
    for c in range(8):
        cx = x0[:, 0] + (c & 1)
        cy = x0[:, 1] + ((c >> 1) & 1)
        cz = x0[:, 2] + (c >> 2)
        if dense:
            idx[:, c] = cx + side * (cy + side * cz)
        else:
            idx[:, c] = (cx ^ ((cy * P1) & 0xFFFFFFFF) ^ ((cz * P2) & 0xFFFFFFFF)) & (T - 1)
        wx = f[:, 0] if c & 1 else np.float32(1) - f[:, 0]
        wy = f[:, 1] if c & 2 else np.float32(1) - f[:, 1]
        wz = f[:, 2] if c & 4 else np.float32(1) - f[:, 2]
        w[:, c] = (wx * wy).astype(np.float32) * wz
    return idx, w


def unit_positions(rec, lo, hi):
    lo = np.asarray(lo, np.float32)
    inv = (np.float32(1) / (np.asarray(hi, np.float32) - lo)).astype(np.float32)
    return np.clip(((rec[:, 0:3] - lo) * inv).astype(np.float32), 0, 1).astype(np.float32)


def encode(rec, grid, lo, hi, res, log2_table, exact=False):
    """(rows, 64) MLP input before rounding. The table is read as fp16 like
    on the GPU, unless `exact`."""
    rec = np.asarray(rec, np.float32)
    T = 1 << log2_table
    g = np.asarray(grid, np.float64) if exact else np.asarray(grid, np.float32).astype(np.float16).astype(np.float64)
    g = g.reshape(LEVELS, T, 2)
    p = unit_positions(rec, lo, hi)
    x = np.zeros((len(rec), IN), np.float64)
    for l in range(LEVELS):
        idx, w = corners(p, res[l], log2_table)
        feats = (w[:, :, None].astype(np.float64) * g[l][idx.astype(np.int64)]).sum(axis=1)
        x[:, 2 * l:2 * l + 2] = feats
    x[:, 32:35] = rec[:, 3:6] * 0.5 + 0.5
    x[:, 35:38] = rec[:, 6:9] * 0.5 + 0.5
    x[:, 38:41] = rec[:, 9:12]
    x[:, 41:44] = rec[:, 12:15]
    x[:, 44] = 1.0
    return x


def forward(x, mlp, exact=False):
    """Returns (prediction (rows, 16), layer inputs X_0..X_5)."""
    rnd = (lambda v: v) if exact else (lambda v: bf16(v).astype(np.float64))
    W = [w.astype(np.float64) if exact else bf16(w).astype(np.float64) for w in weights(mlp)]
    xs = [rnd(x)]
    for l in range(LAYERS - 1):
        xs.append(rnd(np.maximum(xs[-1] @ W[l], 0.0)))
    return xs[-1] @ W[LAYERS - 1], xs


def loss_and_grads(rec, tgt, mlp, grid, lo, hi, res, log2_table, exact=False):
    """Relative L2 loss (sum over rgb, mean over rows), the MLP gradient
    (flat, master layout) and the hash-table gradient (flat)."""
    rnd = (lambda v: v) if exact else (lambda v: bf16(v).astype(np.float64))
    n = len(rec)
    x = encode(rec, grid, lo, hi, res, log2_table, exact)
    pred, xs = forward(x, mlp, exact)
    W = [w.astype(np.float64) if exact else bf16(w).astype(np.float64) for w in weights(mlp)]
    p = pred[:, :3]
    y = np.asarray(tgt, np.float64)[:, :3]
    den = p * p + 0.01
    loss = float(((p - y) ** 2 / den).sum() / n)
    dz = np.zeros((n, OUT))
    dz[:, :3] = 2.0 * (p - y) / den / n
    dz = rnd(dz)
    gmlp = np.zeros(n_params())
    for l in range(LAYERS - 1, -1, -1):
        k, m = layer_shape(l)
        gmlp[layer_off(l):layer_off(l) + k * m] = (xs[l].T @ dz).reshape(-1)
        dx = dz @ W[l].T
        if l > 0:
            dz = rnd(dx * (xs[l] > 0))
    T = 1 << log2_table
    ggrid = np.zeros((LEVELS, T, 2))
    pos = unit_positions(np.asarray(rec, np.float32), lo, hi)
    for l in range(LEVELS):
        idx, w = corners(pos, res[l], log2_table)
        for c in range(8):
            np.add.at(ggrid[l], idx[:, c].astype(np.int64), w[:, c:c + 1].astype(np.float64) * dx[:, 2 * l:2 * l + 2])
    return loss, gmlp, ggrid.reshape(-1), pred[:, :3]
