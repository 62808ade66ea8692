"""CPU oracle of the learned narrow band -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
module, and only as the checker.  The learned band has no counterpart in the
reference (it is an addition of this project), so there is nothing of the
reference to pin it to: it restates libpms's own definitions in float64 numpy,
with the bf16 roundings of the GPU kernels mirrored, so that the GPU forward
pass, gradients, Adam step, features and candidate set can be checked
against an independent implementation.

Definitions (the same as postmps_gb300/csrc/k_learn.cu):
  * coarse density grid: vertex c on fine vertex 2c; particle p at coarse
    coordinate u = ((p - scmin) / cell) * 0.5 (float32, each operation
    rounded) splats w = prod(1 - f or f) onto the 8 vertices around it, as
    rint(w * 2^20) in integers; density = min(sum * 2^-20 * inv_expected, 64);
  * features of cube x: densities of coarse vertices k - 1 + d (even x) or
    k + 2 - d (odd x), k = x >> 1, d = 0..3 per axis, f = (dz*4 + dy)*4 + dx,
    rounded to bf16;
  * candidate: cube inside the grid whose coarse cell's 4^3 patch holds a
    vertex above 0 and one below 0.5 (vertices outside the grid are 0);
  * network: h = relu(x W1 + b1), z = h.w2 + b2 with bf16 W1, w2;
  * loss: mean of pw*y*softplus(-z) + (1-y)*softplus(z);
  * gradients from one bf16 product: dW1 = X^T dh, db1 = sum dh, dw2 = h^T dz with
    dh, h and dz rounded to bf16.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID = 64, 64
OFF_B1, OFF_W2, OFF_B2, N_PARAMS = 4096, 4160, 4224, 4225


# ---------------------------------------------------------------------------
# bf16
# ---------------------------------------------------------------------------
def bf16_bits(x) -> np.ndarray:
    """float32 -> bf16 bits, round to nearest even (NaN kept quiet)."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    nan = np.isnan(np.asarray(x, np.float32))
    r = np.where(nan, (b >> 16) | 0x40, r)
    return r.astype(np.uint16)


def bf16_value(bits) -> np.ndarray:
    return (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32)


def bf16_round(x) -> np.ndarray:
    return bf16_value(bf16_bits(x))


# ---------------------------------------------------------------------------
# coarse grid, features, candidates
# ---------------------------------------------------------------------------
def coarse_dims(scres) -> np.ndarray:
    """Coarse vertices per axis (x, y, z)."""
    return np.asarray(scres, np.int64) // 2 + 2


def inv_expected(sc_cell: float, spacing: float) -> np.float32:
    side = 2.0 * float(np.float32(sc_cell))
    e = (side / float(np.float32(spacing))) ** 3
    return np.float32(1.0 / e if e > 0 else 1.0)


def coarse_counts(pos_sorted: np.ndarray, scmin, sc_cell: float, scres) -> np.ndarray:
    """Fixed-point splat sums [z, y, x] of the coarse density grid."""
    p = np.asarray(pos_sorted, np.float32).reshape(-1, 3)
    scmin = np.asarray(scmin, np.float32)
    cell = np.float32(sc_cell)
    u = ((p - scmin) / cell) * np.float32(0.5)        # float32: subtract, divide, halve
    f0 = np.floor(u)
    cr = coarse_dims(scres)
    ok = np.all((f0 >= 0) & (f0 < (cr - 1).astype(np.float32)), axis=1)
    k = f0[ok].astype(np.int64)
    w1 = (u[ok] - f0[ok]).astype(np.float32)
    w0 = (np.float32(1.0) - w1).astype(np.float32)
    sums = np.zeros((cr[2], cr[1], cr[0]), np.uint64)
    for c in range(8):
        wx = w1[:, 0] if c & 1 else w0[:, 0]
        wy = w1[:, 1] if c & 2 else w0[:, 1]
        wz = w1[:, 2] if c & 4 else w0[:, 2]
        w = ((wx * wy).astype(np.float32) * wz).astype(np.float32)
        fix = np.rint((w * np.float32(1048576.0)).astype(np.float32)).astype(np.uint64)
        np.add.at(sums, (k[:, 2] + (c >> 2), k[:, 1] + ((c >> 1) & 1), k[:, 0] + (c & 1)), fix)
    return sums.astype(np.uint32)


def density(sums: np.ndarray, inv_exp) -> np.ndarray:
    d = (sums.astype(np.float32) * np.float32(1.0 / 1048576.0)).astype(np.float32) * np.float32(inv_exp)
    return np.minimum(d.astype(np.float32), np.float32(64.0))


def features(counts: np.ndarray, scres, inv_exp, cubes) -> np.ndarray:
    """float32 features (bf16-exact) of cubes given by origin vertex id, shape (n, 64)."""
    rx, ry = int(scres[0]), int(scres[1])
    cubes = np.asarray(cubes, np.int64)
    c = np.stack([cubes % rx, (cubes // rx) % ry, cubes // (rx * ry)], axis=1)
    k, s = c >> 1, c & 1
    dens = density(counts, inv_exp)
    cz, cy, cx = counts.shape
    out = np.zeros((len(cubes), 64), np.float32)
    for f in range(64):
        dx, dy, dz = f & 3, (f >> 2) & 3, f >> 4
        idx = []
        for a, dd in ((0, dx), (1, dy), (2, dz)):
            idx.append(np.where(s[:, a] == 1, k[:, a] + 2 - dd, k[:, a] - 1 + dd))
        ix, iy, iz = idx
        inside = (ix >= 0) & (iy >= 0) & (iz >= 0) & (ix < cx) & (iy < cy) & (iz < cz)
        v = np.zeros(len(cubes), np.float32)
        v[inside] = dens[iz[inside], iy[inside], ix[inside]]
        out[:, f] = v
    return bf16_round(out)


def candidates(counts: np.ndarray, scres, inv_exp) -> np.ndarray:
    """Ascending origin vertex ids of the candidate cubes."""
    dens = density(counts, inv_exp)
    cz, cy, cx = dens.shape
    pad = np.zeros((cz + 4, cy + 4, cx + 4), np.float32)    # vertices outside the grid read 0
    pad[1:-3, 1:-3, 1:-3] = dens
    rx, ry, rz = (int(v) for v in scres)
    nk = [(r - 2) // 2 + 1 for r in (rx, ry, rz)]            # coarse cells holding cubes
    anyp = np.zeros((nk[2], nk[1], nk[0]), bool)
    anylo = np.zeros_like(anyp)
    for dz in range(4):
        for dy in range(4):
            for dx in range(4):
                # vertex k - 1 + d sits at padded index k + d
                w = pad[dz:dz + nk[2], dy:dy + nk[1], dx:dx + nk[0]]
                anyp |= w > 0
                anylo |= w < 0.5
    mixed = anyp & anylo
    z, y, x = np.meshgrid(np.arange(rz - 1), np.arange(ry - 1), np.arange(rx - 1), indexing="ij")
    sel = mixed[z >> 1, y >> 1, x >> 1]
    ids = (z[sel].astype(np.int64) * ry + y[sel]) * rx + x[sel]
    return np.sort(ids).astype(np.uint32)


# ---------------------------------------------------------------------------
# network
# ---------------------------------------------------------------------------
def unpack(params: np.ndarray):
    p = np.asarray(params, np.float64)
    return p[:OFF_B1].reshape(N_IN, N_HID), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2], p[OFF_B2]


def forward(params: np.ndarray, x: np.ndarray):
    """logits (float64) with bf16 W1, w2 (fp32 biases); x are bf16-exact floats."""
    w1, b1, w2, b2 = unpack(params)
    w1q = bf16_round(w1.astype(np.float32)).astype(np.float64)
    w2q = bf16_round(w2.astype(np.float32)).astype(np.float64)
    b1f = b1.astype(np.float32).astype(np.float64)
    pre = np.asarray(x, np.float64) @ w1q + b1f
    h = np.maximum(pre, 0.0)
    z = h @ w2q + float(np.float32(b2))
    return z, pre, h, w2q


def softplus(z):
    return np.maximum(z, 0.0) + np.log1p(np.exp(-np.abs(z)))


def loss_and_grad(params: np.ndarray, x: np.ndarray, y: np.ndarray, pos_weight: float):
    """Mean weighted cross-entropy and its gradient in the parameter layout."""
    z, pre, h, w2q = forward(params, x)
    y = np.asarray(y, np.float64)
    B = len(y)
    wy = pos_weight * y
    loss = float(np.sum(wy * softplus(-z) + (1 - y) * softplus(z)) / B)
    p = 1.0 / (1.0 + np.exp(-z))
    dz = (p * (wy + 1 - y) - wy) / B
    dh = np.where(pre > 0, dz[:, None] * w2q[None, :], 0.0)
    dhq = bf16_round(dh.astype(np.float32)).astype(np.float64)
    g = np.zeros(N_PARAMS)
    g[:OFF_B1] = (np.asarray(x, np.float64).T @ dhq).reshape(-1)
    # the kernel forms db1 and dw2 on the tensor cores too: dh, h and dz rounded to bf16
    g[OFF_B1:OFF_W2] = dhq.sum(axis=0)
    hq = bf16_round(h.astype(np.float32)).astype(np.float64)
    dzq = bf16_round(dz.astype(np.float32)).astype(np.float64)
    g[OFF_W2:OFF_B2] = (dzq[:, None] * hq).sum(axis=0)
    g[OFF_B2] = dz.sum()
    return loss, g


def adam(params, grad, m, v, step: int, lr: float, beta1=0.9, beta2=0.999, eps=1e-8):
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v
