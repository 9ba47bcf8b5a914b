"""Random and adversarial 8x8 blocks for the exact-transform tests.

Every transform the library evaluates in fp32 (MJPEG inverse DCT, DV 8-8 and
2-4-8, the encoder's forward DCT + quantisation) must round like the
reference's binary64 operation order. The blocks here aim at the cases where
the fp32 value could fall on the other side of a rounding boundary: dense
blocks with large coefficients (the largest error bound), quantiser-255
products, i32-range DC values, every DC value of a range (exact ties such as
c0 = 4 + 8k), clamping at 0 and 255, and blocks built so that one sample (or
one quotient) lies within 2^-20 of a half-integer.

The near-tie construction is linear algebra on the transform's weights: a
sample is w . c over the coefficients (or samples, for the forward DCT), so
with three free coefficients a meet-in-the-middle search over their values
puts w . c within about 1e-8 of a chosen half-integer. Distances are measured
in float64 with numpy's order of operations (within ~1e-12 of the reference's
binary64 value), which is precise enough to certify "within 2^-20".
"""

from __future__ import annotations

import ctypes

import numpy as np

import oracle

NEAR = 2.0 ** -20


def idct_matrix() -> np.ndarray:
    """The reference's IDCT_MATRIX (transform.rs:2-84) as the oracle holds it, [x][u]."""
    return np.array((ctypes.c_double * 64).in_dll(oracle.lib(), "ORC_IDCT_MATRIX")[:], np.float64).reshape(8, 8)


def jpeg_weights() -> np.ndarray:
    """W[y*8+x, v*8+u] = M[y][v] M[x][u]: sample - 128 = W @ c."""
    M = idct_matrix()
    return np.einsum("yv,xu->yxvu", M, M).reshape(64, 64)


def dv_weights(mode248: bool) -> np.ndarray:
    """Linear weights of DV inverse_88 / inverse_248 (decoder.rs:520-602): value = W @ c
    (before rounding), from the oracle's cos table."""
    cos16 = np.array([oracle.dv_cos(k) for k in range(128)])
    k = np.where(np.arange(8) == 0, 0.7071067811865476, 1.0)
    W = np.zeros((64, 64))
    if not mode248:
        for y in range(8):
            for x in range(8):
                for v in range(8):
                    for u in range(8):
                        W[y * 8 + x, v * 8 + u] = k[u] * k[v] * cos16[(2 * x + 1) * u] * cos16[(2 * y + 1) * v] / 4.0
        return W
    # butterfly b[pair*16+u] = c[pair*16+u] + c[pair*16+8+u], b[pair*16+8+u] = difference;
    # h[row][x] = sum_u k_u b[row][u] cos16[(2x+1)u] / 2; out[(2y+f)][x] = sum_v k_v h[2v+f][x] cos8[(2y+1)v] / 2
    B = np.zeros((64, 64))
    for pair in range(4):
        for u in range(8):
            B[pair * 16 + u, pair * 16 + u] = 1
            B[pair * 16 + u, pair * 16 + 8 + u] = 1
            B[pair * 16 + 8 + u, pair * 16 + u] = 1
            B[pair * 16 + 8 + u, pair * 16 + 8 + u] = -1
    Hm = np.zeros((64, 64))
    for row in range(8):
        for x in range(8):
            for u in range(8):
                Hm[row * 8 + x, row * 8 + u] = k[u] * cos16[(2 * x + 1) * u] / 2.0
    V = np.zeros((64, 64))
    for f in range(2):
        for y in range(4):
            for x in range(8):
                for v in range(4):
                    V[(2 * y + f) * 8 + x, (2 * v + f) * 8 + x] = k[v] * cos16[2 * (2 * y + 1) * v] / 2.0
    return V @ Hm @ B


def _half_distance(value):
    f = value - np.floor(value)
    return np.abs(f - 0.5)


def near_ties(rng, W, n_groups, per_group, base_range, free_range, offset=0.0, targets=None, lo=None, hi=None):
    """Blocks c (int64, (n_groups*per_group, 64)) whose sample `t` (one target per
    group) satisfies W[t] . c + offset within ~1e-8 of a half-integer.

    Each group fixes a target sample and three free positions; the other
    coefficients are uniform in +-base_range (dense), the free ones searched in
    +-free_range. targets (optional) gives the half-integers to aim at (for the
    clamp edges); else any half-integer near the base value. lo/hi clamp the
    result range of the free coefficients."""
    out, dist = [], []
    R = free_range
    vals = np.arange(-R, R + 1, dtype=np.float64)
    for g in range(n_groups):
        t = int(rng.integers(0, 64))
        pos = rng.choice(64, 3, replace=False)
        w = W[t, pos]
        c = rng.integers(-base_range, base_range + 1, (per_group, 64)).astype(np.int64)
        c[:, pos] = 0
        base = c.astype(np.float64) @ W[t] + offset
        A = (vals[:, None] * w[0] + vals[None, :] * w[1]).ravel()  # pairs (c1, c2)
        if targets is None:
            goal = np.floor(base) + 0.5  # the half-integer nearest below, or just above
        else:
            goal = np.full(per_group, float(targets[g % len(targets)]))
        best = np.full(per_group, np.inf)
        pick = np.zeros((per_group, 3), np.int64)
        order = np.argsort(A)
        As = A[order]
        for k3 in vals:
            need = goal - base - k3 * w[2]  # want A ~ need
            j = np.clip(np.searchsorted(As, need), 1, len(As) - 1)
            for jj in (j - 1, j):
                d = np.abs(As[jj] - need)
                better = d < best
                if better.any():
                    best = np.where(better, d, best)
                    idx = order[jj]
                    pick[better, 0] = vals[idx[better] // (2 * R + 1)].astype(np.int64)
                    pick[better, 1] = vals[idx[better] % (2 * R + 1)].astype(np.int64)
                    pick[better, 2] = int(k3)
        c[:, pos] = pick
        if lo is not None:
            c = np.clip(c, lo, hi)
        out.append(c)
        dist.append(_half_distance(c.astype(np.float64) @ W[t] + offset))
    return np.concatenate(out), np.concatenate(dist)


def jpeg_idct_blocks(seed: int, dense: int = 200_000):
    """(coefficients int32 (n, 64), counts by kind, near-tie count) for the inverse DCT."""
    rng = np.random.default_rng(seed)
    parts, kinds = [], {}

    def add(name, c):
        parts.append(np.asarray(c, np.int64))
        kinds[name] = len(c)

    for R in (64, 256, 1024):  # dense, samples mostly in range
        add(f"dense_{R}", rng.integers(-R, R + 1, (dense // 4, 64)))
    add("dense_2^20", rng.integers(-(1 << 20), (1 << 20) + 1, (dense // 8, 64)))
    # quantiser 255 products: levels +-1023 (AC), quantisers 1..255, DC up to +-2^31
    lv = rng.integers(-1023, 1024, (dense // 4, 64)) * (rng.random((dense // 4, 64)) < 0.6)
    qt = rng.integers(1, 256, (dense // 4, 64))
    qt[: dense // 8] = 255
    c = lv * qt
    c[:, 0] = rng.integers(-(1 << 31), (1 << 31), dense // 4)
    add("quant255_i32dc", c)
    # i32-range DC alone, and with small AC
    c = np.zeros((20_000, 64), np.int64)
    c[:, 0] = rng.integers(-(1 << 31), (1 << 31), 20_000)
    c[10_000:, 1:] = rng.integers(-30, 31, (10_000, 63))
    add("i32_dc", c)
    # every DC value in -2^14..2^14 (DC-only blocks: c0 = 4 + 8k lands on x.5 ties)
    c = np.zeros((1 << 15 | 1, 64), np.int64)
    c[:, 0] = np.arange(-(1 << 14), (1 << 14) + 1)
    add("dc_sweep", c)
    # sparse
    c = rng.integers(-2000, 2001, (dense // 4, 64)) * (rng.random((dense // 4, 64)) < 0.08)
    add("sparse", c)
    # near ties: dense bases, three free coefficients; also at the clamp edges (-0.5 and 255.5)
    W = jpeg_weights()
    a, da = near_ties(rng, W, 32, 1024, 120, 300, offset=128.0)
    add("near_tie_dense", a)
    b, db = near_ties(rng, W, 16, 512, 1000, 600, offset=128.0)
    add("near_tie_large", b)
    e, de = near_ties(rng, W, 16, 256, 60, 400, offset=128.0, targets=[-0.5, 255.5])
    add("near_tie_clamp", e)
    near = int((da < NEAR).sum() + (db < NEAR).sum() + (de < NEAR).sum())
    allc = np.concatenate(parts)
    assert allc.min() >= -(1 << 31) and allc.max() < (1 << 31)
    return allc.astype(np.int32), kinds, near


def dv_idct_blocks(seed: int, n: int = 100_000):
    """(coefficients int32 (n, 64) within int16, modes uint8 (n,), counts, near-tie count)."""
    rng = np.random.default_rng(seed)
    parts, modes, kinds = [], [], {}

    def add(name, c, mode):
        parts.append(np.asarray(c, np.int64))
        modes.append(np.full(len(c), mode, np.uint8))
        kinds[name] = len(c)

    near = 0
    for mode in (0, 1):
        tag = "248" if mode else "88"
        add(f"dense_{tag}", rng.integers(-512, 513, (n // 4, 64)), mode)
        add(f"dense_int16_{tag}", rng.integers(-32768, 32768, (n // 8, 64)), mode)
        c = rng.integers(-300, 301, (n // 4, 64)) * (rng.random((n // 4, 64)) < 0.2)
        c[:, 0] = rng.integers(0, 2045, n // 4)  # dc * 4 + 1024 for a 9-bit signed dc
        add(f"sparse_dc_{tag}", c, mode)
        c = np.zeros((8189, 64), np.int64)
        c[:, 0] = np.arange(-4094, 4095)
        add(f"dc_sweep_{tag}", c, mode)
        W = dv_weights(bool(mode))
        a, da = near_ties(rng, W, 32, 512, 150, 400, lo=-32768, hi=32767)
        add(f"near_tie_{tag}", a, mode)
        e, de = near_ties(rng, W, 16, 256, 40, 300, targets=[-0.5, 255.5], lo=-32768, hi=32767)
        add(f"near_tie_clamp_{tag}", e, mode)
        near += int((da < NEAR).sum() + (de < NEAR).sum())
    allc = np.concatenate(parts)
    assert np.abs(allc).max() <= 32768
    return allc.astype(np.int32), np.concatenate(modes), kinds, near


def fdct_blocks(seed: int, n: int = 200_000):
    """(samples uint8 (n, 64), quantisers uint8 (n, 64), counts, near-tie count)."""
    rng = np.random.default_rng(seed)
    S, Q, kinds = [], [], {}

    def add(name, s, q):
        S.append(np.asarray(s, np.uint8))
        Q.append(np.asarray(q, np.uint8))
        kinds[name] = len(s)

    add("noise_q1", rng.integers(0, 256, (n // 4, 64)), np.ones((n // 4, 64)))
    add("noise_qrand", rng.integers(0, 256, (n // 4, 64)), rng.integers(1, 256, (n // 4, 64)))
    checker = ((np.arange(64) // 8 + np.arange(64) % 8) % 2) * 255
    ext = np.stack([np.zeros(64), np.full(64, 255), checker, 255 - checker])
    add("extremes", np.repeat(ext, 64, axis=0), np.tile(np.arange(1, 65)[:, None], (4, 64)))
    # smooth content at q 1 and at the reference's quality-scaled tables
    yy, xx = np.mgrid[0:8, 0:8]
    g = (rng.uniform(0, 30, (n // 4, 1)) * xx.ravel() / 8 + rng.uniform(0, 30, (n // 4, 1)) * yy.ravel() / 8
         + rng.uniform(40, 180, (n // 4, 1)) + rng.normal(0, 4, (n // 4, 64)))
    add("smooth", np.clip(np.rint(g), 0, 255), rng.integers(1, 100, (n // 4, 64)))
    # near ties of one quotient: value / q within ~1e-8 of a half-integer, over three free samples
    M = idct_matrix()
    near = 0
    for g_i in range(24):
        per = 1024
        v, u = int(rng.integers(0, 8)), int(rng.integers(0, 8))
        q = int(rng.choice([1, 1, 2, 3, 7, 16, 99, 255]))
        w = np.einsum("y,x->yx", M[:, v], M[:, u]).ravel() / q  # weight of (sample - 128)
        pos = rng.choice(64, 3, replace=False)
        s = rng.integers(0, 256, (per, 64)).astype(np.float64)
        s[:, pos] = 128
        base = (s - 128.0) @ w
        vals = np.arange(0, 256, dtype=np.float64) - 128.0
        A = (vals[:, None] * w[pos[0]] + vals[None, :] * w[pos[1]]).ravel()
        order = np.argsort(A)
        As = A[order]
        goal = np.floor(base) + 0.5  # the nearest half-integer (the free samples reach +-128 |w|)
        goal = np.where(base - goal > 0.5, goal + 1.0, goal)
        best = np.full(per, np.inf)
        pick = np.zeros((per, 3))
        for k3 in vals:
            need = goal - base - k3 * w[pos[2]]
            j = np.clip(np.searchsorted(As, need), 1, len(As) - 1)
            for jj in (j - 1, j):
                d = np.abs(As[jj] - need)
                better = d < best
                best = np.where(better, d, best)
                idx = order[jj]
                pick[better, 0] = vals[idx[better] // 256]
                pick[better, 1] = vals[idx[better] % 256]
                pick[better, 2] = k3
        s[:, pos] = pick + 128.0
        qt = np.ones((per, 64))
        qt[:, v * 8 + u] = q
        near += int((_half_distance((s - 128.0) @ w) < NEAR).sum())
        add(f"near_tie_{g_i}", s, qt)
    return np.concatenate(S), np.concatenate(Q), _merge(kinds), near


def _merge(kinds):
    out = {}
    for k, v in kinds.items():
        key = "near_tie" if k.startswith("near_tie_") else k
        out[key] = out.get(key, 0) + v
    return out
