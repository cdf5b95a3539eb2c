"""Synthetic tile-displacement fields with planted outliers for the validation tests:
a smooth field, outliers of 4-9 px, secondary peaks that sometimes point back to the
truth, and sometimes fewer peaks than requested."""
import numpy as np


def smooth_case(rng, ni, nj, k, outliers, step=8):
    tops = np.arange(ni, dtype=np.int32) * step + 3
    lefts = np.arange(nj, dtype=np.int32) * step + 5
    yy, xx = np.meshgrid(np.arange(ni), np.arange(nj), indexing="ij")
    u = (0.8 * np.sin(yy / 3.0) + 0.05 * xx).astype(np.float32)
    v = (0.6 * np.cos(xx / 4.0) - 0.03 * yy).astype(np.float32)
    pu = np.zeros((ni, nj, k), np.float32)
    pv = np.zeros((ni, nj, k), np.float32)
    # the main-peak increment is part of the accumulated displacement
    pu[..., 0] = rng.uniform(-0.5, 0.5, (ni, nj)).astype(np.float32)
    pv[..., 0] = rng.uniform(-0.5, 0.5, (ni, nj)).astype(np.float32)
    for p in range(1, k):
        pu[..., p] = rng.uniform(-6, 6, (ni, nj)).astype(np.float32)
        pv[..., p] = rng.uniform(-6, 6, (ni, nj)).astype(np.float32)
    npk = np.full((ni, nj), k, np.int32)
    truth_u, truth_v = u.copy(), v.copy()
    flat = rng.choice(ni * nj, size=outliers, replace=False)
    for f in flat:
        i, j = divmod(int(f), nj)
        bad_u, bad_v = rng.uniform(4, 9) * rng.choice([-1, 1]), rng.uniform(4, 9) * rng.choice([-1, 1])
        u[i, j] += bad_u
        v[i, j] += bad_v
        if k > 1 and rng.random() < 0.5:
            # a secondary peak that points back to the truth
            p = int(rng.integers(1, k))
            pu[i, j, p] = pu[i, j, 0] - bad_u
            pv[i, j, p] = pv[i, j, 0] - bad_v
        if rng.random() < 0.2:
            npk[i, j] = int(rng.integers(1, k + 1))
    return tops, lefts, u, v, pu, pv, npk, truth_u, truth_v


def clustered_case(rng, ni, nj, k, frac, block):
    """smooth_case plus a solid block of outliers (a long chain of adjacent invalid tiles)."""
    tops, lefts, u, v, pu, pv, npk, tu, tv = smooth_case(rng, ni, nj, k, int(frac * ni * nj))
    i0, j0 = ni // 3, nj // 2
    u[i0:i0 + block, j0:j0 + block] += rng.uniform(-9, 9, (min(block, ni - i0), min(block, nj - j0))).astype(np.float32)
    v[i0:i0 + block, j0:j0 + block] += rng.uniform(-9, 9, (min(block, ni - i0), min(block, nj - j0))).astype(np.float32)
    return tops, lefts, u, v, pu, pv, npk, tu, tv
