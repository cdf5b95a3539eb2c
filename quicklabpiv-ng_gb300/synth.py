"""Seeded synthetic PIV image pairs (the reference names no public dataset).

Particles are Gaussian blobs I0 * exp(-8 r^2 / d^2) at uniform random positions
(count = ppp * H * W), with diameter d ~ N(d0, sd_d) and peak I0 ~ N(200, 40) in 8-bit
units.  Frame B re-renders every particle displaced by the flow evaluated at the
particle (no image warping), so the truth field is exact.  Additive Gaussian noise
(sigma in 8-bit units), clip, round.  12-bit data in uint16 scales intensities and
noise by 16.  Flows: Rankine vortex (solid-body core of radius rc, 1/r outside) about
the image centre, plus an optional uniform shear u_col = gamma * (row - centre).
Random numbers: numpy Philox, one stream per (seed, pair id).
"""
from dataclasses import dataclass

import numpy as np


@dataclass
class Flow:
    vmax: float = 4.0          # peak vortex displacement (px)
    rc: float = 64.0           # vortex core radius (px)
    shear: float = 0.0         # d(u_col)/d(row)
    centre: tuple = None       # (row, col); default image centre

    def displacement(self, rows, cols, shape):
        """(d_row, d_col) at the given positions."""
        h, w = shape
        cy, cx = self.centre if self.centre is not None else ((h - 1) / 2.0, (w - 1) / 2.0)
        dy = rows - cy
        dx = cols - cx
        r = np.sqrt(dy * dy + dx * dx)
        with np.errstate(divide="ignore", invalid="ignore"):
            ut = np.where(r <= self.rc, self.vmax * r / self.rc, self.vmax * self.rc / np.maximum(r, 1e-12))
            s = np.where(r > 0, ut / np.maximum(r, 1e-12), 0.0)
        d_row = s * dx            # counter-clockwise rotation in (row, col)
        d_col = -s * dy + self.shear * dy
        return d_row, d_col


def _render(shape, rows, cols, diam, peak):
    h, w = shape
    img = np.zeros(shape, np.float64)
    rad = int(np.ceil(np.max(diam) * 1.2)) + 1
    offs = np.arange(-rad, rad + 1)
    r0 = np.floor(rows).astype(np.int64)
    c0 = np.floor(cols).astype(np.int64)
    inv = 8.0 / (diam * diam)
    for oy in offs:
        yy = r0 + oy
        vy = (yy >= 0) & (yy < h)
        dy2 = (yy - rows) ** 2
        for ox in offs:
            xx = c0 + ox
            ok = vy & (xx >= 0) & (xx < w)
            val = peak * np.exp(-(dy2 + (xx - cols) ** 2) * inv)
            np.add.at(img, (yy[ok], xx[ok]), val[ok])
    return img


def particle_pair(shape, flow, ppp=0.02, diam=3.0, diam_sd=0.5, noise=3.0, bits=8, seed=0, pair_id=0):
    """Returns (frame_a, frame_b) as uint8 (bits=8) or uint16 (bits in 10..16)."""
    rng = np.random.Generator(np.random.Philox(key=[int(seed) & 0xFFFFFFFFFFFFFFFF, int(pair_id)]))
    h, w = shape
    count = int(round(ppp * h * w))
    margin = 8.0
    rows = rng.uniform(-margin, h + margin, count)
    cols = rng.uniform(-margin, w + margin, count)
    d = np.clip(rng.normal(diam, diam_sd, count), 1.0, None) if diam_sd > 0 else np.full(count, float(diam))
    peak = np.clip(rng.normal(200.0, 40.0, count), 20.0, None)
    scale = 1.0 if bits == 8 else float(1 << (bits - 8))
    d_row, d_col = flow.displacement(rows, cols, shape)
    fa = _render(shape, rows, cols, d, peak * scale)
    fb = _render(shape, rows + d_row, cols + d_col, d, peak * scale)
    top = (1 << bits) - 1
    out = []
    for f in (fa, fb):
        f = f + rng.normal(0.0, noise * scale, f.shape)
        f = np.clip(np.rint(f), 0, top)
        out.append(f.astype(np.uint8 if bits == 8 else np.uint16))
    return out[0], out[1]


def config1_pair(seed=1, pair_id=0):
    """512x512 u8, 0.02 ppp, d = 3 +- 0.5, Rankine r_c = 64 max 4 px, noise 3."""
    return particle_pair((512, 512), Flow(vmax=4.0, rc=64.0), ppp=0.02, diam=3.0, diam_sd=0.5, noise=3.0, bits=8,
                         seed=seed, pair_id=pair_id)


def config2_flow():
    """Shear 0.005 px/px plus a Rankine vortex, at most 6 px over a 1024x1024 frame."""
    return Flow(vmax=6.0 - 0.005 * 512, rc=96.0, shear=0.005)


def config2_pair(seed=2, pair_id=0):
    """1024x1024 12-bit in u16, 0.03 ppp, d = 2.5, shear 0.005 + Rankine, max 6 px."""
    return particle_pair((1024, 1024), config2_flow(), ppp=0.03, diam=2.5,
                         diam_sd=0.0, noise=3.0, bits=12, seed=seed, pair_id=pair_id)


def config4_pair(seed=4, pair_id=0):
    """1024x1024 u8 vortex pair, 0.05 ppp, max 3 px (hybrid PIV + dense optical flow)."""
    return particle_pair((1024, 1024), Flow(vmax=3.0, rc=64.0), ppp=0.05, diam=3.0, diam_sd=0.5, noise=3.0, bits=8,
                         seed=seed, pair_id=pair_id)
