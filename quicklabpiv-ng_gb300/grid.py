"""IA grid generation: host-side mirror of the reference's interrogation-area division
strategies, computed with Java float semantics (numpy float32 scalars).

  SuperPosition    S/iareas/AdaptiveInterAreaStrategySuperPosition.java:31-197
  NoSuperPosition  S/iareas/AdaptiveInterAreaStrategyNoSuperPosition.java:32-157
(S/ = src/main/java/pt/quickLabPIV/ in QuickLabPIV-ng.)
"""
import math
from dataclasses import dataclass

import numpy as np

f32 = np.float32


def java_round(x):
    """FastMath.round(float) = (int) floor(x + 0.5f)."""
    return int(math.floor(f32(f32(x) + f32(0.5))))


@dataclass
class StepTiles:
    """IterationStepTiles geometry of one adaptive level."""
    level: int
    n: int
    tiles_i: int
    tiles_j: int
    margin_top: int
    margin_left: int
    margin_bottom: int
    margin_right: int
    tops: np.ndarray    # int32[tiles_i]
    lefts: np.ndarray   # int32[tiles_j]

    @property
    def count(self):
        return self.tiles_i * self.tiles_j

    def origins(self):
        """Row-major flattened (top, left) of every tile."""
        tt, ll = np.meshgrid(self.tops, self.lefts, indexing="ij")
        return tt.ravel().astype(np.int32), ll.ravel().astype(np.int32)

    def centres(self):
        """Tile centres at the centre of the 4 central pixels: top + N/2 - 0.5
        (S/iareas/AdaptiveInterVelocityInheritanceStrategyBiCubicSpline.java:52-58)."""
        half = f32(self.n) / f32(2.0) - f32(0.5)
        return (self.tops.astype(np.float32) + half), (self.lefts.astype(np.float32) + half)


def _floor_div(a, b):
    return a // b


def superposition(height, width, ia_start, level, overlap_factor, margins=(0, 0, 0, 0)):
    """Grid of `level` for the SuperPosition strategy; margins = (top, bottom, left, right).
    overlap_factor = 1 - overlap% / 100 (PIVConfigurationConverterVisitor.java:146), in
    [0.1, 0.9]."""
    ofac = f32(overlap_factor)
    if ofac < f32(1 / 10) or ofac > f32(1 - 1 / 10):
        raise ValueError("Overlap factor must greater than 1/10 and less than 9/10")
    mt, mb, ml, mr = margins
    n = ia_start >> level
    inc = f32(ofac * f32(n))
    nj = int(f32(f32(0.01) + f32(f32(f32(width - (ml + mr)) - f32(f32(n) - inc)) / inc)))
    ni = int(f32(f32(0.01) + f32(f32(f32(height - (mt + mb)) - f32(f32(n) - inc)) / inc)))
    rem_i = height - int(math.ceil(float(f32(f32(f32(ni - 1) * inc) + f32(n))))) - (mt + mb)
    rem_j = width - int(math.ceil(float(f32(f32(f32(nj - 1) * inc) + f32(n))))) - (ml + mr)
    m_top = mt + _floor_div(rem_i, 2)
    m_bottom = mb + int(math.ceil(float(f32(rem_i) / f32(2.0))))
    m_left = ml + _floor_div(rem_j, 2)
    m_right = mr + int(math.ceil(float(f32(rem_j) / f32(2.0))))
    if level == 0:
        tops = [m_top + java_round(f32(f32(k) * inc)) for k in range(ni)]
        lefts = [m_left + java_round(f32(f32(k) * inc)) for k in range(nj)]
    else:
        tops, p = [], f32(m_top)
        for _ in range(ni):
            tops.append(java_round(p))
            p = f32(p + inc)
        lefts, p = [], f32(m_left)
        for _ in range(nj):
            lefts.append(java_round(p))
            p = f32(p + inc)
    return StepTiles(level, n, ni, nj, m_top, m_left, m_bottom, m_right, np.array(tops, np.int32),
                     np.array(lefts, np.int32))


def nosuperposition(height, width, ia_start, level, margins=(0, 0, 0, 0)):
    mt, mb, ml, mr = margins
    n = ia_start >> level
    ni = (height - (mt + mb)) // n
    nj = (width - (ml + mr)) // n
    left_i = height - mt - mb - n * ni
    left_j = width - ml - mr - n * nj
    m_top = mt + left_i // 2
    m_left = ml + left_j // 2
    return StepTiles(level, n, ni, nj, m_top, m_left, height - n * ni - m_top, width - n * nj - m_left,
                     np.arange(ni, dtype=np.int32) * n + m_top, np.arange(nj, dtype=np.int32) * n + m_left)


def adaptive_levels(ia_start, ia_end):
    """Number of adaptive levels: log2(start/end) + 1 (LocalPIVOpenCLGpuJob.java:91);
    start must be a power-of-two multiple of end."""
    if ia_start % ia_end != 0:
        raise ValueError("Interrogation Area start pixels is not a multiple of Interrogation Area end pixels")
    ratio = ia_start // ia_end
    steps = int(math.floor(math.log2(ratio)))
    if 2 ** steps != ratio:
        raise ValueError("step sizes ratio is not a power of two")
    return steps + 1


def level(height, width, ia_start, level, overlap_factor, margins=(0, 0, 0, 0), superposition_start=0):
    """Grid of `level` under AdaptiveInterAreaStrategyMixedSuperPosition
    (S/iareas/AdaptiveInterAreaStrategyMixedSuperPosition.java:31-92): NoSuperPosition before
    superposition_start; from there SuperPosition restarted as at its first step with IA
    ia_start >> superposition_start.  superposition_start 0 is plain SuperPosition."""
    if level < superposition_start:
        return nosuperposition(height, width, ia_start, level, margins)
    g = superposition(height, width, ia_start >> superposition_start, level - superposition_start, overlap_factor,
                      margins)
    g.level = level
    return g
