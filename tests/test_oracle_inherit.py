"""Oracle of the Direct / Area / Distance velocity inheritance pinned to the reference's own tests.

* checkOverlappingFactor known answers of AdaptiveInterAreaVelocityInheritanceByAreaTests.java
  (IA 64 parent, IA 32 child): overlap factor and move flags.
* AdaptiveInterAreaVelocityInheritanceByAreaCompleteTests.java: 171 x 171 image, 32 px margins,
  overlap 1/3, IA 64 -> 32, the 3 x 3 parent field of the test; every child tile's displacement
  against the test's own weighted sum (tolerance 1e-4).
* AdaptiveInterAreaVelocityInheritanceByDistance{,Generic}Tests.java: 139 x 139 image, 16 px
  margins, same field; every child tile against the test's inverse-distance sum (1e-6).
* Direct by construction, and the geometries on which the reference's walk throws.
"""
import math

import numpy as np
import pytest

from conftest import load_package

f32 = np.float32

# (parent top, left, child top, left, factor, up, down, left, right)
AREA_KAT = [
    (0, 0, 16, 16, 1.0, 0, 0, 0, 0), (0, 0, 32, 32, 1.0, 0, 0, 0, 0), (0, 0, 48, 32, 0.5, 0, 0, 0, 0),
    (0, 0, 32, 48, 0.5, 0, 0, 0, 0), (0, 0, 48, 48, 0.25, 0, 0, 0, 0), (0, 0, 56, 56, 0.0625, 0, 0, 0, 0),
    (0, 0, 64, 64, 0.0, 0, 1, 0, 1), (64, 64, 32, 32, 0.0, 1, 0, 1, 0), (16, 16, 0, 0, 0.25, 0, 0, 0, 0),
    (16, 16, 16, 0, 0.5, 0, 0, 0, 0), (16, 16, 0, 16, 0.5, 0, 0, 0, 0), (64, 64, 64, 32, 0.0, 0, 0, 1, 0),
    (64, 64, 32, 64, 0.0, 1, 0, 0, 0), (64, 64, 64, 128, 0.0, 0, 0, 0, 1), (64, 64, 128, 64, 0.0, 0, 1, 0, 0),
]

# parent displacements of the reference's complete tests (u, v per parent tile)
PARENT_U = np.array([[-11, -11, -11], [1, 1, 1], [11, 11, 11]], f32)
PARENT_V = np.array([[-11, 1, 11], [-11, 1, 11], [-11, 1, 11]], f32)


@pytest.fixture(scope="module")
def qp():
    pkg = load_package()
    pkg.build.build()
    return pkg


@pytest.mark.parametrize("case", AREA_KAT)
def test_area_overlap_known_answers(oracle, case):
    pt, pl, ct, cl, factor, up, down, left, right = case
    got = oracle.area_overlap(pt, pl, 64, ct, cl, 32)
    assert abs(got[0] - factor) <= 1e-4
    assert got[1:] == (bool(up), bool(down), bool(left), bool(right))


def _grids(qp, size, margin):
    m = (margin,) * 4
    gp, pt, pl = qp.library_grid(size, size, 64, 0, 1.0 / 3.0, m)
    gc, ct, cl = qp.library_grid(size, size, 64, 1, 1.0 / 3.0, m)
    return pt, pl, ct, cl


def test_area_complete_known_answer(qp, oracle):
    pt, pl, ct, cl = _grids(qp, 171, 32)
    assert len(ct) == len(cl) == 8
    cu, cv = oracle.inherit_tiles(oracle.INHERIT_AREA, 64, pt, pl, PARENT_U, PARENT_V, 32, ct, cl)
    idx = [[0, 1], [0, 1], [0, 1, 2], [0, 1, 2], [0, 1, 2], [0, 1, 2], [1, 2], [1, 2]]
    areas = [[32, 11], [32, 22], [32, 32, 10], [32, 32, 21], [21, 32, 32], [11, 32, 32], [21, 32], [10, 32]]
    for i in range(8):
        for j in range(8):
            tiles = [(a, b) for a in idx[i] for b in idx[j]]
            w = [f32(x * y) for x in areas[i] for y in areas[j]]
            total = f32(0)
            for x in w:
                total = f32(total + x)
            eu = ev = f32(0)
            for (a, b), x in zip(tiles, w):
                eu = f32(eu + f32(f32(x / total) * PARENT_U[a, b]))
                ev = f32(ev + f32(f32(x / total) * PARENT_V[a, b]))
            assert abs(cu[i, j] - eu) <= 1e-4 and abs(cv[i, j] - ev) <= 1e-4, (i, j)


def test_distance_known_answer(qp, oracle):
    pt, pl, ct, cl = _grids(qp, 139, 16)
    assert len(ct) == len(cl) == 8
    cu, cv = oracle.inherit_tiles(oracle.INHERIT_DISTANCE, 64, pt, pl, PARENT_U, PARENT_V, 32, ct, cl)
    sol = [[0], [0], [0, 1], [0, 1], [1, 2], [1, 2], [2], [2]]
    for i in range(8):
        for j in range(8):
            centre = (f32(ct[i]) + f32(16), f32(cl[j]) + f32(16))
            tiles = [(a, b) for a in sol[i] for b in sol[j]]
            dist = []
            for a, b in tiles:
                dy = float(f32(f32(pt[a]) + f32(32) - centre[0]))
                dx = float(f32(f32(pl[b]) + f32(32) - centre[1]))
                dist.append(f32(math.sqrt(dy * dy + dx * dx)))
            zero = [k for k, d in enumerate(dist) if d == 0]
            if zero:
                eu, ev = PARENT_U[tiles[zero[-1]]], PARENT_V[tiles[zero[-1]]]
            else:
                total = f32(0)
                for d in dist:
                    total = f32(total + f32(f32(1) / d))
                eu = ev = f32(0)
                for (a, b), d in zip(tiles, dist):
                    w = f32(f32(f32(1) / d) / total)
                    eu = f32(eu + f32(w * PARENT_U[a, b]))
                    ev = f32(ev + f32(w * PARENT_V[a, b]))
            assert abs(cu[i, j] - eu) <= 1e-6 and abs(cv[i, j] - ev) <= 1e-6, (i, j)


def test_direct(qp, oracle):
    rng = np.random.default_rng(2)
    pu = rng.normal(0, 2, (3, 4)).astype(f32)
    pv = rng.normal(0, 2, (3, 4)).astype(f32)
    pt, pl = np.arange(3) * 20, np.arange(4) * 20
    ct, cl = np.arange(7) * 10, np.arange(9) * 10
    cu, cv = oracle.inherit_tiles(oracle.INHERIT_DIRECT, 40, pt, pl, pu, pv, 20, ct, cl)
    np.testing.assert_array_equal(cu[:6, :8], np.repeat(np.repeat(pu, 2, 0), 2, 1))
    assert not cu[6].any() and not cu[:, 8].any() and not cv[6].any()
    ru, _ = oracle.inherit_tiles(oracle.INHERIT_DIRECT, 40, pt, pl, pu, pv, 20, ct, cl, round_int=True)
    np.testing.assert_array_equal(ru[:6, :8], np.floor(np.repeat(np.repeat(pu, 2, 0), 2, 1) + f32(0.5)))
    with pytest.raises(ValueError):   # fewer than two child tiles per parent tile: index out of range
        oracle.inherit_tiles(oracle.INHERIT_DIRECT, 40, pt, pl, pu, pv, 20, ct[:5], cl)


def test_walk_throws_where_the_reference_does(oracle):
    pu = np.zeros((3, 3), f32)
    pt = pl = np.array([10, 31, 53])
    with pytest.raises(ValueError):   # child column entirely left of the first parent
        oracle.inherit_tiles(oracle.INHERIT_AREA, 64, pt, pl, pu, pu, 32, np.array([10, 21]), np.array([0, 11]) - 30)
    with pytest.raises(ValueError):   # a child column two parents further on: one move is not enough
        oracle.inherit_tiles(oracle.INHERIT_AREA, 16, np.array([0, 16, 32]), np.array([0, 16, 32]), pu, pu, 8,
                             np.array([0, 8]), np.array([0, 40]))
    # the Distance walk never throws on sorted grids
    cu, _ = oracle.inherit_tiles(oracle.INHERIT_DISTANCE, 16, np.array([0, 16, 32]), np.array([0, 16, 32]), pu, pu,
                                 8, np.array([0, 8]), np.array([0, 40]))
    assert cu.shape == (2, 2)
