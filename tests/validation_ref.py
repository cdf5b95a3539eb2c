"""Second, independent restatement (pure Python, small grids only) of the reference's
multi-peak search and vector validation, used to cross-check the C oracle.

Written from the reference sources (S/ = src/main/java/pt/quickLabPIV/):
  * FindMaximumMultiPeaks.findMaximum          S/maximum/FindMaximumMultiPeaks.java:42-162
  * SimpleFixedLengthFloatLinkedList            S/util/SimpleFixedLengthFloatLinkedList.java:53-237
  * VectorValidatorJob.circularVisitor/compute  S/jobs/validator/VectorValidatorJob.java:105-405
  * NormalizedMedianValidator.validateVector    S/iareas/validation/NormalizedMedianValidator.java:63-136
  * SecondaryPeakReplacement.replaceVector      S/iareas/replacement/SecondaryPeakReplacement.java:41-76
  * BilinearReplacement.replaceVector           S/iareas/replacement/BilinearReplacement.java:23-420
  * DifferenceValidator.validateVector          S/iareas/validation/DifferenceValidator.java:30-60
  * Tile constructors, replaceDisplacement      S/iareas/Tile.java:51-67, 156-189
Float arithmetic is carried out with numpy float32 scalars so every rounding step is
Java's single precision.
"""
import math

import numpy as np

f32 = np.float32
FLT_MAX = f32(3.4028234663852886e38)


class PeakList:
    """Linked-list semantics kept as a Python list of [value, i, j], ascending."""

    def __init__(self, max_size, kernel_width):
        self.max_size = max_size
        self.kd = f32((kernel_width - 1) * kernel_width)
        self.items = []

    def _dist(self, i, j, e):
        return f32(float((i - e[1]) ** 2 + (j - e[2]) ** 2))

    def add(self, value, i, j):
        value = f32(value)
        if not self.items:
            self.items.append([value, i, j])
            return True
        idx = 0
        doomed = []
        while idx < len(self.items) and self.items[idx][0] < value:
            e = self.items[idx]
            if self._dist(i, j, e) < self.kd and value > e[0]:
                doomed.append(id(e))
            idx += 1
        if len(self.items) == self.max_size and idx == 0:
            return False
        for e in self.items[idx:]:
            if self._dist(i, j, e) < self.kd and value <= e[0]:
                return False
        before = [e for e in self.items[:idx] if id(e) not in doomed]
        after = self.items[idx:]
        if before:
            self.items = before + [[value, i, j]] + after
            if len(self.items) > self.max_size:
                self.items.pop(0)
        else:
            if len(after) == self.max_size:
                return False
            self.items = [[value, i, j]] + after
        return True


def find_max_multipeaks(m, kernel_width, num_peaks):
    m = np.asarray(m, np.float32)
    di, dj = m.shape
    kw = kernel_width
    si = -(-di // kw)
    sj = -(-dj // kw)
    top_slices = si - si // 2
    left_slices = sj - sj // 2
    peaks = PeakList(num_peaks, kw)
    best_pos = [(0, 0)] * 4
    lowest = FLT_MAX
    for a in range(top_slices):
        for b in range(left_slices):
            origins = [(a * kw, b * kw), (a * kw, (b + left_slices) * kw),
                       ((a + top_slices) * kw, b * kw), ((a + top_slices) * kw, (b + left_slices) * kw)]
            best = [f32(0)] * 4
            for oi in range(kw):
                for oj in range(kw):
                    for q, (ti, tj) in enumerate(origins):
                        i, j = ti + oi, tj + oj
                        if i >= di or j >= dj:
                            continue
                        val = m[i, j]
                        if val > best[q]:
                            best[q] = val
                            best_pos[q] = (i, j)
                        if val < lowest:
                            lowest = val
            for q in range(4):
                peaks.add(best[q], best_pos[q][0], best_pos[q][1])
    out = [(e[1], e[2], float(e[0])) for e in reversed(peaks.items)]
    return out, float(lowest)


def spiral_order(ni, nj):
    """Centre-out rings: right, down, left, up."""
    ci, cj = ni // 2, nj // 2
    hi, hj = 2, 2
    if ni % 2:
        hi = 1
    else:
        ci -= 1
    if nj % 2:
        hj = 1
    else:
        cj -= 1
    seen = set()
    order = []

    def visit(i, j):
        if 0 <= i < ni and 0 <= j < nj and (i, j) not in seen:
            seen.add((i, j))
            order.append(i * nj + j)

    while len(order) < ni * nj:
        i, j = ci, cj
        visit(i, j)
        for _ in range(max(hj - 1, 0)):
            j += 1
            visit(i, j)
        down = max(hi - 1, 0)
        for _ in range(down):
            i += 1
            visit(i, j)
        if down:
            for _ in range(max(hj - 1, 0)):
                j -= 1
                visit(i, j)
            for _ in range(max(hi - 2, 0)):
                i -= 1
                visit(i, j)
        hi += 2
        hj += 2
        ci -= 1
        cj -= 1
    return order


class _Tile:
    __slots__ = ("i", "j", "top", "left", "u", "v", "bu", "bv", "invalid", "locked", "clip")

    def set_invalid(self, state):
        if not self.locked:
            self.invalid = state

    def replace(self, u, v):
        """Tile.replaceDisplacement: under NoOutOfBoundClipping (clip = (n, h, w)) a displacement
        whose rounded value moves the tile out of the image is refused."""
        if self.clip is not None:
            n, h, w = self.clip
            ru = f32(math.floor(f32(u + f32(0.5))))
            rv = f32(math.floor(f32(v + f32(0.5))))
            if (f32(self.top) + ru < 0 or f32(self.top + n) + ru >= h or f32(self.left) + rv < 0 or
                    f32(self.left + n) + rv >= w):
                return False
        self.u, self.v = f32(u), f32(v)
        return True


def _neighbours(tiles, ti, tj):
    ni, nj = len(tiles), len(tiles[0])
    grid = [[None] * 3 for _ in range(3)]
    for a in range(3):
        for b in range(3):
            i, j = ti + a - 1, tj + b - 1
            if 0 <= i < ni and 0 <= j < nj:
                grid[a][b] = tiles[i][j]
    return grid


def _median_validate(t, nb, threshold, eps0):
    lst = [nb[a][b] for a in range(3) for b in range(3) if not (a == 1 and b == 1) and nb[a][b] is not None]
    lst = sorted(lst, key=lambda x: f32(x.u * x.u + x.v * x.v))  # stable, like Collections.sort
    n = len(lst)
    mu = mv = f32(0)
    if n:
        if n % 2 == 0:
            mu = f32((lst[n // 2 - 1].u + lst[n // 2].u) / f32(2))
            mv = f32((lst[n // 2 - 1].v + lst[n // 2].v) / f32(2))
        else:
            mu, mv = lst[n // 2].u, lst[n // 2].v
    r = [FLT_MAX] * 8
    for q, x in enumerate(lst):
        du, dv = f32(mu - x.u), f32(mv - x.v)
        r[q] = f32(du * du + dv * dv)
    r.sort()
    if n - 1 == 0:
        rmed = f32(1)
    elif (n - 1) % 2 == 0:
        rmed = f32(math.sqrt(f32((r[(n - 1) // 2] + r[(n - 1) // 2 + 1]) / f32(2))))
    else:
        rmed = f32(math.sqrt(r[(n - 1) // 2 + 1]))
    du, dv = f32(mu - t.u), f32(mv - t.v)
    dist = f32(f32(math.sqrt(f32(du * du + dv * dv))) / f32(rmed + f32(eps0)))
    t.set_invalid(not (dist < f32(threshold)))


def _difference_validate(t, nb, threshold):
    """adjacents [0][0], [0][1], [1][0]: each valid neighbour overwrites the flag."""
    t2 = f32(f32(threshold) * f32(threshold))
    for a in range(2):
        for b in range(2):
            if a == 1 and b == 1:
                continue
            x = nb[a][b]
            if x is None or x.invalid:
                continue
            du, dv = f32(x.u - t.u), f32(x.v - t.v)
            t.set_invalid(not (f32(du * du + dv * dv) < t2))


def _interp(p1, p2, pi, a1, a2):
    p1, p2, pi = f32(p1), f32(p2), f32(pi)
    w1 = w2 = f32(0)
    if f32(p2 - pi) > f32(1e-6) and f32(pi - p1) > f32(1e-6) and f32(p2 - p1) > f32(1e-6):
        w1 = f32(f32(f32(p2 - pi) / f32(p2 - p1)) * a1)
        w2 = f32(f32(f32(pi - p1) / f32(p2 - p1)) * a2)
    else:
        c = 0
        if abs(f32(pi - p2)) < f32(1e-6):
            w2 = a2
            c += 1
        if abs(f32(pi - p1)) < f32(1e-6):
            w1 = a1
            c += 1
        assert c, "corner case the reference rejects"
        if c > 1:
            w1 = f32(w1 / f32(c))
            w2 = f32(w2 / f32(c))
    return f32(w1 + w2)


def _bilinear(t, nb):
    if not t.invalid:
        return
    ok = lambda x: x is not None and not x.invalid  # noqa: E731
    L, R, T, B = nb[1][0], nb[1][2], nb[0][1], nb[2][1]
    TL, BR, BL, TR = nb[0][0], nb[2][2], nb[2][0], nb[0][2]
    est = []  # (weight u, u, weight v, v)
    if ok(L) and ok(R):
        est.append((1, _interp(L.top, R.top, t.top, L.u, R.u), 2, _interp(L.left, R.left, t.left, L.v, R.v)))
    if ok(B) and ok(T):
        est.append((2, _interp(T.top, B.top, t.top, T.u, B.u), 1, _interp(T.left, B.left, t.left, T.v, B.v)))
    if ok(TL) and ok(BR) and ok(BL) and ok(TR):
        lf = lambda x: f32(x.left)  # noqa: E731
        tp = lambda x: f32(x.top)  # noqa: E731
        wtr = f32(f32(lf(t) - lf(TL)) / f32(lf(TR) - lf(TL)))
        wtl = f32(f32(lf(TR) - lf(t)) / f32(lf(TR) - lf(TL)))
        wbr = f32(f32(lf(t) - lf(BL)) / f32(lf(BR) - lf(BL)))
        wbl = f32(f32(lf(BR) - lf(t)) / f32(lf(BR) - lf(BL)))
        wt = f32(f32(tp(BL) - tp(t)) / f32(tp(BL) - tp(TL)))
        wb = f32(f32(tp(t) - tp(TL)) / f32(tp(BL) - tp(TL)))

        def mix(g):
            top = f32(f32(wtr * g(TR)) + f32(wtl * g(TL)))
            bot = f32(f32(wbr * g(BR)) + f32(wbl * g(BL)))
            return f32(f32(wt * top) + f32(wb * bot))
        est.append((3, mix(lambda x: x.u), 3, mix(lambda x: x.v)))
    else:
        if ok(TL) and ok(BR):
            est.append((1, _interp(TL.top, BR.top, t.top, TL.u, BR.u), 1, _interp(TL.left, BR.left, t.left, TL.v, BR.v)))
        if ok(BL) and ok(TR):
            est.append((1, _interp(TR.top, BL.top, t.top, TR.u, BL.u), 1, _interp(BL.left, TR.left, t.left, BL.v, TR.v)))
    if not est:
        pick = None
        for a in range(3):
            for b in range(3):
                if (a, b) != (1, 1) and ok(nb[a][b]):
                    pick = nb[a][b]   # first valid of the row; later rows overwrite
                    break
        if pick is None:
            t.set_invalid(True)
        elif t.replace(pick.u, pick.v):
            t.set_invalid(False)
        return
    # classification-weighted mean over the four candidate slots (empty slots weigh 0)
    au = av = f32(0)
    wu = wv = 0
    slots = est + [(0, f32(0), 0, f32(0))] * (4 - len(est))
    # slot order in the reference: LR, TB, diagonal(s); empty slots contribute 0 * 0
    for cu, uu, cv, vv in slots:
        av = f32(av + f32(f32(cv) * vv))
        wv += cv
        au = f32(au + f32(f32(cu) * uu))
        wu += cu
    t.replace(f32(au / f32(wu)), f32(av / f32(wv)))
    t.set_invalid(False)


def validate(tops, lefts, u, v, peak_u, peak_v, npeaks, num_peaks, threshold, eps0, max_iterations,
             iterate_until=False, model=1, clip=None):
    """model 1: multi-peak normalised median (num_peaks strategies: secondary peaks, then
    bilinear); 2 / 3: difference validator without / with bilinear replacement; 4 / 5:
    normalised median without / with bilinear replacement.  clip: None or (n, h, w) for
    NoOutOfBoundClipping of the replacements."""
    ni, nj = u.shape
    tiles = [[None] * nj for _ in range(ni)]
    for i in range(ni):
        for j in range(nj):
            t = _Tile()
            t.i, t.j, t.top, t.left = i, j, int(tops[i]), int(lefts[j])
            t.u, t.v = f32(u[i, j]), f32(v[i, j])
            t.bu, t.bv = t.u, t.v
            t.invalid = True          # Tile constructors
            t.locked = False
            t.clip = clip
            tiles[i][j] = t
    strategies = []               # (replacement) per strategy: "peak<p>", "bilinear" or None
    if model == 1:
        strategies = [f"peak{s + 1}" for s in range(num_peaks - 1)] + ["bilinear"]
    else:
        strategies = ["bilinear" if model in (3, 5) else None]

    def check(t, nb):
        if model in (2, 3):
            _difference_validate(t, nb, threshold)
        else:
            _median_validate(t, nb, threshold, eps0)

    order = spiral_order(ni, nj)
    for k in order:
        t = tiles[k // nj][k % nj]
        check(t, _neighbours(tiles, t.i, t.j))
        if not t.invalid:
            t.locked = True
    attempt = 0
    while True:
        corrected = 0
        for k in order:
            t = tiles[k // nj][k % nj]
            nb = _neighbours(tiles, t.i, t.j)
            check(t, nb)
            for repl in strategies:
                if not t.invalid:
                    break
                if repl is not None:
                    t.u, t.v = t.bu, t.bv          # restoreDisplacement
                    if repl == "bilinear":
                        _bilinear(t, nb)
                    else:
                        p = int(repl[4:])
                        if npeaks[t.i, t.j] > p:
                            nu = f32(f32(t.u - f32(peak_u[t.i, t.j, 0])) + f32(peak_u[t.i, t.j, p]))
                            nv = f32(f32(t.v - f32(peak_v[t.i, t.j, 0])) + f32(peak_v[t.i, t.j, p]))
                            if t.replace(nu, nv):
                                t.set_invalid(False)
                check(t, nb)
                if not t.invalid:
                    corrected += 1
                    break
        attempt += 1
        if corrected == 0 or (not iterate_until and attempt >= max_iterations) or attempt >= 1000:
            break
    ou = np.zeros((ni, nj), np.float32)
    ov = np.zeros((ni, nj), np.float32)
    inv = np.zeros((ni, nj), np.uint8)
    for i in range(ni):
        for j in range(nj):
            t = tiles[i][j]
            if t.invalid:
                t.replace(f32(0), f32(0))
            ou[i, j], ov[i, j], inv[i, j] = t.u, t.v, int(t.invalid)
    return ou, ov, inv, attempt
