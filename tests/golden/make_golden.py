"""Generate the small golden fixtures under tests/golden/ from the reference tree.

Run once in a checkout that has the QuickLabPIV-ng reference next to it:
    python tests/golden/make_golden.py /path/to/QuickLabPIV-ng
The outputs are committed; no test reads the reference tree at run time.

Fixtures written (all from files shipped in the reference project):
  rankine_pair.npz     resources/fftBenchmark/rankine_vortex01_{0,1}.tif (512x512 u8,
                       PackBits TIFF), decoded here.
  gpu_fft_golden.npz   every 16th of the 1024 31x31 correlation planes in
                       resources/fftBenchmark/gpuFFTBenchmarkValidationData.matFloat
                       (16x16 IAs, no overlap, own-max normalisation), with their
                       IA indices.
  shift_kat.npz        testFiles/img1.png, img2.png: the synthetic pair shifted by
                       10 px used by ImageCrossCorrelationRealFFTParStdJobTests.
  filter_edges.npz     6-pixel border bands of the Gaussian filter outputs of
                       testFiles/GaussianFilter2D_*.matFloat (padding rules)
  dense_golden.npz     testFiles/Python_denseLucasKanade_PyrLvs2_Fs2_0_Iter5_64x64.matFloat (window 27,
                       1/4/5 iterations) and testFiles/Python_with_JavaLK_denseLiuShen_lambda4_*.matFloat
                       (Liu-Shen images, Java LK input, fixed terms, 5 passes)
  filter_golden.npz    testFiles/GaussianFilter2D_*.matFloat (Gaussian prefilter
                       outputs) cropped to a 96x96 window.
  gauss_kat.npz        the known-answer cases of tests/pt/quickLabPIV/interpolators/
                       Gaussian1DInterpolatorAdvanced{3,5,7}Pixels{Symmetric,Assymmetric,HongWeiGuo}
                       Test.java: per case the window side, the interpolator (0 Gaussian1D least
                       squares, 1 Hongwei Guo with 20 iterations), the centre (uX, uY) and widths
                       (sigmaX, sigmaY) of the analytic peak and the tolerance (8e-3 px).
  tiff_packbits_rankine.tif  the first four PackBits strips (64 rows) of
                       testFiles/rankine_vortex01_0.tif, compressed bytes kept verbatim under a
                       minimal directory; decodes to rankine_pair.npz's a[:64].
  tiff_lzw_chess.tif   the LZW strip of testFiles/coordTestChessA.tif (128x128 u8, four 64x64
                       constant quadrants), compressed bytes kept verbatim.
"""
import struct
import os
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def read_matfloat(path):
    """SimpleFloatMatrixImporterExporter format (big-endian): 'MATFloat\\0', u16 count,
    count x (u16 len, name), then per matrix u16 cols, u16 rows, u16 depth, rows*cols f32."""
    b = Path(path).read_bytes()
    if b[:9] != b"MATFloat\x00":
        raise ValueError("not a .matFloat file")
    p = 9
    (cnt,) = struct.unpack(">H", b[p:p + 2])
    p += 2
    names = []
    for _ in range(cnt):
        (ln,) = struct.unpack(">H", b[p:p + 2])
        p += 2
        names.append(b[p:p + ln].decode())
        p += ln
    mats = []
    for _ in range(cnt):
        sx, sy, _sz = struct.unpack(">HHH", b[p:p + 6])
        p += 6
        mats.append(np.frombuffer(b[p:p + 4 * sx * sy], dtype=">f4").reshape(sy, sx).astype(np.float32))
        p += 4 * sx * sy
    if p != len(b):
        raise ValueError("trailing bytes in .matFloat")
    return names, mats


def read_tiff_gray(path):
    """Baseline grey TIFF, 8/16 bit, uncompressed or PackBits, strip organised."""
    b = Path(path).read_bytes()
    e = "<" if b[:2] == b"II" else ">"
    (off,) = struct.unpack(e + "I", b[4:8])
    (n,) = struct.unpack(e + "H", b[off:off + 2])
    tags = {}
    for k in range(n):
        ent = b[off + 2 + 12 * k: off + 14 + 12 * k]
        t, typ, cnt = struct.unpack(e + "HHI", ent[:8])
        tags[t] = (typ, cnt, ent[8:12])

    def values(t):
        typ, cnt, raw = tags[t]
        size = {3: 2, 4: 4}[typ]
        fmt = e + ("H" if typ == 3 else "I") * cnt
        if cnt * size <= 4:
            return list(struct.unpack(fmt, raw[:cnt * size]))
        (ptr,) = struct.unpack(e + "I", raw)
        return list(struct.unpack(fmt, b[ptr:ptr + cnt * size]))

    w, h = values(256)[0], values(257)[0]
    bps, comp = values(258)[0], values(259)[0]
    data = bytearray()
    for o, c in zip(values(273), values(279)):
        s = b[o:o + c]
        if comp == 1:
            data += s
        elif comp == 32773:
            i = 0
            while i < len(s):
                hdr = s[i] - 256 if s[i] > 127 else s[i]
                i += 1
                if hdr >= 0:
                    data += s[i:i + hdr + 1]
                    i += hdr + 1
                elif hdr != -128:
                    data += bytes([s[i]]) * (1 - hdr)
                    i += 1
        else:
            raise ValueError(f"TIFF compression {comp} not supported")
    dt = np.uint8 if bps == 8 else np.dtype(e + "u2")
    return np.frombuffer(bytes(data), dtype=dt)[: w * h].reshape(h, w).copy()


def tiff_strips(path, first_strips=None):
    """(width, height, bits, compression, rows_per_strip, [strip bytes]) of a TIFF's first page."""
    b = Path(path).read_bytes()
    e = "<" if b[:2] == b"II" else ">"
    (off,) = struct.unpack(e + "I", b[4:8])
    (n,) = struct.unpack(e + "H", b[off:off + 2])
    tags = {}
    for k in range(n):
        ent = b[off + 2 + 12 * k: off + 14 + 12 * k]
        t, typ, cnt = struct.unpack(e + "HHI", ent[:8])
        if typ not in (3, 4):
            continue
        size = 2 if typ == 3 else 4
        fmt = e + ("H" if typ == 3 else "I") * cnt
        if cnt * size <= 4:
            tags[t] = list(struct.unpack(fmt, ent[8:8 + cnt * size]))
        else:
            (ptr,) = struct.unpack(e + "I", ent[8:12])
            tags[t] = list(struct.unpack(fmt, b[ptr:ptr + cnt * size]))
    offs, counts = tags[273], tags[279]
    if first_strips is not None:
        offs, counts = offs[:first_strips], counts[:first_strips]
    rps = tags.get(278, [tags[257][0]])[0]
    return tags[256][0], tags[257][0], tags[258][0], tags[259][0], rps, [b[o:o + c] for o, c in zip(offs, counts)]


def write_min_tiff(dst, width, height, bits, compression, rows_per_strip, strips):
    """Little-endian TIFF with one directory (size, bits, compression, BlackIsZero, strips)."""
    ns = len(strips)
    entries = 9
    ifd = 8
    arrays = ifd + 2 + 12 * entries + 4
    data = arrays + 8 * ns
    offs, pos = [], data
    for s in strips:
        offs.append(pos)
        pos += len(s)
    out = bytearray(b"II" + struct.pack("<HI", 42, ifd))
    out += struct.pack("<H", entries)

    def tag(t, typ, cnt, value):
        return struct.pack("<HHI", t, typ, cnt) + value

    strip_off = struct.pack("<I", offs[0]) if ns == 1 else struct.pack("<I", arrays)
    strip_cnt = struct.pack("<I", len(strips[0])) if ns == 1 else struct.pack("<I", arrays + 4 * ns)
    out += tag(256, 4, 1, struct.pack("<I", width))
    out += tag(257, 4, 1, struct.pack("<I", height))
    out += tag(258, 3, 1, struct.pack("<HH", bits, 0))
    out += tag(259, 3, 1, struct.pack("<HH", compression, 0))
    out += tag(262, 3, 1, struct.pack("<HH", 1, 0))
    out += tag(273, 4, ns, strip_off)
    out += tag(277, 3, 1, struct.pack("<HH", 1, 0))
    out += tag(278, 4, 1, struct.pack("<I", rows_per_strip))
    out += tag(279, 4, ns, strip_cnt)
    out += struct.pack("<I", 0)
    out += struct.pack(f"<{ns}I", *offs) + struct.pack(f"<{ns}I", *[len(s) for s in strips])
    for s in strips:
        out += s
    Path(dst).write_bytes(bytes(out))


def tiff_fixtures(ref):
    ref = Path(ref)
    w, h, bits, comp, rps, strips = tiff_strips(ref / "testFiles/rankine_vortex01_0.tif", first_strips=4)
    assert comp == 32773 and rps == 16
    write_min_tiff(HERE / "tiff_packbits_rankine.tif", w, 4 * rps, bits, comp, rps, strips)
    w, h, bits, comp, rps, strips = tiff_strips(ref / "testFiles/coordTestChessA.tif")
    assert comp == 5 and len(strips) == 1
    write_min_tiff(HERE / "tiff_lzw_chess.tif", w, h, bits, comp, rps, strips)


def read_png_gray(path):
    """8/16-bit greyscale or RGB(A) PNG (non-interlaced); colour images are reduced to
    the first channel.  16-bit samples are big-endian in the file."""
    b = Path(path).read_bytes()
    assert b[:8] == b"\x89PNG\r\n\x1a\n"
    p = 8
    idat = b""
    while p < len(b):
        (ln,) = struct.unpack(">I", b[p:p + 4])
        typ = b[p + 4:p + 8]
        body = b[p + 8:p + 8 + ln]
        p += 12 + ln
        if typ == b"IHDR":
            w, h, depth, ctype, _c, _f, inter = struct.unpack(">IIBBBBB", body)
            assert depth in (8, 16) and inter == 0
        elif typ == b"IDAT":
            idat += body
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype] * (depth // 8)
    raw = zlib.decompress(idat)
    stride = w * ch
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    pos = 0
    for r in range(h):
        f = raw[pos]
        line = np.frombuffer(raw[pos + 1:pos + 1 + stride], dtype=np.uint8).astype(np.int32)
        pos += 1 + stride
        cur = np.zeros(stride, dtype=np.int32)
        for x in range(stride):
            a = cur[x - ch] if x >= ch else 0
            up = prev[x]
            c = prev[x - ch] if x >= ch else 0
            if f == 0:
                v = line[x]
            elif f == 1:
                v = line[x] + a
            elif f == 2:
                v = line[x] + up
            elif f == 3:
                v = line[x] + ((a + up) >> 1)
            else:
                pa, pb, pc = abs(up - c), abs(a - c), abs(a + up - 2 * c)
                pr = a if (pa <= pb and pa <= pc) else (up if pb <= pc else c)
                v = line[x] + pr
            cur[x] = v & 0xFF
        out[r] = cur
        prev = cur
    if depth == 16:
        return (out[:, 0::ch].astype(np.uint16) << 8) | out[:, 1::ch].astype(np.uint16)
    return out[:, ::ch].copy()


def gauss_kat_cases(ref):
    """(dim, kind, uX, uY, sigmaX, sigmaY, tol) of every @Test of the Gaussian 1D KAT files."""
    import re
    rows = []
    d = Path(ref) / "tests/pt/quickLabPIV/interpolators"

    def fexpr(e):
        # Java float literal expressions of the tests: a, +a, -a, a*b, a/b (float arithmetic)
        m = re.fullmatch(r"([+-]?[0-9.]+)f(?:([*/])([0-9.]+)f)?", e.strip())
        a = np.float32(float(m.group(1)))
        if m.group(2) == "*":
            a = np.float32(a * np.float32(float(m.group(3))))
        elif m.group(2) == "/":
            a = np.float32(a / np.float32(float(m.group(3))))
        return float(a)

    for f in sorted(d.glob("Gaussian1DInterpolatorAdvanced*Test.java")):
        text = f.read_text()
        dim = int(re.search(r"int DIM = (\d+);", text).group(1))
        kind = 1 if "HongWeiGuo" in f.name else 0
        for body in text.split("@Test")[1:]:
            vals = {k: fexpr(re.search(rf"float {k} = ([^;]+);", body).group(1))
                    for k in ("uX", "uY", "sigmaX", "sigmaY")}
            assert "createMatrixWithGaussian2DAssymmetric(DIM, DIM, uX, sigmaX, uY, sigmaY)" in body
            assert ("setupPIVContextHongWeiGuo1D" in body) == (kind == 1)
            tols = re.findall(r"getMainPeak[IJ]\(\), ([0-9.e-]+)f\);", body)
            assert len(tols) == 2 and tols[0] == tols[1]
            rows.append((dim, kind, vals["uX"], vals["uY"], vals["sigmaX"], vals["sigmaY"], float(tols[0])))
    return np.array(rows, dtype=np.float64)


def main(ref):
    ref = Path(ref)
    a = read_tiff_gray(ref / "resources/fftBenchmark/rankine_vortex01_0.tif")
    b = read_tiff_gray(ref / "resources/fftBenchmark/rankine_vortex01_1.tif")
    np.savez_compressed(HERE / "rankine_pair.npz", a=a, b=b)

    names, mats = read_matfloat(ref / "resources/fftBenchmark/gpuFFTBenchmarkValidationData.matFloat")
    idx = np.arange(0, len(mats), 16)
    sel_names = [names[i] for i in idx]
    np.savez_compressed(HERE / "gpu_fft_golden.npz", index=idx, planes=np.stack([mats[i] for i in idx]),
                        names=np.array(sel_names))

    i1 = read_png_gray(ref / "testFiles/img1.png")
    i2 = read_png_gray(ref / "testFiles/img2.png")
    np.savez_compressed(HERE / "shift_kat.npz", img1=i1, img2=i2)

    fn1, fm1 = read_matfloat(ref / "testFiles/GaussianFilter2D_3px_2.0f_rankine_vortex01_0.matFloat")
    fn2, fm2 = read_matfloat(ref / "testFiles/GaussianFilter2D_5px_0.48f_rankine_vortex01_0_1.matFloat")
    win = (slice(200, 296), slice(200, 296))
    np.savez_compressed(HERE / "filter_golden.npz", window=np.array([200, 296, 200, 296]),
                        names1=np.array(fn1), names2=np.array(fn2),
                        **{f"f1_{k}": m[win] for k, m in enumerate(fm1)},
                        **{f"f2_{k}": m[win] for k, m in enumerate(fm2)})
    # filter edges: 6-pixel bands along the four image borders (the padding rules); the
    # filtered sources testFiles/rankine_vortex01_{0,1}.tif equal rankine_pair.npz's a, b
    src0 = read_tiff_gray(ref / "testFiles/rankine_vortex01_0.tif")
    src1 = read_tiff_gray(ref / "testFiles/rankine_vortex01_1.tif")
    assert (src0 == a).all() and (src1 == b).all()
    bands = {}
    for tag, mats in (("f1", fm1), ("f2", fm2)):
        for k, m in enumerate(mats):
            bands[f"{tag}_{k}_top"] = m[:6]
            bands[f"{tag}_{k}_bottom"] = m[-6:]
            bands[f"{tag}_{k}_left"] = m[:, :6]
            bands[f"{tag}_{k}_right"] = m[:, -6:]
    np.savez_compressed(HERE / "filter_edges.npz", **bands)

    # dense Lucas-Kanade (window 27, no half-pixel offset) and Liu-Shen (lambda 4) fixtures
    ln, lm = read_matfloat(ref / "testFiles/Python_denseLucasKanade_PyrLvs2_Fs2_0_Iter5_64x64.matFloat")
    lk = dict(zip(ln, lm))
    keep_lk = ["imageA", "imageB"] + [f"{w}LK2nd{k}_{c}" for k in (1, 4, 5) for w in ("before", "after")
                                      for c in ("u", "v")]
    sn, sm = read_matfloat(ref / "testFiles/Python_with_JavaLK_denseLiuShen_lambda4_Rankine_vortex_64x64.matFloat")
    ls = dict(zip(sn, sm))
    keep_ls = ["Im1LS_Filtered", "Im2LS_Filtered", "uLK", "vLK", "cmtx", "IIx", "IIy", "II", "Ixt", "Iyt",
               "A11", "A12", "A22", "B11", "B12", "B22"] + [f"unews{k}" for k in range(5)] + \
              [f"vnews{k}" for k in range(5)]
    np.savez_compressed(HERE / "dense_golden.npz", **{f"lk_{k}": lk[k] for k in keep_lk},
                        **{f"ls_{k}": ls[k] for k in keep_ls})
    np.savez_compressed(HERE / "gauss_kat.npz", cases=gauss_kat_cases(ref))
    tiff_fixtures(ref)
    print("shapes:", a.shape, b.shape, i1.shape, i2.shape, [m.shape for m in fm1], [m.shape for m in fm2],
          fn1, fn2, src0.shape, len(keep_lk), len(keep_ls))


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[2] == "--gauss-kat-only":
        np.savez_compressed(HERE / "gauss_kat.npz", cases=gauss_kat_cases(sys.argv[1]))
        sys.exit(0)
    if len(sys.argv) > 2 and sys.argv[2] == "--tiff-only":
        tiff_fixtures(sys.argv[1])
        sys.exit(0)
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("QLPIV_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <QuickLabPIV-ng checkout> [--gauss-kat-only | --tiff-only] "
                 "(or set QLPIV_REFERENCE)")
    main(ref)
