"""Host data formats either side of the path, no GPU needed.

* TIFF ingest (the frames S/jobs/ImageReaderJob.java reads): the reference's own PackBits and
  LZW strips (tests/golden/tiff_*.tif, compressed bytes kept verbatim) decode to the known
  pixels, and TIFFs written here in every supported form (uncompressed / PackBits / LZW with
  and without the horizontal predictor, 8 / 16 bits, both byte orders, several strips) read back
  exactly.  The encoders below follow the TIFF 6.0 text, independently of the C decoder.
* MATLAB export (S/exporter/StructMultiFrameFloatVelocityExporter.java): the file reads back
  with scipy.io.loadmat with the reference's variable and field names, classes and shapes.
"""
import struct

import numpy as np
import pytest

from conftest import GOLDEN, load_package


@pytest.fixture(scope="module")
def qp():
    pkg = load_package()
    pkg.build.build()
    pkg.load_library()
    return pkg


# ---------------- TIFF writers (test side) ----------------

def packbits(data):
    out, i, n = bytearray(), 0, len(data)
    while i < n:
        run = 1
        while i + run < n and run < 128 and data[i + run] == data[i]:
            run += 1
        if run >= 2:
            out += bytes([(257 - run) & 0xFF, data[i]])
            i += run
            continue
        j = i
        while j < n and j - i < 128 and not (j + 1 < n and data[j + 1] == data[j]):
            j += 1
        j = max(j, i + 1)
        out += bytes([j - i - 1]) + bytes(data[i:j])
        i = j
    return bytes(out)


def lzw(data):
    """TIFF LZW encoder: MSB-first codes, clear (256) at the start and when the table is full,
    end of information (257).  The encoder widens its codes once entry 511 (1023, 2047) is in
    the table; a decoder, one entry behind, widens when its next free entry reaches 511."""
    bits, nbits = [], 0

    def put(code, width):
        for k in range(width - 1, -1, -1):
            bits.append((code >> k) & 1)

    table = {bytes([c]): c for c in range(256)}
    nxt, width = 258, 9
    put(256, width)
    w = b""
    for c in data:
        wc = w + bytes([c])
        if wc in table:
            w = wc
            continue
        put(table[w], width)
        table[wc] = nxt
        nxt += 1
        w = bytes([c])
        if nxt >= 4094:
            put(256, width)
            table = {bytes([x]): x for x in range(256)}
            nxt, width = 258, 9
        else:
            width = 12 if nxt > 2047 else 11 if nxt > 1023 else 10 if nxt > 511 else 9
    if w:
        put(table[w], width)
        nxt += 1
        width = 12 if nxt > 2047 else 11 if nxt > 1023 else 10 if nxt > 511 else 9
    put(257, width)
    while len(bits) % 8:
        bits.append(0)
    return bytes(int("".join(map(str, bits[k:k + 8])), 2) for k in range(0, len(bits), 8))


def write_tiff(path, img, compression=1, big=False, rows_per_strip=None, predictor=1, photometric=1):
    e = ">" if big else "<"
    h, w = img.shape
    bits = img.dtype.itemsize * 8
    rps = rows_per_strip or h
    samples = img.astype(img.dtype.newbyteorder(e))
    if predictor == 2:
        samples = samples.copy()
        samples[:, 1:] = (img[:, 1:].astype(np.int64) - img[:, :-1].astype(np.int64)) % (1 << bits)
    strips = []
    for r in range(0, h, rps):
        raw = samples[r:r + rps].tobytes()
        strips.append(raw if compression == 1 else packbits(raw) if compression == 32773 else lzw(raw))
    tags = [(256, 4, [w]), (257, 4, [h]), (258, 3, [bits]), (259, 3, [compression]), (262, 3, [photometric]),
            (273, 4, None), (277, 3, [1]), (278, 4, [rps]), (279, 4, [len(s) for s in strips])]
    if predictor != 1:
        tags.append((317, 3, [predictor]))
    ifd = 8
    extra = ifd + 2 + 12 * len(tags) + 4
    ns = len(strips)
    data_start = extra + 8 * ns
    offs, pos = [], data_start
    for s in strips:
        offs.append(pos)
        pos += len(s)
    tags[5] = (273, 4, offs)
    out = bytearray((b"MM" if big else b"II") + struct.pack(e + "HI", 42, ifd) + struct.pack(e + "H", len(tags)))
    arrays = extra
    for t, typ, vals in tags:
        if len(vals) == 1:
            val = struct.pack(e + "I", vals[0]) if typ == 4 else struct.pack(e + "HH", vals[0], 0)
        else:
            val = struct.pack(e + "I", arrays)
            arrays += 4 * len(vals)
        out += struct.pack(e + "HHI", t, typ, len(vals)) + val
    out += struct.pack(e + "I", 0)
    for t, typ, vals in tags:
        if len(vals) > 1:
            out += struct.pack(e + f"{len(vals)}I", *vals)
    out += bytes(data_start - len(out))
    for s in strips:
        out += s
    path.write_bytes(bytes(out))


# ---------------- TIFF tests ----------------

def test_reference_packbits_strips(qp, rankine_pair):
    a = qp.read_tiff(GOLDEN / "tiff_packbits_rankine.tif")
    assert a.dtype == np.uint8 and a.shape == (64, 512)
    np.testing.assert_array_equal(a, rankine_pair[0][:64])
    assert qp.tiff_info(GOLDEN / "tiff_packbits_rankine.tif") == (64, 512, 8)


def test_reference_lzw_strip(qp):
    c = qp.read_tiff(GOLDEN / "tiff_lzw_chess.tif")
    assert c.shape == (128, 128)
    expect = np.zeros((128, 128), np.uint8)
    expect[:64, 64:] = 255
    expect[64:, :64] = 127
    expect[64:, 64:] = 48
    np.testing.assert_array_equal(c, expect)


@pytest.mark.parametrize("compression", [1, 32773, 5])
@pytest.mark.parametrize("bits", [8, 16])
@pytest.mark.parametrize("big", [False, True])
def test_written_tiffs_round_trip(qp, tmp_path, compression, bits, big):
    rng = np.random.default_rng(compression + bits + big)
    h, w = 37, 53
    if bits == 8:
        img = rng.integers(0, 256, (h, w), dtype=np.uint8)
    else:
        img = rng.integers(0, 4096, (h, w), dtype=np.uint16)   # 12-bit camera range
    img[5:9] = img[5, 0]                                       # runs for PackBits / long LZW strings
    p = tmp_path / "f.tif"
    write_tiff(p, img, compression=compression, big=big, rows_per_strip=8)
    got = qp.read_tiff(p)
    assert got.dtype == img.dtype
    np.testing.assert_array_equal(got, img)


@pytest.mark.parametrize("bits", [8, 16])
def test_lzw_predictor_and_table_resets(qp, tmp_path, bits):
    rng = np.random.default_rng(bits)
    dt = np.uint8 if bits == 8 else np.uint16
    img = np.cumsum(rng.integers(-3, 4, (96, 200)), axis=1).astype(dt)   # smooth rows: predictor helps
    noisy = rng.integers(0, 1 << bits, (96, 200)).astype(dt)              # fills the 4096-entry table
    for src, pred in ((img, 2), (noisy, 1), (noisy, 2)):
        p = tmp_path / f"p{pred}.tif"
        write_tiff(p, src, compression=5, predictor=pred, rows_per_strip=40)
        np.testing.assert_array_equal(qp.read_tiff(p), src)


def test_white_is_zero(qp, tmp_path):
    img = np.arange(256, dtype=np.uint8).reshape(16, 16)
    p = tmp_path / "w.tif"
    write_tiff(p, 255 - img, photometric=0)
    np.testing.assert_array_equal(qp.read_tiff(p), img)


def test_tiff_rejects(qp, tmp_path):
    img = np.zeros((8, 8), np.uint8)
    p = tmp_path / "pal.tif"
    write_tiff(p, img, photometric=3)
    with pytest.raises(qp.QlpivError) as e:
        qp.read_tiff(p)
    assert e.value.status == qp.E_UNSUPPORTED
    good = tmp_path / "g.tif"
    write_tiff(good, np.arange(64 * 64, dtype=np.uint16).reshape(64, 64))
    cut = tmp_path / "cut.tif"
    cut.write_bytes(good.read_bytes()[:-100])
    with pytest.raises(qp.QlpivError) as e:
        qp.read_tiff(cut)
    assert e.value.status == qp.E_SHAPE
    junk = tmp_path / "j.tif"
    junk.write_bytes(b"PK\x03\x04" + bytes(60))
    with pytest.raises(qp.QlpivError) as e:
        qp.read_tiff(junk)
    assert e.value.status == qp.E_SHAPE
    with pytest.raises(qp.QlpivError) as e:
        qp.read_tiff(tmp_path / "missing.tif")
    assert e.value.status == qp.E_ARG
    lib = qp.load_library()
    buf = np.zeros(10, np.uint8)
    assert lib.qlpiv_tiff_read(str(good).encode(), buf.ctypes.data, buf.nbytes) == qp.E_ARG


# ---------------- MATLAB export ----------------

def _maps(rng, frames):
    maps = []
    for n, (ti, tj), step in ((32, (7, 9), 1), (16, (15, 19), 2)):
        u = rng.normal(0, 2, (frames, ti, tj)).astype(np.float32)
        v = rng.normal(0, 2, (frames, ti, tj)).astype(np.float32)
        inv = rng.random((frames, ti, tj)) < 0.1
        maps.append(dict(u=u, v=v, ia=(n, n), adaptive_step=step, margins=(3, 4, 5, 6), invalid=inv))
    return maps


@pytest.mark.parametrize("nan", [False, True])
@pytest.mark.parametrize("layout,swap", [(0, False), (0, True), (1, False)])
def test_mat_export_reads_back(qp, tmp_path, nan, layout, swap):
    sio = pytest.importorskip("scipy.io")
    rng = np.random.default_rng(int(nan) + 2 * layout + 4 * swap)
    maps = _maps(rng, frames=3)
    p = tmp_path / "v.mat"
    qp.export_mat(p, maps, image_height=300, image_width=340, ia_start=32, ia_end=16, overlap_factor=0.5,
                  swap_uv=swap, mark_invalid_as_nan=nan, export_date="Thu Dec 03 12:00:00 UTC 2026", layout=layout)
    head = p.read_bytes()[:128]
    assert head.startswith(b"MATLAB 5.0 - QuickLabPIV-ng Velocities exported on: Thu Dec 03")
    assert head[124:128] == b"\x00\x01IM"
    m = sio.loadmat(p, squeeze_me=False, struct_as_record=True)
    assert str(m["exportDate"][0]) == "Thu Dec 03 12:00:00 UTC 2026"
    par = m["parameters"][0, 0]
    assert par.dtype.names == ("imageWidth", "imageHeight", "iaStartI", "iaEndI", "iaStartJ", "iaEndJ",
                               "overlapFactor", "hasSwappedUVVectors", "markInvalidAsNaN",
                               "totalNumberOfVelocityMaps", "multiVolumeExport", "multiVolumeLastVolume")
    vals = {k: par[k][0, 0] for k in par.dtype.names}
    assert vals["imageWidth"] == 340 and vals["imageHeight"] == 300
    assert (vals["iaStartI"], vals["iaEndI"], vals["iaStartJ"], vals["iaEndJ"]) == (32, 16, 32, 16)
    assert par["imageWidth"].dtype == np.int32 and par["overlapFactor"].dtype == np.float32
    assert vals["overlapFactor"] == np.float32(0.5) and vals["hasSwappedUVVectors"] == int(swap)
    assert vals["markInvalidAsNaN"] == int(nan) and vals["totalNumberOfVelocityMaps"] == 3
    assert vals["multiVolumeExport"] == 0 and vals["multiVolumeLastVolume"] == 1
    third = "multiVolumeExport" if layout == qp.MAT_RUN else "adaptiveStep"
    for mp in maps:
        name = f"velocities{mp['ia'][0]}x{mp['ia'][1]}"
        s = m[name][0, 0]
        assert s.dtype.names == ("iaHeight", "iaWidth", third, "margins", "u", "v")
        assert s["iaHeight"][0, 0] == mp["ia"][0]
        assert s[third][0, 0] == (0 if layout == qp.MAT_RUN else mp["adaptive_step"])
        mg = s["margins"][0, 0]
        assert mg.dtype.names == ("top", "left", "bottom", "right")
        assert [int(mg[k][0, 0]) for k in mg.dtype.names] == [3, 4, 5, 6]
        # end-of-run maps go through PIVMap: u holds the column displacement unless swapped
        rows_first = layout == qp.MAT_STEP or swap
        for comp, src in (("u", "u" if rows_first else "v"), ("v", "v" if rows_first else "u")):
            arr = s[comp]
            assert arr.dtype == np.float32
            expect = np.moveaxis(mp[src], 0, -1)              # tiles_i x tiles_j x frames
            if nan:
                expect = np.where(np.moveaxis(mp["invalid"], 0, -1), np.float32(np.nan), expect)
            np.testing.assert_array_equal(arr, expect)


def test_mat_export_of_an_adaptive_result(qp, tmp_path):
    """Vector maps laid out like piv_adaptive's output (pairs x tiles_i x tiles_j) export with the
    final level's IA size, grid margins and step."""
    sio = pytest.importorskip("scipy.io")
    desc = qp.adaptive_desc(64, 16, 0.5, margins=(2, 2, 3, 3))
    levels = qp.adaptive_levels(desc, 256, 320)
    last = levels[-1]
    u = np.arange(2 * last["tiles_i"] * last["tiles_j"], dtype=np.float32).reshape(2, last["tiles_i"], -1)
    p = tmp_path / "a.mat"
    qp.export_adaptive_mat(p, desc, 256, 320, u, -u)
    s = sio.loadmat(p)["velocities16x16"][0, 0]
    assert s["u"].shape == (last["tiles_i"], last["tiles_j"], 2)
    assert s["multiVolumeExport"][0, 0] == 0
    mg = s["margins"][0, 0]
    assert [int(mg[k][0, 0]) for k in ("top", "left", "bottom", "right")] == \
        [last["margin_top"], last["margin_left"], last["margin_bottom"], last["margin_right"]]
    np.testing.assert_array_equal(s["u"][:, :, 1], -u[1])    # column displacements first (PIVMap)
    np.testing.assert_array_equal(s["v"][:, :, 1], u[1])
    q = tmp_path / "s.mat"
    qp.export_adaptive_mat(q, desc, 256, 320, u, -u, layout=qp.MAT_STEP)
    t = sio.loadmat(q)["velocities16x16"][0, 0]
    assert t["adaptiveStep"][0, 0] == len(levels) - 1
    np.testing.assert_array_equal(t["u"][:, :, 1], u[1])


def test_mat_export_rejects(qp, tmp_path):
    with pytest.raises(qp.QlpivError):
        qp.export_mat(tmp_path / "x.mat", [dict(u=np.zeros((0, 3, 3), np.float32), v=np.zeros((0, 3, 3), np.float32),
                                                 ia=(16, 16))], 64, 64, 16, 16, 0.5)
    with pytest.raises(qp.QlpivError) as e:
        qp.export_mat(tmp_path / "nodir" / "x.mat", [], 64, 64, 16, 16, 0.5)
    assert e.value.status == qp.E_ARG


def test_mat_dense_export(qp, tmp_path):
    """The optical-flow dense layout: one `velocities` struct, u / v over the pixels inside the
    margins, column displacement first (PIVMap), no NaN marking."""
    sio = pytest.importorskip("scipy.io")
    desc = qp.adaptive_desc(64, 32, 0.5, margins=(3, 4, 5, 6))
    h, w = 200, 230
    rng = np.random.default_rng(4)
    du = rng.normal(0, 1, (2, h, w)).astype(np.float32)
    dv = rng.normal(0, 1, (2, h, w)).astype(np.float32)
    p = tmp_path / "d.mat"
    qp.export_dense_mat(p, desc, h, w, du, dv)
    m = sio.loadmat(p)
    assert "velocities" in m and not any(k.startswith("velocities3") for k in m)
    s = m["velocities"][0, 0]
    assert s.dtype.names == ("iaHeight", "iaWidth", "multiVolumeExport", "margins", "u", "v")
    g = qp.adaptive_levels(desc, h, w)[-1]
    t, l, b, r = g["margin_top"], g["margin_left"], g["margin_bottom"], g["margin_right"]
    assert s["u"].shape == (h - t - b, w - l - r, 2)
    np.testing.assert_array_equal(s["u"][:, :, 1], dv[1, t:h - b, l:w - r])
    np.testing.assert_array_equal(s["v"][:, :, 0], du[0, t:h - b, l:w - r])
    with pytest.raises(qp.QlpivError):
        qp.export_mat(tmp_path / "x.mat", [dict(u=du, v=dv, ia=(32, 32), margins=(0, 0, 0, 0))] * 2, h, w, 64, 32,
                      0.5, layout=qp.MAT_DENSE)


@pytest.mark.parametrize("layout", [0, 2])
def test_mat_export_multi_volume(qp, tmp_path, layout):
    """Split exports (ExecuteLocalPIVWorker.java:172-215, StructMultiFrameFloatVelocityExporter.java:80-115,
    185-262): 7 frames at 3 maps per file give _MV0, _MV1 (3 frames each) and _MV2 (1 frame); each
    volume names the next one and records its first frame, the last one is flagged."""
    sio = pytest.importorskip("scipy.io")
    rng = np.random.default_rng(5 + layout)
    maps = _maps(rng, frames=7)
    if layout == qp.MAT_DENSE:
        maps = maps[1:]
    p = tmp_path / "run_MV0.mat"
    qp.export_mat(p, maps, image_height=300, image_width=340, ia_start=32, ia_end=16, overlap_factor=0.5,
                  export_date="Thu Dec 03 12:00:00 UTC 2026", layout=layout, maps_per_file=3)
    for k, (f0, nf) in enumerate([(0, 3), (3, 3), (6, 1)]):
        m = sio.loadmat(tmp_path / f"run_MV{k}.mat", squeeze_me=False, struct_as_record=True)
        par = m["parameters"][0, 0]
        last = k == 2
        names = ("imageWidth", "imageHeight", "iaStartI", "iaEndI", "iaStartJ", "iaEndJ", "overlapFactor",
                 "hasSwappedUVVectors", "markInvalidAsNaN", "totalNumberOfVelocityMaps", "multiVolumeExport",
                 "multiVolumeLastVolume") + (() if last else ("multiVolumeNextFilename",))
        assert par.dtype.names == names
        assert par["totalNumberOfVelocityMaps"][0, 0] == 7 and par["multiVolumeExport"][0, 0] == 1
        assert par["multiVolumeLastVolume"][0, 0] == int(last)
        if not last:
            assert str(par["multiVolumeNextFilename"][0]) == str(tmp_path / f"run_MV{k + 1}.mat")
        for mp in maps:
            name = "velocities" if layout == qp.MAT_DENSE else f"velocities{mp['ia'][0]}x{mp['ia'][1]}"
            s = m[name][0, 0]
            assert s.dtype.names == ("iaHeight", "iaWidth", "multiVolumeExport", "multiVolumeStartOffset",
                                     "margins", "u", "v")
            assert s["multiVolumeExport"][0, 0] == 1 and s["multiVolumeStartOffset"][0, 0] == f0
            g = mp["margins"] if layout == qp.MAT_DENSE else (0, 0, 0, 0)
            cols = np.moveaxis(mp["v"], 0, -1)[g[0]:mp["v"].shape[1] - g[2], g[1]:mp["v"].shape[2] - g[3]]
            np.testing.assert_array_equal(s["u"], cols[:, :, f0:f0 + nf])
    assert not (tmp_path / "run_MV3.mat").exists()
    with pytest.raises(qp.QlpivError):   # the volume names come from _MV0.mat
        qp.export_mat(tmp_path / "run.mat", maps, image_height=300, image_width=340, ia_start=32, ia_end=16,
                      overlap_factor=0.5, layout=layout, maps_per_file=3)
