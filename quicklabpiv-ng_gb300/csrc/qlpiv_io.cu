// Host-side data formats either side of the path: baseline TIFF ingest and MATLAB level-5 export.
// Declarations: include/qlpiv.h (qlpiv_tiff_*, qlpiv_mat_export).
//
//   TIFF  the images ImageReaderJob reads (S/jobs/ImageReaderJob.java:81-115 through ImageIO):
//         greyscale (BlackIsZero or WhiteIsZero), one sample per pixel, 8 or 16 bits, strips,
//         uncompressed, LZW (5, with or without the horizontal predictor) or PackBits (32773),
//         either byte order ("II" / "MM"); the first image of the file.
//   MAT   StructMultiFrameFloatVelocityExporter (S/exporter/StructMultiFrameFloatVelocityExporter.java):
//         a 128-byte level-5 header, `exportDate` (char), `parameters` (struct of int32 / single
//         scalars) and per velocity map a struct `velocities<H>x<W>`: iaHeight, iaWidth, then
//         multiVolumeExport (end-of-run layout, :185-238) or adaptiveStep (per-step layout,
//         :132-181), margins (struct top, left, bottom, right) and u, v (single,
//         tiles_i x tiles_j x frames, MATLAB column-major order); uncompressed elements.
#include <algorithm>
#include <new>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <limits>
#include <string>
#include <vector>

#include "qlpiv.h"
#include "qlpiv_handle.h"

using qlpiv::fail;

namespace {

// ---------------- TIFF ----------------

struct Tiff {
    int width = 0, height = 0, bps = 0, compression = 1, spp = 1, planar = 1;
    int photometric = 1, predictor = 1, rows_per_strip = 0;
    std::vector<uint32_t> offsets, counts;
    bool big = false;
};

bool read_file(const char *path, std::vector<uint8_t> &buf) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0) {
        std::fclose(f);
        return false;
    }
    buf.resize((size_t)n);
    const size_t got = n > 0 ? std::fread(buf.data(), 1, (size_t)n, f) : 0;
    std::fclose(f);
    return got == (size_t)n;
}

uint32_t rd(const std::vector<uint8_t> &b, size_t off, int bytes, bool big) {
    uint32_t v = 0;
    for (int k = 0; k < bytes; k++) {
        const uint32_t byte = b[off + k];
        v |= big ? byte << (8 * (bytes - 1 - k)) : byte << (8 * k);
    }
    return v;
}

// First image file directory only (later pages, thumbnails and private tags are ignored).
qlpiv_status parse_tiff(const std::vector<uint8_t> &b, Tiff &t) {
    if (b.size() < 8) return fail(QLPIV_E_SHAPE, "not a TIFF file (too short)");
    if (b[0] == 'I' && b[1] == 'I') t.big = false;
    else if (b[0] == 'M' && b[1] == 'M') t.big = true;
    else return fail(QLPIV_E_SHAPE, "not a TIFF file (byte order mark)");
    if (rd(b, 2, 2, t.big) != 42) return fail(QLPIV_E_SHAPE, "not a TIFF file (magic)");
    const size_t ifd = rd(b, 4, 4, t.big);
    if (ifd + 2 > b.size()) return fail(QLPIV_E_SHAPE, "TIFF directory out of the file");
    const int n = (int)rd(b, ifd, 2, t.big);
    if (ifd + 2 + 12 * (size_t)n > b.size()) return fail(QLPIV_E_SHAPE, "TIFF directory truncated");
    for (int k = 0; k < n; k++) {
        const size_t e = ifd + 2 + 12 * (size_t)k;
        const uint32_t tag = rd(b, e, 2, t.big), type = rd(b, e + 2, 2, t.big), cnt = rd(b, e + 4, 4, t.big);
        const int size = type == 3 ? 2 : (type == 4 ? 4 : (type == 1 ? 1 : 0));
        if (size == 0 || cnt == 0) continue;  // types the baseline fields below never use
        if (tag != 273 && tag != 279 && cnt != 1) continue;
        const size_t data = (size_t)size * cnt <= 4 ? e + 8 : rd(b, e + 8, 4, t.big);
        if (data + (size_t)size * cnt > b.size()) return fail(QLPIV_E_SHAPE, "TIFF tag %u out of the file", tag);
        std::vector<uint32_t> vals(cnt);
        for (uint32_t q = 0; q < cnt; q++) vals[q] = rd(b, data + (size_t)q * size, size, t.big);
        switch (tag) {
            case 256: t.width = (int)vals[0]; break;
            case 257: t.height = (int)vals[0]; break;
            case 258: t.bps = (int)vals[0]; break;
            case 259: t.compression = (int)vals[0]; break;
            case 262: t.photometric = (int)vals[0]; break;
            case 273: t.offsets = vals; break;
            case 277: t.spp = (int)vals[0]; break;
            case 278: t.rows_per_strip = (int)vals[0]; break;
            case 279: t.counts = vals; break;
            case 284: t.planar = (int)vals[0]; break;
            case 317: t.predictor = (int)vals[0]; break;
            default: break;
        }
    }
    if (t.width <= 0 || t.height <= 0 || t.width > (1 << 20) || t.height > (1 << 20))
        return fail(QLPIV_E_SHAPE, "TIFF image size %d x %d", t.height, t.width);
    if (t.spp != 1) return fail(QLPIV_E_UNSUPPORTED, "TIFF with %d samples per pixel (greyscale only)", t.spp);
    if (t.photometric != 0 && t.photometric != 1)
        return fail(QLPIV_E_UNSUPPORTED, "TIFF photometric interpretation %d (greyscale only)", t.photometric);
    if (t.bps != 8 && t.bps != 16) return fail(QLPIV_E_UNSUPPORTED, "TIFF with %d bits per sample (8 or 16)", t.bps);
    if (t.compression != 1 && t.compression != 5 && t.compression != 32773)
        return fail(QLPIV_E_UNSUPPORTED, "TIFF compression %d (uncompressed, LZW or PackBits)", t.compression);
    if (t.predictor != 1 && t.predictor != 2) return fail(QLPIV_E_UNSUPPORTED, "TIFF predictor %d", t.predictor);
    if (t.offsets.empty() || t.offsets.size() != t.counts.size())
        return fail(QLPIV_E_SHAPE, "TIFF strips missing or inconsistent");
    if (t.rows_per_strip <= 0 || t.rows_per_strip > t.height) t.rows_per_strip = t.height;
    return QLPIV_OK;
}

// PackBits: header n >= 0 copies n + 1 literal bytes, -127..-1 repeats the next byte 1 - n
// times, -128 is a no-op.
qlpiv_status unpack_bits(const uint8_t *p, size_t n, std::vector<uint8_t> &out, size_t want) {
    size_t i = 0;
    while (i < n && out.size() < want) {
        const int hdr = (int)(int8_t)p[i++];
        if (hdr >= 0) {
            const size_t len = (size_t)hdr + 1;
            if (i + len > n) return fail(QLPIV_E_SHAPE, "PackBits literal run past the strip");
            out.insert(out.end(), p + i, p + i + len);
            i += len;
        } else if (hdr != -128) {
            if (i >= n) return fail(QLPIV_E_SHAPE, "PackBits repeat past the strip");
            out.insert(out.end(), (size_t)(1 - hdr), p[i++]);
        }
    }
    return QLPIV_OK;
}

// TIFF LZW (TIFF 6.0 section 13): codes read most significant bit first, 256 = clear,
// 257 = end of information, the code width grows from 9 to 12 bits one code early (when the
// next free entry reaches 511, 1023, 2047).  Strings are kept as (prefix, last byte, length).
qlpiv_status unlzw(const uint8_t *p, size_t n, std::vector<uint8_t> &out, size_t want) {
    static thread_local uint16_t prefix[4096];
    static thread_local uint8_t last[4096], first[4096];
    static thread_local uint16_t len[4096];
    for (int c = 0; c < 256; c++) {
        prefix[c] = 0xFFFF;
        last[c] = first[c] = (uint8_t)c;
        len[c] = 1;
    }
    size_t bitpos = 0;
    const size_t nbits_total = n * 8;
    int width = 9, next = 258, old = -1;
    uint8_t tmp[4096];
    auto emit = [&](int code) {
        const int l = len[code];
        for (int k = l - 1, c = code; k >= 0; k--, c = prefix[c]) tmp[k] = last[c];
        out.insert(out.end(), tmp, tmp + l);
    };
    while (out.size() < want && bitpos + width <= nbits_total) {
        int code = 0;
        for (int k = 0; k < width; k++, bitpos++) code = (code << 1) | ((p[bitpos >> 3] >> (7 - (bitpos & 7))) & 1);
        if (code == 257) break;
        if (code == 256) {
            width = 9;
            next = 258;
            old = -1;
            continue;
        }
        if (old < 0) {
            if (code > 255) return fail(QLPIV_E_SHAPE, "LZW stream starts with code %d", code);
            emit(code);
            old = code;
            continue;
        }
        if (code > next || (code == next && next >= 4096)) return fail(QLPIV_E_SHAPE, "LZW code %d out of the table", code);
        if (next < 4096) {  // new entry: old string + first byte of the current one
            prefix[next] = (uint16_t)old;
            first[next] = first[old];
            last[next] = code < next ? first[code] : first[old];
            len[next] = (uint16_t)(len[old] + 1);
            next++;
        }
        emit(code);
        old = code;
        width = next >= 2047 ? 12 : next >= 1023 ? 11 : next >= 511 ? 10 : 9;
    }
    return QLPIV_OK;
}

// Decodes every strip into `out` (width x height samples of bps bits, host byte order).
qlpiv_status decode_tiff(const std::vector<uint8_t> &b, const Tiff &t, uint8_t *out) {
    const size_t row = (size_t)t.width * (t.bps / 8), need = row * t.height;
    std::vector<uint8_t> raw;
    raw.reserve(need);
    for (size_t s = 0; s < t.offsets.size() && raw.size() < need; s++) {
        const size_t o = t.offsets[s], c = t.counts[s];
        if (o > b.size() || c > b.size() - o) return fail(QLPIV_E_SHAPE, "TIFF strip %zu out of the file", s);
        const size_t rows = std::min((size_t)t.rows_per_strip, (size_t)t.height - s * t.rows_per_strip);
        const size_t want = raw.size() + rows * row;
        qlpiv_status st = QLPIV_OK;
        if (t.compression == 1) raw.insert(raw.end(), b.begin() + o, b.begin() + o + std::min(c, rows * row));
        else if (t.compression == 32773) st = unpack_bits(b.data() + o, c, raw, want);
        else st = unlzw(b.data() + o, c, raw, want);
        if (st) return st;
        if (raw.size() < want) return fail(QLPIV_E_SHAPE, "TIFF strip %zu decodes to %zu of %zu bytes", s,
                                           raw.size() - (want - rows * row), rows * row);
        raw.resize(want);
    }
    if (raw.size() < need) return fail(QLPIV_E_SHAPE, "TIFF data shorter than the image");
    if (t.bps == 8) {
        std::memcpy(out, raw.data(), need);
    } else {
        uint16_t *o16 = reinterpret_cast<uint16_t *>(out);
        for (size_t k = 0; k < need / 2; k++)
            o16[k] = t.big ? (uint16_t)((raw[2 * k] << 8) | raw[2 * k + 1]) : (uint16_t)(raw[2 * k] | (raw[2 * k + 1] << 8));
    }
    const size_t count = (size_t)t.width * t.height;
    if (t.predictor == 2) {  // horizontal differencing: each sample stores the difference to its left neighbour
        for (int y = 0; y < t.height; y++)
            for (int x = 1; x < t.width; x++) {
                const size_t k = (size_t)y * t.width + x;
                if (t.bps == 8) out[k] = (uint8_t)(out[k] + out[k - 1]);
                else reinterpret_cast<uint16_t *>(out)[k] = (uint16_t)(reinterpret_cast<uint16_t *>(out)[k] +
                                                                         reinterpret_cast<uint16_t *>(out)[k - 1]);
            }
    }
    if (t.photometric == 0) {  // WhiteIsZero: store as BlackIsZero
        for (size_t k = 0; k < count; k++) {
            if (t.bps == 8) out[k] = (uint8_t)(255 - out[k]);
            else reinterpret_cast<uint16_t *>(out)[k] = (uint16_t)(65535 - reinterpret_cast<uint16_t *>(out)[k]);
        }
    }
    return QLPIV_OK;
}

// ---------------- MATLAB level 5 ----------------

enum : uint32_t { miINT8 = 1, miINT32 = 5, miUINT32 = 6, miSINGLE = 7, miMATRIX = 14, miUTF8 = 16 };
enum : uint32_t { mxSTRUCT = 2, mxCHAR = 4, mxSINGLE = 7, mxINT32 = 12 };

struct Buf {
    std::vector<uint8_t> b;
    void u32(uint32_t v) {
        for (int k = 0; k < 4; k++) b.push_back((uint8_t)(v >> (8 * k)));
    }
    void i32(int32_t v) { u32((uint32_t)v); }
    void bytes(const void *p, size_t n) {
        const uint8_t *c = static_cast<const uint8_t *>(p);
        b.insert(b.end(), c, c + n);
    }
    void pad8() {
        while (b.size() % 8) b.push_back(0);
    }
    // one data element: tag (type, byte count) then the data padded to 8 bytes
    void element(uint32_t type, const void *p, size_t n) {
        u32(type);
        u32((uint32_t)n);
        bytes(p, n);
        pad8();
    }
};

// A miMATRIX element: flags, dimensions, name, then `body` (already encoded sub-elements).
void matrix(Buf &out, uint32_t cls, const std::vector<int32_t> &dims, const std::string &name, const Buf &body) {
    Buf m;
    const uint32_t flags[2] = {cls, 0};
    m.element(miUINT32, flags, sizeof(flags));
    m.element(miINT32, dims.data(), sizeof(int32_t) * dims.size());
    m.element(miINT8, name.data(), name.size());
    m.bytes(body.b.data(), body.b.size());
    out.u32(miMATRIX);
    out.u32((uint32_t)m.b.size());
    out.bytes(m.b.data(), m.b.size());
}

void int32_scalar(Buf &out, const std::string &name, int32_t v) {
    Buf body;
    body.element(miINT32, &v, 4);
    matrix(out, mxINT32, {1, 1}, name, body);
}

void single_scalar(Buf &out, const std::string &name, float v) {
    Buf body;
    body.element(miSINGLE, &v, 4);
    matrix(out, mxSINGLE, {1, 1}, name, body);
}

void text(Buf &out, const std::string &name, const std::string &s) {
    Buf body;
    body.element(miUTF8, s.data(), s.size());
    matrix(out, mxCHAR, {1, (int32_t)s.size()}, name, body);
}

// A 1 x 1 struct whose fields are already-encoded unnamed matrices (names in `fields`).
void structure(Buf &out, const std::string &name, const std::vector<std::string> &fields, const Buf &values) {
    Buf body;
    const int32_t len = 32;  // field name length, 31 characters and the terminator
    body.u32(miINT32 | (4u << 16));  // small data element: 4 bytes packed into the tag
    body.i32(len);
    std::vector<char> names(fields.size() * len, 0);
    for (size_t k = 0; k < fields.size(); k++) std::strncpy(&names[k * len], fields[k].c_str(), len - 1);
    body.element(miINT8, names.data(), names.size());
    body.bytes(values.b.data(), values.b.size());
    matrix(out, mxSTRUCT, {1, 1}, name, body);
}

}  // namespace

extern "C" {

qlpiv_status qlpiv_tiff_info(const char *path, int *height, int *width, int *bits_per_sample) {
    if (!path || !height || !width || !bits_per_sample) return fail(QLPIV_E_ARG, "NULL argument");
    try {
        std::vector<uint8_t> b;
        if (!read_file(path, b)) return fail(QLPIV_E_ARG, "cannot read %s", path);
        Tiff t;
        if (qlpiv_status st = parse_tiff(b, t)) return st;
        *height = t.height;
        *width = t.width;
        *bits_per_sample = t.bps;
        return QLPIV_OK;
    } catch (const std::bad_alloc &) {
        return fail(QLPIV_E_OOM, "host memory exhausted while reading %s", path);
    }
}

qlpiv_status qlpiv_tiff_read(const char *path, void *pixels, int64_t capacity_bytes) {
    if (!path || !pixels) return fail(QLPIV_E_ARG, "NULL argument");
    // host allocations (file bytes, decoded strips) can fail on a hostile header: report
    // QLPIV_E_OOM instead of letting std::bad_alloc leave an extern "C" function
    try {
        std::vector<uint8_t> b;
        if (!read_file(path, b)) return fail(QLPIV_E_ARG, "cannot read %s", path);
        Tiff t;
        if (qlpiv_status st = parse_tiff(b, t)) return st;
        const int64_t need = (int64_t)t.width * t.height * (t.bps / 8);
        if (capacity_bytes < need) return fail(QLPIV_E_ARG, "buffer of %lld bytes, image needs %lld",
                                              (long long)capacity_bytes, (long long)need);
        // no strip can expand more than an LZW stream (at most 4096 bytes per 9-bit code)
        int64_t strip_bytes = 0;
        for (size_t s = 0; s < t.counts.size(); s++) strip_bytes += (int64_t)t.counts[s];
        if (need > strip_bytes * 4096 + 4096)
            return fail(QLPIV_E_SHAPE, "image of %lld bytes cannot come from %lld bytes of strips", (long long)need,
                        (long long)strip_bytes);
        return decode_tiff(b, t, static_cast<uint8_t *>(pixels));
    } catch (const std::bad_alloc &) {
        return fail(QLPIV_E_OOM, "host memory exhausted while decoding %s", path);
    }
}

// One MAT file holding frames [f0, f0 + nf) of the maps; multi: one volume of a multi-volume export
// (next: the following volume's file name, empty for the last volume).
static qlpiv_status write_volume(const char *path, const qlpiv_mat_export_params *p, int num_maps,
                                 const qlpiv_mat_velocity_map *maps, int f0, int nf, bool multi,
                                 const std::string &next);

static qlpiv_status mat_export_body(const char *path, const qlpiv_mat_export_params *p, int num_maps,
                                    const qlpiv_mat_velocity_map *maps) {
    if (!path || !p || (num_maps > 0 && !maps)) return fail(QLPIV_E_ARG, "NULL argument");
    if (p->maps_per_file < 0) return fail(QLPIV_E_ARG, "maps_per_file < 0");
    if (p->maps_per_file == 0 || p->maps_per_file >= p->frames)
        return write_volume(path, p, num_maps, maps, 0, p->frames, false, "");
    if (p->layout == QLPIV_MAT_STEP) return fail(QLPIV_E_ARG, "the per-step layout is not split into volumes");
    const std::string base(path);
    const size_t at = base.find("_MV0.mat");
    if (at == std::string::npos) return fail(QLPIV_E_ARG, "a multi-volume export path must contain _MV0.mat");
    auto volume = [&](int k) {
        return base.substr(0, at) + "_MV" + std::to_string(k) + ".mat" + base.substr(at + 8);
    };
    const int volumes = (p->frames + p->maps_per_file - 1) / p->maps_per_file;
    for (int k = 0; k < volumes; k++) {
        const int f0 = k * p->maps_per_file;
        const int nf = p->frames - f0 < p->maps_per_file ? p->frames - f0 : p->maps_per_file;
        const qlpiv_status st =
            write_volume(volume(k).c_str(), p, num_maps, maps, f0, nf, true, k + 1 < volumes ? volume(k + 1) : "");
        if (st != QLPIV_OK) return st;
    }
    return QLPIV_OK;
}

static qlpiv_status write_volume(const char *path, const qlpiv_mat_export_params *p, int num_maps,
                                 const qlpiv_mat_velocity_map *maps, int f0, int nf, bool multi,
                                 const std::string &next) {
    if (num_maps < 0 || p->frames <= 0) return fail(QLPIV_E_ARG, "num_maps < 0 or frames <= 0");
    if (p->layout != QLPIV_MAT_RUN && p->layout != QLPIV_MAT_STEP && p->layout != QLPIV_MAT_DENSE)
        return fail(QLPIV_E_ARG, "layout %d", p->layout);
    if (p->layout == QLPIV_MAT_DENSE && num_maps != 1) return fail(QLPIV_E_ARG, "the dense layout holds one map");
    for (int m = 0; m < num_maps && p->layout == QLPIV_MAT_DENSE; m++) {
        const int *g = maps[m].margins;
        if (g[0] < 0 || g[1] < 0 || g[2] < 0 || g[3] < 0 || g[0] + g[2] >= maps[m].tiles_i ||
            g[1] + g[3] >= maps[m].tiles_j)
            return fail(QLPIV_E_ARG, "dense map: margins leave no pixels");
    }
    for (int m = 0; m < num_maps; m++)
        if (!maps[m].u || !maps[m].v || maps[m].tiles_i <= 0 || maps[m].tiles_j <= 0)
            return fail(QLPIV_E_ARG, "velocity map %d: NULL data or empty grid", m);
    Buf out;
    // 128-byte header: zero-padded text, subsystem offset, version 0x0100, endian indicator "IM"
    char header[116];
    std::memset(header, 0, sizeof(header));
    std::string date;
    if (p->export_date) {
        date = p->export_date;
    } else {
        const std::time_t now = std::time(nullptr);
        char tb[64];
        std::strftime(tb, sizeof(tb), "%a %b %d %H:%M:%S %Y", std::gmtime(&now));
        date = tb;
    }
    const std::string title = "MATLAB 5.0 - QuickLabPIV-ng Velocities exported on: " + date;
    std::memcpy(header, title.data(), title.size() < sizeof(header) ? title.size() : sizeof(header));
    out.bytes(header, sizeof(header));
    const uint8_t subsys[8] = {0};
    out.bytes(subsys, 8);
    const uint16_t version = 0x0100;
    out.bytes(&version, 2);
    out.bytes("IM", 2);
    text(out, "exportDate", date);
    {
        Buf v;
        std::vector<std::string> names = {"imageWidth", "imageHeight", "iaStartI", "iaEndI", "iaStartJ", "iaEndJ",
                                          "overlapFactor", "hasSwappedUVVectors", "markInvalidAsNaN",
                                          "totalNumberOfVelocityMaps", "multiVolumeExport", "multiVolumeLastVolume"};
        if (multi && !next.empty()) names.push_back("multiVolumeNextFilename");
        int32_scalar(v, "", p->image_width);
        int32_scalar(v, "", p->image_height);
        int32_scalar(v, "", p->ia_start);
        int32_scalar(v, "", p->ia_end);
        int32_scalar(v, "", p->ia_start);
        int32_scalar(v, "", p->ia_end);
        single_scalar(v, "", p->overlap_factor);
        int32_scalar(v, "", p->swap_uv ? 1 : 0);
        int32_scalar(v, "", p->mark_invalid_as_nan ? 1 : 0);
        int32_scalar(v, "", p->frames);
        int32_scalar(v, "", multi ? 1 : 0);
        int32_scalar(v, "", multi && !next.empty() ? 0 : 1);
        if (multi && !next.empty()) text(v, "", next);
        structure(out, "parameters", names, v);
    }
    for (int m = 0; m < num_maps; m++) {
        const qlpiv_mat_velocity_map &mp = maps[m];
        Buf v;
        const bool run = p->layout != QLPIV_MAT_STEP, dense = p->layout == QLPIV_MAT_DENSE;
        // dense maps (exportDenseDataToFile, :240-290) cover the image inside the margins
        const int r0 = dense ? mp.margins[0] : 0, c0 = dense ? mp.margins[1] : 0;
        const int rows_out = dense ? mp.tiles_i - mp.margins[0] - mp.margins[2] : mp.tiles_i;
        const int cols_out = dense ? mp.tiles_j - mp.margins[1] - mp.margins[3] : mp.tiles_j;
        int32_scalar(v, "", mp.ia_height);
        int32_scalar(v, "", mp.ia_width);
        int32_scalar(v, "", run ? (multi ? 1 : 0) : mp.adaptive_step);  // multiVolumeExport or adaptiveStep
        if (multi) int32_scalar(v, "", f0);                              // multiVolumeStartOffset
        {
            Buf mv;
            int32_scalar(mv, "", mp.margins[0]);
            int32_scalar(mv, "", mp.margins[1]);
            int32_scalar(mv, "", mp.margins[2]);
            int32_scalar(mv, "", mp.margins[3]);
            structure(v, "", {"top", "left", "bottom", "right"}, mv);
        }
        const size_t per = (size_t)mp.tiles_i * mp.tiles_j;
        for (int comp = 0; comp < 2; comp++) {
            // end-of-run maps go through PIVMap: u is the column displacement unless swapped
            const bool rows = run ? (comp == 0) == (p->swap_uv != 0) : comp == 0;
            const float *src = rows ? mp.u : mp.v;
            // MATLAB order: i fastest, then j, then the frame
            std::vector<float> col((size_t)rows_out * cols_out * nf);
            size_t k = 0;
            for (int f = f0; f < f0 + nf; f++)
                for (int j = 0; j < cols_out; j++)
                    for (int i = 0; i < rows_out; i++) {
                        const size_t s = f * per + (size_t)(i + r0) * mp.tiles_j + (j + c0);
                        const bool bad = !dense && p->mark_invalid_as_nan && mp.invalid && mp.invalid[s];
                        col[k++] = bad ? std::numeric_limits<float>::quiet_NaN() : src[s];
                    }
            Buf body;
            body.element(miSINGLE, col.data(), sizeof(float) * col.size());
            matrix(v, mxSINGLE, {rows_out, cols_out, nf}, "", body);
        }
        const std::string name = dense ? std::string("velocities")
                                       : "velocities" + std::to_string(mp.ia_height) + "x" + std::to_string(mp.ia_width);
        std::vector<std::string> fields = {"iaHeight", "iaWidth", run ? "multiVolumeExport" : "adaptiveStep"};
        if (multi) fields.push_back("multiVolumeStartOffset");
        for (const char *f : {"margins", "u", "v"}) fields.push_back(f);
        structure(out, name, fields, v);
    }
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(QLPIV_E_ARG, "cannot create %s", path);
    const size_t wrote = std::fwrite(out.b.data(), 1, out.b.size(), f);
    const int closed = std::fclose(f);
    if (wrote != out.b.size() || closed != 0) return fail(QLPIV_E_ARG, "short write to %s", path);
    return QLPIV_OK;
}

qlpiv_status qlpiv_mat_export(const char *path, const qlpiv_mat_export_params *p, int num_maps,
                              const qlpiv_mat_velocity_map *maps) {
    try {
        return mat_export_body(path, p, num_maps, maps);
    } catch (const std::bad_alloc &) {
        return fail(QLPIV_E_OOM, "host memory exhausted while building the MAT file");
    }
}

}  // extern "C"
