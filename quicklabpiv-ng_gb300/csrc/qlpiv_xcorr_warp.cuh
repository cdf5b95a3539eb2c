// K1 for IA 16: one warp per interrogation area, every FFT in registers.
//
// Same result contract as xcorr_kernel (qlpiv_xcorr.cuh): tile gather with zero fill, maxima floored
// at 16, v/max*16+1 normalisation, the (2N-1)^2 = 31 x 31 correlation plane of the mirrored-A /
// B real pair, FindMaximumFromCenter's total order (or FindMaximumMultiPeaks), the sub-pixel fit
// queue.  The reference's arithmetic is in S/jobs/xcorr/FastRealFFTXCorr.java:44-116 and
// S/maximum/FindMaximumFromCenter.java:33-183 (S/ = src/main/java/pt/quickLabPIV/).
//
// Each warp works through its own IAs (grid-stride over warps) with no CTA barrier.  With
// M = 32 and z = a' + i b' zero outside [0,16)^2, a lane never holds more than 16 complex values
// of one line: the length-32 transforms are split by the parity of the output index (a
// decimation in frequency done on the inputs), so each lane runs one 16-point transform in
// registers per step.
//   A  row pass     lane (r, p) = (L & 15, L >> 4): R[r][2m+p] = FFT16(z[r][j] w32^(jp))[m]; the
//                   upper half of every row is zero, so the split costs only the twiddles.
//   B  columns      lane L = column k2: Z[2m][L] = FFT16(R[.][L]), Z[2m+1][L] = FFT16(R[i][L] w32^i);
//                   the Hermitian product P = F G / M^2 pairs Z(k) with Z(-k), held by lane
//                   (32 - L) & 31 (shuffles); the inverse column transform of column c is split
//                   between lanes c and 32 - c (even / odd k1 halves, recombined by one exchange);
//                   the two self-mirrored columns 0 and 16 travel packed as P0 + i P16.
//   C  row pairs    lane (p, s): rows 2p, 2p+1 of the Hermitian spectrum packed into one complex
//                   inverse transform, outputs j = 2m + s; the plane goes to shared memory for the
//                   sub-pixel stencil and the multi-peak search, the peak is scored in registers.
// Shared memory per warp: one exchange buffer (rows -> columns, columns -> row pairs), the
// plane, the fit queue.
#pragma once
#include "qlpiv_div.cuh"
#include "qlpiv_xcorr.cuh"

namespace qlpiv {

namespace w16 {

constexpr int kWarps = 4;            // warps (IAs in flight) per CTA
constexpr int kThreads = 32 * kWarps;
constexpr int kMinBlocks = 4;        // 16 warps per SM
constexpr int N = 16, M = 32, D = 31;
constexpr int XS = 17;               // exchange stride A -> B (complex), odd
constexpr int QS = 34;               // exchange stride B -> C (complex), even: 16-byte row pairs
constexpr int PS = 43;               // plane row stride (floats), odd: the multi-peak cell reads
                                     // (3 x 3 cells of 32 records) spread over the banks
constexpr int kXchgCplx = (32 * XS > 17 * QS ? 32 * XS : 17 * QS);  // 578
constexpr int kPlaneFloats = D * PS;
// per-warp shared memory (bytes): exchange, plane, reduction words, fit queue, multi-peak list
constexpr size_t kWarpSmem = sizeof(cplx) * kXchgCplx + sizeof(float) * kPlaneFloats + 8 * 8 +
                             32 * sizeof(FitRec) + 3 * 4 * (QLPIV_MAX_PEAKS + 1) + 4;
constexpr size_t kWarpSmemAligned = (kWarpSmem + 15) & ~(size_t)15;

// cos / sin of 2 pi n / 32, n = 0..16 (exact 0 and 1 at n = 8, 16).
__device__ __forceinline__ constexpr float cos32(int n) {
    return n == 0 ? 1.0f : n == 1 ? 0.98078525066375732f : n == 2 ? 0.92387950420379639f
         : n == 3 ? 0.83146959543228149f : n == 4 ? 0.70710676908493042f : n == 5 ? 0.55557024478912354f
         : n == 6 ? 0.38268342614173889f : n == 7 ? 0.19509032368659973f : n == 8 ? 0.0f
         : n == 9 ? -0.19509032368659973f : n == 10 ? -0.38268342614173889f : n == 11 ? -0.55557024478912354f
         : n == 12 ? -0.70710676908493042f : n == 13 ? -0.83146959543228149f : n == 14 ? -0.92387950420379639f
         : n == 15 ? -0.98078525066375732f : -1.0f;
}
__device__ __forceinline__ constexpr float sin32(int n) { return n <= 8 ? cos32(8 - n) : cos32(n - 8); }

// x * w32^(sgn e) with w32 = exp(-2 pi i / 32): forward (INV false) multiplies by
// (cos, -sin), inverse by (cos, +sin).  e in 0..16, compile-time.
template <bool INV>
__device__ __forceinline__ cplx tw32(cplx x, int e) {
    const float c = cos32(e), s = INV ? sin32(e) : -sin32(e);
    if (e == 0) return x;
    if (e == 8) return INV ? cplx{-x.y, x.x} : cplx{x.y, -x.x};
    return cplx{x.x * c - x.y * s, x.x * s + x.y * c};
}

// 16-point DFT in registers, natural order in and out: radix 4 x 4 (index n = q + 4t,
// k = k1 + 4 k2), twiddles w16^(q k1) = w32^(2 q k1).
template <bool INV>
__device__ __forceinline__ void fft16(cplx *x) {
    cplx b[16];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        cplx a0 = x[q], a1 = x[q + 4], a2 = x[q + 8], a3 = x[q + 12];
        dft4<INV>(a0, a1, a2, a3);
        b[q * 4 + 0] = a0;
        b[q * 4 + 1] = tw32<INV>(a1, 2 * q);
        b[q * 4 + 2] = tw32<INV>(a2, 4 * q);
        b[q * 4 + 3] = tw32<INV>(a3, 6 * q > 16 ? 0 : 6 * q);
    }
    // w32^(6q) for q = 3 is w32^18 = -w32^2
    if (true) {
        const cplx t = tw32<INV>(b[3 * 4 + 3], 2);
        b[3 * 4 + 3] = cplx{-t.x, -t.y};
    }
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
        cplx c0 = b[0 * 4 + k1], c1 = b[1 * 4 + k1], c2 = b[2 * 4 + k1], c3 = b[3 * 4 + k1];
        dft4<INV>(c0, c1, c2, c3);
        x[k1] = c0;
        x[k1 + 4] = c1;
        x[k1 + 8] = c2;
        x[k1 + 12] = c3;
    }
}

struct WarpSmem {
    cplx *x;       // exchange buffer
    float *plane;  // D rows of PS floats
    uint64_t *red;
    FitRec *fitq;
    float *mp_lv;
    int *mp_li, *mp_lj;
};

__device__ __forceinline__ WarpSmem warp_smem(unsigned char *base, int warp) {
    unsigned char *p = base + (size_t)warp * kWarpSmemAligned;
    WarpSmem s;
    s.x = reinterpret_cast<cplx *>(p);
    s.plane = reinterpret_cast<float *>(s.x + kXchgCplx);
    s.red = reinterpret_cast<uint64_t *>(s.plane + kPlaneFloats + (kPlaneFloats & 1));
    s.fitq = reinterpret_cast<FitRec *>(s.red + 8);
    s.mp_lv = reinterpret_cast<float *>(s.fitq + 32);
    s.mp_li = reinterpret_cast<int *>(s.mp_lv + QLPIV_MAX_PEAKS + 1);
    s.mp_lj = s.mp_li + QLPIV_MAX_PEAKS + 1;
    return s;
}

}  // namespace w16

// One IA of the warp kernel by the 32 lanes of one warp (shared memory sm, P-point stencils at
// fitv): fits queued at sm.fitq[qn..) and flushed every 32, or (BATCH) staged as entry nb of mpb.
template <typename Pix, bool PP, bool BATCH>
__device__ __forceinline__ void xcorr16_warp_ia(const IaJob &job, long ia, const w16::WarpSmem &sm, float *fitv,
                                                int lane, int &qn, MpBatch *mpb, int &nb) {
    using namespace w16;
    const int multi = job.num_peaks;
    const int KQ = multi > 0 ? multi : 1;
    // lane roles
    const int r_row = lane & 15, r_par = lane >> 4;        // phase A and C: line and output parity
    const int partner = (lane == 0) ? 16 : (lane == 16 ? 0 : 32 - lane);
    const bool role_o = lane >= 16;                        // lanes 16..31: odd half of column 32 - L
    // column of the inverse column task: lanes 0 and 16 share the packed columns 0 + i 16
    const int colL = lane == 16 ? 0 : (lane < 16 ? lane : 32 - lane);
    const int src_mirror = (32 - lane) & 31;               // holder of Z(., -L)
    auto P = [&](int i, int j) -> float { return sm.plane[i * PS + j]; };
    const Pix *imgA, *imgB;
    long pitch_a, pitch_b;
    int img_h, img_w;
    if (job.frames != nullptr) {
        const int fi = job.frame_idx[ia];
        const qlpiv_frame fr = (unsigned)fi < (unsigned)job.num_frames ? job.frames[fi] : qlpiv_frame{};
        imgA = reinterpret_cast<const Pix *>(fr.img_a);
        imgB = reinterpret_cast<const Pix *>(fr.img_b);
        pitch_a = pitch_b = (long)fr.pitch;
        img_h = fr.height;
        img_w = fr.width;
    } else {
        imgA = reinterpret_cast<const Pix *>(job.img_a);
        imgB = reinterpret_cast<const Pix *>(job.img_b);
        pitch_a = job.pitch_a;
        pitch_b = job.pitch_b;
        img_h = job.h;
        img_w = job.w;
    }
    int at, al, bt, bl;
    if (job.a_top != nullptr) {
        at = job.a_top[ia]; al = job.a_left[ia];
        bt = job.b_top[ia]; bl = job.b_left[ia];
    } else {
        at = bt = (int)(ia * N);
        al = bl = 0;
    }

    // ---- A. row r_row of z: A mirrored (row N-1-r, columns reversed), B direct ----
    float ra[16], rb[16];
    float mxa = 0.0f, mxb = 0.0f;
    if (at >= 0 && al >= 0 && at + N <= img_h && al + N <= img_w && bt >= 0 && bl >= 0 && bt + N <= img_h &&
        bl + N <= img_w) {
        // both tiles inside the image: plain loads from the two row bases
        const Pix *rowA = imgA + (long)(at + N - 1 - r_row) * pitch_a + al;
        const Pix *rowB = imgB + (long)(bt + r_row) * pitch_b + bl;
#pragma unroll
        for (int j = 0; j < 16; j++) {
            ra[j] = (float)__ldg(rowA + (N - 1 - j));
            rb[j] = (float)__ldg(rowB + j);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 16; j++) {
            ra[j] = load_pix(imgA, pitch_a, img_h, img_w, at + (N - 1 - r_row), al + (N - 1 - j));
            rb[j] = load_pix(imgB, pitch_b, img_h, img_w, bt + r_row, bl + j);
        }
    }
#pragma unroll
    for (int j = 0; j < 16; j++) {
        mxa = fmaxf(mxa, ra[j]);
        mxb = fmaxf(mxb, rb[j]);
    }
    float maxA, maxB;
    if (job.max_mode == QLPIV_MAX_COMPUTE || job.max_mode == QLPIV_MAX_FIXED_A ||
        job.max_mode == QLPIV_MAX_FIXED_B) {
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {  // lanes r and r + 16 hold the same row
            mxa = fmaxf(mxa, __shfl_xor_sync(0xffffffffu, mxa, o));
            mxb = fmaxf(mxb, __shfl_xor_sync(0xffffffffu, mxb, o));
        }
        maxA = job.max_mode == QLPIV_MAX_FIXED_A ? job.fixed_max_a : fmaxf(mxa, 16.0f);
        maxB = job.max_mode == QLPIV_MAX_FIXED_B ? job.fixed_max_b : fmaxf(mxb, 16.0f);
    } else if (job.max_mode == QLPIV_MAX_GIVEN) {
        maxA = job.max_a[ia];
        maxB = job.max_b[ia];
    } else {
        maxA = job.fixed_max_a;
        maxB = job.fixed_max_b;
    }
    if (job.norm_mode == QLPIV_NORM_MAX_A) maxB = maxA;
    const bool normalize = job.norm_mode != QLPIV_NORM_NONE;
    cplx x[16];
    {
        // integer pixels and integer maxima up to 65535: the correction-step division is exact
        const bool int_div = sizeof(Pix) <= 2 && maxA == rintf(maxA) && maxB == rintf(maxB) && maxA >= 1.0f &&
                             maxB >= 1.0f && maxA <= 65535.0f && maxB <= 65535.0f;
        const float rA = __frcp_rn(maxA), rB = __frcp_rn(maxB);
        if (normalize && int_div) {
#pragma unroll
            for (int j = 0; j < 16; j++) {
                ra[j] = __fadd_rn(__fmul_rn(div_int(ra[j], maxA, rA), 16.0f), 1.0f);
                rb[j] = __fadd_rn(__fmul_rn(div_int(rb[j], maxB, rB), 16.0f), 1.0f);
            }
        } else if (normalize) {
#pragma unroll
            for (int j = 0; j < 16; j++) {
                ra[j] = __fadd_rn(__fmul_rn(__fdiv_rn(ra[j], maxA), 16.0f), 1.0f);
                rb[j] = __fadd_rn(__fmul_rn(__fdiv_rn(rb[j], maxB), 16.0f), 1.0f);
            }
        }
#pragma unroll
        for (int j = 0; j < 16; j++) {
            // odd outputs: inputs times w32^j
            const cplx v{ra[j], rb[j]};
            const cplx t = tw32<false>(v, j);
            x[j] = r_par ? t : v;
        }
    }
    fft16<false>(x);
    cplx *X = sm.x;
#pragma unroll
    for (int m = 0; m < 16; m++) X[(2 * m + r_par) * XS + r_row] = x[m];
    __syncwarp();

    // ---- B. column lane = k2 ----
    cplx E[16], O[16];
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const cplx y = X[lane * XS + i];
        E[i] = y;
        O[i] = tw32<false>(y, i);
    }
    fft16<false>(E);  // Z[2m][lane]
    fft16<false>(O);  // Z[2m+1][lane]
    // Hermitian product P = F G / M^2 with the mirror Z(-k1, -k2) from lane (32 - L) & 31:
    // even k1 = 2m pairs with 2((16 - m) & 15), odd 2m + 1 with 2(15 - m) + 1
    constexpr float kScale = 0.25f / (float)(M * M);
    auto prod = [](cplx a, cplx zm) -> cplx {
        const float fr = a.x + zm.x, fi = a.y - zm.y;
        const float gr = a.y + zm.y, gi = zm.x - a.x;
        return cplx{(fr * gr - fi * gi) * kScale, (fr * gi + fi * gr) * kScale};
    };
#pragma unroll
    for (int m = 0; m <= 8; m++) {
        const int mm = (16 - m) & 15;
        const cplx sa = E[mm], sb = E[m];
        cplx za, zb;
        za.x = __shfl_sync(0xffffffffu, sa.x, src_mirror);
        za.y = __shfl_sync(0xffffffffu, sa.y, src_mirror);
        if (mm != m) {
            zb.x = __shfl_sync(0xffffffffu, sb.x, src_mirror);
            zb.y = __shfl_sync(0xffffffffu, sb.y, src_mirror);
        }
        E[m] = prod(E[m], za);
        if (mm != m) E[mm] = prod(E[mm], zb);
    }
#pragma unroll
    for (int m = 0; m < 8; m++) {
        const int mm = 15 - m;
        const cplx sa = O[mm], sb = O[m];
        cplx za, zb;
        za.x = __shfl_sync(0xffffffffu, sa.x, src_mirror);
        za.y = __shfl_sync(0xffffffffu, sa.y, src_mirror);
        zb.x = __shfl_sync(0xffffffffu, sb.x, src_mirror);
        zb.y = __shfl_sync(0xffffffffu, sb.y, src_mirror);
        O[m] = prod(O[m], za);
        O[mm] = prod(O[mm], zb);
    }
    // inverse column transform of column colL, split over the lane pair: the even-k1 half on
    // lanes 0..15 (lane 0: columns 0 and 16 packed), the odd-k1 half on lanes 16..31, rebuilt
    // from P(2m+1, c) = conj(P(2(15-m)+1, 32-c)); lanes 0 / 16 trade their packed halves
#pragma unroll
    for (int m = 0; m < 16; m++) {
        const cplx snd = lane == 16 ? E[m] : O[m];
        cplx got;
        got.x = __shfl_sync(0xffffffffu, snd.x, lane ^ 16);
        got.y = __shfl_sync(0xffffffffu, snd.y, lane ^ 16);
        cplx in;
        if (!role_o) {
            in = E[m];
            if (lane == 0) in = cplx{E[m].x - got.y, E[m].y + got.x};   // P0 + i P16 (even half)
        } else {
            const cplx c = O[15 - m];
            in = cplx{c.x, -c.y};
            if (lane == 16) in = cplx{got.x - O[m].y, got.y + O[m].x};  // P0 + i P16 (odd half)
        }
        E[m] = in;
    }
    fft16<true>(E);  // lanes 0..15: e(i) of column colL; lanes 16..31: o(i)
    // q(i) = e(i) + w32^-i o(i), q(i + 16) = e(i) - w32^-i o(i)
    __syncwarp();    // every lane has read its column from the exchange buffer
#pragma unroll
    for (int i = 0; i < 16; i += 2) {
        // two consecutive rows per 16-byte store (8 lanes per wavefront, no bank conflict)
        cplx q2[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            cplx other;
            other.x = __shfl_sync(0xffffffffu, E[i + h].x, partner);
            other.y = __shfl_sync(0xffffffffu, E[i + h].y, partner);
            const cplx e = role_o ? other : E[i + h];
            const cplx o = tw32<true>(role_o ? E[i + h] : other, i + h);
            q2[h] = role_o ? cplx{e.x - o.x, e.y - o.y} : cplx{e.x + o.x, e.y + o.y};
        }
        *reinterpret_cast<float4 *>(X + colL * QS + (role_o ? 16 : 0) + i) =
            make_float4(q2[0].x, q2[0].y, q2[1].x, q2[1].y);
    }
    __syncwarp();

    // ---- C. row pair (2p, 2p+1), outputs j = 2m + s ----
    const int i1 = 2 * r_row, i2 = i1 + 1;
    {
        cplx y[16];
        // rows i1, i2 of one column as one 16-byte load: (q(i1, c), q(i2, c))
        auto rows = [&](int c) -> float4 { return *reinterpret_cast<const float4 *>(X + c * QS + i1); };
        const float4 ab0 = rows(0);  // column 0: (q(., 0), q(., 16)) packed, both real
        const float sgn = r_par ? -1.0f : 1.0f;
#pragma unroll
        for (int n = 0; n < 16; n++) {
            cplx lo, hi;  // y[n], y[n + 16]
            if (n == 0) {
                lo = cplx{ab0.x, ab0.z};
                hi = cplx{ab0.y, ab0.w};
            } else {
                const float4 ab = rows(n), ab2 = rows(16 - n);
                lo = cplx{ab.x - ab.w, ab.y + ab.z};
                hi = cplx{ab2.x + ab2.w, ab2.z - ab2.y};  // conj(q1(16-n)) + i conj(q2(16-n))
            }
            const cplx s = cplx{lo.x + sgn * hi.x, lo.y + sgn * hi.y};
            const cplx t = tw32<true>(s, n);
            y[n] = r_par ? t : s;
        }
        fft16<true>(y);
        // plane rows i1, i2 (i2 = 31 lies outside the 31 x 31 plane)
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int j = 2 * m + r_par;
            x[m] = y[m];
            if (j < D) {
                sm.plane[i1 * PS + j] = y[m].x;
                if (i2 < D) sm.plane[i2 * PS + j] = y[m].y;
            }
            if (job.planes != nullptr && j < D) {
                float *pl = job.planes + ia * (long)(D * D);
                pl[i1 * D + j] = y[m].x;
                if (i2 < D) pl[i2 * D + j] = y[m].y;
            }
        }
    }
    __syncwarp();

    // ---- peak: FindMaximumFromCenter over rows / columns 1..D-1, or FindMaximumMultiPeaks ----
    float minf = 3.402823466e38f;
    if (!BATCH && multi == 0) {
        float mv = -3.402823466e38f;
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int j = 2 * m + r_par;
            const bool jok = j >= 1 && j <= D - 1;
            if (jok && i1 >= 1) { mv = fmaxf(mv, x[m].x); minf = fminf(minf, x[m].x); }
            if (jok && i2 <= D - 1) { mv = fmaxf(mv, x[m].y); minf = fminf(minf, x[m].y); }
        }
        uint64_t best = 0ull;
        uint32_t best_ij = 0u;
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int j = 2 * m + r_par;
            const bool jok = j >= 1 && j <= D - 1;
            if (jok && i1 >= 1 && x[m].x == mv) {
                const uint64_t k = peak_key(x[m].x, i1, j, N);
                if (k > best) { best = k; best_ij = ((uint32_t)i1 << 16) | (uint32_t)j; }
            }
            if (jok && i2 <= D - 1 && x[m].y == mv) {
                const uint64_t k = peak_key(x[m].y, i2, j, N);
                if (k > best) { best = k; best_ij = ((uint32_t)i2 << 16) | (uint32_t)j; }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const uint64_t ok = __shfl_xor_sync(0xffffffffu, best, o);
            const uint32_t oij = __shfl_xor_sync(0xffffffffu, best_ij, o);
            if (ok > best) { best = ok; best_ij = oij; }
            minf = fminf(minf, __shfl_xor_sync(0xffffffffu, minf, o));
        }
        if (lane == 0) {
            FitRec r;
            r.ia = ia;
            r.mn = minf;
            r.pi = 0;
            r.pj = 0;
            r.pv = 0.0f;
            if (best != 0ull) {
                r.pi = (int)(best_ij >> 16);
                r.pj = (int)(best_ij & 0xffffu);
                r.pv = __uint_as_float((uint32_t)(best >> 32));
            }
            r.slot = 0;
            r.npk = 1;
            fit_stencil<D>(r, job, P, fitv + qn * 2 * job.subpix_pixels);
            sm.fitq[qn] = r;
        }
    } else {
        // FindMaximumMultiPeaks visits every cell of the plane
#pragma unroll
        for (int m = 0; m < 16; m++) {
            const int j = 2 * m + r_par;
            if (j <= D - 1) {
                minf = fminf(minf, x[m].x);
                if (i2 <= D - 1) minf = fminf(minf, x[m].y);
            }
        }
        if (!BATCH) {
            multipeak_core<D, 32>(job, ia, minf, P, sm.x, sm.red, sm.fitq, fitv, qn, sm.mp_lv, sm.mp_li,
                                  sm.mp_lj);
        } else {
            multipeak_stage<D, 32>(job, ia, minf, P, sm.x, sm.red, mpb, nb);
            if (++nb == kMpBatch) {
                mp_batch_run<D, PP>(mpb, nb, lane, job, sm.fitq, fitv);
                nb = 0;
            }
        }
    }
    if (!BATCH) {
        qn += KQ;
        if (qn + KQ > 32) {
            fit_flush<D, PP>(sm.fitq, fitv, qn, lane, job);
            qn = 0;
        }
    }
    __syncwarp();  // the exchange buffer and the plane are rewritten by the next IA
}

// BATCH: the instantiation for the batched multi-peak replay, launched for multi-peak jobs with
// batch buffers only; a warp that finds no free batch leaves its IAs to the per-IA retry launch.
template <typename Pix, bool PP, bool BATCH>
__global__ void __launch_bounds__(w16::kThreads, w16::kMinBlocks) xcorr16_warp_kernel(IaJob job) {
    using namespace w16;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // P-point stencils of the whole CTA's fit queues follow the per-warp blocks
    float *fitv_all = reinterpret_cast<float *>(smem_raw + kWarps * kWarpSmemAligned);
    float *fitv = fitv_all + (size_t)warp * 32 * 2 * (job.subpix_pixels > 0 ? job.subpix_pixels : 1);
    const WarpSmem sm = warp_smem(smem_raw, warp);
    const int multi = job.num_peaks;
    int qn = 0;
    const long warps_total = (long)gridDim.x * kWarps;

    // batched multi-peak replay: a batch claimed for this warp and its fill
    MpBatch *mpb = nullptr;
    const long count = job.ia_list != nullptr ? (long)job.ia_list[0] : job.count;
    if (BATCH) {
        int slot = -1;
        if (lane == 0 && multi > 0 && mp_batched(job))
            slot = mp_claim(job.mp_slots, job.mp_batch_units, (int)((blockIdx.x * kWarps + warp) % 1024u));
        slot = __shfl_sync(0xffffffffu, slot, 0);
        if (slot < 0) {
            // no free batch: every IA of this warp runs in the per-IA launch
            for (long k = (long)blockIdx.x * kWarps + warp + (long)lane * warps_total; k < count;
                 k += 32 * warps_total)
                job.mp_retry[1 + atomicAdd(job.mp_retry, 1)] = (int)k;
            return;
        }
        mpb = job.mp_batch + slot;
    }
    int nb = 0;
    for (long k = (long)blockIdx.x * kWarps + warp; k < count; k += warps_total) {
        const long ia = job.ia_list != nullptr ? (long)job.ia_list[1 + k] : k;
        xcorr16_warp_ia<Pix, PP, BATCH>(job, ia, sm, fitv, lane, qn, mpb, nb);
    }
    if (!BATCH && qn > 0) fit_flush<D, PP>(sm.fitq, fitv, qn, lane, job);
    if (BATCH) {
        if (nb > 0) mp_batch_run<D, PP>(mpb, nb, lane, job, sm.fitq, fitv);
        if (lane == 0) mp_release(job.mp_slots, (int)(mpb - job.mp_batch));
    }
}

}  // namespace qlpiv
