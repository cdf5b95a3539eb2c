// In-warp shared-memory FFT building blocks for the fused FFT-PIV kernel.
//
// A length-M transform (M = 8G, G in {4, 8, 16, 32}) is computed by a group of G
// consecutive lanes of one warp.  Between passes the data sits in "stride-G layout":
// lane g of the group holds elements g + G*m, m = 0..7, in registers.  Passes are
// Stockham radix-R steps (R in {8, 4, 2}); each pass reads the stride-G layout and,
// except for the last one, writes its outputs to a per-group shared-memory buffer
// from which the next pass reads the stride-G layout again.  The last pass leaves
// the natural-order result in stride-G layout, so forward and inverse transforms
// chain without data movement.  Groups never span warps, so the exchanges need only
// __syncwarp().  Buffer indices are padded (xpad) to spread the accesses over banks.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace qlpiv {

struct cplx {
    float x, y;
};

__device__ __forceinline__ cplx cadd(cplx a, cplx b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cplx csub(cplx a, cplx b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cplx cmul(cplx a, cplx b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ cplx mul_mi(cplx a) {
    return INV ? cplx{-a.y, a.x} : cplx{a.y, -a.x};
}

__device__ __forceinline__ int pad8(int e) { return e + (e >> 3); }

// Exchange-buffer index of element e written by pass PASS of a length-M transform, layout L.
// Layout 0: e + e/8 after every pass.  Layout 1 makes the 8-byte accesses of a 16-lane half-warp
// hit 16 distinct bank pairs when one group fills the half-warp (M >= 128):
//   pass 0 (radix 8) writes x[8g + t], the next pass reads x[g + G m]:     e + e/16;
//   pass 1 (radix 8 after radix 8) writes x[64a + 8t + b] from lane 8a + b: e + 4 (e/32).
// For M = 64 (two groups per half-warp) e + e/8 is conflict-free when the two groups' buffers
// start 8 (mod 16) complex apart.
template <int M, int L, int PASS>
__device__ __forceinline__ int xpad(int e) {
    if constexpr (L == 1 && M >= 128) return PASS == 0 ? e + (e >> 4) : e + 4 * (e >> 5);
    else return e + (e >> 3);
}
// Complex elements an exchange buffer of layout L must hold.
template <int M, int L>
constexpr int xbuf_size() {
    return L == 1 && M >= 128 ? M + 4 * (M / 32 - 1) : M + M / 8;
}

// Radix kernels, forward (e^{-2 pi i/R}) or inverse (e^{+2 pi i/R}), in place.
template <bool INV>
__device__ __forceinline__ void dft2(cplx &a, cplx &b) {
    const cplx t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(cplx &a0, cplx &a1, cplx &a2, cplx &a3) {
    const cplx s0 = cadd(a0, a2), d0 = csub(a0, a2);
    const cplx s1 = cadd(a1, a3), d1 = mul_mi<INV>(csub(a1, a3));
    a0 = cadd(s0, s1);
    a2 = csub(s0, s1);
    a1 = cadd(d0, d1);
    a3 = csub(d0, d1);
}

template <bool INV>
__device__ __forceinline__ void dft8(cplx *v) {
    // split into even/odd DFT4s, then combine with w8^k
    cplx e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    cplx o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<INV>(e0, e1, e2, e3);
    dft4<INV>(o0, o1, o2, o3);
    const float r = 0.70710678118654752440f;
    // w8^1 = (1 -+ i)/sqrt2, w8^2 = -+i, w8^3 = (-1 -+ i)/sqrt2
    const cplx t1 = INV ? cplx{(o1.x - o1.y) * r, (o1.x + o1.y) * r} : cplx{(o1.x + o1.y) * r, (o1.y - o1.x) * r};
    const cplx t2 = mul_mi<INV>(o2);
    const cplx t3 = INV ? cplx{-(o3.x + o3.y) * r, (o3.x - o3.y) * r} : cplx{(o3.y - o3.x) * r, -(o3.x + o3.y) * r};
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, t1);
    v[5] = csub(e1, t1);
    v[2] = cadd(e2, t2);
    v[6] = csub(e2, t2);
    v[3] = cadd(e3, t3);
    v[7] = csub(e3, t3);
}

// One Stockham pass of radix R over M = 8G points.  Input: stride-G layout in v[]
// (lane g holds x[g + G*m]).  Butterfly s of lane g is i = g + G*s (s < 8/R); its
// inputs are x[i + t*M/R] = v[s + (8/R)*t].  With p = product of the radices of the
// previous passes and k = i mod p, inputs are multiplied by w^(t*k*M/(p*R)) (w = the
// M-th root of unity in `tw`), transformed, and output t goes to y[(i-k)*R + k + t*p].
// If LAST, p*R == M and the output is y[i + t*p] = stride-G layout: kept in v[].
// Otherwise the outputs are written to buf (padded index).
template <int M, int R, int P, bool INV, bool LAST, int L = 0, int PASS = 0>
__device__ __forceinline__ void stockham_pass(cplx *v, int g, cplx *buf, const cplx *tw) {
    constexpr int G = M / 8;
    constexpr int B = 8 / R;  // butterflies per lane
    cplx u[8];
#pragma unroll
    for (int s = 0; s < B; s++) {
        const int i = g + G * s;
        const int k = i & (P - 1);
#pragma unroll
        for (int t = 0; t < R; t++) {
            cplx x = v[s + B * t];
            if (P > 1 && t > 0) {
                const int e = (t * k * (M / (P * R))) & (M - 1);
                cplx w = tw[e];
                if (INV) w.y = -w.y;
                x = cmul(x, w);
            }
            u[s * R + t] = x;
        }
        if (R == 8) dft8<INV>(&u[s * R]);
        if (R == 4) dft4<INV>(u[s * R], u[s * R + 1], u[s * R + 2], u[s * R + 3]);
        if (R == 2) dft2<INV>(u[s * R], u[s * R + 1]);
    }
    if (LAST) {
#pragma unroll
        for (int s = 0; s < B; s++)
#pragma unroll
            for (int t = 0; t < R; t++) v[s + B * t] = u[s * R + t];
    } else {
        __syncwarp();
#pragma unroll
        for (int s = 0; s < B; s++) {
            const int i = g + G * s;
            const int k = i & (P - 1);
            const int j = (i - k) * R + k;
#pragma unroll
            for (int t = 0; t < R; t++) buf[xpad<M, L, PASS>(j + t * P)] = u[s * R + t];
        }
        __syncwarp();
#pragma unroll
        for (int m = 0; m < 8; m++) v[m] = buf[xpad<M, L, PASS>(g + G * m)];
    }
}

// Full length-M FFT on stride-G layout data (in and out), using buf (xbuf_size<M, L>()
// complex, private to the group) for the exchanges.
template <int M, bool INV, int L = 0>
__device__ __forceinline__ void fft_group(cplx *v, int g, cplx *buf, const cplx *tw) {
    static_assert(M == 32 || M == 64 || M == 128 || M == 256, "unsupported FFT size");
    if constexpr (M == 32) {
        stockham_pass<32, 8, 1, INV, false, L, 0>(v, g, buf, tw);
        stockham_pass<32, 4, 8, INV, true, L, 1>(v, g, buf, tw);
    } else if constexpr (M == 64) {
        stockham_pass<64, 8, 1, INV, false, L, 0>(v, g, buf, tw);
        stockham_pass<64, 8, 8, INV, true, L, 1>(v, g, buf, tw);
    } else if constexpr (M == 128) {
        stockham_pass<128, 8, 1, INV, false, L, 0>(v, g, buf, tw);
        stockham_pass<128, 8, 8, INV, false, L, 1>(v, g, buf, tw);
        stockham_pass<128, 2, 64, INV, true, L, 2>(v, g, buf, tw);
    } else {
        stockham_pass<256, 8, 1, INV, false, L, 0>(v, g, buf, tw);
        stockham_pass<256, 8, 8, INV, false, L, 1>(v, g, buf, tw);
        stockham_pass<256, 4, 64, INV, true, L, 2>(v, g, buf, tw);
    }
}

}  // namespace qlpiv
