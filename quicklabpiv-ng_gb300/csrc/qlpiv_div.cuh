// Tile normalisation v / max without the general division sequence.
#pragma once
#include <cuda_runtime.h>

namespace qlpiv {

// The correctly rounded quotient v / m for integer-valued v in [0, 65535] and integer m in
// [1, 65535], given rm = RN(1 / m): y = RN(v rm) is within an ulp of the quotient, and one
// correction step with the exact FMA residual, q = RN(y + rm RN(v - m y)) (Markstein, "Computation
// of elementary functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990),
// rounds it correctly.  qlpiv_probe_division checks the whole domain against IEEE division.
__device__ __forceinline__ float div_int(float v, float m, float rm) {
    const float y = __fmul_rn(v, rm);
    const float e = __fmaf_rn(-y, m, v);
    return __fmaf_rn(e, rm, y);
}

}  // namespace qlpiv
