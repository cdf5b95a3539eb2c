// Vector validation after a correlation level (qlpiv_validate.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace qlpiv {

// Iterate-until-no-corrections stops after this many sweeps at most (the reference has
// no bound; a sweep sequence that keeps correcting vectors would not end).
constexpr int kMaxValidationSweeps = 1000;

struct ValidateParams {
    int ni, nj;          // tiles per axis of one frame
    int num_peaks;       // multi-peak model: k strategies (k - 1 secondary peaks, then bilinear)
    float threshold, epsilon0;
    int max_iterations, iterate_until_no_corrections;
    int model;           // qlpiv_validation (QLPIV_VALIDATE_MULTIPEAK_MEDIAN .. QLPIV_VALIDATE_MEDIAN)
    int clip_n, clip_h, clip_w;  // NoOutOfBoundClipping of the replacements (clip_n == 0: allowed)
};

// Per-level device arrays, [pairs][ni*nj] unless noted.
struct ValidateBufs {
    float *u, *v;              // accumulated displacements (validated in place)
    float *bu, *bv;            // backups (written)
    const float2 *peak_uv;     // [pairs][ni*nj][k] peak increments, peak 0 = main (multi-peak model)
    const uint8_t *npeaks;     // peaks found per tile (multi-peak model)
    uint8_t *state;            // bit 0 invalid, bit 1 locked (written)
    const int *tops, *lefts;   // [ni], [nj] tile top / left pixels
    const int *order, *rank;   // [ni*nj] spiral visit order and each tile's rank in it
    int *list, *done;          // scratch
    int *sweeps;               // optional [pairs] correction sweeps made
};

// circularVisitor order of an ni x nj grid (flat tile indices), host side.
void spiral_order(int ni, int nj, int *order);

cudaError_t launch_validate(cudaStream_t s, int pairs, const ValidateParams &vp, const ValidateBufs &b);

}  // namespace qlpiv
