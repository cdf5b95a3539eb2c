/*
 * qlpiv -- C ABI of the GB300 FFT-PIV hot path (libqlpiv_gpu.so).
 *
 * Drop-in boundary for QuickLabPIV-ng's PIV stage plugins.  Every entry point takes
 * plain pointers and sizes, returns a qlpiv_status, and on failure leaves a message
 * for qlpiv_last_error() (thread-local).  Host pointers are borrowed for the duration
 * of the call; device buffers, streams and pinned staging belong to the handle.
 * Calls on one handle are serialised by the handle; distinct handles are
 * independent (the reference runs one job instance per host thread,
 * S/jobs/managers/OpenClGpuManager.java:121-148).
 *
 * Citations: paths inside QuickLabPIV-ng, S/ = src/main/java/pt/quickLabPIV/.
 */
#ifndef QLPIV_H
#define QLPIV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QLPIV_ABI_VERSION 5

/* Status codes.  The Java shim maps QLPIV_E_SHAPE/QLPIV_E_ARG to JobAnalyzeException
 * (S/jobs/xcorr/CrossCorrelationFFTTemplate.java:594-642 shape checks) and the others
 * to JobComputeException. */
typedef enum {
    QLPIV_OK = 0,
    QLPIV_E_ARG = 1,         /* null pointer, bad enum, count < 0 */
    QLPIV_E_SHAPE = 2,       /* unsupported IA size, tiles of different size */
    QLPIV_E_OOM = 3,         /* device or pinned allocation failed */
    QLPIV_E_CUDA = 4,        /* a CUDA runtime call failed */
    QLPIV_E_TIMEOUT = 5,     /* a bounded device wait expired */
    QLPIV_E_CANCELLED = 6,   /* request cancelled */
    QLPIV_E_UNSUPPORTED = 7, /* feature not available in this build */
    QLPIV_E_NO_DEVICE = 8    /* no CUDA device */
} qlpiv_status;

/* Pixel type of images and tiles. */
typedef enum {
    QLPIV_PIX_U8 = 0,  /* MatrixByte, 8-bit images */
    QLPIV_PIX_U16 = 1, /* MatrixInt16, 10/12/16-bit images */
    QLPIV_PIX_F32 = 2  /* MatrixFloat */
} qlpiv_pixel;

/* Tile normalisation v/max*16+1 (no mean subtraction). */
typedef enum {
    QLPIV_NORM_MAX_A = 0,   /* both tiles by tile A's max: FastRealFFTXCorr.java:53-54 (CPU job) */
    QLPIV_NORM_OWN_MAX = 1, /* each tile by its own max: CrossCorrelationRealFFTParStdJob.java:128-129 */
    QLPIV_NORM_NONE = 3     /* raw values */
} qlpiv_norm;

/* Where the tile maxima come from. */
typedef enum {
    QLPIV_MAX_COMPUTE = 0, /* max of the clipped tile, floored at 16 (MatrixByte.java:16-33) */
    QLPIV_MAX_GIVEN = 1,   /* per-IA arrays supplied by the caller (Matrix.getMaxValue()) */
    QLPIV_MAX_FIXED = 2,   /* one constant per image (full-image warp tiles, MatrixByte.java:366-384) */
    QLPIV_MAX_FIXED_A = 3, /* A tiles fixed_max_a, B tiles computed (FirstImage warping: A cut from the
                              warped frame, B clipped from the original) */
    QLPIV_MAX_FIXED_B = 4  /* A tiles computed, B tiles fixed_max_b (SecondImage warping) */
} qlpiv_max_mode;

typedef enum {
    QLPIV_SUBPIX_NONE = 0,
    QLPIV_SUBPIX_GAUSS3 = 1,      /* Gaussian1DPolynomialInterpolator (3-point, 1D-1D) */
    QLPIV_SUBPIX_GAUSS_LM = 2,    /* Gaussian1DInterpolator: least-squares Gaussian through
                                     subpix_pixels points per axis
                                     (S/interpolators/Gaussian1DInterpolator.java:36-115) */
    QLPIV_SUBPIX_HONGWEI_GUO = 3  /* Gaussian1DHongweiGuoInterpolator: y^2-weighted log fit,
                                     subpix_iterations re-weightings
                                     (S/interpolators/Gaussian1DHongweiGuoInterpolator.java:47-250) */
} qlpiv_subpix;

/* Stencil pixels of the P-point interpolators: odd, 3..QLPIV_MAX_SUBPIX_PIXELS. */
#define QLPIV_MAX_SUBPIX_PIXELS 15

/* qlpiv_vector.flags */
#define QLPIV_F_SUB_I 1u     /* sub-pixel fit accepted along I (rows) */
#define QLPIV_F_SUB_J 2u     /* sub-pixel fit accepted along J (columns) */
#define QLPIV_F_PARABOLIC 4u /* a stencil value was negative: parabolic fallback */
#define QLPIV_F_EDGE 8u      /* 3-point stencil leaves the plane: integer peak kept */
#define QLPIV_F_NO_PEAK 16u  /* no non-negative cell: peak left at (0,0) */
#define QLPIV_F_ABSENT 32u   /* multi-peak slot beyond the peaks found (vector zeroed) */
#define QLPIV_F_FLOOR 64u    /* min floor below the P-point interpolator's limit (-3.15 least
                                squares, -5.15 Hongwei Guo; the reference throws
                                InterpolateException): integer peak kept */

/* FindMaximumMultiPeaks limits of this library: 1..QLPIV_MAX_PEAKS peaks per IA and a
 * cell width of at least 2 (the per-cell maxima of one IA are staged on chip). */
#define QLPIV_MAX_PEAKS 16

/* One IA result (32 bytes): MaxCrossResult main peak after interpolation.
 * u/v are the displacement increments along rows/columns
 * (MaxCrossResult.getNthDisplacementU/V, S/maximum/MaxCrossResult.java:304-326,412-437);
 * sub_i/sub_j the sub-pixel peak in plane coordinates; peak_i/peak_j the integer peak
 * of FindMaximumFromCenter; min_floor the minimum over the visited cells. */
typedef struct qlpiv_vector {
    float u, v;
    float sub_i, sub_j;
    float peak_value;
    float min_floor;
    int16_t peak_i, peak_j;
    uint32_t flags;
} qlpiv_vector;

/* One correlation pass: IA side and tile/peak semantics. */
typedef struct qlpiv_pass_desc {
    int n;              /* IA side: 16, 32, 64 or 128 (128: a two-CTA cluster per IA) */
    int norm_mode;      /* qlpiv_norm */
    int max_mode;       /* qlpiv_max_mode */
    float fixed_max_a;  /* QLPIV_MAX_FIXED: max of every A tile */
    float fixed_max_b;  /* QLPIV_MAX_FIXED: max of every B tile */
    int subpix_mode;    /* qlpiv_subpix */
    int num_peaks;      /* 0: FindMaximumFromCenter, one vector per IA.  k >= 1:
                           FindMaximumMultiPeaks (S/maximum/FindMaximumMultiPeaks.java:42-162),
                           k vectors per IA, largest peak first, every peak fitted */
    int peak_kernel;    /* FindMaximumMultiPeaks cell width (kernelWidth), >= 2 */
    int subpix_pixels;  /* QLPIV_SUBPIX_GAUSS_LM / HONGWEI_GUO: stencil pixels (odd) */
    int subpix_iterations; /* QLPIV_SUBPIX_HONGWEI_GUO: re-weightings, 6..50 */
    int reserved[2];
} qlpiv_pass_desc;

/* One image pair of a batch.  Pixels are row-major with `pitch` elements per row; both
 * frames share height, width, pitch and the batch's pixel type. */
typedef struct qlpiv_frame {
    const void *img_a;
    const void *img_b;
    int32_t height;
    int32_t width;
    int64_t pitch;
} qlpiv_frame;

/* Geometry of one adaptive level's IA grid (IterationStepTiles). */
typedef struct qlpiv_grid {
    int n;            /* IA side */
    int tiles_i, tiles_j;
    int margin_top, margin_left, margin_bottom, margin_right;
} qlpiv_grid;

typedef enum {
    QLPIV_WARP_NONE = 0,          /* NoImageWarping: B tiles at round(origin + displacement) */
    QLPIV_WARP_BOTH_BILINEAR = 1, /* BothImagesBiLinearWarping (BiLinearImageWarpingStrategy): both
                                     frames warped by half the field */
    QLPIV_WARP_FIRST_BILINEAR = 2,  /* FirstImageBiLinearWarping: A warped by the whole field, B tiles
                                       clipped from the original frame */
    QLPIV_WARP_SECOND_BILINEAR = 3, /* SecondImageBiLinearWarping: B warped, A tiles clipped */
    /* BiLinearImageMicroAndMiniWarpingStrategy (S/images/BiLinearImageMicroAndMiniWarpingStrategy.java):
     * every tile warped on its own; micro: by its fractional displacement, mini: by a bicubic
     * spline over its up to 7 x 7 neighbour tiles.  Warped tiles keep the full-scale maximum,
     * clipped ones their own; level 0 clips both tiles. */
    QLPIV_WARP_FIRST_MICRO = 4,
    QLPIV_WARP_SECOND_MICRO = 5,
    QLPIV_WARP_BOTH_MICRO = 6,
    QLPIV_WARP_FIRST_MINI = 7,
    QLPIV_WARP_SECOND_MINI = 8,
    QLPIV_WARP_BOTH_MINI = 9
} qlpiv_warp_mode;

/* Velocity inheritance between adaptive levels (InterAreaVelocityStrategiesFactoryEnum,
 * S/iareas/InterAreaVelocityStrategiesFactoryEnum.java:12-29). */
typedef enum {
    QLPIV_INHERIT_BICUBIC_SPLINE = 0, /* AdaptiveInterVelocityInheritanceStrategyBiCubicSpline */
    QLPIV_INHERIT_DIRECT = 1,         /* ...StrategyDirect: child (2i + a, 2j + b) <- parent (i, j) */
    QLPIV_INHERIT_AREA = 2,           /* ...StrategyArea: overlap-area weighted parents */
    QLPIV_INHERIT_DISTANCE = 3        /* ...StrategyDistanceGeneric: inverse-distance weighted
                                         surrounding parents */
} qlpiv_inherit_mode;

/* Adaptive multi-pass PIV parameters (PIVInputParameters fields of the path). */
typedef struct qlpiv_adaptive_desc {
    int ia_start;          /* IA side of the first level (getInterrogationAreaStartIPixels) */
    int ia_end;            /* IA side of the last level; ia_start / ia_end a power of two */
    float overlap_factor;  /* 1 - overlap% / 100, in [0.1, 0.9] (SuperPosition division) */
    int margins[4];        /* top, bottom, left, right */
    int warp_mode;         /* qlpiv_warp_mode */
    int norm_mode;         /* qlpiv_norm */
    int max_mode;          /* QLPIV_MAX_COMPUTE or QLPIV_MAX_FIXED */
    float fixed_max;       /* QLPIV_MAX_FIXED tile max, 0 = full scale (255 / 65535) */
    int subpix_mode;       /* qlpiv_subpix */
    int int16_warp_quirk;  /* 1: store warped 16-bit pixels through a signed byte like
                              MatrixInt16.setElement(float) (S/MatrixInt16.java:95-101) */
    int validation;        /* qlpiv_validation: vector validation after every level */
    int num_peaks;         /* QLPIV_VALIDATE_MULTIPEAK_MEDIAN: peaks per IA = strategies */
    int peak_kernel;       /* FindMaximumMultiPeaks cell width */
    float median_threshold;   /* NormalizedMedianValidator / DifferenceValidator distance threshold */
    float median_epsilon0;    /* NormalizedMedianValidator epsilon0 */
    int max_correction_iterations;      /* VectorValidatorConfiguration */
    int iterate_until_no_corrections;   /* VectorValidatorConfiguration */
    int subpix_pixels;     /* as qlpiv_pass_desc */
    int subpix_iterations; /* as qlpiv_pass_desc */
    int inherit_mode;      /* qlpiv_inherit_mode (getVelocityInheritanceStrategy) */
    int clipping_mode;     /* qlpiv_clipping (PIVInputParameters.getClippingMode) */
    int superposition_start; /* interrogation-area division: levels before this one split without
                              superposition (AdaptiveInterAreaStrategyNoSuperPosition), the rest
                              with it, SuperPosition restarting at this level as at its first
                              step (AdaptiveInterAreaStrategyMixedSuperPosition,
                              S/iareas/AdaptiveInterAreaStrategyMixedSuperPosition.java:31-92,
                              getSuperPositionIterationStepStart).  0: SuperPosition throughout
                              (AdaptiveInterAreaStrategySuperPosition); >= the level count:
                              NoSuperPosition throughout.  qlpiv_grid_level gives every level. */
    int stable_mode;       /* qlpiv_stable: when a level's correlation is repeated */
    float stable_max_displacement;  /* QLPIV_STABLE_MAX_DISPLACEMENT: getMaxDisplacement (px) */
    int stable_max_retries;         /* QLPIV_STABLE_MAX_DISPLACEMENT: getMaxRetries (>= 1) */
    int reserved[5];
} qlpiv_adaptive_desc;

/* Tile stabilisation per level (InterAreaStableStrategiesFactoryEnum,
 * S/iareas/InterAreaStableStrategiesFactoryEnum.java:9-27; the loop of
 * S/jobs/LocalPIVOpenCLGpuJob.java:233-405).  Pass r = 1, 2, ... of a level re-warps the frames
 * with every tile's current displacement (no warping at the first level), correlates the tiles
 * still EVALUATING and accumulates their increments; a tile's state then follows
 * InterAreaDisplacementStableStrategy.computeStableState (S/iareas/InterAreaDisplacementStableStrategy.java:19-36):
 * |increment| = (float) sqrt(du^2 + dv^2) in double above the maximum keeps it EVALUATING while
 * r < max_retries (UNSTABLE at r = max_retries), else it is STABLE.  At the first level the
 * BothImages strategy does not warp, so a repeated pass correlates the same tiles again and adds
 * the same increment, as the reference does.  Not combined with vector validation (the
 * reference's validator then visits only the re-correlated tiles): QLPIV_E_ARG. */
typedef enum {
    QLPIV_STABLE_SIMPLE = 0,            /* InterAreaSimpleStableStrategy: one correlation per level */
    QLPIV_STABLE_MAX_DISPLACEMENT = 1   /* InterAreaDisplacementStableStrategy */
} qlpiv_stable;

/* ClippingModeEnum (S/ClippingModeEnum.java:9-13).  Under QLPIV_CLIP_NO_OUT_OF_BOUND every
 * displacement update of a tile -- inheritance, the correlation increment, a validation
 * replacement, the zeroing of still-invalid vectors, the optical-flow tile replacement -- is
 * refused when the tile of side n at (top, left), moved by the rounded displacement
 * (FastMath.round), would leave the image by the reference's test: top + round(u) < 0,
 * top + n + round(u) >= height, or the same for columns (Tile.accumulateDisplacement /
 * replaceDisplacement, S/iareas/Tile.java:103-136,156-189).  A refused correlation increment is
 * dropped; a refused replacement leaves the displacement as it is.  The reference's throw for
 * NoImageWarping B tiles that need clipping (S/images/NoImageWarpingStrategy.java:48-70) cannot
 * trigger then: the refusals keep every displaced tile inside the image.  LOGGED behaves as
 * ALLOWED (the reference only logs). */
typedef enum {
    QLPIV_CLIP_ALLOWED = 0,           /* AllowedOutOfBoundClipping (the converter's default) */
    QLPIV_CLIP_LOGGED = 1,            /* LoggedOutOfBoundClipping */
    QLPIV_CLIP_NO_OUT_OF_BOUND = 2    /* NoOutOfBoundClipping */
} qlpiv_clipping;

/* Vector validation after each level (VectorValidatorJob, S/jobs/validator/VectorValidatorJob.java:242-405),
 * the five models the converter builds (PIVConfigurationConverterVisitor.visit,
 * ui/src/main/java/pt/quickLabPIV/business/transfer/PIVConfigurationConverterVisitor.java:546-641).
 * Still-invalid vectors are set to 0 in every model. */
typedef enum {
    QLPIV_VALIDATE_NONE = 0,
    /* VelocityValidationOptionsMultiPeakNormalizedMedianModel: FindMaximumMultiPeaks with
     * num_peaks peaks, strategies 0..k-2 = normalised median + SecondaryPeakReplacement of
     * peak s+1, strategy k-1 = normalised median + BilinearReplacement. */
    QLPIV_VALIDATE_MULTIPEAK_MEDIAN = 1,
    /* The four single-strategy models, all with FindMaximumFromCenter peaks:
     * DifferenceValidator (S/iareas/validation/DifferenceValidator.java:30-60; distance
     * threshold median_threshold px) without / with BilinearReplacement, and
     * NormalizedMedianValidator without / with BilinearReplacement.  The difference validator
     * compares a tile only with its valid top-left, top and left neighbours, and every tile
     * starts invalid, so in the reference it never validates a vector: these two models set
     * every vector to 0 (subject to the clipping mode), and so does this library. */
    QLPIV_VALIDATE_DIFFERENCE_ONLY = 2,
    QLPIV_VALIDATE_DIFFERENCE = 3,
    QLPIV_VALIDATE_MEDIAN_ONLY = 4,
    QLPIV_VALIDATE_MEDIAN = 5
} qlpiv_validation;

typedef struct qlpiv_params {
    int device;         /* CUDA device ordinal */
    int reserved[7];
} qlpiv_params;

typedef struct qlpiv_handle qlpiv_handle;

int qlpiv_abi_version(void);
const char *qlpiv_last_error(void);

/* Creates a handle bound to one device: a non-blocking stream, device workspace and
 * pinned staging that grow on demand.  Replaces the device set-up of the xcorr job
 * constructors (S/jobs/xcorr/CrossCorrelationRealFFTParStdJob.java:58-78). */
qlpiv_status qlpiv_create(const qlpiv_params *params, qlpiv_handle **out);
/* Job.dispose() (S/jobs/Job.java:58): frees everything the handle owns. */
qlpiv_status qlpiv_destroy(qlpiv_handle *h);
/* Waits for all work queued on the handle's stream. */
qlpiv_status qlpiv_synchronize(qlpiv_handle *h);

/* Job<List<Tile>, XCorrelationResults> compute() for the cross-correlation job:
 * `count` tile pairs of n x n pixels (row-major, contiguous per tile) in host memory,
 * tile maxima per IA (max_a/max_b; NULL = compute, floor 16), normalisation mode.
 * Writes count (2n-1)^2 float planes, the JOB_RESULT_CROSS_MATRICES of
 * CrossCorrelationRealFFTParStdJob / CrossCorrelationSoftRealFFTJob
 * (S/jobs/xcorr/XCorrelationResults.java:14-55). */
qlpiv_status qlpiv_xcorr_planes(qlpiv_handle *h, int n, long count, int pixel_type, const void *tiles_a,
                                const void *tiles_b, const float *max_a, const float *max_b, int norm_mode,
                                float *planes_out);

/* Fused xcorr + FindMaximumFromCenter.findMaximum (S/maximum/FindMaximumFromCenter.java:47-183)
 * + ICrossCorrelationInterpolator.interpolate (Gaussian1DPolynomialInterpolator.java:25-106)
 * on host tiles; writes count vectors.  Same tile arguments as qlpiv_xcorr_planes. */
qlpiv_status qlpiv_xcorr_peaks(qlpiv_handle *h, int n, long count, int pixel_type, const void *tiles_a,
                               const void *tiles_b, const float *max_a, const float *max_b, int norm_mode,
                               int subpix_mode, qlpiv_vector *out);

/* Fused xcorr + FindMaximumMultiPeaks.findMaximum (S/maximum/FindMaximumMultiPeaks.java:42-162,
 * S/util/SimpleFixedLengthFloatLinkedList.java:98-237) + the sub-pixel fit of every peak:
 * out receives count x num_peaks vectors, largest peak first; slots beyond the peaks
 * found carry QLPIV_F_ABSENT.  min_floor is the minimum over the whole plane. */
qlpiv_status qlpiv_xcorr_multipeaks(qlpiv_handle *h, int n, long count, int pixel_type, const void *tiles_a,
                                    const void *tiles_b, const float *max_a, const float *max_b, int norm_mode,
                                    int subpix_mode, int num_peaks, int peak_kernel, qlpiv_vector *out);

/* One correlation pass over an image pair in host memory (height x width, row-major):
 * warp/clip (IImageWarpingStrategy.warpAndClipImage, S/images/NoImageWarpingStrategy.java:27-89,
 * tiles partially outside the image are zero-filled), xcorr, peak and sub-pixel for
 * `count` IAs whose tile origins are given per IA (a_top/a_left in image A,
 * b_top/b_left in image B: rounded displaced origins, FastMath.round).  Synchronous;
 * writes count vectors to host memory. */
qlpiv_status qlpiv_pass(qlpiv_handle *h, const qlpiv_pass_desc *desc, const void *img_a, const void *img_b,
                        int height, int width, int pixel_type, long count, const int32_t *a_top,
                        const int32_t *a_left, const int32_t *b_top, const int32_t *b_left, qlpiv_vector *out);

/* Same as qlpiv_pass with every pointer in device memory (inputs resident in HBM);
 * queued on the handle's stream and returns without waiting. */
qlpiv_status qlpiv_pass_device(qlpiv_handle *h, const qlpiv_pass_desc *desc, const void *img_a,
                               const void *img_b, int height, int width, int pixel_type, long count,
                               const int32_t *a_top, const int32_t *a_left, const int32_t *b_top,
                               const int32_t *b_left, qlpiv_vector *out);

/* Batched pass over many image pairs of possibly different sizes (one launch for the
 * whole flattened IA work list): IA k belongs to frames[frame_of_ia[k]].  This replaces
 * the reference's fan-out of one job per frame pair and thread
 * (S/InputFiles.java:215-224, S/jobs/managers/OpenClGpuManager.java:85-186).  Host
 * variant: frames[] point to host images, all other arrays are host arrays; synchronous. */
qlpiv_status qlpiv_pass_batch(qlpiv_handle *h, const qlpiv_pass_desc *desc, int pixel_type, int num_frames,
                              const qlpiv_frame *frames, long count, const int32_t *frame_of_ia,
                              const int32_t *a_top, const int32_t *a_left, const int32_t *b_top,
                              const int32_t *b_left, qlpiv_vector *out);

/* Device variant: `frames` is a device array of num_frames entries whose image pointers
 * are device pointers; every other array is in device memory; queued on the handle's
 * stream. */
qlpiv_status qlpiv_pass_batch_device(qlpiv_handle *h, const qlpiv_pass_desc *desc, int pixel_type,
                                     int num_frames, const qlpiv_frame *frames, long count,
                                     const int32_t *frame_of_ia, const int32_t *a_top, const int32_t *a_left,
                                     const int32_t *b_top, const int32_t *b_left, qlpiv_vector *out);

/* The CUDA stream (cudaStream_t) the handle queues work on. */
qlpiv_status qlpiv_get_stream(qlpiv_handle *h, void **stream);
/* Queue subsequent work on a caller-owned stream (NULL restores the handle's own). */
qlpiv_status qlpiv_set_stream(qlpiv_handle *h, void *stream);

/* IA grid of one level: AdaptiveInterAreaStrategySuperPosition / NoSuperPosition
 * (S/iareas/AdaptiveInterAreaStrategySuperPosition.java:31-197,
 *  S/iareas/AdaptiveInterAreaStrategyNoSuperPosition.java:32-157).  margins = top, bottom,
 * left, right.  tops/lefts (capacity `cap`) may be NULL to query the size only.  Host only. */
qlpiv_status qlpiv_grid_superposition(int height, int width, const int margins[4], int ia_start, int level,
                                      float overlap_factor, qlpiv_grid *grid, int32_t *tops, int32_t *lefts,
                                      int cap);
qlpiv_status qlpiv_grid_nosuperposition(int height, int width, const int margins[4], int ia_start, int level,
                                        qlpiv_grid *grid, int32_t *tops, int32_t *lefts, int cap);
/* The grid of adaptive level `level` under the mixed division (AdaptiveInterAreaStrategy-
 * MixedSuperPosition, S/iareas/AdaptiveInterAreaStrategyMixedSuperPosition.java:31-92): levels
 * before superposition_start as qlpiv_grid_nosuperposition, the rest as qlpiv_grid_superposition
 * of IA ia_start >> superposition_start at level - superposition_start.  Host only. */
qlpiv_status qlpiv_grid_level(int height, int width, const int margins[4], int ia_start, int level,
                              float overlap_factor, int superposition_start, qlpiv_grid *grid, int32_t *tops,
                              int32_t *lefts, int cap);

/* Number of adaptive levels and the grid of each (`grids` may be NULL).  Host only. */
qlpiv_status qlpiv_adaptive_levels(const qlpiv_adaptive_desc *desc, int height, int width, int *levels,
                                   qlpiv_grid *grids, int max_levels);

/* Velocity inheritance between levels, IterationStepTiles.reuseTiles with the
 * BiCubicSpline strategy (S/iareas/AdaptiveInterVelocityInheritanceStrategyBiCubicSpline.java:27-136):
 * parent displacements pu/pv (pni x pnj) at parent centres p_ci/p_cj, child centres
 * c_ci/c_cj (float, top + N/2 - 0.5); round_int for non-warping modes.  Host arrays. */
qlpiv_status qlpiv_inherit(qlpiv_handle *h, int pni, int pnj, const double *p_ci, const double *p_cj, const float *pu,
                           const float *pv, int cni, int cnj, const float *c_ci, const float *c_cj, int round_int,
                           float *cu, float *cv);

/* Velocity inheritance with the Direct, Area or Distance strategy
 * (S/iareas/AdaptiveInterVelocityInheritanceStrategy{Direct,Area,DistanceGeneric}.java): parent
 * grid (side pn, rows p_tops[pni], columns p_lefts[pnj]) with displacements pu/pv, child grid
 * (side cn, c_tops[cni], c_lefts[cnj]); round_int for non-warping modes.  Geometries on which
 * the reference's walk throws are rejected with QLPIV_E_SHAPE.  Host arrays. */
qlpiv_status qlpiv_inherit_tiles(qlpiv_handle *h, int mode, int pn, int pni, int pnj, const int32_t *p_tops,
                                 const int32_t *p_lefts, const float *pu, const float *pv, int cn, int cni, int cnj,
                                 const int32_t *c_tops, const int32_t *c_lefts, int round_int, float *cu, float *cv);

/* Per-pixel displacement field of a level (BiCubicSplineInterpolatorWithBiLinearBackup.
 * interpolateDisplacements, S/iareas/BiCubicSplineInterpolatorWithBiLinearBackup.java:57-107):
 * tile displacements u/v (ni x nj) at centres ci/cj -> fu/fv (height x width).  Host arrays. */
qlpiv_status qlpiv_displacement_field(qlpiv_handle *h, int height, int width, int ni, int nj, const double *ci,
                                      const double *cj, const float *u, const float *v, float *fu, float *fv);

/* IImageWarpingStrategy.warpAndClipImage for full-image bilinear warping
 * (S/images/BiLinearImageWarpingStrategy.java:38-265) through the level's tile displacements:
 * warp_mode QLPIV_WARP_BOTH_BILINEAR warps both images by half the field, FIRST warps image A
 * (sampled at (i - u, j - v)) and SECOND image B (at (i + u, j + v)) by the whole field; the
 * image that is not warped is copied unchanged.  Host arrays, out_a/out_b as the input pixel type
 * (u8 or u16). */
qlpiv_status qlpiv_warp_pair(qlpiv_handle *h, int pixel_type, int warp_mode, const void *img_a, const void *img_b,
                             int height, int width, int ni, int nj, const double *ci, const double *cj, const float *u,
                             const float *v, int int16_quirk, void *out_a, void *out_b);

/* Micro / mini per-tile warping of one pair's tiles (BiLinearImageMicroAndMiniWarpingStrategy
 * .warpAndClipImage, S/images/BiLinearImageMicroAndMiniWarpingStrategy.java:39-407): grid rows
 * tops[ni], columns lefts[nj], side n, tile displacements u / v (ni x nj, rows / columns);
 * warp_mode one of QLPIV_WARP_{FIRST,SECOND,BOTH}_{MICRO,MINI}.  tiles_a / tiles_b receive
 * ni x nj x n x n pixels of the image type, max_a / max_b the tiles' maxima (warped: full_max,
 * clipped: own, floor 16).  Host arrays. */
qlpiv_status qlpiv_tile_warp(qlpiv_handle *h, int pixel_type, const void *img_a, const void *img_b, int height,
                             int width, int n, int ni, int nj, const int32_t *tops, const int32_t *lefts,
                             const float *u, const float *v, int warp_mode, float full_max, void *tiles_a,
                             void *tiles_b, float *max_a, float *max_b);

/* Whole adaptive PIV of num_pairs image pairs of one size (LocalPIVOpenCLGpuJob's level
 * loop, S/jobs/LocalPIVOpenCLGpuJob.java:188-411, SimpleStrategy): per level grid ->
 * inheritance -> warp/clip -> xcorr + peak + sub-pixel -> accumulate -> validation
 * (desc->validation), all on the device.  frames[] are host images (pitch in elements); out_u/out_v receive
 * num_pairs x (tiles_i x tiles_j) displacements of the last level (rows, columns). */
qlpiv_status qlpiv_piv_adaptive(qlpiv_handle *h, const qlpiv_adaptive_desc *desc, int pixel_type, int height,
                                int width, int num_pairs, const qlpiv_frame *frames, float *out_u, float *out_v);

/* Device variant: frames is a device frame table, out_u/out_v device buffers; queued
 * on the handle's stream. */
qlpiv_status qlpiv_piv_adaptive_device(qlpiv_handle *h, const qlpiv_adaptive_desc *desc, int pixel_type, int height,
                                       int width, int num_pairs, const qlpiv_frame *frames, float *out_u,
                                       float *out_v);

/* VectorValidatorJob.compute (S/jobs/validator/VectorValidatorJob.java:242-405) for one
 * frame's ni x nj tiles with the multi-peak normalised-median model: u/v (row-major,
 * main peak already accumulated) are validated and replaced in place; peak_u/peak_v hold
 * the k = desc->num_peaks displacement increments per tile (peak 0 = main), npeaks the
 * peaks found per tile; tops/lefts the tile rows' top and columns' left pixels.
 * invalid_out (may be NULL) receives the final invalid flags.  Host arrays; synchronous.
 * Uses desc->num_peaks, median_threshold, median_epsilon0, max_correction_iterations,
 * iterate_until_no_corrections. */
qlpiv_status qlpiv_validate(qlpiv_handle *h, const qlpiv_adaptive_desc *desc, int ni, int nj, const int32_t *tops,
                            const int32_t *lefts, float *u, float *v, const float *peak_u, const float *peak_v,
                            const int32_t *npeaks, uint8_t *invalid_out);

/* qlpiv_validate for any desc->validation model, with the tile side n and the image size the
 * clipping mode needs (desc->clipping_mode; qlpiv_validate itself refuses
 * QLPIV_CLIP_NO_OUT_OF_BOUND).  peak_u / peak_v / npeaks are read by the multi-peak model only
 * and may be NULL for the others (k = 1 strategy).  VectorValidatorJob.compute with the
 * replacements' Tile.replaceDisplacement bounds (S/iareas/Tile.java:156-189). */
qlpiv_status qlpiv_validate_tiles(qlpiv_handle *h, const qlpiv_adaptive_desc *desc, int n, int height, int width,
                                  int ni, int nj, const int32_t *tops, const int32_t *lefts, float *u, float *v,
                                  const float *peak_u, const float *peak_v, const int32_t *npeaks,
                                  uint8_t *invalid_out);

/* Velocity inheritance that allocates nothing (no counterpart in the reference).
 * For callers that cannot let the library allocate device memory during a call -- a
 * Java host passing device buffers from its own pool with a fixed memory budget, or an
 * acquisition loop that must not take cudaMalloc's implicit synchronisation while frames
 * stream in.  Same result as qlpiv_inherit, but every argument is in device memory (float
 * centres) and the work is queued on `stream` (NULL: the legacy default stream); the call
 * returns without waiting.  The stage-1 scratch is a fixed device array of
 * 2 x QLPIV_NOALLOC_MAX_ROWS floats (4 MiB) that every GPU loading the library holds until
 * exit; cni x pnj above QLPIV_NOALLOC_MAX_ROWS is rejected with QLPIV_E_SHAPE.  The first
 * call on a device looks up that array's device address (cudaGetSymbolAddress), so make
 * the first call on each device before any stream capture.  All calls share the array:
 * calls that overlap on the GPU race.  No entry needs clearing between calls (every
 * entry read is written earlier in the same call). */
#define QLPIV_NOALLOC_MAX_ROWS 524288
qlpiv_status qlpiv_inherit_noalloc(int device, void *stream, int pni, int pnj, const float *p_ci, const float *p_cj,
                                   const float *pu, const float *pv, int cni, int cnj, const float *c_ci,
                                   const float *c_cj, int round_int, float *cu, float *cv);

/* ---- Dense optical flow after PIV (LiuShenWithLucasKanade / LucasKanade interpolators) ---- */

/* GaussianFilter2D.applyFilter (S/images/filters/GaussianFilter2D.java:31-128,
 * GaussianFilter2DInternal.java:49-97): separable Gaussian of `kernel_px` (odd) points and
 * `sigma`, rows then columns, the reference's border padding; img of pixel_type (height x width,
 * contiguous rows) -> out float.  sigma < 1e-5 copies the image.  Host arrays; synchronous. */
qlpiv_status qlpiv_gaussian_filter(qlpiv_handle *h, int pixel_type, const void *img, int height, int width,
                                   float sigma, int kernel_px, float *out);
/* ImageFloat.normalize (S/images/ImageFloat.java:571-596): out = img / max.  Host arrays. */
qlpiv_status qlpiv_normalize(qlpiv_handle *h, const float *img, int height, int width, float *out);
/* DenseLucasKanadeAparapiJob.compute (S/jobs/interpolators/DenseLucasKanadeAparapiJob.java:56-215,
 * DenseLucasKanadeGpuKernel.java:203-751): dense Lucas-Kanade on two (filtered) float images;
 * us (columns) / vs (rows) hold the initial field and receive the result.  window odd 3..31,
 * iterations >= 1, half_pixel: the 2x2-average sampling (half-pixel offset).  Host arrays. */
qlpiv_status qlpiv_dense_lk(qlpiv_handle *h, const float *img_a, const float *img_b, int height, int width, float *us,
                            float *vs, int window, int iterations, int half_pixel);
/* DenseLiuShenAparapiJob.compute (S/jobs/interpolators/DenseLiuShenAparapiJob.java:64-255,
 * DenseLiuShenGpuKernel.java:66-588): the Lucas-Kanade pass on lk_a/lk_b (skipped when
 * iterations_lk == 0) followed by iterations_ls Liu-Shen passes with multiplier lambda on the
 * (filtered, normalised) images ls_a/ls_b.  us (columns) / vs (rows) in and out.  Host arrays. */
qlpiv_status qlpiv_liu_shen(qlpiv_handle *h, const float *lk_a, const float *lk_b, const float *ls_a,
                            const float *ls_b, int height, int width, float *us, float *vs, int window,
                            int iterations_lk, float lambda, int iterations_ls, int half_pixel);

/* Optical flow after PIV (IOpticalFlowInterpolator.interpolate(stepTilesA, stepTilesB) of the
 * LucasKanade and LiuShenWithLucasKanade interpolators,
 * S/interpolators/DenseLucasKanadeAparapiJobInterpolator.java:247-334,
 * S/interpolators/DenseLiuShenAparapiJobInterpolator.java:226-341). */
typedef enum {
    QLPIV_FLOW_LUCAS_KANADE = 1,  /* dense Lucas-Kanade */
    QLPIV_FLOW_LIU_SHEN = 2       /* dense Lucas-Kanade followed by Liu-Shen */
} qlpiv_flow_mode;

/* IgnorePIVBaseDisplacementsModeEnum (S/IgnorePIVBaseDisplacementsModeEnum.java): what the flow
 * stage keeps of the PIV field before Lucas-Kanade (the interpolators' interpolate(stepTilesA,
 * stepTilesB)).  IGNORE_V / IGNORE_U name the reference's axes: IGNORE_V fills the row
 * component, IGNORE_U the column component, with 0 (dense export) or 0.5; AUTO / AUTO_SMALL zero
 * components below 3 / 0.9 px in magnitude. */
typedef enum {
    QLPIV_IGNORE_PIV_NONE = 0,
    QLPIV_IGNORE_PIV_U = 1,
    QLPIV_IGNORE_PIV_V = 2,
    QLPIV_IGNORE_PIV_UV = 3,
    QLPIV_IGNORE_PIV_AUTO = 4,
    QLPIV_IGNORE_PIV_AUTO_SMALL = 5
} qlpiv_ignore_piv;

typedef struct qlpiv_flow_desc {
    int mode;               /* qlpiv_flow_mode */
    float filter_sigma_lk;  /* Lucas-Kanade prefilter (GaussianFilter2D) */
    int filter_px_lk;
    float filter_sigma_ls;  /* Liu-Shen prefilter, followed by normalisation */
    int filter_px_ls;
    int window_lk;          /* odd, 3..31 */
    int iterations_lk;
    float lambda_ls;        /* Liu-Shen Lagrange multiplier */
    int iterations_ls;
    int dense_export;       /* denseVectors: whole-pixel field and dense output */
    int ignore_piv;         /* qlpiv_ignore_piv: ignorePIVBaseDisplacements(Mode) */
    int pyramid_levels;     /* Lucas-Kanade coarse to fine over 1..4 levels (0 or 1: full resolution
                               only, as the reference): 2 x 2 box down-sampling of the prefiltered
                               images and of the field (halved), each level's result up-sampled
                               (nearest, doubled) as the next finer level's start.  This library's
                               own design; the reference's dense LK has no pyramid */
    int clipping_mode;      /* qlpiv_clipping of the tile replacement (qlpiv_flow_after_piv; the
                               PIV + flow entry points take the PIV descriptor's) */
    int reserved[3];
} qlpiv_flow_desc;

/* The optical flow after PIV of one frame pair on the last adaptive step's grid (tiles of side
 * n, rows tops[ni], columns lefts[nj]): images prefiltered (Liu-Shen images normalised), the tile
 * displacements tile_u/tile_v (rows, columns; ni x nj, updated in place) interpolated per pixel
 * (bicubic spline at pixel + 0.5, or + 0 with dense export), Lucas-Kanade (+ Liu-Shen) with the
 * half-pixel offset unless dense export, tiles replaced from the pixel at top + n/2 - 1 (the 2x2
 * average there with dense export).  dense_u/dense_v (rows, columns; may be NULL) receive the
 * dense field.  Host arrays; synchronous. */
qlpiv_status qlpiv_flow_after_piv(qlpiv_handle *h, const qlpiv_flow_desc *desc, int pixel_type, const void *img_a,
                                  const void *img_b, int height, int width, int n, int ni, int nj,
                                  const int32_t *tops, const int32_t *lefts, float *tile_u, float *tile_v,
                                  float *dense_u, float *dense_v);

/* Adaptive PIV of num_pairs host frame pairs (as qlpiv_piv_adaptive) followed on the device by
 * the optical flow after PIV of every pair (LocalPIVOpenCLGpuJob.java:414).  out_u/out_v:
 * num_pairs x last-level tiles; dense_u/dense_v (may be NULL): num_pairs x height x width. */
qlpiv_status qlpiv_piv_flow(qlpiv_handle *h, const qlpiv_adaptive_desc *piv, const qlpiv_flow_desc *flow,
                            int pixel_type, int height, int width, int num_pairs, const qlpiv_frame *frames,
                            float *out_u, float *out_v, float *dense_u, float *dense_v);

/* qlpiv_piv_flow on frames and outputs resident on the device; asynchronous on the handle's
 * stream. */
qlpiv_status qlpiv_piv_flow_device(qlpiv_handle *h, const qlpiv_adaptive_desc *piv, const qlpiv_flow_desc *flow,
                                   int pixel_type, int height, int width, int num_pairs, const qlpiv_frame *frames,
                                   float *out_u, float *out_v, float *dense_u, float *dense_v);

/* ---------------- mixed batches ----------------
 * Many frame pairs of uneven sizes, each with its own IA size (16, 32, 64, 128) and overlap
 * factor, correlated as one flattened work list per IA size (the pair's level-0 SuperPosition
 * grid) and replayed from one captured CUDA graph.  Two schedules:
 *   QLPIV_SCHEDULE_PER_SIZE    one launch per IA size, each on its own graph branch (the sizes
 *                              run concurrently);
 *   QLPIV_SCHEDULE_PERSISTENT  IA 16, 32 and 64 in one persistent launch (one CTA per SM drains
 *                              the three work lists, largest IAs first), IA 128 on its own branch;
 *                              FindMaximumFromCenter with the 3-point (or no) sub-pixel fit.
 * Both write the same vectors.  `autotune`: QLPIV_AUTOTUNE_OFF (per-size launches, default
 * grids), QLPIV_AUTOTUNE_ON (the grid of each size's launch chosen by timing 1, 2, 4, 8, 16 and
 * 32 waves of resident CTAs on its work list, then the faster schedule over the whole batch),
 * QLPIV_AUTOTUNE_PERSISTENT (the persistent schedule where it applies, default grids).
 * `frames` is a host table of device images; the plan keeps a device copy and the output.
 * Output vectors are size-major and pair-contiguous: pair q's tiles_i x tiles_j tiles
 * (row-major) start at pair_offset[q]. */
typedef struct qlpiv_mixed_plan qlpiv_mixed_plan;
enum qlpiv_autotune { QLPIV_AUTOTUNE_OFF = 0, QLPIV_AUTOTUNE_ON = 1, QLPIV_AUTOTUNE_PERSISTENT = 2 };
enum qlpiv_schedule { QLPIV_SCHEDULE_PER_SIZE = 0, QLPIV_SCHEDULE_PERSISTENT = 1 };
qlpiv_status qlpiv_mixed_plan_create(qlpiv_handle *h, const qlpiv_pass_desc *tmpl, int pixel_type, int num_pairs,
                                     const qlpiv_frame *frames, const int32_t *ia_size, const float *overlap_factor,
                                     int autotune, qlpiv_mixed_plan **plan);
/* The schedule the plan's graph runs (qlpiv_schedule). */
qlpiv_status qlpiv_mixed_plan_schedule(const qlpiv_mixed_plan *plan, int32_t *schedule);
/* total_vectors; pair_offset[num_pairs + 1] (the last entry = total); tiles_ij[2 num_pairs]
 * (tiles_i, tiles_j); waves[4]
 * chosen for sizes 16, 32, 64, 128 (0: default).  Any output may be NULL. */
qlpiv_status qlpiv_mixed_plan_info(const qlpiv_mixed_plan *plan, int64_t *total_vectors, int64_t *pair_offset,
                                   int32_t *tiles_ij, int32_t *waves);
/* Queues the plan's graph on the handle's stream; *device_out receives the device vectors. */
qlpiv_status qlpiv_mixed_plan_run(qlpiv_handle *h, qlpiv_mixed_plan *plan, qlpiv_vector **device_out);
/* Waits for the handle's stream and copies the plan's vectors to the host. */
qlpiv_status qlpiv_mixed_plan_download(qlpiv_handle *h, qlpiv_mixed_plan *plan, qlpiv_vector *host_out);
qlpiv_status qlpiv_mixed_plan_destroy(qlpiv_mixed_plan *plan);

/* ---------------- adaptive batches ----------------
 * Frame pairs of uneven sizes, each with its own adaptive schedule (one of num_schedules
 * descriptors, schedule_of_pair[q]), replayed from one captured CUDA graph.  The pairs that share
 * frame size and schedule form a group that runs qlpiv_piv_adaptive_device's loop over all its
 * pairs (every level one flattened work list); the groups are branches of the graph, forked from
 * and joined into the handle's stream.  `frames` is a host table of device images (u8 or u16);
 * the batch keeps a device copy per group.  Outputs: the last level's displacements of every
 * pair, pair q's tiles_i x tiles_j tiles (row-major) at pair_offset[q], each pair's the same as
 * qlpiv_piv_adaptive gives for it alone.  The reference runs one such job per pair and host
 * thread (S/jobs/OpenClGpuManager.java:121-148). */
typedef struct qlpiv_adaptive_batch qlpiv_adaptive_batch;
qlpiv_status qlpiv_adaptive_batch_create(qlpiv_handle *h, int pixel_type, int num_pairs, const qlpiv_frame *frames,
                                         const qlpiv_adaptive_desc *schedules, int num_schedules,
                                         const int32_t *schedule_of_pair, qlpiv_adaptive_batch **batch);
/* total_tiles; pair_offset[num_pairs + 1]; tiles_ij[2 num_pairs]; groups.  Any output may be NULL. */
qlpiv_status qlpiv_adaptive_batch_info(const qlpiv_adaptive_batch *batch, int64_t *total_tiles,
                                       int64_t *pair_offset, int32_t *tiles_ij, int32_t *groups);
/* Queues the batch's graph on the handle's stream; *device_u / *device_v receive the device
 * displacements (rows, columns). */
qlpiv_status qlpiv_adaptive_batch_run(qlpiv_handle *h, qlpiv_adaptive_batch *batch, float **device_u,
                                      float **device_v);
/* Waits for the handle's stream and copies the displacements to the host. */
qlpiv_status qlpiv_adaptive_batch_download(qlpiv_handle *h, qlpiv_adaptive_batch *batch, float *host_u,
                                           float *host_v);
qlpiv_status qlpiv_adaptive_batch_destroy(qlpiv_adaptive_batch *batch);

/* ---------------- request server (continuous batching) ----------------
 * The reference runs one job per frame pair and host thread (S/jobs/LocalPIVOpenCLGpuJob.java,
 * pooled by OpenClGpuManager.java:121-148); it has no server.  A qlpiv_server owns one device
 * and a device-owner thread: requests (frame pairs of any size, each with its own adaptive
 * schedule) are copied into pinned staging at submit, admitted while their device memory fits
 * the HBM budget and a slot (a CUDA stream with its own plan) is free, run concurrently with the
 * requests already on the device, and complete independently.  A request's displacements are
 * those qlpiv_piv_adaptive gives for the same pair, whatever else is in flight. */
typedef struct qlpiv_server qlpiv_server;

typedef struct qlpiv_server_params {
    int device;
    int slots;                /* concurrent requests on the device; 0: 16 */
    int64_t hbm_budget;       /* device bytes for in-flight requests; 0: 80 % of the free memory */
    int64_t staging_bytes;    /* pinned host bytes for queued inputs and results; 0: 1 GiB */
    int submit_timeout_ms;    /* how long qlpiv_submit waits for staging space; 0: 10 s */
    int reserved[7];
} qlpiv_server_params;

typedef struct qlpiv_request {
    const qlpiv_adaptive_desc *schedule;  /* copied at submit */
    int pixel_type;                       /* QLPIV_PIX_U8 or QLPIV_PIX_U16 */
    int height, width;
    int64_t pitch;                        /* elements per row, >= width */
    const void *img_a, *img_b;            /* copied at submit */
    float *out_u, *out_v;                 /* last-level tiles (rows, columns); written before
                                             qlpiv_poll reports the request done, so they must stay
                                             valid until then */
} qlpiv_request;

typedef struct qlpiv_result {
    int status;               /* qlpiv_status of the request */
    int tiles_i, tiles_j;     /* last-level grid */
    double queue_ms;          /* submit -> admitted to the device */
    double device_ms;         /* admitted -> results on the host */
    double total_ms;          /* submit -> results on the host */
} qlpiv_result;

typedef struct qlpiv_server_stats {
    int64_t submitted, completed, failed, pending, in_flight;
    int64_t device_bytes_in_flight, hbm_budget;
    int64_t reserved[4];
} qlpiv_server_stats;

qlpiv_status qlpiv_server_create(const qlpiv_server_params *params, qlpiv_server **out);
/* Cancels the queued requests (their qlpiv_poll reports QLPIV_E_CANCELLED), waits for those on
 * the device and frees everything. */
qlpiv_status qlpiv_server_destroy(qlpiv_server *s);
/* Checks and copies the request; returns a ticket.  QLPIV_E_TIMEOUT when the staging stayed full
 * for submit_timeout_ms, QLPIV_E_OOM when the request can never fit the budget or the staging. */
qlpiv_status qlpiv_submit(qlpiv_server *s, const qlpiv_request *req, uint64_t *ticket);
/* Waits up to timeout_ms (< 0: forever) for the request.  QLPIV_OK: done, *result filled and the
 * ticket released (check result->status); QLPIV_E_TIMEOUT: not done yet; QLPIV_E_ARG: unknown
 * ticket. */
qlpiv_status qlpiv_poll(qlpiv_server *s, uint64_t ticket, qlpiv_result *result, int timeout_ms);
qlpiv_status qlpiv_server_stats_read(qlpiv_server *s, qlpiv_server_stats *stats);
/* Device bytes an adaptive plan of `pairs` frame pairs uses (the server's admission estimate). */
qlpiv_status qlpiv_adaptive_plan_bytes(const qlpiv_adaptive_desc *desc, int pixel_type, int height, int width,
                                       int pairs, int64_t *bytes);

/* ---------------- Host data formats either side of the path (no device use) ----------------
 *
 * Image ingest replaces S/jobs/ImageReaderJob.java:81-115 (ImageIO read of the frame files) for
 * baseline greyscale TIFF: one sample per pixel, 8 or 16 bits, strips, uncompressed, LZW or PackBits,
 * either byte order.  Other TIFFs are rejected with QLPIV_E_UNSUPPORTED, malformed ones with
 * QLPIV_E_SHAPE.  16-bit samples are returned in host order (12-bit cameras store 0..4095). */
qlpiv_status qlpiv_tiff_info(const char *path, int *height, int *width, int *bits_per_sample);
/* Decodes the image row-major into `pixels` (uint8 or uint16 per bits_per_sample). */
qlpiv_status qlpiv_tiff_read(const char *path, void *pixels, int64_t capacity_bytes);

/* MATLAB level-5 export of the vector maps with the variables of
 * S/exporter/StructMultiFrameFloatVelocityExporter.java (one struct per IA size):
 *   exportDate                      char
 *   parameters                      struct: imageWidth, imageHeight, iaStartI, iaEndI, iaStartJ,
 *                                   iaEndJ (int32), overlapFactor (single), hasSwappedUVVectors,
 *                                   markInvalidAsNaN, totalNumberOfVelocityMaps, multiVolumeExport,
 *                                   multiVolumeLastVolume (int32)                      (:80-115)
 *   velocities<iaHeight>x<iaWidth>  QLPIV_MAT_RUN (the end-of-run export, exportDataToFile(PIVResults),
 *                                   :185-238): iaHeight, iaWidth, multiVolumeExport (int32),
 *                                   margins (struct top, left, bottom, right), u, v (single,
 *                                   tiles_i x tiles_j x frames) taken through PIVMap
 *                                   (S/PIVMap.java:119-133): u = column displacement and v = row
 *                                   displacement unless swap_uv;
 *                                   QLPIV_MAT_STEP (exportDataToFile(frame, IterationStepTiles),
 *                                   :132-181): iaHeight, iaWidth, adaptiveStep, margins, u = row and
 *                                   v = column displacement.
 * Invalid vectors are written as NaN when mark_invalid_as_nan is set. */
/* QLPIV_MAT_DENSE (exportDenseDataToFile, :240-290, the optical-flow dense export): one struct
 * `velocities` with the same fields as QLPIV_MAT_RUN; the map's tiles_i x tiles_j is the whole
 * frame (the dense field of qlpiv_flow_after_piv) and u, v are written for the pixels inside the
 * margins, (H - top - bottom) x (W - left - right) x frames, in PIVMap's U/V order. */
typedef enum { QLPIV_MAT_RUN = 0, QLPIV_MAT_STEP = 1, QLPIV_MAT_DENSE = 2 } qlpiv_mat_layout;

typedef struct qlpiv_mat_export_params {
    int image_width, image_height;
    int ia_start, ia_end;       /* first and last adaptive IA side (square IAs) */
    float overlap_factor;
    int frames;                 /* velocity maps per IA size */
    int swap_uv;                /* PIVMap swapUVOrder, recorded as hasSwappedUVVectors */
    int mark_invalid_as_nan;    /* invalid vectors written as NaN */
    const char *export_date;    /* NULL: the current UTC time */
    int layout;                 /* qlpiv_mat_layout */
    int maps_per_file;          /* multi-volume export (ExecuteLocalPIVWorker's split exports,
                                   ui/.../business/transfer/ExecuteLocalPIVWorker.java:172-215): with
                                   0 < maps_per_file < frames (RUN / DENSE layouts) the frames go to
                                   volumes of maps_per_file maps, volume k written to `path` with its
                                   "_MV0.mat" replaced by "_MV<k>.mat"; each records
                                   multiVolumeExport = 1, totalNumberOfVelocityMaps = frames,
                                   multiVolumeLastVolume and (but the last) multiVolumeNextFilename,
                                   and its velocities structs multiVolumeStartOffset (the first frame
                                   index).  0: one file. */
    int reserved[2];
} qlpiv_mat_export_params;

typedef struct qlpiv_mat_velocity_map {
    int ia_height, ia_width, adaptive_step;
    int tiles_i, tiles_j;
    int margins[4];             /* top, left, bottom, right */
    const float *u, *v;         /* tile displacements along rows (u) and columns (v),
                                   frames x tiles_i x tiles_j, row-major */
    const uint8_t *invalid;     /* same shape, nonzero = invalid; may be NULL */
} qlpiv_mat_velocity_map;

qlpiv_status qlpiv_mat_export(const char *path, const qlpiv_mat_export_params *params, int num_maps,
                              const qlpiv_mat_velocity_map *maps);

/* Stage timing of the adaptive pipeline (CUDA events around every launch on the
 * handle's stream).  Accumulates while enabled; qlpiv_profile_read synchronises the
 * stream, returns the totals per (stage, level) and clears them. */
typedef struct qlpiv_stage_time {
    char stage[24];     /* "inherit", "spline", "warp", "xcorr", "origins" */
    int level;          /* adaptive level, IA side = ia_start >> level */
    int ia_side;
    long launches;      /* kernel launches accumulated */
    long items;         /* IAs (xcorr) or pixels (warp) or tiles processed */
    double ms;          /* summed device time */
} qlpiv_stage_time;

qlpiv_status qlpiv_profile_enable(qlpiv_handle *h, int enable);
qlpiv_status qlpiv_profile_read(qlpiv_handle *h, qlpiv_stage_time *out, int cap, int *count);

/* Instrumentation: FP32 FMA throughput of `device` measured with a short probe kernel
 * (TFLOP/s, best of three), the compute roofline denominator of the FFT kernels. */
qlpiv_status qlpiv_measure_fp32_peak(int device, double *tflops);

/* Instrumentation: the sub-pixel fit's float-pair logarithm beside CUDA's double log for n
 * positive normal floats (host arrays), to check its error bound on the device. */
qlpiv_status qlpiv_probe_log(int device, const float *x, long n, double *mine, double *ref);

/* Instrumentation: the IA-16 kernel's tile normalisation divides integer pixels by integer
 * maxima with a reciprocal and one exact correction step instead of the general division; this
 * runs it against IEEE division for every v in [0, 65535] and divisor in [1, 65535] and returns
 * the number of quotients that differ (0 expected). */
qlpiv_status qlpiv_probe_division(int device, int64_t *mismatches);

/* Number of kernel launches issued by this handle since creation (instrumentation). */
long qlpiv_launch_count(qlpiv_handle *h);

#ifdef __cplusplus
}
#endif

#endif /* QLPIV_H */
