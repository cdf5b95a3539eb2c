// C ABI of libqlpiv_gpu.so: handles, workspace, argument checking, transfers.
// Declarations and reference citations: include/qlpiv.h.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "qlpiv_handle.h"
#include "qlpiv_internal.h"
#include "qlpiv_xcorr.cuh"

namespace {

thread_local std::string g_last_error;
thread_local qlpiv::AsyncAlloc g_async_alloc;

}  // namespace

namespace qlpiv {

AsyncAlloc &async_alloc_tls() { return g_async_alloc; }

qlpiv_status fail(qlpiv_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

qlpiv_status cuda_fail(cudaError_t e, const char *what) {
    if (e == cudaErrorMemoryAllocation) return fail(QLPIV_E_OOM, "%s: %s", what, cudaGetErrorString(e));
    return fail(QLPIV_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

qlpiv_status check_subpix(int mode, int pixels, int iterations) {
    if (mode == QLPIV_SUBPIX_NONE || mode == QLPIV_SUBPIX_GAUSS3) return QLPIV_OK;
    if (mode != QLPIV_SUBPIX_GAUSS_LM && mode != QLPIV_SUBPIX_HONGWEI_GUO)
        return fail(QLPIV_E_ARG, "unknown sub-pixel mode %d", mode);
    if (pixels < 3 || pixels > QLPIV_MAX_SUBPIX_PIXELS || pixels % 2 != 1)
        return fail(QLPIV_E_ARG, "Number of interpolation pixels must be an odd number (3..%d), got %d",
                    QLPIV_MAX_SUBPIX_PIXELS, pixels);
    if (mode == QLPIV_SUBPIX_HONGWEI_GUO && (iterations < 6 || iterations > 50))
        return fail(QLPIV_E_ARG, "Invalid number of interpolations: should be >= 6 and <= 50, got %d", iterations);
    return QLPIV_OK;
}

}  // namespace qlpiv

using qlpiv::cuda_fail;
using qlpiv::DeviceScope;
using qlpiv::DevBuf;
using qlpiv::fail;

namespace {


qlpiv_status check_desc(const qlpiv_pass_desc *d) {
    if (!d) return fail(QLPIV_E_ARG, "pass descriptor is NULL");
    if (!qlpiv::xcorr_size_supported(d->n))
        return fail(QLPIV_E_SHAPE, "IA size %d is not supported (16, 32, 64, 128)", d->n);
    if (d->norm_mode != QLPIV_NORM_MAX_A && d->norm_mode != QLPIV_NORM_OWN_MAX && d->norm_mode != QLPIV_NORM_NONE)
        return fail(QLPIV_E_ARG, "unknown normalisation mode %d", d->norm_mode);
    if (d->max_mode != QLPIV_MAX_COMPUTE && d->max_mode != QLPIV_MAX_FIXED && d->max_mode != QLPIV_MAX_FIXED_A &&
        d->max_mode != QLPIV_MAX_FIXED_B)
        return fail(QLPIV_E_ARG, "max mode %d not valid for a frame pass", d->max_mode);
    if ((d->max_mode == QLPIV_MAX_FIXED || d->max_mode == QLPIV_MAX_FIXED_A) && !(d->fixed_max_a > 0.0f))
        return fail(QLPIV_E_ARG, "fixed tile maxima must be positive");
    if ((d->max_mode == QLPIV_MAX_FIXED || d->max_mode == QLPIV_MAX_FIXED_B) && !(d->fixed_max_b > 0.0f))
        return fail(QLPIV_E_ARG, "fixed tile maxima must be positive");
    if (qlpiv_status st = qlpiv::check_subpix(d->subpix_mode, d->subpix_pixels, d->subpix_iterations)) return st;
    if (d->num_peaks != 0 && !qlpiv::multipeak_supported(d->n, d->num_peaks, d->peak_kernel))
        return fail(QLPIV_E_ARG, "multi-peak search: %d peaks with cell width %d not supported for IA %d "
                    "(1..%d peaks, cell width >= 2)", d->num_peaks, d->peak_kernel, d->n, QLPIV_MAX_PEAKS);
    return QLPIV_OK;
}

// vectors written per IA: one, or num_peaks in multi-peak mode
long vectors_per_ia(const qlpiv_pass_desc *d) { return d->num_peaks > 0 ? d->num_peaks : 1; }

qlpiv_status check_pixel(int pixel_type) {
    if (pixel_type != QLPIV_PIX_U8 && pixel_type != QLPIV_PIX_U16 && pixel_type != QLPIV_PIX_F32)
        return fail(QLPIV_E_ARG, "unknown pixel type %d", pixel_type);
    return QLPIV_OK;
}

qlpiv_status launch(qlpiv_handle *h, const qlpiv::IaJob &job, int n, int pixel_type) {
    qlpiv::IaJob j = job;
    cudaError_t e;
    if (j.num_peaks >= 1 && j.num_peaks <= 4 && n <= 64 &&
        (j.subpix == QLPIV_SUBPIX_NONE || j.subpix == QLPIV_SUBPIX_GAUSS3)) {
        // the batched multi-peak replay (the handle's buffers: its calls share one stream)
        if (h->mp_units == 0) {
            long units = 0;
            const size_t bytes = qlpiv::xcorr_batch_bytes(h->num_sms, &units);
            const size_t sb = qlpiv::xcorr_batch_slot_bytes(units);
            if ((e = h->mp_batch.ensure(bytes)) != cudaSuccess || (e = h->mp_slots.ensure(sb)) != cudaSuccess ||
                (e = cudaMemsetAsync(h->mp_slots.p, 0, sb, h->stream)) != cudaSuccess)
                return cuda_fail(e, "multi-peak batch buffers");
            h->mp_units = units;
        }
        if ((e = h->mp_retry.ensure(sizeof(int) * (size_t)(1 + j.count))) != cudaSuccess)
            return cuda_fail(e, "multi-peak retry list");
        j.mp_batch = h->mp_batch.as<qlpiv::MpBatch>();
        j.mp_batch_units = h->mp_units;
        j.mp_slots = h->mp_slots.as<unsigned>();
        j.mp_retry = h->mp_retry.as<int>();
    }
    int nk = 1;
    e = qlpiv::launch_xcorr(j, n, pixel_type, h->stream, h->num_sms, &nk);
    if (e != cudaSuccess) return cuda_fail(e, "xcorr kernel launch");
    h->launches += nk;
    return QLPIV_OK;
}

// Shared body of qlpiv_xcorr_planes / qlpiv_xcorr_peaks: tiles of n x n pixels,
// contiguous per tile, form a virtual image of count*n rows and n columns.
qlpiv_status tiles_call(qlpiv_handle *h, int n, long count, int pixel_type, const void *ta, const void *tb,
                        const float *max_a, const float *max_b, int norm_mode, int subpix_mode,
                        qlpiv_vector *vec_out, float *planes_out, int num_peaks = 0, int peak_kernel = 0) {
    if (!h) return fail(QLPIV_E_ARG, "handle is NULL");
    if (count < 0) return fail(QLPIV_E_ARG, "count < 0");
    if (count == 0) return QLPIV_OK;
    if (!ta || !tb) return fail(QLPIV_E_ARG, "tile arrays are NULL");
    if ((max_a == nullptr) != (max_b == nullptr)) return fail(QLPIV_E_ARG, "give both tile max arrays or none");
    if (!qlpiv::xcorr_size_supported(n)) return fail(QLPIV_E_SHAPE, "IA size %d is not supported (16, 32, 64, 128)", n);
    qlpiv_status st = check_pixel(pixel_type);
    if (st != QLPIV_OK) return st;
    if (norm_mode != QLPIV_NORM_MAX_A && norm_mode != QLPIV_NORM_OWN_MAX && norm_mode != QLPIV_NORM_NONE)
        return fail(QLPIV_E_ARG, "unknown normalisation mode %d", norm_mode);
    if ((long)n * n * count > (1L << 31) - 1) return fail(QLPIV_E_SHAPE, "tile batch too large for one call");
    if (num_peaks != 0 && !qlpiv::multipeak_supported(n, num_peaks, peak_kernel))
        return fail(QLPIV_E_ARG, "multi-peak search: %d peaks with cell width %d not supported for IA %d "
                    "(1..%d peaks, cell width >= 2)", num_peaks, peak_kernel, n, QLPIV_MAX_PEAKS);
    const long kq = num_peaks > 0 ? num_peaks : 1;

    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    const size_t tile_bytes = (size_t)n * n * qlpiv::pixel_bytes(pixel_type) * count;
    const int d = 2 * n - 1;
    cudaError_t e;
    if ((e = h->tiles_a.ensure(tile_bytes)) != cudaSuccess) return cuda_fail(e, "tile buffer");
    if ((e = h->tiles_b.ensure(tile_bytes)) != cudaSuccess) return cuda_fail(e, "tile buffer");
    if (max_a) {
        if ((e = h->max_a.ensure(sizeof(float) * count)) != cudaSuccess) return cuda_fail(e, "max buffer");
        if ((e = h->max_b.ensure(sizeof(float) * count)) != cudaSuccess) return cuda_fail(e, "max buffer");
    }
    if ((e = h->vectors.ensure(sizeof(qlpiv_vector) * count * kq)) != cudaSuccess)
        return cuda_fail(e, "vector buffer");
    if (planes_out && (e = h->planes.ensure(sizeof(float) * (size_t)d * d * count)) != cudaSuccess)
        return cuda_fail(e, "plane buffer");

    if ((e = cudaMemcpyAsync(h->tiles_a.p, ta, tile_bytes, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(h->tiles_b.p, tb, tile_bytes, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess)
        return cuda_fail(e, "tile upload");
    if (max_a) {
        if ((e = cudaMemcpyAsync(h->max_a.p, max_a, sizeof(float) * count, cudaMemcpyHostToDevice, h->stream)) !=
                cudaSuccess ||
            (e = cudaMemcpyAsync(h->max_b.p, max_b, sizeof(float) * count, cudaMemcpyHostToDevice, h->stream)) !=
                cudaSuccess)
            return cuda_fail(e, "max upload");
    }

    qlpiv::IaJob job{};
    job.img_a = h->tiles_a.p;
    job.img_b = h->tiles_b.p;
    job.pitch_a = job.pitch_b = n;
    job.h = (int)(count * n);
    job.w = n;
    job.frames = nullptr;
    job.frame_idx = nullptr;
    job.a_top = job.a_left = job.b_top = job.b_left = nullptr;  // tile k at row k*n
    job.max_a = max_a ? (const float *)h->max_a.p : nullptr;
    job.max_b = max_b ? (const float *)h->max_b.p : nullptr;
    job.count = count;
    job.norm_mode = norm_mode;
    job.max_mode = max_a ? QLPIV_MAX_GIVEN : QLPIV_MAX_COMPUTE;
    job.subpix = subpix_mode;  // tile entry points: none or 3-point
    job.out = (qlpiv_vector *)h->vectors.p;
    job.planes = planes_out ? (float *)h->planes.p : nullptr;
    job.num_peaks = num_peaks;
    job.peak_kernel = peak_kernel;
    if ((st = launch(h, job, n, pixel_type)) != QLPIV_OK) return st;

    if (vec_out && (e = cudaMemcpyAsync(vec_out, h->vectors.p, sizeof(qlpiv_vector) * count * kq,
                                        cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess)
        return cuda_fail(e, "vector download");
    if (planes_out && (e = cudaMemcpyAsync(planes_out, h->planes.p, sizeof(float) * (size_t)d * d * count,
                                           cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess)
        return cuda_fail(e, "plane download");
    if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return cuda_fail(e, "xcorr");
    return QLPIV_OK;
}

qlpiv::IaJob frame_job(const qlpiv_pass_desc *desc, const void *img_a, const void *img_b, int height, int width,
                       long count, const int32_t *at, const int32_t *al, const int32_t *bt, const int32_t *bl,
                       qlpiv_vector *out) {
    qlpiv::IaJob job{};
    job.img_a = img_a;
    job.img_b = img_b;
    job.pitch_a = job.pitch_b = width;
    job.h = height;
    job.w = width;
    job.frames = nullptr;
    job.frame_idx = nullptr;
    job.a_top = at;
    job.a_left = al;
    job.b_top = bt;
    job.b_left = bl;
    job.max_a = job.max_b = nullptr;
    job.count = count;
    job.norm_mode = desc->norm_mode;
    job.max_mode = desc->max_mode;
    job.fixed_max_a = desc->fixed_max_a;
    job.fixed_max_b = desc->fixed_max_b;
    job.subpix = desc->subpix_mode;
    job.subpix_pixels = desc->subpix_mode >= QLPIV_SUBPIX_GAUSS_LM ? desc->subpix_pixels : 0;
    job.subpix_iters = desc->subpix_iterations;
    job.out = out;
    job.planes = nullptr;
    job.num_peaks = desc->num_peaks;
    job.peak_kernel = desc->peak_kernel;
    return job;
}

qlpiv_status check_frame(qlpiv_handle *h, const qlpiv_pass_desc *desc, const void *img_a, const void *img_b,
                         int height, int width, int pixel_type, long count, const int32_t *at, const int32_t *al,
                         const int32_t *bt, const int32_t *bl, const void *out) {
    if (!h) return fail(QLPIV_E_ARG, "handle is NULL");
    qlpiv_status st = check_desc(desc);
    if (st != QLPIV_OK) return st;
    if ((st = check_pixel(pixel_type)) != QLPIV_OK) return st;
    if (count < 0) return fail(QLPIV_E_ARG, "count < 0");
    if (height <= 0 || width <= 0) return fail(QLPIV_E_SHAPE, "image size %d x %d", height, width);
    if (count > 0 && (!img_a || !img_b || !at || !al || !bt || !bl || !out))
        return fail(QLPIV_E_ARG, "NULL image, origin or output pointer");
    return QLPIV_OK;
}


qlpiv_status check_batch(qlpiv_handle *h, const qlpiv_pass_desc *desc, int pixel_type, int num_frames,
                         const qlpiv_frame *frames, long count, const int32_t *fi, const int32_t *at,
                         const int32_t *al, const int32_t *bt, const int32_t *bl, const void *out) {
    if (!h) return fail(QLPIV_E_ARG, "handle is NULL");
    qlpiv_status st = check_desc(desc);
    if (st != QLPIV_OK) return st;
    if ((st = check_pixel(pixel_type)) != QLPIV_OK) return st;
    if (count < 0 || num_frames < 0) return fail(QLPIV_E_ARG, "negative count");
    if (count > 0 && (num_frames == 0 || !frames || !fi || !at || !al || !bt || !bl || !out))
        return fail(QLPIV_E_ARG, "NULL frame table, work list or output pointer");
    return QLPIV_OK;
}

qlpiv::IaJob batch_job(const qlpiv_pass_desc *desc, const qlpiv_frame *frames_dev, int num_frames, long count,
                       const int32_t *fi, const int32_t *at, const int32_t *al, const int32_t *bt, const int32_t *bl,
                       qlpiv_vector *out) {
    qlpiv::IaJob job = frame_job(desc, nullptr, nullptr, 0, 0, count, at, al, bt, bl, out);
    job.frames = frames_dev;
    job.frame_idx = fi;
    job.num_frames = num_frames;
    return job;
}

}  // namespace

extern "C" {

int qlpiv_abi_version(void) { return QLPIV_ABI_VERSION; }

const char *qlpiv_last_error(void) { return g_last_error.c_str(); }

qlpiv_status qlpiv_create(const qlpiv_params *params, qlpiv_handle **out) {
    if (!out) return fail(QLPIV_E_ARG, "output handle pointer is NULL");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(QLPIV_E_NO_DEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
    const int dev = params ? params->device : 0;
    if (dev < 0 || dev >= ndev || dev >= qlpiv::kMaxDevices) return fail(QLPIV_E_ARG, "device %d out of range", dev);
    qlpiv_handle *h = new qlpiv_handle();
    h->device = dev;
    DeviceScope ds(dev);
    if (ds.err != cudaSuccess) {
        delete h;
        return cuda_fail(ds.err, "cudaSetDevice");
    }
    if ((e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking)) != cudaSuccess) {
        delete h;
        return cuda_fail(e, "handle set-up");
    }
    h->stream = h->own_stream;
    // FFT twiddle tables: uploaded here, before any stream of this handle can be captured
    const qlpiv::cplx *tw = nullptr;
    if ((e = qlpiv::ensure_twiddles(dev, &tw)) != cudaSuccess) {
        cudaStreamDestroy(h->own_stream);
        delete h;
        return cuda_fail(e, "twiddle tables");
    }
    *out = h;
    return QLPIV_OK;
}

qlpiv_status qlpiv_destroy(qlpiv_handle *h) {
    if (!h) return QLPIV_OK;
    {
        DeviceScope ds(h->device);
        if (h->stream) cudaStreamSynchronize(h->stream);
        if (h->own_stream) {
            cudaStreamSynchronize(h->own_stream);
            cudaStreamDestroy(h->own_stream);
        }
        for (DevBuf *b : {&h->tiles_a, &h->tiles_b, &h->max_a, &h->max_b, &h->origins, &h->vectors, &h->planes,
                          &h->frames, &h->mp_batch, &h->mp_slots, &h->mp_retry})
            b->release();
        for (DevBuf &b : h->scratch) b.release();
        for (qlpiv::StageEvent &ev : h->prof_pending) {
            cudaEventDestroy(ev.begin);
            cudaEventDestroy(ev.end);
        }
        if (h->plan) qlpiv::destroy_plan(h->plan);
        h->plan = nullptr;
    }
    delete h;
    return QLPIV_OK;
}

qlpiv_status qlpiv_synchronize(qlpiv_handle *h) {
    if (!h) return fail(QLPIV_E_ARG, "handle is NULL");
    DeviceScope ds(h->device);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "synchronize");
    return QLPIV_OK;
}

long qlpiv_launch_count(qlpiv_handle *h) { return h ? h->launches : -1; }

qlpiv_status qlpiv_xcorr_planes(qlpiv_handle *h, int n, long count, int pixel_type, const void *tiles_a,
                                const void *tiles_b, const float *max_a, const float *max_b, int norm_mode,
                                float *planes_out) {
    if (count > 0 && !planes_out) return fail(QLPIV_E_ARG, "planes_out is NULL");
    return tiles_call(h, n, count, pixel_type, tiles_a, tiles_b, max_a, max_b, norm_mode, QLPIV_SUBPIX_NONE, nullptr,
                      planes_out);
}

qlpiv_status qlpiv_xcorr_peaks(qlpiv_handle *h, int n, long count, int pixel_type, const void *tiles_a,
                               const void *tiles_b, const float *max_a, const float *max_b, int norm_mode,
                               int subpix_mode, qlpiv_vector *out) {
    if (count > 0 && !out) return fail(QLPIV_E_ARG, "output vector array is NULL");
    if (subpix_mode != QLPIV_SUBPIX_NONE && subpix_mode != QLPIV_SUBPIX_GAUSS3)
        return fail(QLPIV_E_ARG, "unknown sub-pixel mode %d", subpix_mode);
    return tiles_call(h, n, count, pixel_type, tiles_a, tiles_b, max_a, max_b, norm_mode, subpix_mode, out, nullptr);
}

qlpiv_status qlpiv_xcorr_multipeaks(qlpiv_handle *h, int n, long count, int pixel_type, const void *tiles_a,
                                    const void *tiles_b, const float *max_a, const float *max_b, int norm_mode,
                                    int subpix_mode, int num_peaks, int peak_kernel, qlpiv_vector *out) {
    if (count > 0 && !out) return fail(QLPIV_E_ARG, "output vector array is NULL");
    if (subpix_mode != QLPIV_SUBPIX_NONE && subpix_mode != QLPIV_SUBPIX_GAUSS3)
        return fail(QLPIV_E_ARG, "unknown sub-pixel mode %d", subpix_mode);
    if (num_peaks < 1) return fail(QLPIV_E_ARG, "num_peaks must be >= 1");
    return tiles_call(h, n, count, pixel_type, tiles_a, tiles_b, max_a, max_b, norm_mode, subpix_mode, out, nullptr,
                      num_peaks, peak_kernel);
}

qlpiv_status qlpiv_pass(qlpiv_handle *h, const qlpiv_pass_desc *desc, const void *img_a, const void *img_b,
                        int height, int width, int pixel_type, long count, const int32_t *a_top,
                        const int32_t *a_left, const int32_t *b_top, const int32_t *b_left, qlpiv_vector *out) {
    qlpiv_status st = check_frame(h, desc, img_a, img_b, height, width, pixel_type, count, a_top, a_left, b_top,
                                  b_left, out);
    if (st != QLPIV_OK || count == 0) return st;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    const size_t img_bytes = (size_t)height * width * qlpiv::pixel_bytes(pixel_type);
    cudaError_t e;
    if ((e = h->tiles_a.ensure(img_bytes)) != cudaSuccess || (e = h->tiles_b.ensure(img_bytes)) != cudaSuccess ||
        (e = h->origins.ensure(sizeof(int32_t) * 4 * count)) != cudaSuccess ||
        (e = h->vectors.ensure(sizeof(qlpiv_vector) * count * vectors_per_ia(desc))) != cudaSuccess)
        return cuda_fail(e, "workspace");
    int32_t *org = (int32_t *)h->origins.p;
    if ((e = cudaMemcpyAsync(h->tiles_a.p, img_a, img_bytes, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(h->tiles_b.p, img_b, img_bytes, cudaMemcpyHostToDevice, h->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(org, a_top, sizeof(int32_t) * count, cudaMemcpyHostToDevice, h->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(org + count, a_left, sizeof(int32_t) * count, cudaMemcpyHostToDevice, h->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(org + 2 * count, b_top, sizeof(int32_t) * count, cudaMemcpyHostToDevice, h->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(org + 3 * count, b_left, sizeof(int32_t) * count, cudaMemcpyHostToDevice, h->stream)) !=
            cudaSuccess)
        return cuda_fail(e, "upload");
    qlpiv::IaJob job = frame_job(desc, h->tiles_a.p, h->tiles_b.p, height, width, count, org, org + count,
                                 org + 2 * count, org + 3 * count, (qlpiv_vector *)h->vectors.p);
    if ((st = launch(h, job, desc->n, pixel_type)) != QLPIV_OK) return st;
    if ((e = cudaMemcpyAsync(out, h->vectors.p, sizeof(qlpiv_vector) * count * vectors_per_ia(desc),
                             cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess)
        return cuda_fail(e, "download");
    if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return cuda_fail(e, "pass");
    return QLPIV_OK;
}

qlpiv_status qlpiv_pass_device(qlpiv_handle *h, const qlpiv_pass_desc *desc, const void *img_a,
                               const void *img_b, int height, int width, int pixel_type, long count,
                               const int32_t *a_top, const int32_t *a_left, const int32_t *b_top,
                               const int32_t *b_left, qlpiv_vector *out) {
    qlpiv_status st = check_frame(h, desc, img_a, img_b, height, width, pixel_type, count, a_top, a_left, b_top,
                                  b_left, out);
    if (st != QLPIV_OK || count == 0) return st;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    qlpiv::IaJob job = frame_job(desc, img_a, img_b, height, width, count, a_top, a_left, b_top, b_left, out);
    return launch(h, job, desc->n, pixel_type);
}

qlpiv_status qlpiv_pass_batch(qlpiv_handle *h, const qlpiv_pass_desc *desc, int pixel_type, int num_frames,
                              const qlpiv_frame *frames, long count, const int32_t *frame_of_ia,
                              const int32_t *a_top, const int32_t *a_left, const int32_t *b_top,
                              const int32_t *b_left, qlpiv_vector *out) {
    qlpiv_status st = check_batch(h, desc, pixel_type, num_frames, frames, count, frame_of_ia, a_top, a_left, b_top,
                                  b_left, out);
    if (st != QLPIV_OK || count == 0) return st;
    for (long k = 0; k < count; k++)
        if (frame_of_ia[k] < 0 || frame_of_ia[k] >= num_frames)
            return fail(QLPIV_E_ARG, "frame_of_ia[%ld] = %d is outside [0, %d)", k, frame_of_ia[k], num_frames);
    const size_t pb = qlpiv::pixel_bytes(pixel_type);
    size_t total = 0;
    for (int f = 0; f < num_frames; f++) {
        const qlpiv_frame &fr = frames[f];
        if (fr.height <= 0 || fr.width <= 0 || fr.pitch < fr.width || !fr.img_a || !fr.img_b)
            return fail(QLPIV_E_SHAPE, "frame %d: bad geometry or NULL image", f);
        total += 2 * (((size_t)fr.height * fr.width * pb + 255) & ~(size_t)255);
    }
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    cudaError_t e;
    if ((e = h->tiles_a.ensure(total)) != cudaSuccess || (e = h->frames.ensure(sizeof(qlpiv_frame) * num_frames)) !=
        cudaSuccess || (e = h->origins.ensure(sizeof(int32_t) * 5 * count)) != cudaSuccess ||
        (e = h->vectors.ensure(sizeof(qlpiv_vector) * count * vectors_per_ia(desc))) != cudaSuccess)
        return cuda_fail(e, "workspace");
    // pack the images densely (pitch = width) and rebuild the frame table for the device
    std::vector<qlpiv_frame> dev_frames(num_frames);
    char *base = (char *)h->tiles_a.p;
    size_t off = 0;
    for (int f = 0; f < num_frames; f++) {
        const qlpiv_frame &fr = frames[f];
        const size_t row = (size_t)fr.width * pb, bytes = row * fr.height;
        char *da = base + off;
        off += (bytes + 255) & ~(size_t)255;
        char *db = base + off;
        off += (bytes + 255) & ~(size_t)255;
        // rows packed in the host image (pitch == width): one linear copy per image
        const size_t spitch = (size_t)fr.pitch * pb;
        auto upload = [&](char *d, const void *src) {
            return spitch == row ? cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, h->stream)
                                 : cudaMemcpy2DAsync(d, row, src, spitch, row, fr.height, cudaMemcpyHostToDevice,
                                                     h->stream);
        };
        if ((e = upload(da, fr.img_a)) != cudaSuccess || (e = upload(db, fr.img_b)) != cudaSuccess)
            return cuda_fail(e, "frame upload");
        dev_frames[f] = {da, db, fr.height, fr.width, (int64_t)fr.width};
    }
    int32_t *org = (int32_t *)h->origins.p;
    const int32_t *src[5] = {frame_of_ia, a_top, a_left, b_top, b_left};
    for (int k = 0; k < 5; k++)
        if ((e = cudaMemcpyAsync(org + k * count, src[k], sizeof(int32_t) * count, cudaMemcpyHostToDevice,
                                 h->stream)) != cudaSuccess)
            return cuda_fail(e, "work list upload");
    if ((e = cudaMemcpyAsync(h->frames.p, dev_frames.data(), sizeof(qlpiv_frame) * num_frames,
                             cudaMemcpyHostToDevice, h->stream)) != cudaSuccess)
        return cuda_fail(e, "frame table upload");
    qlpiv::IaJob job = batch_job(desc, (const qlpiv_frame *)h->frames.p, num_frames, count, org, org + count,
                                 org + 2 * count,
                                 org + 3 * count, org + 4 * count, (qlpiv_vector *)h->vectors.p);
    if ((st = launch(h, job, desc->n, pixel_type)) != QLPIV_OK) return st;
    if ((e = cudaMemcpyAsync(out, h->vectors.p, sizeof(qlpiv_vector) * count * vectors_per_ia(desc),
                             cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess)
        return cuda_fail(e, "download");
    // the frame table lives in pageable host memory: wait before it goes out of scope
    if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return cuda_fail(e, "batch pass");
    return QLPIV_OK;
}

qlpiv_status qlpiv_pass_batch_device(qlpiv_handle *h, const qlpiv_pass_desc *desc, int pixel_type,
                                     int num_frames, const qlpiv_frame *frames, long count,
                                     const int32_t *frame_of_ia, const int32_t *a_top, const int32_t *a_left,
                                     const int32_t *b_top, const int32_t *b_left, qlpiv_vector *out) {
    qlpiv_status st = check_batch(h, desc, pixel_type, num_frames, frames, count, frame_of_ia, a_top, a_left, b_top,
                                  b_left, out);
    if (st != QLPIV_OK || count == 0) return st;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    qlpiv::IaJob job = batch_job(desc, frames, num_frames, count, frame_of_ia, a_top, a_left, b_top, b_left, out);
    return launch(h, job, desc->n, pixel_type);
}

qlpiv_status qlpiv_get_stream(qlpiv_handle *h, void **stream) {
    if (!h || !stream) return fail(QLPIV_E_ARG, "NULL argument");
    *stream = (void *)h->stream;
    return QLPIV_OK;
}

qlpiv_status qlpiv_set_stream(qlpiv_handle *h, void *stream) {
    if (!h) return fail(QLPIV_E_ARG, "handle is NULL");
    std::lock_guard<std::mutex> lock(h->mu);
    h->stream = stream ? (cudaStream_t)stream : h->own_stream;
    return QLPIV_OK;
}

}  // extern "C"
