// Velocity inheritance without any device allocation.
//
// Some callers cannot let the library allocate device memory inside a call: a Java
// host that hands over device buffers from its own pool through JNI or Panama and keeps
// a fixed device-memory budget, or an acquisition loop that must not pay cudaMalloc's
// implicit synchronisation (and the failure it can bring when memory is short) while
// frames stream in.  qlpiv_inherit_noalloc serves them: the caller passes every input and
// output in device memory, and the one scratch buffer the two-stage inheritance needs
// (the stage-1 row table) is a file-scope device array of fixed size that lives as long
// as the library is loaded on the device.
#include <cuda_runtime.h>

#include <mutex>

#include "qlpiv_adaptive.h"
#include "qlpiv_handle.h"
#include "qlpiv_internal.h"

namespace {

// Stage-1 row table: u values then v values, QLPIV_NOALLOC_MAX_ROWS floats each (4 MiB).
static __device__ __align__(256) float g_inherit_rows[2 * QLPIV_NOALLOC_MAX_ROWS];

std::mutex g_mu;
float *g_rows_addr[qlpiv::kMaxDevices] = {nullptr};

// Device address of g_inherit_rows on `dev` (the current device), looked up once.
cudaError_t rows_address(int dev, float **out) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_rows_addr[dev] == nullptr) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_inherit_rows);
        if (e != cudaSuccess) return e;
        g_rows_addr[dev] = static_cast<float *>(p);
    }
    *out = g_rows_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" qlpiv_status qlpiv_inherit_noalloc(int device, void *stream, int pni, int pnj, const float *p_ci,
                                              const float *p_cj, const float *pu, const float *pv, int cni, int cnj,
                                              const float *c_ci, const float *c_cj, int round_int, float *cu,
                                              float *cv) {
    if (!p_ci || !p_cj || !pu || !pv || !c_ci || !c_cj || !cu || !cv) return qlpiv::fail(QLPIV_E_ARG, "NULL argument");
    if (pni < 1 || pnj < 1 || cni < 1 || cnj < 1) return qlpiv::fail(QLPIV_E_SHAPE, "empty grid");
    if ((long)cni * pnj > QLPIV_NOALLOC_MAX_ROWS)
        return qlpiv::fail(QLPIV_E_SHAPE,
                           "child rows x parent columns = %ld exceeds the fixed scratch of %d entries "
                           "(QLPIV_NOALLOC_MAX_ROWS); use qlpiv_inherit",
                           (long)cni * pnj, QLPIV_NOALLOC_MAX_ROWS);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return qlpiv::fail(QLPIV_E_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= ndev || device >= qlpiv::kMaxDevices)
        return qlpiv::fail(QLPIV_E_ARG, "device %d out of range", device);
    qlpiv::DeviceScope ds(device);
    if (ds.err != cudaSuccess) return qlpiv::cuda_fail(ds.err, "cudaSetDevice");
    float *rows = nullptr;
    cudaError_t e = rows_address(device, &rows);
    if (e != cudaSuccess) return qlpiv::cuda_fail(e, "cudaGetSymbolAddress");
    // Stage 1 writes every row-table entry stage 2 reads, so nothing needs clearing.
    e = qlpiv::launch_inherit(static_cast<cudaStream_t>(stream), 1, p_ci, pni, p_cj, pnj, pu, pv, c_ci, cni, c_cj, cnj,
                              round_int, rows, rows + QLPIV_NOALLOC_MAX_ROWS, cu, cv);
    if (e != cudaSuccess) return qlpiv::cuda_fail(e, "inherit");
    return QLPIV_OK;
}
