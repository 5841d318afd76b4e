// cb_solve_noalloc: the tangent solve for callers that cannot allocate GPU
// memory.
//
// Some callers of this library may not call cudaMalloc at the point where
// they need a solve: a host application that reserved the GPU's memory up
// front for its own allocator or a fixed pool (cudaMalloc then fails or
// takes memory the pool counts on), or a real-time loop whose memory
// footprint must not change after start-up. cb_solve_noalloc serves them.
// It runs the same solve kernels as cb_factor_solve, but its three work
// vectors and its grid-barrier counters live in the file-scope device array
// below instead of in memory the handle allocated, and it allocates
// nothing: no cudaMalloc, no cudaFree.
#include <cuda_runtime.h>

#include <mutex>

#include "cubens_gb300.h"
#include "internal.hpp"

// Scratch for the solve: 256 bytes of grid-barrier counters, then the three
// work vectors (3 * npad elements of the factor's precision), at most
// 3 * CB_NOALLOC_MAX_EQ doubles (12 MiB). Every GPU that loads this library
// holds it until the process exits.
#define CB_NOALLOC_MAX_EQ (1L << 19)
static __device__ __align__(256) unsigned char g_solve_scratch[256 + 3 * CB_NOALLOC_MAX_EQ * sizeof(double)];

extern "C" cb::BandFactor *cb_internal_factor(cb_model *m, cudaStream_t *st, int *device);
extern "C" void cb_internal_set_error(cb_model *m, const char *msg);

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on `device`, looked up once per
// device with that device current. In host code the symbol is only a
// host-side stand-in, so kernels must be given this address instead. The
// address is kept for the life of the process: a cudaDeviceReset of the
// device invalidates it, and the entry point is not to be used after one.
cudaError_t scratch_address(int device, void **out)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    if (!g_scratch_addr[device]) {
        int prev = 0;
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) return e;
        if (prev != device && (e = cudaSetDevice(device)) != cudaSuccess) return e;
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_solve_scratch);
        if (prev != device) cudaSetDevice(prev);
        if (e != cudaSuccess) return e;
        g_scratch_addr[device] = p;
    }
    *out = g_scratch_addr[device];
    return cudaSuccess;
}

}  // namespace

extern "C" int cb_solve_noalloc(cb_model *m, const double *rhs, double *x)
{
    if (!m || !rhs || !x) return CB_ERR_ARG;
    cudaStream_t st = nullptr;
    int device = 0;
    cb::BandFactor *f = cb_internal_factor(m, &st, &device);
    if (!f || !f->band) return CB_ERR_STATE;
    const size_t need = cb::band_work_bytes(*f);
    if (need > sizeof(g_solve_scratch)) {
        cb_internal_set_error(m, "cb_solve_noalloc: the model needs more solve scratch than the static "
                                 "limit of 3 x 524288 doubles (padded equations > 524288 with an FP64 "
                                 "factor, > 1048576 with an FP32 factor)");
        return CB_ERR_LIMIT;
    }
    void *scratch = nullptr;
    cudaError_t e = scratch_address(device, &scratch);
    if (e != cudaSuccess) {
        cb_internal_set_error(m, cudaGetErrorString(e));
        return CB_ERR_CUDA;
    }
    int prev = 0;
    cudaGetDevice(&prev);
    if (prev != device) cudaSetDevice(device);
    // the grid and chain barriers sit at the start of the scratch; a wait that
    // gave up sets the grid barrier's error flag (the chain barrier's too)
    cb::GridBarrier bar[2] = {};
    try {
        cb::band_solve_with_work(*f, rhs, x, scratch, st);
        e = cudaMemcpyAsync(bar, scratch, sizeof bar, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    } catch (const std::exception &ex) {
        cb_internal_set_error(m, ex.what());
        e = cudaErrorUnknown;
    }
    if (prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess) {
        if (e != cudaErrorUnknown) cb_internal_set_error(m, cudaGetErrorString(e));
        return CB_ERR_CUDA;
    }
    if (bar[0].err || bar[1].err) {
        cb_internal_set_error(m, "cb_solve_noalloc: a grid barrier of the solve timed out; x is incomplete");
        return CB_ERR_TIMEOUT;
    }
    return CB_OK;
}
