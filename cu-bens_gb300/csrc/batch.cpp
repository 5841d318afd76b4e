// Many independent analyses at once (the batched imperfection sweep): a pool
// of host threads, each taking the next handle and running its arc-length
// loop. Every handle owns its CUDA stream, so the small, latency-bound
// kernels of different analyses overlap on the GPU; each handle's results
// are exactly those of running it alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "cubens_gb300.h"

extern "C" void cb_internal_share_gpu(cb_model *m, int shared);

namespace {

int run_one(cb_model *m, int steps, cb_step *out)
{
    cb_info info;
    if (cb_model_info(m, &info) != CB_OK) return CB_ERR_ARG;
    int rc = cb_msal_begin(m, &out[0]);
    for (int k = 1; k < steps; ++k) {
        if (rc != CB_OK || out[k - 1].done) {
            out[k] = cb_step{};
            out[k].done = 1;
            continue;
        }
        rc = cb_msal_step(m, &out[k]);
    }
    return rc;
}

}  // namespace

extern "C" int cb_batch_msal(cb_model **models, int n, int steps, int threads, cb_step *out, int *status)
{
    if (!models || n <= 0 || steps <= 0 || !out) return CB_ERR_ARG;
    for (int i = 0; i < n; ++i)
        if (!models[i]) return CB_ERR_ARG;
    threads = std::max(1, std::min(threads, n));
    int device = 0;
    cudaGetDevice(&device);
    std::atomic<int> next{0};
    auto worker = [&]() {
        cudaSetDevice(device);
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= n) break;
            const int rc = run_one(models[i], steps, out + (size_t)i * steps);
            if (status) status[i] = rc;
        }
    };
    for (int i = 0; i < n; ++i) cb_internal_share_gpu(models[i], threads > 1);
    std::vector<std::thread> pool;
    pool.reserve(threads);
    for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
    for (auto &t : pool) t.join();
    for (int i = 0; i < n; ++i) cb_internal_share_gpu(models[i], 0);
    if (status)
        for (int i = 0; i < n; ++i)
            if (status[i] != CB_OK) return status[i];
    return CB_OK;
}
