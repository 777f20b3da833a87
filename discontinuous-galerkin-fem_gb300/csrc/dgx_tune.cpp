// Launch-shape autotuner for the persistent stage kernels.
//
// The stage kernels walk their 128-element tiles with a grid stride, so the grid size is
// free: one CTA per tile (no persistence), or a multiple of the SM count so that every CTA
// stays resident and walks several tiles.  Which is faster depends on the order (register
// and shared-memory footprint, hence CTAs per SM), on the element count (the last partial
// wave) and, for batched solves, on the mix of orders.  The tuner times each candidate
// grid on the caller's stream with CUDA events (one warm-up launch, then the mean of three
// launches) the first time a (kernel, order, element count) key is seen, and keeps the
// fastest for the life of the process.
//
// DGX_AUTOTUNE=0 in the environment turns timing off: every key gets one CTA per tile.
// DGX_AUTOTUNE_VERBOSE=1 prints each decision to stderr.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "dgx_context.h"

namespace dgx {

namespace {
std::mutex g_tune_mu;
std::map<std::string, int> g_tuned;

bool env_is(const char* name, const char* value) {
    const char* v = std::getenv(name);
    return v && std::strcmp(v, value) == 0;
}
}  // namespace

std::vector<int> grid_candidates(int ntiles) {
    std::vector<int> c{ntiles};
    int sms = 152, dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaGetLastError();
    for (int k : {1, 2, 3, 4, 6, 8})
        if (sms * k < ntiles) c.push_back(sms * k);
    return c;
}

int tune_grid(const std::string& key, const std::vector<int>& candidates, const GridLaunch& launch, cudaStream_t s,
              int* best) {
    if (candidates.empty()) return set_error(DGX_ERR_RUNTIME, "autotuner: no candidate launch shapes");
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            *best = it->second;
            return DGX_OK;
        }
    }
    if (env_is("DGX_AUTOTUNE", "0") || candidates.size() == 1) {
        *best = candidates[0];
        return DGX_OK;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        if (e0) cudaEventDestroy(e0);
        return set_error(DGX_ERR_CUDA, "autotuner: cudaEventCreate failed");
    }
    constexpr int REPS = 3;
    int pick = candidates[0];
    float pick_ms = 0.0f;
    int rc = DGX_OK;
    for (int g : candidates) {
        if (launch(g, s)) {
            rc = set_error(DGX_ERR_CUDA, std::string("autotuner: launch failed: ") +
                                             launch_error_text());
            break;
        }
        cudaEventRecord(e0, s);
        for (int r = 0; r < REPS && !rc; ++r)
            if (launch(g, s))
                rc = set_error(DGX_ERR_CUDA, std::string("autotuner: launch failed: ") +
                                                 launch_error_text());
        cudaEventRecord(e1, s);
        float ms = 0.0f;
        if (rc || cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
            if (!rc) rc = set_error(DGX_ERR_CUDA, std::string("autotuner: timing failed: ") +
                                                      cudaGetErrorString(cudaGetLastError()));
            break;
        }
        ms /= REPS;
        if (env_is("DGX_AUTOTUNE_VERBOSE", "1")) std::fprintf(stderr, "[dgx tune] %s grid=%d %.4f ms\n", key.c_str(), g, ms);
        if (g == candidates[0] || ms < pick_ms) {
            pick = g;
            pick_ms = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tuned[key] = pick;
    }
    *best = pick;
    return DGX_OK;
}

}  // namespace dgx
