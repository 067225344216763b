// abi.cu -- status helpers shared by every entry point of libgbla.so.
#include <atomic>
#include "common.cuh"

namespace gbla {

static std::atomic<int> g_last_cuda_error{0};

gbla_status from_cuda(cudaError_t e) {
    if (e == cudaSuccess) return GBLA_SUCCESS;
    g_last_cuda_error.store((int)e);
    return GBLA_CUDA_ERROR;
}

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (cached[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        cached[dev] = v;
    }
    return cached[dev];
}

int64_t persistent_grid(const void *func, int threads, size_t smem, int64_t work) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    int64_t grid = (int64_t)sm_count() * per_sm;
    if (grid > work) grid = work;
    return grid < 1 ? 1 : grid;
}

}  // namespace gbla

GBLA_API const char *gbla_status_string(gbla_status s) {
    switch (s) {
        case GBLA_SUCCESS: return "GBLA_SUCCESS";
        case GBLA_INVALID_VALUE: return "GBLA_INVALID_VALUE";
        case GBLA_NOT_SUPPORTED: return "GBLA_NOT_SUPPORTED";
        case GBLA_CUDA_ERROR: return "GBLA_CUDA_ERROR";
        case GBLA_WORKSPACE_TOO_SMALL: return "GBLA_WORKSPACE_TOO_SMALL";
    }
    return "GBLA_UNKNOWN_STATUS";
}

GBLA_API int gbla_version(void) { return 100; }

GBLA_API int gbla_last_cuda_error(void) { return gbla::g_last_cuda_error.load(); }
