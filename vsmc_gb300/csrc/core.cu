// Status strings, error bookkeeping, grid sizing and stream-ordered scratch.
#include "common.cuh"

#include <atomic>

namespace vsmc_cuda
{

static std::atomic<int> g_last_cuda_error{0};

void set_last_cuda_error(cudaError_t e)
{
    g_last_cuda_error.store(static_cast<int>(e));
}

int num_sms()
{
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return 152;
    if (cached[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) !=
                cudaSuccess ||
            n <= 0)
            n = 152;
        cached[dev] = n;
    }
    return cached[dev];
}

int grid_for(
    size_t work_items, int block, int items_per_thread, int blocks_per_sm)
{
    const size_t per_block =
        static_cast<size_t>(block) * static_cast<size_t>(items_per_thread);
    size_t need = (work_items + per_block - 1) / per_block;
    const size_t cap =
        static_cast<size_t>(num_sms()) * static_cast<size_t>(blocks_per_sm);
    if (need > cap)
        need = cap;
    if (need < 1)
        need = 1;
    return static_cast<int>(need);
}

Scratch::~Scratch()
{
    // stream-ordered: each block is released after the work queued before
    for (void *p : ptrs_)
        cudaFreeAsync(p, stream_);
}

void *Scratch::alloc(size_t bytes)
{
    void *p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, bytes ? bytes : 1, stream_);
    if (e != cudaSuccess) {
        set_last_cuda_error(e);
        return nullptr;
    }
    ptrs_.push_back(p);
    return p;
}

} // namespace vsmc_cuda

extern "C" {

const char *vsmc_cuda_status_string(int status)
{
    switch (status) {
        case VSMC_CUDA_OK: return "ok";
        case VSMC_CUDA_ERR_ARG: return "invalid argument";
        case VSMC_CUDA_ERR_SIZE: return "length out of the supported range";
        case VSMC_CUDA_ERR_NONFINITE:
            return "non-finite or negative weight";
        case VSMC_CUDA_ERR_TIMEOUT: return "bounded device wait gave up";
        case VSMC_CUDA_ERR_CUDA: return "CUDA runtime error";
        case VSMC_CUDA_ERR_ALLOC: return "device allocation failed";
        case VSMC_CUDA_ERR_INTERNAL: return "internal consistency check failed";
        default: return "unknown status";
    }
}

int vsmc_cuda_last_cuda_error(void)
{
    return vsmc_cuda::g_last_cuda_error.load();
}

int vsmc_cuda_version(void) { return 100; }

} // extern "C"
