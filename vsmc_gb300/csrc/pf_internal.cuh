// Host-side filter object shared by the FP32 and FP64 drivers.
#pragma once

#include "common.cuh"
#include "pf32_types.cuh"

namespace vsmc_cuda
{

struct Pf64State; // FP64 driver state (pf64.cu)

} // namespace vsmc_cuda

struct vsmc_cuda_pf {
    size_t n = 0;
    size_t stride = 0; // SoA row stride (n rounded up to 256 elements)
    size_t dim = 4;     // state components (rows)
    size_t mon_dim = 2; // monitored leading components
    bool custom = false; // precision 32 with the caller's model (no CV model)
    bool host_equal = false; // custom: weights set equal by the host
    int precision = 32;
    int scheme = VSMC_CUDA_SYSTEMATIC;
    double threshold = 0.5;
    uint32_t seed = 0;
    vsmc_cuda_cv_model model = {};
    size_t max_steps = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false; // created here when the caller passed NULL
    size_t t = 0;           // next step on the host side
    bool mean_pending = false;
    bool use_graph = true;

    // device buffers
    void *state = nullptr;  // dim rows of `stride` (float or double)
    void *state2 = nullptr; // FP32: second buffer; a step reads one, writes the other
    int cur = 0;            // FP32: buffer holding the current state (0: state)
    void *weight = nullptr; // FP32: log-weights (float); FP64: W (double)
    double *obs = nullptr;  // max_steps x 2
    double *h_mean = nullptr; // max_steps x mon_dim
    double *h_ess = nullptr, *h_logz = nullptr;
    int *h_res = nullptr;
    vsmc_cuda::PfScalars *sc = nullptr;
    vsmc_cuda::PfScalars *sc_host = nullptr; // pinned copy for status reads
    vsmc_cuda::PfScalars *sc_host_dev = nullptr; // its mapped device address

    // FP32 fused-step workspace
    size_t max_grid = 0; // records in `part`
    int grid_step = 0;
    int grid_rs = 0;
    uint32_t chunk_rs = 0;
    uint32_t shift = 0;
    vsmc_cuda::PfPartial *part = nullptr;
    uint64_t *qpart = nullptr;
    uint32_t *epart = nullptr, *cpart = nullptr;
    int32_t *rep = nullptr;
    int32_t *idx = nullptr;
    uint32_t *empties = nullptr;
    uint32_t mcmc_sweeps = 0; // FP32 resample-move: sweeps after resampling
    float mcmc_scale = 0;
    uint32_t *h_acc = nullptr; // accepted MCMC steps per step (max_steps)
    int32_t *gen = nullptr; // FP32 genealogy rows (max_steps x n) or null
    bool record_gen = false;
    cudaGraph_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr}; // by buffer parity

    vsmc_cuda::Pf64State *p64 = nullptr;
};

namespace vsmc_cuda
{

int pf64_create(vsmc_cuda_pf *pf);
void pf64_destroy(vsmc_cuda_pf *pf);
int pf64_step(vsmc_cuda_pf *pf, bool first);
int pf64_final_mean(vsmc_cuda_pf *pf);

} // namespace vsmc_cuda
