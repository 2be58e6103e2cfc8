// Data layout of the FP32 filter's resampling passes (the step kernel's
// layout, PfScalars / PfPartial / PfStepArgs, is in vsmc_cuda_filter.cuh).
#pragma once

#include "common.cuh"
#include "pf_model.cuh"

namespace vsmc_cuda
{

struct Rs32Args {
    const float *lw;
    const uint64_t *q; // integer weights given directly (lw unused), or null
    uint32_t n;
    uint32_t shift;  // fixed-point K
    uint32_t chunk;  // particles per block (multiple of kPfTile)
    int scheme;      // VSMC_CUDA_STRATIFIED or VSMC_CUDA_SYSTEMATIC
    int force;       // resample whatever the step decided (host decision)
    // per warp range (block * kRsWarps + warp): the range's sum of q, its
    // empty slots and its copies (sum of rep), each turned into exclusive
    // prefix sums by the last block of the pass that wrote it
    uint64_t *qpart;
    uint32_t *epart;
    uint32_t *cpart;
    int32_t *rep;
    int32_t *idx;      // per slot: itself (>= 0) or -(empty rank + 1)
    uint32_t *srcs;    // N entries: source of the k-th empty slot
    PfScalars *sc;
    // monitor of the resampled particles: sum_i rep_i x_{d,i} / n over the
    // first mon_dim rows of mon_state (the state the resample draws from);
    // mon_dim 0 skips it
    const float *mon_state;
    size_t stride;
    uint32_t mon_dim;
    uint32_t max_steps;
    PfPartial *mon_part; // per-block sums (at least one record per block)
    double *h_mean;   // max_steps x mon_dim (the resampling step's entry)
    int *h_res;       // the step's resampled flag (forced resamples set it)
};

} // namespace vsmc_cuda
