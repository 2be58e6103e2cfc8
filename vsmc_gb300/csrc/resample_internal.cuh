// Device-side resampling / weight building blocks shared by the C ABI
// (resample.cu) and the FP64 filter driver (pf64.cu).
#pragma once

#include "common.cuh"

namespace vsmc_cuda
{

int u01_rep_device(size_t m, size_t n, const double *w, const double *u,
    int *rep, const int *integ, uint32_t *err, Scratch &scratch,
    cudaStream_t st, bool sorted = false);
int rep_index_device(size_t m, size_t n, const int *rep, int *idx,
    uint32_t *err, Scratch &scratch, cudaStream_t st);
int scheme_device(size_t m, size_t n, vsmc_cuda_rng *rng, const double *w,
    int *rep, int scheme, Scratch &scratch, cudaStream_t st);
int weight_normalize_device(size_t n, double *W, double *ess_dev,
    uint32_t *err, Scratch &scratch, cudaStream_t st);
int weight_post_set_log_device(size_t n, double *W, double *ess_dev,
    uint32_t *err, Scratch &scratch, cudaStream_t st);
int weight_set_equal_device(size_t n, double *W, double *ess_dev,
    uint32_t *err, Scratch &scratch, cudaStream_t st);
int weight_add_log_device(size_t n, const double *l, double *W,
    double *ess_dev, uint32_t *err, Scratch &scratch, cudaStream_t st);
template <typename T>
int monitor_mean_device(size_t n, size_t dim, size_t ld, const T *state,
    const double *W, double *out, Scratch &scratch, cudaStream_t st);
template <typename T>
int state_copy_device(size_t n, size_t dim, size_t ld, const int *idx,
    T *state, uint32_t *err, cudaStream_t st);

} // namespace vsmc_cuda
