// Bit-exact left-to-right double summation (see seqsum.cu).
#pragma once

#include "common.cuh"

namespace vsmc_cuda
{

// prefix (n doubles) and/or *total (device) of x[0..n), non-negative terms;
// allow_inf: +inf terms are summed as a sequential loop would (inf onward).
// Device error bits go to *err (DEV_ERR_NONFINITE for negative / NaN terms).
int seqsum_device(size_t n, const double *x, double *prefix, double *total,
    uint32_t *err, Scratch &scratch, cudaStream_t st, bool allow_inf = false);

// copy the device error word to the host (synchronizes) and map it to a
// status
int read_err(uint32_t *err_dev, cudaStream_t st, int *status);

} // namespace vsmc_cuda
