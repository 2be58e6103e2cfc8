// Genealogy and the sampler summary text.
//
//   * Lineage tracing over a history of resampling index rows, the
//     ResampleIndex of the reference (resample/index.hpp:46-206) on the
//     device: row k holds, for each particle after iteration k, the index
//     of its parent among the particles before it (the identity when the
//     iteration did not resample).  index(id, iter) follows a particle of
//     the last iteration back to iteration iter; index_matrix gives every
//     particle's whole line in row-major ([N][iters]) or column-major
//     ([iters][N]) layout.
//   * Sampler::print (core/sampler.hpp:646-689): the TSV summary with
//     "Size", "Resampled", one "Accept.k" per move, "ESS" and the monitor
//     columns, each field followed by the separator.
#include "common.cuh"

#include <cstdio>
#include <cstring>
#include <string>

using namespace vsmc_cuda;

namespace vsmc_cuda
{

// out[id] = the ancestor at iteration `iter` of particle id of the last
// iteration: follow rows iters-1, ..., iter
__global__ void k_index_trace(uint32_t N, uint32_t iters, const int *rows,
    uint32_t iter, int *out, uint32_t *err)
{
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < N;
         id += gridDim.x * blockDim.x) {
        int a = rows[static_cast<size_t>(iters - 1) * N + id];
        for (uint32_t k = iters - 1; k > iter; --k) {
            if (a < 0 || static_cast<uint32_t>(a) >= N) {
                atomicOr(err, DEV_ERR_INTERNAL);
                a = 0;
            }
            a = rows[static_cast<size_t>(k - 1) * N + a];
        }
        out[id] = a;
    }
}

// The whole line of each particle of the last iteration: out[id][k]
// (row-major) or out[k][id] (column-major) is the ancestor at iteration k.
__global__ void k_index_matrix(uint32_t N, uint32_t iters, const int *rows,
    int col_major, int *out, uint32_t *err)
{
    for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < N;
         id += gridDim.x * blockDim.x) {
        int a = rows[static_cast<size_t>(iters - 1) * N + id];
        for (uint32_t k = iters; k-- > 0;) {
            if (k + 1 < iters) {
                if (a < 0 || static_cast<uint32_t>(a) >= N) {
                    atomicOr(err, DEV_ERR_INTERNAL);
                    a = 0;
                }
                a = rows[static_cast<size_t>(k) * N + a];
            }
            if (col_major)
                out[static_cast<size_t>(k) * N + id] = a;
            else
                out[static_cast<size_t>(id) * iters + k] = a;
        }
    }
}

static int check_err(uint32_t *err, cudaStream_t st)
{
    uint32_t h = 0;
    VSMC_CUDA_TRY(cudaMemcpyAsync(
        &h, err, sizeof(h), cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    return h ? VSMC_CUDA_ERR_ARG : VSMC_CUDA_OK;
}

// ostream's default formatting of a double (precision 6, %g style)
static void put_double(std::string &s, double v)
{
    char b[64];
    std::snprintf(b, sizeof(b), "%g", v);
    s += b;
}

static void put_size(std::string &s, unsigned long long v)
{
    char b[32];
    std::snprintf(b, sizeof(b), "%llu", v);
    s += b;
}

} // namespace vsmc_cuda

extern "C" {

int vsmc_cuda_resample_index_trace(size_t N, size_t iters, const int *rows,
    size_t iter, int *out, void *stream)
{
    if (rows == nullptr || out == nullptr || iters == 0 || iter >= iters)
        return VSMC_CUDA_ERR_ARG;
    if (N == 0)
        return VSMC_CUDA_OK;
    if (N >= (size_t(1) << 31) || iters > 0xFFFFFFFFull)
        return VSMC_CUDA_ERR_SIZE;
    cudaStream_t st = as_stream(stream);
    Scratch scratch(st);
    uint32_t *err = scratch.get<uint32_t>(1);
    if (err == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    VSMC_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    k_index_trace<<<grid_for(N, 256, 1, 8), 256, 0, st>>>(
        static_cast<uint32_t>(N), static_cast<uint32_t>(iters), rows,
        static_cast<uint32_t>(iter), out, err);
    VSMC_CUDA_CHECK_LAUNCH();
    return check_err(err, st);
}

int vsmc_cuda_resample_index_matrix(size_t N, size_t iters, const int *rows,
    int layout, int *out, void *stream)
{
    if (rows == nullptr || out == nullptr || (layout != 0 && layout != 1))
        return VSMC_CUDA_ERR_ARG;
    if (N == 0 || iters == 0)
        return VSMC_CUDA_OK;
    if (N >= (size_t(1) << 31) || iters > 0xFFFFFFFFull)
        return VSMC_CUDA_ERR_SIZE;
    cudaStream_t st = as_stream(stream);
    Scratch scratch(st);
    uint32_t *err = scratch.get<uint32_t>(1);
    if (err == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    VSMC_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    k_index_matrix<<<grid_for(N, 256, 1, 8), 256, 0, st>>>(
        static_cast<uint32_t>(N), static_cast<uint32_t>(iters), rows, layout,
        out, err);
    VSMC_CUDA_CHECK_LAUNCH();
    return check_err(err, st);
}

int vsmc_cuda_sampler_print(size_t T, size_t N, const int *resampled,
    const double *ess, size_t nmon, const char *mon_name, const double *mon,
    size_t naccept, const size_t *accept, char sep, char *buf, size_t cap,
    size_t *len)
{
    if (accept == nullptr)
        naccept = 1; // one move accepting every particle
    if (len == nullptr || (T > 0 && (resampled == nullptr || ess == nullptr)) ||
        (nmon > 0 && (mon_name == nullptr || mon == nullptr)) ||
        (cap > 0 && buf == nullptr))
        return VSMC_CUDA_ERR_ARG;
    std::string s;
    if (T > 0) {
        s += "Size";
        s += sep;
        s += "Resampled";
        s += sep;
        for (size_t k = 0; k < naccept; ++k) {
            s += "Accept.";
            put_size(s, k);
            s += sep;
        }
        s += "ESS";
        s += sep;
        for (size_t d = 0; d < nmon; ++d) {
            s += mon_name;
            s += '.';
            put_size(s, d);
            s += sep;
        }
        s += '\n';
        for (size_t t = 0; t < T; ++t) {
            put_size(s, N);
            s += sep;
            put_size(s, resampled[t] ? 1 : 0);
            s += sep;
            for (size_t k = 0; k < naccept; ++k) {
                put_size(s, accept ? accept[t * naccept + k] : N);
                s += sep;
            }
            put_double(s, ess[t]);
            s += sep;
            for (size_t d = 0; d < nmon; ++d) {
                put_double(s, mon[t * nmon + d]);
                s += sep;
            }
            s += '\n';
        }
    }
    *len = s.size();
    if (cap == 0)
        return VSMC_CUDA_OK;
    if (s.size() + 1 > cap) {
        std::memcpy(buf, s.data(), cap - 1);
        buf[cap - 1] = 0;
        return VSMC_CUDA_ERR_SIZE;
    }
    std::memcpy(buf, s.data(), s.size());
    buf[s.size()] = 0;
    return VSMC_CUDA_OK;
}

} // extern "C"
