// Shared device code for libvsmc_cuda: counter-based generators, u01
// conversions, counter arithmetic, status handling and block-level scans.
//
// Everything here is sm_103a device code written for this library.  The
// generator constants are the published Random123 ones, as they appear in
// the reference (rng/philox.hpp:76-101, rng/threefry.hpp:71-146).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

#include "../../include/vsmc_cuda.h"
#include "../../include/vsmc_cuda_device.cuh"
#include "../../include/vsmc_cuda_filter.cuh"

namespace vsmc_cuda
{

// ------------------------------------------------------------------ status

// Sticky per-process record of the last CUDA runtime error seen.
void set_last_cuda_error(cudaError_t e);

#define VSMC_CUDA_TRY(expr)                                                   \
    do {                                                                      \
        cudaError_t vsmc_cuda_err_ = (expr);                                  \
        if (vsmc_cuda_err_ != cudaSuccess) {                                  \
            ::vsmc_cuda::set_last_cuda_error(vsmc_cuda_err_);                 \
            return VSMC_CUDA_ERR_CUDA;                                        \
        }                                                                     \
    } while (0)

#define VSMC_CUDA_CHECK_LAUNCH() VSMC_CUDA_TRY(cudaGetLastError())

inline cudaStream_t as_stream(void *s) { return static_cast<cudaStream_t>(s); }

// The device-side error word bits DEV_ERR_* come from vsmc_cuda_filter.cuh.

// ------------------------------------------------------- counter arithmetic

// 128-bit counter as four 32-bit limbs (Philox4x32) -- c += v with carry.
__host__ __device__ inline void ctr32_add(uint32_t c[4], uint64_t v)
{
    uint64_t acc = static_cast<uint64_t>(c[0]) + (v & 0xFFFFFFFFull);
    c[0] = static_cast<uint32_t>(acc);
    acc = static_cast<uint64_t>(c[1]) + (v >> 32) + (acc >> 32);
    c[1] = static_cast<uint32_t>(acc);
    acc = static_cast<uint64_t>(c[2]) + (acc >> 32);
    c[2] = static_cast<uint32_t>(acc);
    c[3] = static_cast<uint32_t>(static_cast<uint64_t>(c[3]) + (acc >> 32));
}

// carry of one into limb 1 and up (the reference's increment_single<1>)
__host__ __device__ inline void ctr32_carry1(uint32_t c[4])
{
    if (++c[1] != 0)
        return;
    if (++c[2] != 0)
        return;
    ++c[3];
}

// 256-bit counter as four 64-bit limbs (Threefry4x64) -- c += v with carry.
__host__ __device__ inline void ctr64_add(uint64_t c[4], uint64_t v)
{
    uint64_t old = c[0];
    c[0] += v;
    if (c[0] >= old)
        return;
    if (++c[1] != 0)
        return;
    if (++c[2] != 0)
        return;
    ++c[3];
}

__host__ __device__ inline void ctr64_carry1(uint64_t c[4])
{
    if (++c[1] != 0)
        return;
    if (++c[2] != 0)
        return;
    ++c[3];
}

// ------------------------------------------------------------- generators

struct u64x4 {
    uint64_t x, y, z, w;
};

__device__ __forceinline__ uint64_t rotl64(uint64_t x, int r)
{
    return (x << r) | (x >> (64 - r));
}

// Threefry4x64-20 on one counter block (no pre-increment): key injection
// before round 1 and after every fourth round, with +s on word 3.
__device__ __forceinline__ u64x4 threefry4x64_20(
    u64x4 c, uint64_t k0, uint64_t k1, uint64_t k2, uint64_t k3)
{
    const uint64_t k4 = 0x1BD11BDAA9FC1A22ull ^ k0 ^ k1 ^ k2 ^ k3;
    const uint64_t ks[5] = {k0, k1, k2, k3, k4};
    uint64_t s0 = c.x + k0, s1 = c.y + k1, s2 = c.z + k2, s3 = c.w + k3;
    constexpr int R0[8] = {14, 52, 23, 5, 25, 46, 58, 32};
    constexpr int R1[8] = {16, 57, 40, 37, 33, 12, 22, 32};
#pragma unroll
    for (int n = 1; n <= 20; ++n) {
        const int r = (n - 1) % 8;
        if (n % 2) {
            s0 += s1;
            s1 = rotl64(s1, R0[r]) ^ s0;
            s2 += s3;
            s3 = rotl64(s3, R1[r]) ^ s2;
        } else {
            s0 += s3;
            s3 = rotl64(s3, R0[r]) ^ s0;
            s2 += s1;
            s1 = rotl64(s1, R1[r]) ^ s2;
        }
        if (n % 4 == 0) {
            const int inc = n / 4;
            s0 += ks[(inc + 0) % 5];
            s1 += ks[(inc + 1) % 5];
            s2 += ks[(inc + 2) % 5];
            s3 += ks[(inc + 3) % 5] + static_cast<uint64_t>(inc);
        }
    }
    return {s0, s1, s2, s3};
}

// u32x4, philox4x32_10, the u01 maps, kPi2 and normal_pair_f come from
// vsmc_cuda_device.cuh.

// ------------------------------------------------------------ block scans

constexpr int kWarp = 32;

template <typename T, typename Op>
__device__ __forceinline__ T warp_inclusive_scan(T v, Op op)
{
    const int lane = threadIdx.x & (kWarp - 1);
#pragma unroll
    for (int d = 1; d < kWarp; d <<= 1) {
        T o = __shfl_up_sync(0xFFFFFFFFu, v, d);
        if (lane >= d)
            v = op(o, v);
    }
    return v;
}

template <typename T, typename Op>
__device__ __forceinline__ T warp_reduce(T v, Op op)
{
#pragma unroll
    for (int d = kWarp / 2; d > 0; d >>= 1)
        v = op(v, __shfl_xor_sync(0xFFFFFFFFu, v, d));
    return v;
}

// Block-wide inclusive scan of one value per thread; returns the inclusive
// value and writes the block total to *total.  smem needs blockDim/32 + 1
// entries.  Must be called by all threads of the block.
template <typename T, typename Op>
__device__ __forceinline__ T block_inclusive_scan(
    T v, Op op, T identity, T *smem, T *total)
{
    const int lane = threadIdx.x & (kWarp - 1);
    const int wid = threadIdx.x / kWarp;
    const int nw = (blockDim.x + kWarp - 1) / kWarp;
    T x = warp_inclusive_scan(v, op);
    if (lane == kWarp - 1)
        smem[wid] = x;
    __syncthreads();
    if (wid == 0) {
        T w = lane < nw ? smem[lane] : identity;
        w = warp_inclusive_scan(w, op);
        if (lane < nw)
            smem[lane] = w;
    }
    __syncthreads();
    if (wid > 0)
        x = op(smem[wid - 1], x);
    *total = smem[nw - 1];
    __syncthreads();
    return x;
}

template <typename T, typename Op>
__device__ __forceinline__ T block_reduce(T v, Op op, T identity, T *smem)
{
    const int lane = threadIdx.x & (kWarp - 1);
    const int wid = threadIdx.x / kWarp;
    const int nw = (blockDim.x + kWarp - 1) / kWarp;
    v = warp_reduce(v, op);
    if (lane == 0)
        smem[wid] = v;
    __syncthreads();
    T r = identity;
    if (wid == 0) {
        r = lane < nw ? smem[lane] : identity;
        r = warp_reduce(r, op);
        if (lane == 0)
            smem[0] = r;
    }
    __syncthreads();
    r = smem[0];
    __syncthreads();
    return r;
}

struct OpAdd {
    template <typename T>
    __device__ __forceinline__ T operator()(T a, T b) const
    {
        return a + b;
    }
};

struct OpMax {
    template <typename T>
    __device__ __forceinline__ T operator()(T a, T b) const
    {
        return a < b ? b : a;
    }
};

// ----------------------------------------------------- device-wide helpers

int num_sms();

// Grid size for a grid-stride kernel: a multiple of the SM count, capped so
// that a small problem does not launch idle blocks.
int grid_for(size_t work_items, int block, int items_per_thread,
    int blocks_per_sm = 4);

// Stream-ordered scratch allocation (cudaMallocAsync on the caller's
// stream).  RAII: freed on the same stream when it goes out of scope.
class Scratch
{
    public:
    explicit Scratch(cudaStream_t s) : stream_(s) {}
    ~Scratch();
    Scratch(const Scratch &) = delete;
    Scratch &operator=(const Scratch &) = delete;

    // returns nullptr on failure (and records the CUDA error)
    void *alloc(size_t bytes);

    template <typename T>
    T *get(size_t n)
    {
        return static_cast<T *>(alloc(sizeof(T) * (n ? n : 1)));
    }

    private:
    cudaStream_t stream_;
    std::vector<void *> ptrs_;
};

} // namespace vsmc_cuda
