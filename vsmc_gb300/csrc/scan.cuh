// Device-wide scans in three kernels (reduce tiles, scan tile totals, scan
// tiles with their offsets).  No inter-block waiting of any kind.
//
// Load:  T operator()(size_t i) const   -- element i (i < n)
// Store: void operator()(size_t i, T inclusive) const
#pragma once

#include "common.cuh"

#include <cstring>

namespace vsmc_cuda
{

constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;

// shuffle any 4-byte-multiple trivially copyable value
template <typename T>
__device__ __forceinline__ T shfl_up_any(T v, int d)
{
    static_assert(sizeof(T) % 4 == 0, "shuffle size");
    constexpr int W = sizeof(T) / 4;
    uint32_t w[W];
    memcpy(w, &v, sizeof(T));
#pragma unroll
    for (int k = 0; k < W; ++k)
        w[k] = __shfl_up_sync(0xFFFFFFFFu, w[k], d);
    T r;
    memcpy(&r, w, sizeof(T));
    return r;
}

template <typename T, typename Op>
__device__ __forceinline__ T warp_incl_any(T v, Op op)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const T o = shfl_up_any(v, d);
        if (lane >= d)
            v = op(o, v);
    }
    return v;
}

// block-wide exclusive scan of one value per thread (kB threads, at most
// 1024); *total = block total
template <typename T, typename Op, int kB = kScanBlock>
__device__ __forceinline__ T block_excl_any(T v, Op op, T id, T *total)
{
    __shared__ T sh[kB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const T incl = warp_incl_any(v, op);
    if (lane == 31)
        sh[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        T w = lane < kB / 32 ? sh[lane] : id;
        w = warp_incl_any(w, op);
        if (lane < kB / 32)
            sh[lane] = w;
    }
    __syncthreads();
    T excl = shfl_up_any(incl, 1);
    if (lane == 0)
        excl = id;
    if (wid > 0)
        excl = op(sh[wid - 1], excl);
    *total = sh[kB / 32 - 1];
    __syncthreads();
    return excl;
}

template <typename T, typename Op, typename Load>
__global__ void __launch_bounds__(kScanBlock) k_scan_reduce(
    size_t n, Load load, Op op, T id, T *part)
{
    const size_t base = static_cast<size_t>(blockIdx.x) * kScanTile;
    T acc = id;
    for (int k = 0; k < kScanItems; ++k) {
        const size_t i = base + static_cast<size_t>(k) * kScanBlock + threadIdx.x;
        if (i < n)
            acc = op(acc, load(i));
    }
    // order inside a tile does not matter for associative exact ops; for
    // floating point the down-sweep recomputes in its own order anyway
    T tot;
    (void)block_excl_any(acc, op, id, &tot);
    if (threadIdx.x == 0)
        part[blockIdx.x] = tot;
}

// exclusive scan of part[0..nb) in place (one block of kPartsBlock
// threads): each thread takes a contiguous stretch (its loads issued
// together), one block scan of the stretches' totals, then each thread
// writes its stretch's prefixes
constexpr int kPartsBlock = 1024;

template <typename T, typename Op>
__global__ void __launch_bounds__(kPartsBlock) k_scan_parts(
    size_t nb, T *part, Op op, T id)
{
    constexpr int kK = 8; // loads of a stretch issued together
    const size_t per = (nb + kPartsBlock - 1) / kPartsBlock;
    const size_t b0 = min(nb, threadIdx.x * per);
    const size_t b1 = min(nb, b0 + per);
    T acc = id;
    for (size_t i0 = b0; i0 < b1; i0 += kK) {
        T v[kK];
#pragma unroll
        for (int k = 0; k < kK; ++k)
            v[k] = i0 + k < b1 ? part[i0 + k] : id;
#pragma unroll
        for (int k = 0; k < kK; ++k)
            acc = op(acc, v[k]);
    }
    T tot;
    T run = block_excl_any<T, Op, kPartsBlock>(acc, op, id, &tot);
    for (size_t i0 = b0; i0 < b1; i0 += kK) {
        T v[kK];
#pragma unroll
        for (int k = 0; k < kK; ++k)
            v[k] = i0 + k < b1 ? part[i0 + k] : id;
#pragma unroll
        for (int k = 0; k < kK; ++k)
            if (i0 + k < b1) {
                part[i0 + k] = run;
                run = op(run, v[k]);
            }
    }
}

// The tile's values are loaded and stored striped (element k * kScanBlock +
// t by thread t: coalesced) through shared memory, and scanned blocked
// (thread t owns elements t * kScanItems .. + kScanItems - 1); one padding
// slot per 32 elements spreads the blocked accesses over the banks.
template <typename T, typename Op, typename Load, typename Store>
__global__ void __launch_bounds__(kScanBlock) k_scan_down(
    size_t n, Load load, Store store, Op op, T id, const T *part)
{
    __shared__ T sv[kScanTile + kScanTile / 32];
    const size_t tile0 = static_cast<size_t>(blockIdx.x) * kScanTile;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int j = k * kScanBlock + threadIdx.x;
        const size_t i = tile0 + j;
        sv[j + j / 32] = i < n ? load(i) : id;
    }
    __syncthreads();
    T v[kScanItems];
    T acc = id;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int j = threadIdx.x * kScanItems + k;
        v[k] = sv[j + j / 32];
        acc = op(acc, v[k]);
    }
    T tot;
    T run = block_excl_any(acc, op, id, &tot); // its barriers end the reads
    run = op(part[blockIdx.x], run);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int j = threadIdx.x * kScanItems + k;
        run = op(run, v[k]);
        sv[j + j / 32] = run;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int j = k * kScanBlock + threadIdx.x;
        const size_t i = tile0 + j;
        if (i < n)
            store(i, sv[j + j / 32]);
    }
}

// Inclusive scan of load(0..n) into store(); `part` needs scan_parts(n)
// elements of T.
inline size_t scan_parts(size_t n) { return (n + kScanTile - 1) / kScanTile; }

template <typename T, typename Op, typename Load, typename Store>
int device_scan(size_t n, Load load, Store store, Op op, T id, T *part,
    cudaStream_t st)
{
    if (n == 0)
        return VSMC_CUDA_OK;
    const size_t nb = scan_parts(n);
    if (nb > 0x7FFFFFFFull)
        return VSMC_CUDA_ERR_SIZE;
    k_scan_reduce<T, Op, Load><<<static_cast<unsigned>(nb), kScanBlock, 0, st>>>(
        n, load, op, id, part);
    k_scan_parts<T, Op><<<1, kPartsBlock, 0, st>>>(nb, part, op, id);
    k_scan_down<T, Op, Load, Store>
        <<<static_cast<unsigned>(nb), kScanBlock, 0, st>>>(
            n, load, store, op, id, part);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

} // namespace vsmc_cuda
