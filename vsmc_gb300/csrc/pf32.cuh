// FP32 bootstrap-filter step on the device.
//
// One fused kernel per step moves every particle, evaluates its
// log-likelihood, updates its FP32 log-weight and reduces, per block in FP64:
//   * the previous step's weighted position mean (from the state it reads),
//   * (max, sum exp, sum exp^2) of the new log-weights (log-sum-exp, ESS),
// and the last block to finish combines the blocks' records (no waiting:
// a thread-fenced completion counter) into the step's ESS, log-evidence
// increment and resampling decision.
//
// Resampling, when the decision says so, runs on an exact 64-bit fixed-point
// CDF: q_i = floor(exp(lw_i - max) * 2^K) with K = 63 - ceil(log2 N), so the
// integer prefix sums cannot overflow and do not depend on summation order.
// Systematic / stratified uniforms u_j = (j + a_j 2^-32) / N are counted
// against C_i / Q exactly: a fixed-point reciprocal of Q gives
// floor((C_i N - G) / Q) per particle, and an exact 128-bit comparison
// settles the rare value next to a uniform (pf32_dev.cuh).  Three passes
// (sum, count, assign), one warp per range of particles.  Replication counts
// then go to parent indices with the reference's slot layout
// (resample/transform.hpp:116-133): parents keep their slot, empty slots
// take surplus copies in order.  Only empty slots are written by the
// gather.
#pragma once

#include "common.cuh"
#include "pf_model.cuh"
#include "pf32_types.cuh"
#include "pf32_dev.cuh"

namespace vsmc_cuda
{

// ------------------------------------------------------------ fused step
//
// The step kernel itself is the model template k_pf_step of
// vsmc_cuda_filter.cuh; the library instantiates it with CvModel below.

// The constant-velocity / Student-t model of the benchmark as a step-kernel
// model: dim 4 (x, y, vx, vy), the weighted mean of (x, y) recorded.
// Observation t (clamped to the last one past max_steps, for profiling
// loops that run past the horizon) is read once per thread and step.
struct CvModel {
    static constexpr int dim = 4;
    static constexpr int monitor_dim = 2;
    struct step_type {
        float ox, oy;
    };

    CvConst<float> c;
    const double *obs; // max_steps x 2 (device)
    uint32_t max_steps;

    __device__ __forceinline__ step_type step(uint32_t t) const
    {
        const uint32_t to = t < max_steps ? t : max_steps - 1;
        return {static_cast<float>(obs[2 * to + 0]),
            static_cast<float>(obs[2 * to + 1])};
    }

    __device__ __forceinline__ void init(
        const step_type &, ParticleRng &rng, float (&x)[4]) const
    {
        float z1, z2, z3, z4;
        rng.normal_pair(z1, z2);
        rng.normal_pair(z3, z4);
        x[0] = c.sd_pos0 * z1;
        x[1] = c.sd_pos0 * z2;
        x[2] = c.sd_vel0 * z3;
        x[3] = c.sd_vel0 * z4;
    }

    __device__ __forceinline__ void move(
        const step_type &, ParticleRng &rng, float (&x)[4]) const
    {
        float z1, z2;
        rng.normal_pair(z1, z2);
        cv_move(c, c.sigma_a * z1, c.sigma_a * z2, x[0], x[1], x[2], x[3]);
    }

    __device__ __forceinline__ float log_likelihood(
        const step_type &s, const float (&x)[4]) const
    {
        return cv_loglik(c, s.ox, s.oy, x[0], x[1]);
    }
};

__device__ __forceinline__ float4 ld4(const float *p, uint32_t i)
{
    return pf_ld4(p + i);
}

// Monitor from per-thread sums: block sums of the first mon_dim rows (FP32
// per thread, FP64 across warps) go to part[block].mon, the block's weight
// total (weighted) to part[block].prev_w; the last block to finish
// (sc->done2) writes the mean (sums over the weight total, or times inv_n
// for equal weights) to sc->mean and, for a recorded step, to h_mean[t].
// Called by every thread of the block; wblock is the block's weight total.
__device__ __forceinline__ void mean_finish(const float (&acc)[kMaxMonitorDim],
    double wblock, bool weighted, double inv_n, uint32_t mon_dim,
    PfPartial *part, PfScalars *sc, double *h_mean, uint32_t t,
    uint32_t max_steps)
{
    constexpr int kW = kPfBlock / 32;
    __shared__ double sh[kMaxMonitorDim + 1][kW];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < kMaxMonitorDim; ++d) {
        double v = acc[d];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        if (lane == 0)
            sh[d][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        PfPartial p = {};
        for (int w = 0; w < kW; ++w)
#pragma unroll
            for (int d = 0; d < kMaxMonitorDim; ++d)
                p.mon[d] += sh[d][w];
        p.prev_w = wblock;
        part[blockIdx.x] = p;
        __threadfence();
        is_last = atomicAdd(&sc->done2, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last)
        return;
    // the last block: every thread sums a stride of the blocks' records
    __threadfence();
    double tot[kMaxMonitorDim + 1] = {};
    for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
#pragma unroll
        for (int d = 0; d < kMaxMonitorDim; ++d)
            tot[d] += __ldcg(&part[b].mon[d]);
        tot[kMaxMonitorDim] += __ldcg(&part[b].prev_w);
    }
#pragma unroll
    for (int d = 0; d <= kMaxMonitorDim; ++d) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            tot[d] += __shfl_xor_sync(0xFFFFFFFFu, tot[d], o);
        if (lane == 0)
            sh[d][wid] = tot[d];
    }
    __syncthreads();
    if (threadIdx.x != 0)
        return;
    double wsum = 0;
    for (int w = 0; w < kW; ++w)
        wsum += sh[kMaxMonitorDim][w];
    const double scale = weighted ? 1.0 / wsum : inv_n;
#pragma unroll
    for (int d = 0; d < kMaxMonitorDim; ++d) {
        if (static_cast<uint32_t>(d) >= mon_dim)
            break;
        double v = 0;
        for (int w = 0; w < kW; ++w)
            v += sh[d][w];
        sc->mean[d] = v * scale;
        if (t < max_steps)
            h_mean[static_cast<size_t>(t) * mon_dim + d] = v * scale;
    }
    sc->done2 = 0;
}

// the mean of equal-weight particles (sums times 1 / n)
__device__ __forceinline__ void equal_mean_finish(
    const float (&acc)[kMaxMonitorDim], uint32_t mon_dim, double inv_n,
    PfPartial *part, PfScalars *sc, double *h_mean, uint32_t t,
    uint32_t max_steps)
{
    mean_finish(acc, 0.0, false, inv_n, mon_dim, part, sc, h_mean, t,
        max_steps);
}

// out = in gathered through idx (materializes a pending resample)
__global__ void __launch_bounds__(kPfBlock) k_pf32_materialize(
    const PfStepArgs a, uint32_t dim)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += gridDim.x * blockDim.x) {
        uint32_t src = pf_source(a.srcs, a.idx[i]);
        if (src >= a.n) {
            atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
            src = 0;
        }
        for (uint32_t d = 0; d < dim; ++d)
            a.out[d * a.stride + i] = a.in[d * a.stride + src];
    }
}

// The last step's monitor, for runs whose steps record the previous step's
// (the filter's own runs): the weighted mean of the current particles,
// read through a pending gather; equal weights after a resample,
// exp(lw - M) otherwise.  FP32 within a thread and a warp, FP64 across
// warps and blocks, as the step kernel forms it.
__global__ void __launch_bounds__(kPfBlock) k_pf32_final_mean(
    const PfStepArgs a, uint32_t mon_dim)
{
    const int resampled = a.sc->resampled;
    const bool gather = a.sc->gather != 0;
    const float M = static_cast<float>(a.sc->M);
    float macc[kMaxMonitorDim] = {};
    float sw = 0.0f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += gridDim.x * blockDim.x) {
        uint32_t src = gather ? pf_source(a.srcs, a.idx[i]) : i;
        if (src >= a.n) {
            atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
            src = 0;
        }
        const float w = resampled ? 1.0f : __expf(a.lw[i] - M);
        sw += w;
#pragma unroll
        for (int d = 0; d < kMaxMonitorDim; ++d)
            if (static_cast<uint32_t>(d) < mon_dim)
                macc[d] = fmaf(w, a.in[d * a.stride + src], macc[d]);
    }
    // the block's weight total (FP64 across warps) for the mean's divisor
    constexpr int kW = kPfBlock / 32;
    __shared__ double shw[kW];
    __shared__ double wtot;
    double v = sw;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        shw[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < kW; ++w)
            s += shw[w];
        wtot = s;
    }
    __syncthreads();
    mean_finish(macc, wtot, true, 0.0, mon_dim, a.part, a.sc, a.h_mean,
        a.sc->step - 1, a.max_steps);
}

__global__ void k_pf32_clear_gather(PfScalars *sc)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        sc->gather = 0;
}

// ------------------------------------------------------------ resampling

__device__ __forceinline__ void chunk_range(
    uint32_t n, uint32_t chunk, uint32_t &lo, uint32_t &hi)
{
    lo = blockIdx.x * chunk;
    hi = lo + chunk;
    if (lo > n)
        lo = n;
    if (hi > n)
        hi = n;
}

__device__ __forceinline__ uint64_t q_at(
    const Rs32Args &a, uint32_t i, float M)
{
    return a.q ? a.q[i] : fixed_q(a.lw[i], M, a.shift);
}

// Resident blocks per SM of the resampling passes (their grid is SMs times
// this; 64 registers a thread).
constexpr int kRsBlocksPerSm = 4;

// Each block's chunk is split into kRsWarps equal warp ranges (the chunk
// is a multiple of kPfTile, so a range is a multiple of 128 particles); the
// passes address a range by (block, warp).
constexpr uint32_t kRsWarps = kPfBlock / 32;

__device__ __forceinline__ void warp_range(
    uint32_t lo, uint32_t hi, uint32_t chunk, uint32_t w, uint32_t &wlo,
    uint32_t &whi)
{
    const uint32_t span = chunk / kRsWarps;
    wlo = lo + w * span;
    whi = wlo + span;
    if (wlo > hi)
        wlo = hi;
    if (whi > hi)
        whi = hi;
}

// The block that finishes a resampling pass last (a thread-fenced ticket on
// sc->done3; nothing waits), in every thread of that block.  Its thread 0
// resets the ticket for the next pass.
__device__ __forceinline__ bool rs_last_block(PfScalars *sc)
{
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        last = atomicAdd(&sc->done3, 1u) == gridDim.x - 1;
        if (last)
            sc->done3 = 0;
    }
    __syncthreads();
    if (last)
        __threadfence();
    return last;
}

// Partials of a resampling pass: entry block * kRsWarps + warp for each
// warp range, then one entry per block from gridDim.x * kRsWarps on.  The
// last block of the pass turns the block entries into exclusive prefix
// sums; a range's offset is its block's prefix plus the ranges before it in
// its block.
template <typename T>
__device__ __forceinline__ T *blk_parts(T *v)
{
    return v + gridDim.x * kRsWarps;
}

// Records each warp's value x (the same in every lane) and the block's
// total.  Called by the whole block; sh holds kRsWarps entries.
template <typename T>
__device__ __forceinline__ void put_parts(T *v, T x, T *sh)
{
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        v[blockIdx.x * kRsWarps + w] = x;
        sh[w] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        T t = 0;
#pragma unroll
        for (int k = 0; k < kRsWarps; ++k)
            t += sh[k];
        blk_parts(v)[blockIdx.x] = t;
    }
}

// The offset of the calling warp's range (every lane gets it), once the
// block entries hold their prefix sums.
template <typename T>
__device__ __forceinline__ T range_offset(const T *v)
{
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T x = lane < w ? __ldcg(v + blockIdx.x * kRsWarps + lane) : T(0);
    if (lane == 31)
        x = __ldcg(v + gridDim.x * kRsWarps + blockIdx.x);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        x += __shfl_xor_sync(0xFFFFFFFFu, x, o);
    return x;
}

// v[0..m) replaced by its exclusive prefix sums by one block (each thread a
// contiguous stretch, its loads issued together); returns the total.
// sh: kPfBlock / 32 + 1 entries.
template <typename T>
__device__ __forceinline__ T scan_blocks_in_place(T *v, uint32_t m, T *sh)
{
    constexpr uint32_t kK = 4;
    const uint32_t per = (m + blockDim.x - 1) / blockDim.x;
    const uint32_t b0 = min(m, threadIdx.x * per);
    const uint32_t b1 = min(m, b0 + per);
    T s = 0;
    T x[kK];
    for (uint32_t i = b0; i < b1; i += kK) {
#pragma unroll
        for (uint32_t k = 0; k < kK; ++k)
            x[k] = i + k < b1 ? __ldcg(v + i + k) : T(0);
#pragma unroll
        for (uint32_t k = 0; k < kK; ++k)
            s += x[k];
    }
    T tot;
    T run = block_inclusive_scan(s, OpAdd(), T(0), sh, &tot) - s;
    if (per <= kK) {
#pragma unroll
        for (uint32_t k = 0; k < kK; ++k)
            if (b0 + k < b1) {
                v[b0 + k] = run;
                run += x[k];
            }
    } else {
        for (uint32_t i = b0; i < b1; ++i) {
            const T y = __ldcg(v + i);
            v[i] = run;
            run += y;
        }
    }
    return tot;
}

// log-weights i..i+3 (i a multiple of 4) below hi, -inf past it
__device__ __forceinline__ float4 load_lw4(
    const float *lw, uint32_t i, uint32_t hi)
{
    if (i + 3 < hi)
        return __ldcg(reinterpret_cast<const float4 *>(lw + i));
    float4 v = make_float4(-INFINITY, -INFINITY, -INFINITY, -INFINITY);
    if (i < hi)
        v.x = lw[i];
    if (i + 1 < hi)
        v.y = lw[i + 1];
    if (i + 2 < hi)
        v.z = lw[i + 2];
    return v;
}

// Sum of q over each warp range (four groups of four per lane in flight)
// and over each block, into qpart.  The last block to finish turns the
// block sums into prefix sums and sets the event's CDF constants: the total
// Q and the reciprocal terms.
__global__ void __launch_bounds__(kPfBlock, kRsBlocksPerSm) k_rs32_qsum(
    const Rs32Args a)
{
    if (!(a.force || a.sc->resampled))
        return;
    if (a.force && blockIdx.x == 0 && threadIdx.x == 0) {
        // a host decision: the later passes see the flag set
        a.sc->resampled = 1;
        const uint32_t t = a.sc->step - 1;
        if (a.h_res != nullptr && t < a.max_steps)
            a.h_res[t] = 1;
    }
    const float M = static_cast<float>(a.sc->M);
    uint32_t lo, hi;
    chunk_range(a.n, a.chunk, lo, hi);
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t wlo, whi;
    warp_range(lo, hi, a.chunk, w, wlo, whi);
    uint64_t acc = 0;
    constexpr int kG = 4;
    constexpr uint32_t kSpan = kG * 128;
    if (a.q == nullptr) {
        // groups of kG float4 per lane; the next group's loads are issued
        // before this group's weights, and a float4 past the range reads as
        // -inf (weight 0), so the range's last group needs no other path
        float4 v[kG], nv[kG];
#pragma unroll
        for (int h = 0; h < kG; ++h)
            v[h] = load_lw4(a.lw, wlo + h * 128 + lane * 4, whi);
        for (uint32_t base = wlo; base < whi; base += kSpan) {
#pragma unroll
            for (int h = 0; h < kG; ++h)
                nv[h] = load_lw4(a.lw, base + kSpan + h * 128 + lane * 4, whi);
#pragma unroll
            for (int h = 0; h < kG; ++h)
                acc += fixed_q(v[h].x, M, a.shift) +
                    fixed_q(v[h].y, M, a.shift) +
                    fixed_q(v[h].z, M, a.shift) + fixed_q(v[h].w, M, a.shift);
#pragma unroll
            for (int h = 0; h < kG; ++h)
                v[h] = nv[h];
        }
    } else {
        for (uint32_t base = wlo; base < whi; base += kSpan)
            for (int h = 0; h < kG; ++h) {
                const uint32_t i0 = base + h * 128 + lane * 4;
                for (uint32_t i = i0; i < whi && i < i0 + 4; ++i)
                    acc += a.q[i];
            }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
    __shared__ uint64_t shs[kPfBlock / 32 + 1];
    put_parts(a.qpart, acc, shs);
    if (!rs_last_block(a.sc))
        return;
    const uint64_t Q = scan_blocks_in_place(blk_parts(a.qpart), gridDim.x, shs);
    if (threadIdx.x == 0) {
        uint32_t err = 0;
        cdf_constants(*a.sc, Q, a.n, a.scheme == VSMC_CUDA_SYSTEMATIC, err);
        if (err)
            a.sc->err |= err;
    }
}

// End of a counting pass: each warp's empty and copy counts (the same in
// every lane) go to epart / cpart with the block totals; the last block
// turns the block totals into prefix sums (with the ranges' own entries,
// the offsets the assign pass starts each range from) and records the
// totals.
__device__ __forceinline__ void count_finish(
    const Rs32Args &a, uint32_t empties, uint32_t copies)
{
    __shared__ uint32_t sh[kPfBlock / 32 + 1];
    __shared__ uint32_t sh2[kRsWarps];
    put_parts(a.epart, empties, sh);
    put_parts(a.cpart, copies, sh2);
    if (!rs_last_block(a.sc))
        return;
    const uint32_t et = scan_blocks_in_place(blk_parts(a.epart), gridDim.x, sh);
    const uint32_t ct = scan_blocks_in_place(blk_parts(a.cpart), gridDim.x, sh);
    if (threadIdx.x == 0) {
        a.sc->nempty = et;
        if (ct != a.n)
            a.sc->err |= DEV_ERR_INTERNAL;
    }
}

// Replication counts, one warp per warp range, no block barrier.  Particle
// i's count is F(C_i) - F(C_{i-1}) for the CDF C_i: exact 64-bit prefix sums
// (the range's offset from qsum, a warp scan per group of 128 particles).
// F(C), the uniforms at or below C / Q, comes from the fixed-point
// reciprocal of Q (cdf_floor): no division and no position carried from
// particle to particle.  Stratified also reads each particle's word a_{j*}:
// a group's j* are nondecreasing, so the warp generates the Philox blocks
// holding them once into its shared-memory row (a word past the row is
// generated where it is needed).  Per-range empty and copy counts go to
// epart / cpart.
constexpr uint32_t kStratRow = 64; // Philox blocks per warp row (256 words)

// One warp's range; Usual picks the reciprocal's case for the whole pass.
template <bool Sys, bool Usual>
__device__ __forceinline__ void count_range(const Rs32Args &a,
    const CdfRcp &p, const EnginePos &e, uint4 *row, uint32_t wlo,
    uint32_t whi, uint32_t &empties, uint32_t &copies)
{
    const uint32_t lane = threadIdx.x & 31;
    const float M = static_cast<float>(a.sc->M);
    const bool checked = a.q != nullptr;
    const uint32_t n = a.n;
    uint64_t carry = range_offset(a.qpart); // the CDF before the range
    uint32_t Fprev = 0;
    if (wlo != 0 && wlo < whi) {
        if (Sys) {
            Fprev = sys_F<Usual>(carry, p);
        } else {
            uint64_t r;
            const uint32_t j = strat_j<Usual>(carry, p, r);
            Fprev = strat_F(j, r, p, e, row, 0, 0);
        }
    }
    float4 nxt = make_float4(0, 0, 0, 0);
    if (!checked && wlo + lane * 4 + 3 < whi)
        nxt = __ldcg(reinterpret_cast<const float4 *>(a.lw + wlo + lane * 4));
    for (uint32_t base = wlo; base < whi; base += 128) {
        const uint32_t i0 = base + lane * 4;
        const float4 v = nxt;
        if (!checked && i0 + 128 + 3 < whi)
            nxt = __ldcg(reinterpret_cast<const float4 *>(a.lw + i0 + 128));
        uint64_t q[4];
        if (i0 + 3 < whi && !checked) {
            q[0] = fixed_q(v.x, M, a.shift);
            q[1] = fixed_q(v.y, M, a.shift);
            q[2] = fixed_q(v.z, M, a.shift);
            q[3] = fixed_q(v.w, M, a.shift);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                q[k] = (i0 + k < whi) ? q_at(a, i0 + k, M) : 0;
        }
        uint64_t s[4];
        s[0] = q[0];
        s[1] = s[0] + q[1];
        s[2] = s[1] + q[2];
        s[3] = s[2] + q[3];
        const uint64_t incl = warp_inclusive_scan(s[3], OpAdd());
        const uint64_t tot = __shfl_sync(0xFFFFFFFFu, incl, 31);
        const uint64_t cb = carry + (incl - s[3]);
        uint32_t F[4];
        if (Sys) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                F[k] = i0 + k + 1 >= n ? n : sys_F<Usual>(cb + s[k], p);
        } else {
            uint32_t j[4];
            uint64_t r[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                j[k] = strat_j<Usual>(cb + s[k], p, r[k]);
            // the group's words: j[0] of lane 0 .. j[3] of lane 31 (j = n
            // needs none)
            uint32_t jv = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (j[k] < n)
                    jv = j[k];
            const uint32_t jl = __reduce_min_sync(0xFFFFFFFFu, j[0]);
            const uint32_t jh = __reduce_max_sync(0xFFFFFFFFu, jv);
            uint32_t b0 = 0, nb = 0;
            if (jl < n) {
                b0 = (e.index + jl) >> 2;
                const uint32_t bl = (e.index + (jh > jl ? jh : jl)) >> 2;
                nb = bl - b0 + 1;
                if (nb > kStratRow)
                    nb = kStratRow;
            }
            __syncwarp();
            for (uint32_t d = lane; d < nb; d += 32)
                row[d] = engine_block(e, b0 + d);
            __syncwarp();
#pragma unroll
            for (int k = 0; k < 4; ++k)
                F[k] = i0 + k + 1 >= n ? n
                                       : strat_F(j[k], r[k], p, e, row, b0, nb);
        }
        uint32_t Fl = __shfl_up_sync(0xFFFFFFFFu, F[3], 1);
        if (lane == 0)
            Fl = Fprev;
        int32_t r[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            r[k] = static_cast<int32_t>(F[k] - Fl);
            Fl = F[k];
        }
        if (i0 + 3 < whi) {
            *reinterpret_cast<int4 *>(a.rep + i0) =
                make_int4(r[0], r[1], r[2], r[3]);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                empties += r[k] == 0 ? 1u : 0u;
                copies += static_cast<uint32_t>(r[k]);
            }
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (i0 + k < whi) {
                    a.rep[i0 + k] = r[k];
                    empties += r[k] == 0 ? 1u : 0u;
                    copies += static_cast<uint32_t>(r[k]);
                }
        }
        carry += tot;
        Fprev = __shfl_sync(0xFFFFFFFFu, F[3], 31);
    }
}

template <bool Sys>
__global__ void __launch_bounds__(kPfBlock, kRsBlocksPerSm) k_rs32_count(
    const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    uint32_t lo, hi;
    chunk_range(a.n, a.chunk, lo, hi);
    const uint32_t w = threadIdx.x >> 5;
    const CdfRcp p = load_cdf_rcp(*a.sc, a.n);
    EnginePos e = {};
    if (!Sys)
        e = engine_pos(*a.sc);
    __shared__ uint4 rows[Sys ? 1 : kRsWarps][Sys ? 1 : kStratRow];
    uint4 *row = rows[Sys ? 0 : w];
    uint32_t wlo, whi;
    warp_range(lo, hi, a.chunk, w, wlo, whi);
    uint32_t empties = 0, copies = 0;
    if (p.s != 0)
        count_range<Sys, true>(a, p, e, row, wlo, whi, empties, copies);
    else
        count_range<Sys, false>(a, p, e, row, wlo, whi, empties, copies);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        empties += __shfl_xor_sync(0xFFFFFFFFu, empties, o);
        copies += __shfl_xor_sync(0xFFFFFFFFu, copies, o);
    }
    count_finish(a, empties, copies);
}

// the counting kernel of the scheme (systematic or stratified)
inline void launch_rs32_count(int grid, cudaStream_t st, const Rs32Args &a)
{
    if (a.scheme == VSMC_CUDA_SYSTEMATIC)
        k_rs32_count<true><<<grid, kPfBlock, 0, st>>>(a);
    else
        k_rs32_count<false><<<grid, kPfBlock, 0, st>>>(a);
}

// Slot assignment, one warp per warp range (no block barrier).  With
// c = copies before slot i and e = empty slots before i, the first surplus
// rank of i is c - (i - e) (every non-empty slot before i keeps one of its
// copies).  idx[i] = i for a parent (it keeps its slot), idx[i] = -(e + 1)
// for the e-th empty slot, and srcs[first surplus rank .. + r - 1) = i for a
// parent with r >= 2 copies: the reference's layout
// (resample/transform.hpp:116-133) in one pass over the counts.  Each range
// starts from its offsets (c, e) that the counting pass left in cpart /
// epart, and a warp scan of (copies, empties) carries them through its
// 128-particle groups.
template <bool Mon>
__global__ void __launch_bounds__(kPfBlock, kRsBlocksPerSm) k_rs32_assign(
    const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    uint32_t lo, hi;
    chunk_range(a.n, a.chunk, lo, hi);
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t etotal = a.sc->nempty;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        PfScalars &sc = *a.sc;
        sc.gather = 1;
        // words the scheme consumed: U01SequenceSystematic draws once in its
        // constructor; U01SequenceStratified draws lazily up to the first
        // uniform above the second-to-last cumulative weight
        // (rng/u01_sequence.hpp:177-259, resample/transform.hpp:61-70)
        if (a.scheme == VSMC_CUDA_SYSTEMATIC) {
            engine_advance(sc, 1);
        } else if (a.n >= 2) {
            const uint32_t jf = a.n - static_cast<uint32_t>(a.rep[a.n - 1]);
            engine_advance(sc, jf < a.n ? jf + 1 : a.n);
        }
    }
    uint32_t wlo, whi;
    warp_range(lo, hi, a.chunk, w, wlo, whi);
    uint32_t coff = range_offset(a.cpart), eoff = range_offset(a.epart);
    // monitor of the resampled particles, sum_i rep_i x_{d,i}, when the
    // host asks for it right after resampling (mon_dim > 0); the rows, like
    // the counts, are loaded one group ahead
    const uint32_t md = Mon ? a.mon_dim : 0u;
    float macc[kMaxMonitorDim] = {};
    float4 mrow[kMaxMonitorDim], mnxt[kMaxMonitorDim];
#pragma unroll
    for (int d = 0; d < kMaxMonitorDim; ++d)
        mnxt[d] = static_cast<uint32_t>(d) < md
            ? load_row4(a.mon_state + d * a.stride, wlo + lane * 4, whi)
            : make_float4(0, 0, 0, 0);
    uint32_t err = 0;
    __shared__ __align__(16) uint32_t shm[kPfBlock / 32][kRunChunk];
    int4 nxt = load_rep4(a.rep, wlo + lane * 4, whi);
    for (uint32_t base = wlo; base < whi; base += 128) {
        const uint32_t i0 = base + lane * 4;
        const int4 cur = nxt;
        if (base + 128 < whi)
            nxt = load_rep4(a.rep, i0 + 128, whi);
#pragma unroll
        for (int d = 0; d < kMaxMonitorDim; ++d) {
            mrow[d] = mnxt[d];
            if (static_cast<uint32_t>(d) < md && base + 128 < whi)
                mnxt[d] = load_row4(a.mon_state + d * a.stride, i0 + 128, whi);
        }
        const int32_t r[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
        for (int d = 0; d < kMaxMonitorDim; ++d)
            if (static_cast<uint32_t>(d) < md)
                macc[d] += static_cast<float>(max(r[0], 0)) * mrow[d].x +
                    static_cast<float>(max(r[1], 0)) * mrow[d].y +
                    static_cast<float>(max(r[2], 0)) * mrow[d].z +
                    static_cast<float>(max(r[3], 0)) * mrow[d].w;

        uint32_t tr = 0, te = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (r[k] >= 0) {
                tr += static_cast<uint32_t>(r[k]);
                te += r[k] == 0 ? 1u : 0u;
            }
        // (copies, empties) before each lane: one 32-bit scan of
        // copies * 256 + empties (a group has at most 128 empties) unless a
        // lane has 2^16 or more copies
        uint32_t c, e, tc, tn;
        if (__any_sync(0xFFFFFFFFu, tr >= (1u << 16))) {
            const uint64_t v = (static_cast<uint64_t>(tr) << 32) | te;
            const uint64_t incl = warp_inclusive_scan(v, OpAdd());
            const uint64_t tot = __shfl_sync(0xFFFFFFFFu, incl, 31);
            const uint64_t ex = incl - v;
            c = coff + static_cast<uint32_t>(ex >> 32);
            e = eoff + static_cast<uint32_t>(ex & 0xFFFFFFFFu);
            tc = static_cast<uint32_t>(tot >> 32);
            tn = static_cast<uint32_t>(tot & 0xFFFFFFFFu);
        } else {
            const uint32_t v = (tr << 8) | te;
            const uint32_t incl = warp_inclusive_scan(v, OpAdd());
            const uint32_t tot = __shfl_sync(0xFFFFFFFFu, incl, 31);
            const uint32_t ex = incl - v;
            c = coff + (ex >> 8);
            e = eoff + (ex & 0xFFu);
            tc = tot >> 8;
            tn = tot & 0xFFu;
        }
        const uint32_t c0 = c, e0 = e;
        int32_t out[4];
        uint32_t rs[4], rl[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t i = i0 + k;
            rs[k] = 0;
            rl[k] = 0;
            if (r[k] == 0) {
                out[k] = -static_cast<int32_t>(e) - 1;
                ++e;
            } else {
                out[k] = static_cast<int32_t>(i);
                if (r[k] >= 2) {
                    rs[k] = c - (i - e);
                    rl[k] = static_cast<uint32_t>(r[k]) - 1;
                }
            }
            if (r[k] > 0)
                c += static_cast<uint32_t>(r[k]);
        }
        // the group's surplus ranks: copies minus kept slots before its
        // first particle, and the sum of its runs
        {
            const uint32_t first = c0 - (i0 - e0);
            const uint32_t W0 = __shfl_sync(0xFFFFFFFFu, first, 0);
            const uint32_t Sw =
                __reduce_add_sync(0xFFFFFFFFu, rl[0] + rl[1] + rl[2] + rl[3]);
            if (Sw != 0) {
                if (Sw > etotal || W0 > etotal - Sw) {
                    err |= DEV_ERR_INTERNAL; // ranks past the empty slots
                } else {
                    write_surplus_runs(a.srcs, rs, rl, i0, W0, Sw, shm[w], err);
                }
            }
        }
        if (i0 + 3 < whi) {
            *reinterpret_cast<int4 *>(a.idx + i0) =
                make_int4(out[0], out[1], out[2], out[3]);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (r[k] >= 0)
                    a.idx[i0 + k] = out[k];
        }
        coff += tc;
        eoff += tn;
    }
    if (err)
        atomicOr(&a.sc->err, err);
    if (Mon && md > 0)
        equal_mean_finish(macc, md, 1.0 / static_cast<double>(a.n),
            a.mon_part, a.sc, a.h_mean, a.sc->step - 1, a.max_steps);
}

// the assign pass, with the resampled particles' mean when asked for
inline void launch_rs32_assign(int grid, cudaStream_t st, const Rs32Args &a)
{
    if (a.mon_dim > 0)
        k_rs32_assign<true><<<grid, kPfBlock, 0, st>>>(a);
    else
        k_rs32_assign<false><<<grid, kPfBlock, 0, st>>>(a);
}

// Genealogy row of the step just finished (t = step - 1): each particle's
// parent among the step's particles before resampling, or itself when the
// step did not resample.
__global__ void __launch_bounds__(kPfBlock) k_pf32_record(
    const PfStepArgs a, int32_t *rows)
{
    const uint32_t t = a.sc->step - 1;
    if (t >= a.max_steps)
        return;
    const bool res = a.sc->resampled != 0;
    int32_t *row = rows + static_cast<size_t>(t) * a.n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += gridDim.x * blockDim.x) {
        uint32_t src = res ? pf_source(a.srcs, a.idx[i]) : i;
        if (src >= a.n) {
            atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
            src = 0;
        }
        row[i] = static_cast<int32_t>(src);
    }
}

// Resample-move: after a step that resampled (t >= 1), `sweeps` random-walk
// Metropolis steps (cv_mcmc_step) on each particle's acceleration, on the
// gathered state read from a.in (the step's output); the result goes to
// a.out (the step's input buffer, so the next step reads it with no
// gather).  Steps that did not resample (weights not equal) copy the state
// through unchanged.  acc_hist[t] += the accepted steps.  After moving, the
// monitor (sc->mean, h_mean[t]) is the equal-weight mean of the moved
// particles, as the reference's monitor sees them after the mcmc queue
// (core/sampler.hpp:746-754).
__global__ void __launch_bounds__(kPfBlock) k_pf32_mcmc(const PfStepArgs a,
    CvConst<float> c, const double *obs, uint32_t sweeps, float s_rw,
    float inv_var, uint32_t *acc_hist)
{
    const uint32_t t = a.sc->step - 1;
    const bool gather = a.sc->gather != 0;
    const bool move = a.sc->resampled != 0 && t >= 1;
    const uint32_t to = t < a.max_steps ? t : a.max_steps - 1;
    const float obx = static_cast<float>(obs[2 * to + 0]);
    const float oby = static_cast<float>(obs[2 * to + 1]);
    const size_t ld = a.stride;
    uint32_t acc = 0;
    float macc[kMaxMonitorDim] = {};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += gridDim.x * blockDim.x) {
        uint32_t src = gather ? pf_source(a.srcs, a.idx[i]) : i;
        if (src >= a.n) {
            atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
            src = 0;
        }
        float x = a.in[src], y = a.in[ld + src], vx = a.in[2 * ld + src],
              vy = a.in[3 * ld + src];
        if (move) {
            float ax, ay;
            cv_innovation(c, t, a.seed, src, ax, ay);
            float lt = -0.5f * inv_var * (ax * ax + ay * ay) +
                cv_loglik(c, obx, oby, x, y);
            for (uint32_t k = 0; k < sweeps; ++k)
                acc += cv_mcmc_step(c, obx, oby, s_rw, inv_var, t, a.seed, i,
                    k, x, y, vx, vy, ax, ay, lt);
            macc[0] += x;
            macc[1] += y;
        }
        a.out[i] = x;
        a.out[ld + i] = y;
        a.out[2 * ld + i] = vx;
        a.out[3 * ld + i] = vy;
    }
    __shared__ uint32_t sh[kPfBlock / 32 + 1];
    acc = block_reduce(acc, OpAdd(), 0u, sh);
    if (threadIdx.x == 0 && acc && t < a.max_steps)
        atomicAdd(acc_hist + t, acc);
    if (move)
        equal_mean_finish(macc, 2, 1.0 / static_cast<double>(a.n), a.part,
            a.sc, a.h_mean, t, a.max_steps);
}

// parent index of every slot from the encoded idx (reference layout)
__global__ void __launch_bounds__(kPfBlock) k_rs32_decode(
    const Rs32Args a, int32_t *parent)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += gridDim.x * blockDim.x) {
        const int32_t v = a.idx[i];
        parent[i] = v >= 0 ? v : static_cast<int32_t>(a.srcs[-v - 1]);
    }
}

__global__ void k_rs32_setup(PfScalars *sc, uint32_t k0, uint32_t k1,
    uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t index)
{
    PfScalars z = {};
    z.resampled = 1;
    z.rkey[0] = k0;
    z.rkey[1] = k1;
    z.rctr[0] = c0;
    z.rctr[1] = c1;
    z.rctr[2] = c2;
    z.rctr[3] = c3;
    z.rindex = index;
    *sc = z;
}

} // namespace vsmc_cuda
