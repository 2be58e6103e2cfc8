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
// Systematic / stratified uniforms u_j = (j + a_j 2^-32) / N are compared with
// C_i / Q exactly in 128-bit integers.  Replication counts then go to parent
// indices with the reference's slot layout (resample/transform.hpp:116-133):
// parents keep their slot, empty slots take surplus copies in order.  Only
// empty slots are written by the gather.
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

// Sum of q over each warp range (four groups of four per lane in flight):
// qpart[block * kRsWarps + warp].
__global__ void __launch_bounds__(kPfBlock) k_rs32_qsum(const Rs32Args a)
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
    for (uint32_t base = wlo; base < whi; base += kG * 128) {
        if (a.q == nullptr && base + kG * 128 <= whi) {
            float4 v[kG];
#pragma unroll
            for (int h = 0; h < kG; ++h)
                v[h] = __ldcg(reinterpret_cast<const float4 *>(
                    a.lw + base + h * 128 + lane * 4));
#pragma unroll
            for (int h = 0; h < kG; ++h)
                acc += fixed_q(v[h].x, M, a.shift) +
                    fixed_q(v[h].y, M, a.shift) +
                    fixed_q(v[h].z, M, a.shift) + fixed_q(v[h].w, M, a.shift);
        } else {
            for (int h = 0; h < kG; ++h) {
                const uint32_t i0 = base + h * 128 + lane * 4;
                for (uint32_t i = i0; i < whi && i < i0 + 4; ++i)
                    acc += q_at(a, i, M);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
    if (lane == 0)
        a.qpart[blockIdx.x * kRsWarps + w] = acc;
}

// sum of part[0..upto) and of part[0..total) over the block
template <typename T>
__device__ __forceinline__ void block_prefix_of_parts(
    const T *part, uint32_t upto, uint32_t total, T &prefix, T &all, T *sh)
{
    T p = 0, q = 0;
    for (uint32_t b = threadIdx.x; b < total; b += blockDim.x) {
        const T v = part[b];
        q += v;
        if (b < upto)
            p += v;
    }
    prefix = block_reduce(p, OpAdd(), T(0), sh);
    all = block_reduce(q, OpAdd(), T(0), sh);
}

// Replication counts from the fixed-point CDF; per-block empty and copy
// counts.
template <bool Sys>
__global__ void __launch_bounds__(kPfBlock, 4) k_rs32_count(const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    const float M = static_cast<float>(a.sc->M);
    uint32_t lo, hi;
    chunk_range(a.n, a.chunk, lo, hi);
    __shared__ uint64_t shq[kPfBlock / 32 + 1];
    __shared__ QR shqr[kPfBlock / 32];
    __shared__ uint32_t she[kPfBlock / 32 + 1];
    __shared__ QR start0;
    __shared__ uint4 wbuf[2 * kPfBlock];        // stratified words of a tile
    __shared__ uint32_t wsh[2 * (kPfBlock / 32)];
    uint64_t offset, Q;
    block_prefix_of_parts(a.qpart, blockIdx.x * kRsWarps,
        gridDim.x * kRsWarps, offset, Q, shq);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        a.sc->Q = Q;
    const PfScalars sc = *a.sc;
    constexpr bool sys = Sys; // the scheme (a.scheme) picked the instance
    const bool checked = a.q != nullptr;
    const uint32_t n = a.n;
    const CountP cp = make_count_params(Q, n, engine_word(sc, 0));
    const float invQ = __frcp_rn(__ull2float_rn(Q));
    uint32_t err = 0;
    if (threadIdx.x == 0) {
        // the block's first CDF value, offset, by one 128-bit division
        const uint64_t G = sys ? cp.G : 0;
        long long j;
        uint64_t r;
        QR s;
        if (cn_divmod(offset, G, cp, j, r, err)) {
            s.j = static_cast<uint32_t>(j + 1);
            s.r = r;
        } else { // offset n < G < Q: X = -(G - offset n)
            s.j = 0;
            s.r = Q - (G - offset * static_cast<uint64_t>(n));
        }
        start0 = s;
    }
    __syncthreads();
    QR carry = start0;
    uint32_t empties = 0, copies = 0;
    // the next tile's log-weights are loaded while this one is counted
    float4 nxt = make_float4(0, 0, 0, 0);
    if (!checked && lo + threadIdx.x * 4 + 3 < hi)
        nxt = __ldcg(reinterpret_cast<const float4 *>(
            a.lw + lo + threadIdx.x * 4));
    for (uint32_t base = lo; base < hi; base += kPfTile) {
        const uint32_t i0 = base + threadIdx.x * 4;
        const float4 v = nxt;
        if (!checked && i0 + kPfTile + 3 < hi)
            nxt = __ldcg(reinterpret_cast<const float4 *>(a.lw + i0 + kPfTile));
        uint64_t q[4];
        if (i0 + 3 < hi && !checked) {
            q[0] = fixed_q(v.x, M, a.shift);
            q[1] = fixed_q(v.y, M, a.shift);
            q[2] = fixed_q(v.z, M, a.shift);
            q[3] = fixed_q(v.w, M, a.shift);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                q[k] = (i0 + k < hi) ? q_at(a, i0 + k, M) : 0;
        }
        // positions after each of this thread's particles, from its start
        QR loc[4];
        QR acc = {0, 0};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            qr_push(acc, q[k], n, checked, Q, invQ, cp, err);
            loc[k] = acc;
        }
        QR tile_total;
        const QR ex = block_exclusive_qr(acc, Q, shqr, &tile_total);
        const QR st = qr_add(carry, ex, Q);
        WordBuf wv = {wbuf, 0, 0};
        if (!sys) {
            uint32_t wlo, whi;
            words_span(st, qr_add(st, loc[3], Q), n, sc, wlo, whi);
            wv = fill_words<kPfBlock>(sc, wlo, whi, wbuf, 2 * kPfBlock, wsh);
        }
        uint32_t F[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t i = i0 + k;
            if (i + 1 >= n)
                F[k] = n; // the last particle takes the rest
            else if (i < hi)
                F[k] = f_of_buf(qr_add(st, loc[k], Q), sys, n, Q, sc, wv);
            else
                F[k] = 0;
        }
        // F before this thread's first particle is F at the thread's start
        // position (particle 0 has nothing before it)
        uint32_t Fprev = i0 == 0 ? 0u : f_of_buf(st, sys, n, Q, sc, wv);
        int32_t r[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            r[k] = static_cast<int32_t>(F[k] - Fprev);
            Fprev = F[k];
        }
        if (i0 + 3 < hi) {
            *reinterpret_cast<int4 *>(a.rep + i0) = make_int4(r[0], r[1], r[2], r[3]);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                empties += r[k] == 0 ? 1u : 0u;
                copies += static_cast<uint32_t>(r[k]);
            }
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (i0 + k < hi) {
                    a.rep[i0 + k] = r[k];
                    empties += r[k] == 0 ? 1u : 0u;
                    copies += static_cast<uint32_t>(r[k]);
                }
        }
        carry = qr_add(carry, tile_total, Q);
    }
    if (err)
        atomicOr(&a.sc->err, err);
    empties = block_reduce(empties, OpAdd(), 0u, she);
    copies = block_reduce(copies, OpAdd(), 0u, she);
    if (threadIdx.x == 0) {
        a.epart[blockIdx.x] = empties;
        a.cpart[blockIdx.x] = copies;
    }
}

// Warp-wide exclusive scan of positions; *total gets the warp's sum.
__device__ __forceinline__ QR warp_exclusive_qr(QR v, uint64_t Q, QR *total)
{
    const uint32_t lane = threadIdx.x & 31;
    QR x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        QR o;
        o.j = __shfl_up_sync(0xFFFFFFFFu, x.j, d);
        o.r = __shfl_up_sync(0xFFFFFFFFu, x.r, d);
        if (lane >= static_cast<uint32_t>(d))
            x = qr_add(o, x, Q);
    }
    total->j = __shfl_sync(0xFFFFFFFFu, x.j, 31);
    total->r = __shfl_sync(0xFFFFFFFFu, x.r, 31);
    QR ex;
    ex.j = __shfl_up_sync(0xFFFFFFFFu, x.j, 1);
    ex.r = __shfl_up_sync(0xFFFFFFFFu, x.r, 1);
    if (lane == 0)
        ex = QR{0, 0};
    return ex;
}

// Systematic counts, one warp per warp range: the range's first CDF
// position comes from the per-range q sums (one 128-bit division by the
// range's lane 0), then the warp walks its range 128 particles at a time
// with warp scans of the positions and no block barrier.  The counts are
// the same integers as k_rs32_count<true> gives.
__global__ void __launch_bounds__(kPfBlock, 4) k_rs32_count_sys(const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    const float M = static_cast<float>(a.sc->M);
    uint32_t lo, hi;
    chunk_range(a.n, a.chunk, lo, hi);
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __shared__ uint64_t shq[kPfBlock / 32 + 1];
    __shared__ uint32_t she[kPfBlock / 32 + 1];
    // offset of the block (every earlier range) and of this warp's range
    uint64_t boff, Q;
    block_prefix_of_parts(a.qpart, blockIdx.x * kRsWarps,
        gridDim.x * kRsWarps, boff, Q, shq);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        a.sc->Q = Q;
    uint64_t woff =
        lane < w ? a.qpart[blockIdx.x * kRsWarps + lane] : uint64_t(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        woff += __shfl_xor_sync(0xFFFFFFFFu, woff, o);
    woff += boff;
    uint32_t wlo, whi;
    warp_range(lo, hi, a.chunk, w, wlo, whi);
    const bool checked = a.q != nullptr;
    const uint32_t n = a.n;
    const CountP cp = make_count_params(Q, n, engine_word(*a.sc, 0));
    const float invQ = __frcp_rn(__ull2float_rn(Q));
    uint32_t err = 0;
    // the range's first CDF position (lane 0), broadcast
    QR carry = {0, 0};
    if (lane == 0 && wlo < whi) {
        long long j;
        uint64_t r;
        if (cn_divmod(woff, cp.G, cp, j, r, err)) {
            carry.j = static_cast<uint32_t>(j + 1);
            carry.r = r;
        } else { // woff n < G < Q: X = -(G - woff n)
            carry.j = 0;
            carry.r = Q - (cp.G - woff * static_cast<uint64_t>(n));
        }
    }
    carry.j = __shfl_sync(0xFFFFFFFFu, carry.j, 0);
    carry.r = __shfl_sync(0xFFFFFFFFu, carry.r, 0);
    uint32_t empties = 0, copies = 0;
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
        QR loc[4];
        QR acc = {0, 0};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            qr_push(acc, q[k], n, checked, Q, invQ, cp, err);
            loc[k] = acc;
        }
        QR total;
        const QR ex = warp_exclusive_qr(acc, Q, &total);
        const QR st = qr_add(carry, ex, Q);
        uint32_t F[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t i = i0 + k;
            if (i + 1 >= n) {
                F[k] = n; // the last particle takes the rest
            } else if (i < whi) {
                const QR x = qr_add(st, loc[k], Q);
                F[k] = x.j < n ? x.j : n;
            } else {
                F[k] = 0;
            }
        }
        uint32_t Fprev = i0 == 0 ? 0u : (st.j < n ? st.j : n);
        int32_t r[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            r[k] = static_cast<int32_t>(F[k] - Fprev);
            Fprev = F[k];
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
        carry = qr_add(carry, total, Q);
    }
    if (err)
        atomicOr(&a.sc->err, err);
    empties = block_reduce(empties, OpAdd(), 0u, she);
    copies = block_reduce(copies, OpAdd(), 0u, she);
    if (threadIdx.x == 0) {
        a.epart[blockIdx.x] = empties;
        a.cpart[blockIdx.x] = copies;
    }
}

// the counting kernel of the scheme (systematic or stratified)
inline void launch_rs32_count(int grid, cudaStream_t st, const Rs32Args &a)
{
    if (a.scheme == VSMC_CUDA_SYSTEMATIC)
        k_rs32_count_sys<<<grid, kPfBlock, 0, st>>>(a);
    else
        k_rs32_count<false><<<grid, kPfBlock, 0, st>>>(a);
}

// Slot assignment.  With c = copies before slot i and e = empty slots before
// i, the first surplus rank of i is c - (i - e) (every non-empty slot before
// i keeps one of its copies).  idx[i] = i for a parent (it keeps its slot),
// idx[i] = -(e + 1) for the e-th empty slot, and srcs[first surplus rank ..
// + r - 1) = i for a parent with r >= 2 copies: the reference's layout
// (resample/transform.hpp:116-133) in one pass over the counts.
template <bool Mon>
__global__ void __launch_bounds__(kPfBlock) k_rs32_assign(const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    uint32_t lo, hi;
    chunk_range(a.n, a.chunk, lo, hi);
    __shared__ uint32_t sh32[kPfBlock / 32 + 1];
    __shared__ uint64_t sh64[kPfBlock / 32 + 1];
    uint32_t eoff, etotal, coff, ctotal;
    block_prefix_of_parts(a.epart, blockIdx.x, gridDim.x, eoff, etotal, sh32);
    block_prefix_of_parts(a.cpart, blockIdx.x, gridDim.x, coff, ctotal, sh32);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        PfScalars &sc = *a.sc;
        sc.nempty = etotal;
        sc.gather = 1;
        if (ctotal != a.n)
            sc.err |= DEV_ERR_INTERNAL;
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
    // monitor of the resampled particles, sum_i rep_i x_{d,i}, when the
    // host asks for it right after resampling (mon_dim > 0); the rows, like
    // the counts, are loaded one tile ahead
    const uint32_t md = Mon ? a.mon_dim : 0u;
    float macc[kMaxMonitorDim] = {};
    float4 mrow[kMaxMonitorDim], mnxt[kMaxMonitorDim];
#pragma unroll
    for (int d = 0; d < kMaxMonitorDim; ++d)
        mnxt[d] = static_cast<uint32_t>(d) < md
            ? load_row4(a.mon_state + d * a.stride, lo + threadIdx.x * 4, hi)
            : make_float4(0, 0, 0, 0);
    uint32_t err = 0;
    __shared__ __align__(16) uint32_t shm[kPfBlock / 32][kRunChunk];
    // the next tile's counts are loaded while this one is scanned
    int4 nxt = load_rep4(a.rep, lo + threadIdx.x * 4, hi);
    for (uint32_t base = lo; base < hi; base += kPfTile) {
        const uint32_t i0 = base + threadIdx.x * 4;
        const int4 cur = nxt;
        if (base + kPfTile < hi)
            nxt = load_rep4(a.rep, i0 + kPfTile, hi);
#pragma unroll
        for (int d = 0; d < kMaxMonitorDim; ++d) {
            mrow[d] = mnxt[d];
            if (static_cast<uint32_t>(d) < md && base + kPfTile < hi)
                mnxt[d] = load_row4(a.mon_state + d * a.stride,
                    i0 + kPfTile, hi);
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
        const uint64_t v = (static_cast<uint64_t>(tr) << 32) | te;
        uint64_t tot;
        const uint64_t incl =
            block_inclusive_scan(v, OpAdd(), uint64_t(0), sh64, &tot);
        const uint64_t ex = incl - v;
        uint32_t c = coff + static_cast<uint32_t>(ex >> 32);
        uint32_t e = eoff + static_cast<uint32_t>(ex & 0xFFFFFFFFu);
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
        // the warp's surplus ranks: copies minus kept slots before its first
        // particle, and the sum of its runs
        {
            const uint32_t first = c0 - (i0 - e0);
            const uint32_t W0 = __shfl_sync(0xFFFFFFFFu, first, 0);
            uint32_t Sw = rl[0] + rl[1] + rl[2] + rl[3];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                Sw += __shfl_xor_sync(0xFFFFFFFFu, Sw, o);
            if (Sw != 0) {
                if (Sw > etotal || W0 > etotal - Sw)
                    err |= DEV_ERR_INTERNAL; // ranks past the empty slots
                else
                    write_surplus_runs(a.srcs, rs, rl, i0, W0, Sw,
                        shm[threadIdx.x >> 5], err);
            }
        }
        if (i0 + 3 < hi) {
            *reinterpret_cast<int4 *>(a.idx + i0) =
                make_int4(out[0], out[1], out[2], out[3]);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (r[k] >= 0)
                    a.idx[i0 + k] = out[k];
        }
        coff += static_cast<uint32_t>(tot >> 32);
        eoff += static_cast<uint32_t>(tot & 0xFFFFFFFFu);
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
