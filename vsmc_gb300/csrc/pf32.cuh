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

// Per-particle body of the fused kernel.  First: draw the prior at t = 0.
// x..vy hold the particle as read (after any resampling gather) on entry and
// the moved particle on exit.
template <bool First>
__device__ __forceinline__ void step_one(const Pf32Args &a, uint32_t i,
    uint32_t t, float ox, float oy, int resampled, float Mprev, float &x,
    float &y, float &vx, float &vy, float &lw, float &m, float &s, float &s2,
    float &sx, float &sy, float &sw)
{
    const u32x4 w = particle_block(t, a.seed, i);
    float lw_old = 0.0f;
    if (First) {
        float z1, z2, z3, z4;
        normal_pair_f(w.x, w.y, z1, z2);
        normal_pair_f(w.z, w.w, z3, z4);
        x = a.c.sd_pos0 * z1;
        y = a.c.sd_pos0 * z2;
        vx = a.c.sd_vel0 * z3;
        vy = a.c.sd_vel0 * z4;
    } else {
        lw_old = resampled ? 0.0f : lw - Mprev;
        const float wo = resampled ? 1.0f : __expf(lw_old);
        sx += wo * x;
        sy += wo * y;
        sw += wo;
        float z1, z2;
        normal_pair_f(w.x, w.y, z1, z2);
        cv_move(a.c, a.c.sigma_a * z1, a.c.sigma_a * z2, x, y, vx, vy);
    }
    lw = lw_old + cv_loglik(a.c, ox, oy, x, y);
    lse_push(lw, m, s, s2);
}

__device__ __forceinline__ float4 ld4(const float *p, uint32_t i)
{
    return __ldcs(reinterpret_cast<const float4 *>(p + i));
}

__device__ __forceinline__ void st4(float *p, uint32_t i, float4 v)
{
    __stcs(reinterpret_cast<float4 *>(p + i), v);
}

// source slot of slot i after a resample: idx[i] >= 0 is the slot itself
// (a parent), idx[i] = -(e + 1) is the e-th empty slot, filled from srcs[e]
__device__ __forceinline__ uint32_t source_of(
    const int32_t *idx, const uint32_t *srcs, int32_t v)
{
    return v >= 0 ? static_cast<uint32_t>(v) : __ldcg(srcs + (-v - 1));
    (void)idx;
}

// Reads the state of particles i0..i0+3 (gathered through idx after a
// resample).
__device__ __forceinline__ void load_group(const Pf32Args &a, uint32_t i0,
    bool gather, float4 &X, float4 &Y, float4 &VX, float4 &VY)
{
    if (gather) {
        const int4 I = __ldcs(reinterpret_cast<const int4 *>(a.idx + i0));
        const int b = static_cast<int>(i0);
        if (I.x == b && I.y == b + 1 && I.z == b + 2 && I.w == b + 3) {
            X = ld4(a.ax, i0);
            Y = ld4(a.ay, i0);
            VX = ld4(a.avx, i0);
            VY = ld4(a.avy, i0);
        } else {
            uint32_t s0 = source_of(a.idx, a.srcs, I.x);
            uint32_t s1 = source_of(a.idx, a.srcs, I.y);
            uint32_t s2 = source_of(a.idx, a.srcs, I.z);
            uint32_t s3 = source_of(a.idx, a.srcs, I.w);
            if (max(max(s0, s1), max(s2, s3)) >= a.n) {
                // an index outside the particles: record it, read slot 0
                atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
                s0 = s0 < a.n ? s0 : 0;
                s1 = s1 < a.n ? s1 : 0;
                s2 = s2 < a.n ? s2 : 0;
                s3 = s3 < a.n ? s3 : 0;
            }
            X = make_float4(a.ax[s0], a.ax[s1], a.ax[s2], a.ax[s3]);
            Y = make_float4(a.ay[s0], a.ay[s1], a.ay[s2], a.ay[s3]);
            VX = make_float4(a.avx[s0], a.avx[s1], a.avx[s2], a.avx[s3]);
            VY = make_float4(a.avy[s0], a.avy[s1], a.avy[s2], a.avy[s3]);
        }
    } else {
        X = ld4(a.ax, i0);
        Y = ld4(a.ay, i0);
        VX = ld4(a.avx, i0);
        VY = ld4(a.avy, i0);
    }
}

template <bool First>
__global__ void __launch_bounds__(kPfBlock, 4) k_pf32_step(const Pf32Args a)
{
    const uint32_t t = a.sc->step;
    const int resampled = First ? 1 : a.sc->resampled;
    const bool gather = First ? false : (a.sc->gather != 0);
    const float Mprev = First ? 0.0f : static_cast<float>(a.sc->M);
    // steps past the capacity (profiling loops) reuse the last observation
    // and record nothing
    const uint32_t to = t < a.max_steps ? t : a.max_steps - 1;
    const float ox = static_cast<float>(a.obs[2 * to + 0]);
    const float oy = static_cast<float>(a.obs[2 * to + 1]);
    const uint32_t n = a.n;
    float m = -INFINITY, s = 0, s2 = 0, sx = 0, sy = 0, sw = 0;

    const uint32_t ntiles = (n + kPfTile - 1) / kPfTile;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint32_t i0 = tile * kPfTile + threadIdx.x * 4;
        if (i0 + 3 < n) {
            float4 X, Y, VX, VY, LW;
            if (!First) {
                load_group(a, i0, gather, X, Y, VX, VY);
                LW = resampled ? make_float4(0, 0, 0, 0) : ld4(a.lw, i0);
            }
            step_one<First>(a, i0 + 0, t, ox, oy, resampled, Mprev, X.x, Y.x,
                VX.x, VY.x, LW.x, m, s, s2, sx, sy, sw);
            step_one<First>(a, i0 + 1, t, ox, oy, resampled, Mprev, X.y, Y.y,
                VX.y, VY.y, LW.y, m, s, s2, sx, sy, sw);
            step_one<First>(a, i0 + 2, t, ox, oy, resampled, Mprev, X.z, Y.z,
                VX.z, VY.z, LW.z, m, s, s2, sx, sy, sw);
            step_one<First>(a, i0 + 3, t, ox, oy, resampled, Mprev, X.w, Y.w,
                VX.w, VY.w, LW.w, m, s, s2, sx, sy, sw);
            st4(a.bx, i0, X);
            st4(a.by, i0, Y);
            st4(a.bvx, i0, VX);
            st4(a.bvy, i0, VY);
            st4(a.lw, i0, LW);
        } else {
            for (uint32_t i = i0; i < n && i < i0 + 4; ++i) {
                float X = 0, Y = 0, VX = 0, VY = 0, LW = 0;
                if (!First) {
                    uint32_t src =
                        gather ? source_of(a.idx, a.srcs, a.idx[i]) : i;
                    if (src >= a.n) {
                        atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
                        src = 0;
                    }
                    X = a.ax[src];
                    Y = a.ay[src];
                    VX = a.avx[src];
                    VY = a.avy[src];
                    LW = resampled ? 0.0f : a.lw[i];
                }
                step_one<First>(a, i, t, ox, oy, resampled, Mprev, X, Y, VX,
                    VY, LW, m, s, s2, sx, sy, sw);
                a.bx[i] = X;
                a.by[i] = Y;
                a.bvx[i] = VX;
                a.bvy[i] = VY;
                a.lw[i] = LW;
            }
        }
    }

    // ---- warp level in FP32
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const float om = __shfl_xor_sync(0xFFFFFFFFu, m, d);
        const float os = __shfl_xor_sync(0xFFFFFFFFu, s, d);
        const float os2 = __shfl_xor_sync(0xFFFFFFFFu, s2, d);
        sx += __shfl_xor_sync(0xFFFFFFFFu, sx, d);
        sy += __shfl_xor_sync(0xFFFFFFFFu, sy, d);
        sw += __shfl_xor_sync(0xFFFFFFFFu, sw, d);
        lse_merge_f(m, s, s2, om, os, os2);
    }
    // ---- block level in FP32 (warp 0 merges the warps' records), then one
    // FP64 record per block
    constexpr int kW = kPfBlock / 32;
    __shared__ float shw[6][kW];
    __shared__ double sh[5][kW];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        shw[0][wid] = m;
        shw[1][wid] = s;
        shw[2][wid] = s2;
        shw[3][wid] = sx;
        shw[4][wid] = sy;
        shw[5][wid] = sw;
    }
    __syncthreads();
    if (wid == 0) {
        const bool in = lane < kW;
        float wm = in ? shw[0][lane] : -INFINITY;
        float ws = in ? shw[1][lane] : 0.0f, ws2 = in ? shw[2][lane] : 0.0f;
        float wx = in ? shw[3][lane] : 0.0f, wy = in ? shw[4][lane] : 0.0f;
        float ww = in ? shw[5][lane] : 0.0f;
#pragma unroll
        for (int d = kW / 2; d > 0; d >>= 1) {
            const float om = __shfl_xor_sync(0xFFFFFFFFu, wm, d);
            const float os = __shfl_xor_sync(0xFFFFFFFFu, ws, d);
            const float os2 = __shfl_xor_sync(0xFFFFFFFFu, ws2, d);
            wx += __shfl_xor_sync(0xFFFFFFFFu, wx, d);
            wy += __shfl_xor_sync(0xFFFFFFFFu, wy, d);
            ww += __shfl_xor_sync(0xFFFFFFFFu, ww, d);
            lse_merge_f(wm, ws, ws2, om, os, os2);
        }
        if (lane == 0) {
            const MovePartial p = {wx, wy, ww, wm, ws, ws2};
            a.part[blockIdx.x] = p;
            __threadfence();
            is_last = atomicAdd(&a.sc->done, 1u) == gridDim.x - 1;
        }
    }
    __syncthreads();
    if (!is_last)
        return;

    // ---- last block: combine every block's record
    __threadfence();
    float M = -INFINITY;
    for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x)
        M = fmaxf(M, static_cast<float>(a.part[b].m));
    __shared__ float shmax[kPfBlock / 32 + 1];
    M = block_reduce(M, OpMax(), -INFINITY, shmax);
    double S = 0, S2 = 0, SX = 0, SY = 0, SW = 0;
    for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
        const MovePartial p = a.part[b];
        SX += p.sx;
        SY += p.sy;
        SW += p.sw;
        if (p.m > -INFINITY) {
            const double f = __expf(static_cast<float>(p.m) - M);
            S += p.s * f;
            S2 += p.s2 * f * f;
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        S += __shfl_xor_sync(0xFFFFFFFFu, S, d);
        S2 += __shfl_xor_sync(0xFFFFFFFFu, S2, d);
        SX += __shfl_xor_sync(0xFFFFFFFFu, SX, d);
        SY += __shfl_xor_sync(0xFFFFFFFFu, SY, d);
        SW += __shfl_xor_sync(0xFFFFFFFFu, SW, d);
    }
    __syncthreads();
    if (lane == 0) {
        sh[0][wid] = S;
        sh[1][wid] = S2;
        sh[2][wid] = SX;
        sh[3][wid] = SY;
        sh[4][wid] = SW;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double S1 = 0, S21 = 0, SX1 = 0, SY1 = 0, SW1 = 0;
        for (int w = 0; w < kPfBlock / 32; ++w) {
            S1 += sh[0][w];
            S21 += sh[1][w];
            SX1 += sh[2][w];
            SY1 += sh[3][w];
            SW1 += sh[4][w];
        }
        PfScalars &sc = *a.sc;
        const double prev_mass = First ? static_cast<double>(n) : SW1;
        const bool rec = t < a.max_steps;
        if (!First && rec) {
            a.h_mean[2 * (t - 1) + 0] = SX1 / SW1;
            a.h_mean[2 * (t - 1) + 1] = SY1 / SW1;
        }
        const double ess = S1 * S1 / S21;
        const double M1 = static_cast<double>(M);
        sc.logz += M1 + log(S1) - log(prev_mass);
        if (!(S1 > 0) || !(ess > 0))
            sc.err |= DEV_ERR_NONFINITE;
        const int flag = ess < a.threshold * static_cast<double>(n) ? 1 : 0;
        if (rec) {
            a.h_ess[t] = ess;
            a.h_logz[t] = sc.logz;
            a.h_res[t] = flag;
        }
        sc.M = M1;
        sc.S = S1;
        sc.ess = ess;
        sc.resampled = flag;
        sc.gather = 0; // every block has read it; a resample sets it again
        sc.step = t + 1;
        sc.done = 0;
    }
}

// Weighted mean of the current particles (the last step's monitor).
__global__ void __launch_bounds__(kPfBlock) k_pf32_final_mean(
    const Pf32Args a, uint32_t t_rec)
{
    const int resampled = a.sc->resampled;
    const bool gather = a.sc->gather != 0;
    const float M = static_cast<float>(a.sc->M);
    const uint32_t n = a.n;
    // FP32 within a thread and a warp, FP64 across warps and blocks, as
    // the step kernel forms the monitor sums; four particles per thread
    // step (float4 rows when nothing is gathered)
    float sx = 0, sy = 0, sw = 0;
    auto add = [&](uint32_t i, float x, float y) {
        const float w = resampled ? 1.0f : __expf(a.lw[i] - M);
        sx += w * x;
        sy += w * y;
        sw += w;
    };
    const uint32_t ngroups = n / 4;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < ngroups;
         g += gridDim.x * blockDim.x) {
        const uint32_t i0 = 4 * g;
        if (!gather) {
            const float4 X = ld4(a.ax, i0), Y = ld4(a.ay, i0);
            add(i0 + 0, X.x, Y.x);
            add(i0 + 1, X.y, Y.y);
            add(i0 + 2, X.z, Y.z);
            add(i0 + 3, X.w, Y.w);
        } else {
            for (uint32_t i = i0; i < i0 + 4; ++i) {
                uint32_t src = source_of(a.idx, a.srcs, a.idx[i]);
                if (src >= n) {
                    atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
                    src = 0;
                }
                add(i, a.ax[src], a.ay[src]);
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < n - 4 * ngroups) { // the last 1-3
        const uint32_t i = 4 * ngroups + threadIdx.x;
        uint32_t src = gather ? source_of(a.idx, a.srcs, a.idx[i]) : i;
        if (src >= n) {
            atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
            src = 0;
        }
        add(i, a.ax[src], a.ay[src]);
    }
    __shared__ double sh[3][kPfBlock / 32];
    __shared__ bool is_last;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        sx += __shfl_xor_sync(0xFFFFFFFFu, sx, d);
        sy += __shfl_xor_sync(0xFFFFFFFFu, sy, d);
        sw += __shfl_xor_sync(0xFFFFFFFFu, sw, d);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][wid] = sx;
        sh[1][wid] = sy;
        sh[2][wid] = sw;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        MovePartial p = {0, 0, 0, 0, 0, 0};
        for (int w = 0; w < kPfBlock / 32; ++w) {
            p.sx += sh[0][w];
            p.sy += sh[1][w];
            p.sw += sh[2][w];
        }
        a.part[blockIdx.x] = p;
        __threadfence();
        is_last = atomicAdd(&a.sc->done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last || threadIdx.x != 0)
        return;
    __threadfence();
    double SX = 0, SY = 0, SW = 0;
    for (uint32_t b = 0; b < gridDim.x; ++b) {
        SX += a.part[b].sx;
        SY += a.part[b].sy;
        SW += a.part[b].sw;
    }
    if (t_rec < a.max_steps) {
        a.h_mean[2 * t_rec + 0] = SX / SW;
        a.h_mean[2 * t_rec + 1] = SY / SW;
    }
    a.sc->done = 0;
}

// B = A gathered through idx (materializes a pending resample)
__global__ void __launch_bounds__(kPfBlock) k_pf32_materialize(
    const Pf32Args a)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += gridDim.x * blockDim.x) {
        uint32_t src = source_of(a.idx, a.srcs, a.idx[i]);
        if (src >= a.n) {
            atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
            src = 0;
        }
        a.bx[i] = a.ax[src];
        a.by[i] = a.ay[src];
        a.bvx[i] = a.avx[src];
        a.bvy[i] = a.avy[src];
    }
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

// block sum of q over the block's chunk (four groups of four per thread in
// flight)
__global__ void __launch_bounds__(kPfBlock) k_rs32_qsum(const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    const float M = static_cast<float>(a.sc->M);
    uint32_t lo, hi;
    chunk_range(a.n, a.chunk, lo, hi);
    uint64_t acc = 0;
    constexpr int kG = 4;
    for (uint32_t base = lo; base < hi; base += kG * kPfTile) {
        if (a.q == nullptr && base + kG * kPfTile <= hi) {
            float4 v[kG];
#pragma unroll
            for (int h = 0; h < kG; ++h)
                v[h] = __ldcg(reinterpret_cast<const float4 *>(
                    a.lw + base + h * kPfTile + threadIdx.x * 4));
#pragma unroll
            for (int h = 0; h < kG; ++h)
                acc += fixed_q(v[h].x, M, a.shift) +
                    fixed_q(v[h].y, M, a.shift) +
                    fixed_q(v[h].z, M, a.shift) + fixed_q(v[h].w, M, a.shift);
        } else {
            for (int h = 0; h < kG; ++h) {
                const uint32_t i0 = base + h * kPfTile + threadIdx.x * 4;
                for (uint32_t i = i0; i < hi && i < i0 + 4; ++i)
                    acc += q_at(a, i, M);
            }
        }
    }
    __shared__ uint64_t sh[kPfBlock / 32 + 1];
    acc = block_reduce(acc, OpAdd(), uint64_t(0), sh);
    if (threadIdx.x == 0)
        a.qpart[blockIdx.x] = acc;
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
    block_prefix_of_parts(a.qpart, blockIdx.x, gridDim.x, offset, Q, shq);
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

// the counting kernel of the scheme (systematic or stratified)
inline void launch_rs32_count(int grid, cudaStream_t st, const Rs32Args &a)
{
    if (a.scheme == VSMC_CUDA_SYSTEMATIC)
        k_rs32_count<true><<<grid, kPfBlock, 0, st>>>(a);
    else
        k_rs32_count<false><<<grid, kPfBlock, 0, st>>>(a);
}

// Slot assignment.  With c = copies before slot i and e = empty slots before
// i, the first surplus rank of i is c - (i - e) (every non-empty slot before
// i keeps one of its copies).  idx[i] = i for a parent (it keeps its slot),
// idx[i] = -(e + 1) for the e-th empty slot (its source is srcs[e], filled
// below); marks[first surplus rank of a parent with two or more copies] =
// parent + 1.
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
    // the next tile's counts are loaded while this one is scanned
    int4 nxt = load_rep4(a.rep, lo + threadIdx.x * 4, hi);
    for (uint32_t base = lo; base < hi; base += kPfTile) {
        const uint32_t i0 = base + threadIdx.x * 4;
        const int4 cur = nxt;
        if (base + kPfTile < hi)
            nxt = load_rep4(a.rep, i0 + kPfTile, hi);
        const int32_t r[4] = {cur.x, cur.y, cur.z, cur.w};
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
        int32_t out[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t i = i0 + k;
            if (r[k] == 0) {
                out[k] = -static_cast<int32_t>(e) - 1;
                ++e;
            } else {
                out[k] = static_cast<int32_t>(i);
                if (r[k] >= 2) {
                    const uint32_t rank = c - (i - e);
                    if (rank < a.n)
                        a.marks[rank] = i + 1;
                    else
                        atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
                }
            }
            if (r[k] > 0)
                c += static_cast<uint32_t>(r[k]);
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
}

__device__ __forceinline__ void rank_range(
    uint32_t K, uint32_t &lo, uint32_t &hi)
{
    uint32_t per = (K + gridDim.x - 1) / gridDim.x;
    per = (per + 3) / 4 * 4;
    lo = blockIdx.x * per;
    hi = lo + per;
    if (lo > K)
        lo = K;
    if (hi > K)
        hi = K;
}

// per-block max of the marks over the block's share of the surplus ranks
__global__ void __launch_bounds__(kPfBlock) k_rs32_markmax(const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    uint32_t lo, hi;
    rank_range(min(a.sc->nempty, a.n), lo, hi);
    uint32_t mx = 0;
    const uint32_t step = 4 * blockDim.x;
    for (uint32_t k0 = lo + threadIdx.x * 4; k0 < hi; k0 += 2 * step) {
        const uint4 v = load_marks4(a.marks, k0, hi);
        const uint4 w = k0 + step < hi ? load_marks4(a.marks, k0 + step, hi)
                                       : make_uint4(0, 0, 0, 0);
        mx = max(mx, max(max(v.x, v.y), max(v.z, v.w)));
        mx = max(mx, max(max(w.x, w.y), max(w.z, w.w)));
    }
    __shared__ uint32_t sh[kPfBlock / 32 + 1];
    mx = block_reduce(mx, OpMax(), 0u, sh);
    if (threadIdx.x == 0)
        a.mpart[blockIdx.x] = mx;
}

// Running max of the marks gives the parent of each surplus rank:
// srcs[k] = that parent; the marks are cleared for the next resample.
__global__ void __launch_bounds__(kPfBlock) k_rs32_fill(const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    uint32_t lo, hi;
    rank_range(min(a.sc->nempty, a.n), lo, hi);
    __shared__ uint32_t sh[kPfBlock / 32 + 1];
    __shared__ uint32_t shl[kPfBlock / 32];
    uint32_t carry = 0;
    for (uint32_t b = threadIdx.x; b < blockIdx.x; b += blockDim.x)
        carry = max(carry, a.mpart[b]);
    carry = block_reduce(carry, OpMax(), 0u, sh);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t step = 4 * blockDim.x;
    // the next group's marks are loaded while this one is scanned
    uint4 nxt = load_marks4(a.marks, lo + threadIdx.x * 4, hi);
    uint32_t err = 0;
    for (uint32_t base = lo; base < hi; base += step) {
        const uint32_t k0 = base + threadIdx.x * 4;
        const uint4 cur = nxt;
        if (base + step < hi)
            nxt = load_marks4(a.marks, k0 + step, hi);
        const uint32_t mk[4] = {cur.x, cur.y, cur.z, cur.w};
        uint32_t run[4];
        uint32_t tmax = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            tmax = max(tmax, mk[k]);
            run[k] = tmax;
        }
        uint32_t tot;
        const uint32_t incl = block_inclusive_scan(tmax, OpMax(), 0u, sh, &tot);
        // exclusive max: the previous lane's inclusive value, or the
        // previous warp's total for lane 0
        uint32_t before = __shfl_up_sync(0xFFFFFFFFu, incl, 1);
        if (lane == 31)
            shl[wid] = incl;
        __syncthreads();
        if (lane == 0)
            before = wid > 0 ? shl[wid - 1] : 0u;
        __syncthreads();
        before = max(before, carry);
        uint32_t out[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t rk = max(run[k], before);
            if (k0 + k < hi && (rk == 0 || rk - 1 >= a.n))
                err |= DEV_ERR_INTERNAL;
            out[k] = rk - 1;
        }
        if (k0 + 3 < hi) {
            *reinterpret_cast<uint4 *>(a.srcs + k0) =
                make_uint4(out[0], out[1], out[2], out[3]);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k0 + k < hi)
                    a.srcs[k0 + k] = out[k];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (mk[k] && k0 + k < hi)
                a.marks[k0 + k] = 0;
        carry = max(carry, tot);
    }
    if (err)
        atomicOr(&a.sc->err, err);
}

// Genealogy row of the step just finished (t = step - 1): each particle's
// parent among the step's particles before resampling, or itself when the
// step did not resample.
__global__ void __launch_bounds__(kPfBlock) k_pf32_record(
    const Pf32Args a, int32_t *rows)
{
    const uint32_t t = a.sc->step - 1;
    if (t >= a.max_steps)
        return;
    const bool res = a.sc->resampled != 0;
    int32_t *row = rows + static_cast<size_t>(t) * a.n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += gridDim.x * blockDim.x) {
        uint32_t src = res ? source_of(a.idx, a.srcs, a.idx[i]) : i;
        if (src >= a.n) {
            atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
            src = 0;
        }
        row[i] = static_cast<int32_t>(src);
    }
}

// Resample-move: after a step that resampled (t >= 1), `sweeps` random-walk
// Metropolis steps (cv_mcmc_step) on each particle's acceleration, on the
// gathered state; the result goes to the other buffer (out).  Steps that
// did not resample (weights not equal) copy the state through unchanged.
// acc_hist[t] += the accepted steps.
__global__ void __launch_bounds__(kPfBlock) k_pf32_mcmc(const Pf32Args a,
    float *ox_, float *oy_, float *ovx, float *ovy, uint32_t sweeps,
    float s_rw, float inv_var, uint32_t *acc_hist)
{
    const uint32_t t = a.sc->step - 1;
    const bool gather = a.sc->gather != 0;
    const bool move = a.sc->resampled != 0 && t >= 1;
    const uint32_t to = t < a.max_steps ? t : a.max_steps - 1;
    const float obx = static_cast<float>(a.obs[2 * to + 0]);
    const float oby = static_cast<float>(a.obs[2 * to + 1]);
    uint32_t acc = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += gridDim.x * blockDim.x) {
        uint32_t src = gather ? source_of(a.idx, a.srcs, a.idx[i]) : i;
        if (src >= a.n) {
            atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
            src = 0;
        }
        // the step's output is in the b buffer
        float x = a.bx[src], y = a.by[src], vx = a.bvx[src], vy = a.bvy[src];
        if (move) {
            float ax, ay;
            cv_innovation(a.c, t, a.seed, src, ax, ay);
            float lt = -0.5f * inv_var * (ax * ax + ay * ay) +
                cv_loglik(a.c, obx, oby, x, y);
            for (uint32_t k = 0; k < sweeps; ++k)
                acc += cv_mcmc_step(a.c, obx, oby, s_rw, inv_var, t, a.seed, i,
                    k, x, y, vx, vy, ax, ay, lt);
        }
        ox_[i] = x;
        oy_[i] = y;
        ovx[i] = vx;
        ovy[i] = vy;
    }
    __shared__ uint32_t sh[kPfBlock / 32 + 1];
    acc = block_reduce(acc, OpAdd(), 0u, sh);
    if (threadIdx.x == 0 && acc && t < a.max_steps)
        atomicAdd(acc_hist + t, acc);
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
