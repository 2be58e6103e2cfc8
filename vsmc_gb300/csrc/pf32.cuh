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

namespace vsmc_cuda
{

// ------------------------------------------------------- small utilities

__device__ __forceinline__ void lse_push(float v, float &m, float &s, float &s2)
{
    if (!(v > -INFINITY)) // -inf and NaN carry no weight
        return;
    if (v > m) {
        const float e = __expf(m - v);
        s = s * e + 1.0f;
        s2 = s2 * e * e + 1.0f;
        m = v;
    } else {
        const float e = __expf(v - m);
        s += e;
        s2 += e * e;
    }
}

__device__ __forceinline__ void lse_merge(
    double &m, double &s, double &s2, double m2, double t, double t2)
{
    if (!(m2 > -INFINITY))
        return;
    if (!(m > -INFINITY)) {
        m = m2;
        s = t;
        s2 = t2;
        return;
    }
    if (m2 > m) {
        const double e = exp(m - m2);
        s = s * e + t;
        s2 = s2 * e * e + t2;
        m = m2;
    } else {
        const double e = exp(m2 - m);
        s += t * e;
        s2 += t2 * e * e;
    }
}

// 64 x 64 -> 128 bit product, compared as (hi, lo)
struct U128 {
    uint64_t hi, lo;
};

__device__ __forceinline__ U128 mul_u64(uint64_t a, uint64_t b)
{
    return {__umul64hi(a, b), a * b};
}

__device__ __forceinline__ bool le_u128(const U128 &a, const U128 &b)
{
    return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo);
}

// word k (k >= 0) of the scalar stream of an engine at (key, ctr, index):
// gen(ctr + (index + k) / 4)[(index + k) % 4]
__device__ __forceinline__ uint32_t engine_word(const PfScalars &sc, uint64_t k)
{
    const uint64_t pos = static_cast<uint64_t>(sc.rindex) + k;
    uint32_t c[4] = {sc.rctr[0], sc.rctr[1], sc.rctr[2], sc.rctr[3]};
    ctr32_add(c, pos / 4);
    const u32x4 b = philox4x32_10(c[0], c[1], c[2], c[3], sc.rkey[0], sc.rkey[1]);
    const uint32_t i = static_cast<uint32_t>(pos % 4);
    return i == 0 ? b.x : (i == 1 ? b.y : (i == 2 ? b.z : b.w));
}

// advance the engine by k >= 1 words
__device__ __forceinline__ void engine_advance(PfScalars &sc, uint64_t k)
{
    if (k == 0)
        return;
    const uint64_t last = static_cast<uint64_t>(sc.rindex) + k - 1;
    uint32_t c[4] = {sc.rctr[0], sc.rctr[1], sc.rctr[2], sc.rctr[3]};
    ctr32_add(c, last / 4);
    for (int i = 0; i < 4; ++i)
        sc.rctr[i] = c[i];
    sc.rindex = static_cast<uint32_t>(last % 4) + 1;
}

// Fixed-point comparison setup shared by the count kernels.
struct CountP {
    uint64_t Q;  // CDF total
    uint64_t D;  // N * 2^32
    uint32_t n;
    int sh;      // Q >> sh < 2^24
    float scale; // n / (Q >> sh)
};

__device__ __forceinline__ CountP make_count_params(uint64_t Q, uint32_t n)
{
    CountP p;
    p.Q = Q;
    p.D = static_cast<uint64_t>(n) << 32;
    p.n = n;
    const int bits = 64 - __clzll(static_cast<long long>(Q));
    p.sh = bits > 24 ? bits - 24 : 0;
    p.scale = static_cast<float>(n) / static_cast<float>(Q >> p.sh);
    return p;
}

// Number of uniforms u_j = (j + a_j 2^-32) / N (j < N) with u_j <= C / Q.
// The u_j are strictly increasing, so this is also the index of the first
// uniform above C.  a(j) returns a_j.  The float estimate is within a few
// units; the 128-bit checks make the answer exact.
template <typename AFn>
__device__ __forceinline__ uint32_t count_le(
    uint64_t C, const CountP &p, AFn a, uint32_t &err)
{
    const U128 X = mul_u64(C, p.D);
    auto cond = [&](long long jj) -> bool {
        const uint64_t num = (static_cast<uint64_t>(jj) << 32) + a(jj);
        return le_u128(mul_u64(num, p.Q), X);
    };
    const long long nn = static_cast<long long>(p.n);
    const float f = static_cast<float>(static_cast<uint32_t>(C >> p.sh)) * p.scale;
    long long j = static_cast<long long>(floorf(f)) - 1; // estimate of the answer - 1
    if (j > nn - 1)
        j = nn - 1;
    if (j < -1)
        j = -1;
    // walk a few steps from the estimate; the largest j with cond(j) is the
    // answer - 1 (cond is monotone: true then false)
    for (int g = 0; g < 8 && j >= 0 && !cond(j); ++g)
        --j;
    long long lo, hi; // cond(lo) true or lo == -1; cond(hi) false or hi == n
    if (j >= 0 && !cond(j)) {
        lo = -1;
        hi = j;
    } else {
        for (int g = 0; g < 8 && j + 1 < nn && cond(j + 1); ++g)
            ++j;
        if (j + 1 >= nn || !cond(j + 1))
            return static_cast<uint32_t>(j + 1);
        lo = j + 1;
        hi = nn;
    }
    // estimate was far off (very large N): exact bisection
    int guard = 0;
    while (hi - lo > 1) {
        const long long mid = lo + (hi - lo) / 2;
        if (cond(mid))
            lo = mid;
        else
            hi = mid;
        if (++guard > 64) {
            err |= DEV_ERR_BOUND;
            break;
        }
    }
    return static_cast<uint32_t>(lo + 1);
}

__device__ __forceinline__ uint64_t fixed_q(float lw, float M, uint32_t shift)
{
    if (!(lw > -INFINITY))
        return 0;
    const float w = __expf(lw - M); // in (0, 1]
    return __float2ull_rz(ldexpf(fminf(w, 1.0f), static_cast<int>(shift)));
}

// ------------------------------------------------------------ fused step

// Per-particle body of the fused kernel.  First: draw the prior at t = 0.
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

template <bool First>
__global__ void __launch_bounds__(kPfBlock) k_pf32_step(const Pf32Args a)
{
    const uint32_t t = a.sc->step;
    const int resampled = First ? 1 : a.sc->resampled;
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
                X = __ldcs(reinterpret_cast<const float4 *>(a.x + i0));
                Y = __ldcs(reinterpret_cast<const float4 *>(a.y + i0));
                VX = __ldcs(reinterpret_cast<const float4 *>(a.vx + i0));
                VY = __ldcs(reinterpret_cast<const float4 *>(a.vy + i0));
                if (!resampled)
                    LW = __ldcs(reinterpret_cast<const float4 *>(a.lw + i0));
                else
                    LW = make_float4(0, 0, 0, 0);
            }
            step_one<First>(a, i0 + 0, t, ox, oy, resampled, Mprev, X.x, Y.x,
                VX.x, VY.x, LW.x, m, s, s2, sx, sy, sw);
            step_one<First>(a, i0 + 1, t, ox, oy, resampled, Mprev, X.y, Y.y,
                VX.y, VY.y, LW.y, m, s, s2, sx, sy, sw);
            step_one<First>(a, i0 + 2, t, ox, oy, resampled, Mprev, X.z, Y.z,
                VX.z, VY.z, LW.z, m, s, s2, sx, sy, sw);
            step_one<First>(a, i0 + 3, t, ox, oy, resampled, Mprev, X.w, Y.w,
                VX.w, VY.w, LW.w, m, s, s2, sx, sy, sw);
            __stcs(reinterpret_cast<float4 *>(a.x + i0), X);
            __stcs(reinterpret_cast<float4 *>(a.y + i0), Y);
            __stcs(reinterpret_cast<float4 *>(a.vx + i0), VX);
            __stcs(reinterpret_cast<float4 *>(a.vy + i0), VY);
            __stcs(reinterpret_cast<float4 *>(a.lw + i0), LW);
        } else {
            for (uint32_t i = i0; i < n && i < i0 + 4; ++i) {
                float X = 0, Y = 0, VX = 0, VY = 0, LW = 0;
                if (!First) {
                    X = a.x[i];
                    Y = a.y[i];
                    VX = a.vx[i];
                    VY = a.vy[i];
                    LW = resampled ? 0.0f : a.lw[i];
                }
                step_one<First>(a, i, t, ox, oy, resampled, Mprev, X, Y, VX,
                    VY, LW, m, s, s2, sx, sy, sw);
                a.x[i] = X;
                a.y[i] = Y;
                a.vx[i] = VX;
                a.vy[i] = VY;
                a.lw[i] = LW;
            }
        }
    }

    // ---- block reduction: FP32 per thread, FP64 across warps
    double dm = m, ds = s, ds2 = s2, dsx = sx, dsy = sy, dsw = sw;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const double om = __shfl_xor_sync(0xFFFFFFFFu, dm, d);
        const double os = __shfl_xor_sync(0xFFFFFFFFu, ds, d);
        const double os2 = __shfl_xor_sync(0xFFFFFFFFu, ds2, d);
        lse_merge(dm, ds, ds2, om, os, os2);
        dsx += __shfl_xor_sync(0xFFFFFFFFu, dsx, d);
        dsy += __shfl_xor_sync(0xFFFFFFFFu, dsy, d);
        dsw += __shfl_xor_sync(0xFFFFFFFFu, dsw, d);
    }
    __shared__ double sh[6][kPfBlock / 32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][wid] = dsx;
        sh[1][wid] = dsy;
        sh[2][wid] = dsw;
        sh[3][wid] = dm;
        sh[4][wid] = ds;
        sh[5][wid] = ds2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        MovePartial p = {0, 0, 0, -INFINITY, 0, 0};
        for (int w = 0; w < kPfBlock / 32; ++w) {
            p.sx += sh[0][w];
            p.sy += sh[1][w];
            p.sw += sh[2][w];
            lse_merge(p.m, p.s, p.s2, sh[3][w], sh[4][w], sh[5][w]);
        }
        a.part[blockIdx.x] = p;
        __threadfence();
        is_last = atomicAdd(&a.sc->done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last)
        return;

    // ---- last block: combine all block records in FP64
    __threadfence();
    double M = -INFINITY, S = 0, S2 = 0, SX = 0, SY = 0, SW = 0;
    for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
        const MovePartial p = a.part[b];
        SX += p.sx;
        SY += p.sy;
        SW += p.sw;
        lse_merge(M, S, S2, p.m, p.s, p.s2);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const double om = __shfl_xor_sync(0xFFFFFFFFu, M, d);
        const double os = __shfl_xor_sync(0xFFFFFFFFu, S, d);
        const double os2 = __shfl_xor_sync(0xFFFFFFFFu, S2, d);
        lse_merge(M, S, S2, om, os, os2);
        SX += __shfl_xor_sync(0xFFFFFFFFu, SX, d);
        SY += __shfl_xor_sync(0xFFFFFFFFu, SY, d);
        SW += __shfl_xor_sync(0xFFFFFFFFu, SW, d);
    }
    __syncthreads();
    if (lane == 0) {
        sh[0][wid] = SX;
        sh[1][wid] = SY;
        sh[2][wid] = SW;
        sh[3][wid] = M;
        sh[4][wid] = S;
        sh[5][wid] = S2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double M1 = -INFINITY, S1 = 0, S21 = 0, SX1 = 0, SY1 = 0, SW1 = 0;
        for (int w = 0; w < kPfBlock / 32; ++w) {
            SX1 += sh[0][w];
            SY1 += sh[1][w];
            SW1 += sh[2][w];
            lse_merge(M1, S1, S21, sh[3][w], sh[4][w], sh[5][w]);
        }
        PfScalars &sc = *a.sc;
        const double prev_mass = First ? static_cast<double>(n) : SW1;
        const bool rec = t < a.max_steps;
        if (!First && rec) {
            a.h_mean[2 * (t - 1) + 0] = SX1 / SW1;
            a.h_mean[2 * (t - 1) + 1] = SY1 / SW1;
        }
        const double ess = S1 * S1 / S21;
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
        sc.step = t + 1;
        sc.done = 0;
    }
}

// Weighted mean of the current particles (the last step's monitor).
__global__ void __launch_bounds__(kPfBlock) k_pf32_final_mean(
    const Pf32Args a, uint32_t t_rec)
{
    const int resampled = a.sc->resampled;
    const float M = static_cast<float>(a.sc->M);
    double sx = 0, sy = 0, sw = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += gridDim.x * blockDim.x) {
        const float w = resampled ? 1.0f : __expf(a.lw[i] - M);
        sx += w * a.x[i];
        sy += w * a.y[i];
        sw += w;
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

// block sum of q over the block's chunk
__global__ void __launch_bounds__(kPfBlock) k_rs32_qsum(const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    const float M = static_cast<float>(a.sc->M);
    uint32_t lo, hi;
    chunk_range(a.n, a.chunk, lo, hi);
    uint64_t acc = 0;
    for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x)
        acc += fixed_q(a.lw[i], M, a.shift);
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

struct StratA {
    const PfScalars *sc;
    __device__ uint64_t operator()(long long j) const
    {
        return engine_word(*sc, static_cast<uint64_t>(j));
    }
};

struct SystA {
    uint64_t a0;
    __device__ uint64_t operator()(long long) const { return a0; }
};

// Replication counts from the fixed-point CDF; per-block empty counts.
__global__ void __launch_bounds__(kPfBlock) k_rs32_count(const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    const float M = static_cast<float>(a.sc->M);
    uint32_t lo, hi;
    chunk_range(a.n, a.chunk, lo, hi);
    __shared__ uint64_t shq[kPfBlock / 32 + 1];
    __shared__ uint32_t she[kPfBlock / 32 + 1];
    uint64_t offset, Q;
    block_prefix_of_parts(a.qpart, blockIdx.x, gridDim.x, offset, Q, shq);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        a.sc->Q = Q;
    const CountP cp = make_count_params(Q, a.n);
    const uint64_t a0 = engine_word(*a.sc, 0);
    StratA strat{a.sc};
    SystA syst{a0};
    uint32_t err = 0;
    uint32_t empties = 0, copies = 0;
    for (uint32_t base = lo; base < hi; base += kPfTile) {
        const uint32_t i0 = base + threadIdx.x * 4;
        uint64_t q[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            q[k] = (i0 + k < hi) ? fixed_q(a.lw[i0 + k], M, a.shift) : 0;
        const uint64_t tsum = q[0] + q[1] + q[2] + q[3];
        uint64_t tile_total;
        const uint64_t incl =
            block_inclusive_scan(tsum, OpAdd(), uint64_t(0), shq, &tile_total);
        uint64_t C = offset + incl - tsum; // exclusive prefix of this thread
        uint32_t Fprev = a.scheme == VSMC_CUDA_STRATIFIED
            ? count_le(C, cp, strat, err)
            : count_le(C, cp, syst, err);
        if (i0 == 0)
            Fprev = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t i = i0 + k;
            if (i >= hi)
                break;
            C += q[k];
            uint32_t F;
            if (i + 1 == a.n)
                F = a.n; // the last particle takes the rest
            else
                F = a.scheme == VSMC_CUDA_STRATIFIED
                    ? count_le(C, cp, strat, err)
                    : count_le(C, cp, syst, err);
            const int32_t r = static_cast<int32_t>(F - Fprev);
            a.rep[i] = r;
            empties += r == 0 ? 1u : 0u;
            copies += static_cast<uint32_t>(r);
            Fprev = F;
        }
        offset += tile_total;
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

// Slot assignment: marks[surplus rank of p] = p + 1 for parents with two or
// more copies, empties[empty rank of d] = d.  With c = copies before slot i
// and e = empty slots before i, the first surplus rank of i is c - (i - e)
// (every non-empty slot before i keeps one of its copies).
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
    for (uint32_t base = lo; base < hi; base += kPfTile) {
        const uint32_t i0 = base + threadIdx.x * 4;
        int32_t r[4];
        uint32_t tr = 0, te = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            r[k] = (i0 + k < hi) ? a.rep[i0 + k] : -1;
            if (r[k] >= 0) {
                tr += static_cast<uint32_t>(r[k]);
                te += r[k] == 0 ? 1u : 0u;
            }
        }
        const uint64_t v = (static_cast<uint64_t>(tr) << 32) | te;
        uint64_t tot;
        const uint64_t incl =
            block_inclusive_scan(v, OpAdd(), uint64_t(0), sh64, &tot);
        const uint64_t ex = incl - v;
        uint32_t c = coff + static_cast<uint32_t>(ex >> 32);
        uint32_t e = eoff + static_cast<uint32_t>(ex & 0xFFFFFFFFu);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (r[k] < 0)
                break;
            const uint32_t i = i0 + k;
            if (r[k] == 0) {
                if (e < a.n)
                    a.empties[e] = i;
                else
                    atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
                ++e;
            } else if (r[k] >= 2) {
                const uint32_t rank = c - (i - e);
                if (rank < a.n)
                    a.marks[rank] = i + 1;
                else
                    atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
            }
            c += static_cast<uint32_t>(r[k]);
        }
        coff += static_cast<uint32_t>(tot >> 32);
        eoff += static_cast<uint32_t>(tot & 0xFFFFFFFFu);
    }
}

__device__ __forceinline__ void rank_range(
    uint32_t K, uint32_t &lo, uint32_t &hi)
{
    const uint32_t per = (K + gridDim.x - 1) / gridDim.x;
    lo = blockIdx.x * per;
    hi = lo + per;
    if (lo > K)
        lo = K;
    if (hi > K)
        hi = K;
}

// per-block max of the marks over the block's share of the K surplus ranks
__global__ void __launch_bounds__(kPfBlock) k_rs32_markmax(const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    uint32_t lo, hi;
    rank_range(min(a.sc->nempty, a.n), lo, hi);
    uint32_t mx = 0;
    for (uint32_t k = lo + threadIdx.x; k < hi; k += blockDim.x)
        mx = max(mx, a.marks[k]);
    __shared__ uint32_t sh[kPfBlock / 32 + 1];
    mx = block_reduce(mx, OpMax(), 0u, sh);
    if (threadIdx.x == 0)
        a.mpart[blockIdx.x] = mx;
}

// Running max of the marks gives the parent of each surplus rank; copy the
// parent into the empty slot of the same rank, and clear the marks.
__global__ void __launch_bounds__(kPfBlock) k_rs32_gather(const Rs32Args a)
{
    if (!a.sc->resampled)
        return;
    uint32_t lo, hi;
    rank_range(min(a.sc->nempty, a.n), lo, hi);
    __shared__ uint32_t sh[kPfBlock / 32 + 1];
    uint32_t carry = 0;
    for (uint32_t b = threadIdx.x; b < blockIdx.x; b += blockDim.x)
        carry = max(carry, a.mpart[b]);
    carry = block_reduce(carry, OpMax(), 0u, sh);
    for (uint32_t base = lo; base < hi; base += blockDim.x) {
        const uint32_t k = base + threadIdx.x;
        const uint32_t mk = k < hi ? a.marks[k] : 0u;
        uint32_t tot;
        uint32_t run = block_inclusive_scan(mk, OpMax(), 0u, sh, &tot);
        run = max(run, carry);
        carry = max(carry, tot);
        if (k < hi) {
            const uint32_t src = run - 1;
            const uint32_t dst = a.empties[k];
            if (run == 0 || src >= a.n || dst >= a.n) {
                atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
                continue;
            }
            a.x[dst] = a.x[src];
            a.y[dst] = a.y[src];
            a.vx[dst] = a.vx[src];
            a.vy[dst] = a.vy[src];
            if (mk)
                a.marks[k] = 0;
        }
    }
}

} // namespace vsmc_cuda
