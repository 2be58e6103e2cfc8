// Batched FP32 bootstrap filters.
//
// Thousands of independent filters, each with its own particle count,
// horizon, model constants and seed, advance together: per global step one
// persistent kernel moves, weights and reduces the particles of every filter
// still running, and three kernels resample the filters whose ESS fell below
// the threshold, in equal chunks listed by the step kernel.  A whole run
// (every step of the longest horizon) is one CUDA graph.
//
// Filter f behaves exactly as a single precision-32 filter (pf.cu) with seed
// seeds[f]: the same particle streams (Philox4x32 key {step, seed}, counter
// {0, particle, 0, 0}), the same FP32 move / likelihood / log-weight
// arithmetic, the same resampling engine (key {0, seed}, counter {0, 0, 1, 0})
// and the same exact fixed-point counting, so its particles, counts and
// resampling decisions match; only the order of the FP64 block sums differs.
//
// Layout.  Filters are stored by horizon, longest first, so the filters still
// running at step t are a prefix and so are their tiles (a tile is
// kBlock * kPPT consecutive particles of one filter).  Particle arrays are the
// filters' segments concatenated, each starting on a multiple of 4 elements.
// Resampling indices are local to the filter's segment.
//
// The step and tile shapes (threads per block, particles per thread) are
// chosen by vsmc_cuda_batch_autotune from timed runs of the actual batch.
//
// No reference counterpart: the reference would run one Sampler<T> per
// filter (core/sampler.hpp:107-114) with the pf example's move
// (example/pf/include/pf.hpp:154-170).
#include "bearings.cuh"
#include "cv_sim.cuh"
#include "mlp.cuh"
#include "pf32_dev.cuh"
#include "pf_model.cuh"

#include <algorithm>
#include <type_traits>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

using namespace vsmc_cuda;

namespace vsmc_cuda
{

// Static description of one filter (internal order).
struct BFilter {
    uint32_t n;        // particles
    uint32_t off;      // first particle in the concatenated arrays
    uint32_t tile0;    // first tile of the step kernel
    uint32_t ntiles;   // tiles of the step kernel
    uint32_t T;        // horizon: steps 0..T-1, step T records the last mean
    uint32_t obs_off;  // first observation pair (caller's filter order)
    uint32_t hist_off; // first history entry (caller's filter order)
    uint32_t seed;
    uint32_t shift;    // fixed-point K = 63 - ceil(log2 n)
    uint32_t rs_chunk; // resampling chunk: a multiple of 4096 particles
    union {
        CvConst<float> c;   // position / Student-t model
        BearingsConst bc;   // bearings-only model
    };
};

// A block's record of the tiles of one filter: FP32 sums, as the block
// forms them (the single filter widens the same values to FP64).
struct TileRecord {
    float sx, sy, sw; // previous-step monitor sums
    float m, s, s2;   // new log-weights: max, sum exp, sum exp^2
};

// filter kinds
constexpr int kKindCv = 0;       // CV + Student-t positions, bootstrap
constexpr int kKindBearings = 1; // bearings-only, bootstrap
constexpr int kKindLearned = 2;  // bearings-only, learned proposal

struct BatchArgs {
    const BFilter *flt;
    PfScalars *st;               // dynamic state, one per filter
    const uint32_t *tile_filter; // filter of each tile
    const uint32_t *active;      // [tmax + 1] tiles of the filters with T >= t
    const float *ax, *ay, *avx, *avy; // state in
    float *bx, *by, *bvx, *bvy;       // state out
    float *lw;
    int32_t *rep, *idx;
    uint32_t *srcs;
    TileRecord *part; // per tile
    const float *obs; // the observations in FP32 (converted once per run)
    const float2 *obs_sc; // bearings kinds: (sin z, cos z) of each bearing
    double *h_mean, *h_ess, *h_logz;
    int *h_res;
    uint32_t *step; // global step counter
    // resampling list of the step: rs_list[rpar * rs_cap + v] = {filter,
    // chunk}, rs_count[rpar] entries; per-entry totals of the passes
    uint2 *rs_list;
    uint32_t *rs_count;
    uint32_t *work; // step kernel's tile counters, by step parity
    uint64_t *rs_q;
    uint32_t *rs_e, *rs_c;
    uint32_t rs_cap, rpar;
    const uint32_t *packed; // proposal network (learned kind)
    uint32_t nfilters, tmax;
    int scheme;
    double threshold;
};

// The FP32 per-particle body of the single filter (step_one in pf32.cuh),
// with the filter's constants and seed.
template <bool First>
__device__ __forceinline__ void batch_one(const CvConst<float> &c,
    uint32_t seed, uint32_t i, uint32_t t, float ox, float oy, int resampled,
    float Mprev, float &x, float &y, float &vx, float &vy, float &lw, float &m,
    float &s, float &s2, float &sx, float &sy, float &sw)
{
    const u32x4 w = particle_block(t, seed, i);
    float lw_old = 0.0f;
    if (First) {
        float z1, z2, z3, z4;
        normal_pair_f(w.x, w.y, z1, z2);
        normal_pair_f(w.z, w.w, z3, z4);
        x = c.sd_pos0 * z1;
        y = c.sd_pos0 * z2;
        vx = c.sd_vel0 * z3;
        vy = c.sd_vel0 * z4;
    } else {
        lw_old = resampled ? 0.0f : lw - Mprev;
        const float wo = resampled ? 1.0f : __expf(lw_old);
        sx += wo * x;
        sy += wo * y;
        sw += wo;
        float z1, z2;
        normal_pair_f(w.x, w.y, z1, z2);
        cv_move(c, c.sigma_a * z1, c.sigma_a * z2, x, y, vx, vy);
    }
    lw = lw_old + cv_loglik(c, ox, oy, x, y);
    lse_push(lw, m, s, s2);
}

template <int kPPT>
__device__ __forceinline__ void load_run(const float *p, float (&v)[kPPT])
{
    if constexpr (kPPT == 4) {
        const float4 q = __ldcs(reinterpret_cast<const float4 *>(p));
        v[0] = q.x;
        v[1] = q.y;
        v[2] = q.z;
        v[3] = q.w;
    } else if constexpr (kPPT == 2) {
        const float2 q = __ldcs(reinterpret_cast<const float2 *>(p));
        v[0] = q.x;
        v[1] = q.y;
    } else {
        v[0] = __ldcs(p);
    }
}

template <int kPPT>
__device__ __forceinline__ void store_run(float *p, const float (&v)[kPPT])
{
    if constexpr (kPPT == 4) {
        __stcs(reinterpret_cast<float4 *>(p),
            make_float4(v[0], v[1], v[2], v[3]));
    } else if constexpr (kPPT == 2) {
        __stcs(reinterpret_cast<float2 *>(p), make_float2(v[0], v[1]));
    } else {
        __stcs(p, v[0]);
    }
}

// The record of `count` consecutive tiles of one filter done by this block
// (FP32 within a warp, FP64 across warps), written at the first of them
// (the others get empty records) and, in the block that completes the
// filter's last tile, the filter's FP64 combination: ESS, log-evidence
// increment, resampling decision and histories (or, at t == T, the last
// weighted mean).  All threads of the block call it.
template <int kBlock, bool First>
__device__ __forceinline__ void tile_finish(const BatchArgs &a, uint32_t tile,
    uint32_t count, uint32_t f, const BFilter &F, PfScalars &S, uint32_t t,
    bool mon, float m, float s, float s2, float sx, float sy, float sw,
    float *shm, float (*shw)[kBlock / 32], bool &is_last)
{
    constexpr int kW = kBlock / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
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
    if (lane == 0) {
        shm[wid] = m;
        shw[0][wid] = s;
        shw[1][wid] = s2;
        shw[2][wid] = sx;
        shw[3][wid] = sy;
        shw[4][wid] = sw;
    }
    __syncthreads();
    if (wid == 0) {
        // warp 0 merges the warps' records in FP32
        const bool in = lane < kW;
        float wm = in ? shm[lane] : -INFINITY;
        float ws = in ? shw[0][lane] : 0.0f, ws2 = in ? shw[1][lane] : 0.0f;
        float wx = in ? shw[2][lane] : 0.0f, wy = in ? shw[3][lane] : 0.0f;
        float ww = in ? shw[4][lane] : 0.0f;
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
            const TileRecord p = {wx, wy, ww, wm, ws, ws2};
            a.part[tile] = p;
            const TileRecord empty = {0, 0, 0, -INFINITY, 0, 0};
            for (uint32_t k = 1; k < count; ++k)
                a.part[tile + k] = empty;
            __threadfence();
            is_last = atomicAdd(&S.done, count) == F.ntiles - count;
        }
    }
    __syncthreads();
    if (!is_last)
        return;
    // ---- the filter's last tile: warp 0 combines its tile records in FP64
    __threadfence();
    if (wid != 0)
        return;
    float M = -INFINITY;
    for (uint32_t b = lane; b < F.ntiles; b += 32)
        M = fmaxf(M, __ldcg(&a.part[F.tile0 + b].m));
    M = warp_reduce(M, OpMax());
    double T1 = 0, T2 = 0, TX = 0, TY = 0, TW = 0;
    for (uint32_t b = lane; b < F.ntiles; b += 32) {
        const TileRecord p = a.part[F.tile0 + b];
        TX += p.sx;
        TY += p.sy;
        TW += p.sw;
        if (p.m > -INFINITY) {
            const double fct = __expf(p.m - M);
            T1 += p.s * fct;
            T2 += p.s2 * fct * fct;
        }
    }
    T1 = warp_reduce(T1, OpAdd());
    T2 = warp_reduce(T2, OpAdd());
    TX = warp_reduce(TX, OpAdd());
    TY = warp_reduce(TY, OpAdd());
    TW = warp_reduce(TW, OpAdd());
    uint32_t rs_first = ~0u; // first list entry of the filter's chunks
    if (lane == 0) {
        if (mon) {
            a.h_mean[2 * (F.hist_off + F.T - 1) + 0] = TX / TW;
            a.h_mean[2 * (F.hist_off + F.T - 1) + 1] = TY / TW;
            S.resampled = 0; // finished: nothing left to resample
            S.gather = 0;
        } else {
            // the previous weights' mass: their own normalizer (the
            // single filter's step kernel uses the same one)
            const double prev_mass =
                First || S.resampled ? static_cast<double>(F.n) : S.S;
            if (!First) {
                a.h_mean[2 * (F.hist_off + t - 1) + 0] = TX / TW;
                a.h_mean[2 * (F.hist_off + t - 1) + 1] = TY / TW;
            }
            const double ess = T1 * T1 / T2;
            const double M1 = static_cast<double>(M);
            S.logz += M1 + log(T1) - log(prev_mass);
            if (!(T1 > 0) || !(ess > 0))
                S.err |= DEV_ERR_NONFINITE;
            const int flag =
                ess < a.threshold * static_cast<double>(F.n) ? 1 : 0;
            a.h_ess[F.hist_off + t] = ess;
            a.h_logz[F.hist_off + t] = S.logz;
            a.h_res[F.hist_off + t] = flag;
            S.M = M1;
            S.Mf = M;
            S.S = T1;
            S.ess = ess;
            S.resampled = flag;
            S.gather = 0;
            S.step = t + 1;
            if (flag) {
                const uint32_t nc = (F.n + F.rs_chunk - 1) / F.rs_chunk;
                const uint32_t v = atomicAdd(a.rs_count + a.rpar, nc);
                if (v + nc <= a.rs_cap)
                    rs_first = v;
                else
                    S.err |= DEV_ERR_INTERNAL;
            }
        }
        S.done = 0;
    }
    rs_first = __shfl_sync(0xFFFFFFFFu, rs_first, 0);
    if (rs_first != ~0u) {
        // list the filter's resampling chunks
        uint2 *list = a.rs_list + static_cast<size_t>(a.rpar) * a.rs_cap;
        const uint32_t nc = (F.n + F.rs_chunk - 1) / F.rs_chunk;
        for (uint32_t j = lane; j < nc; j += 32)
            list[rs_first + j] = make_uint2(f, j);
    }
}

// slot i's source inside the filter after a resample (bounds-checked)
__device__ __forceinline__ uint32_t batch_source(
    const BatchArgs &a, const BFilter &F, PfScalars &S, uint32_t i)
{
    const int32_t v = a.idx[F.off + i];
    const uint32_t e = static_cast<uint32_t>(-(v + 1));
    uint32_t src = v >= 0 ? static_cast<uint32_t>(v)
                          : (e < F.n ? __ldcg(a.srcs + F.off + e) : F.n);
    if (src >= F.n) {
        atomicOr(&S.err, DEV_ERR_INTERNAL);
        src = 0;
    }
    return src;
}

// bootstrap body of the bearings-only model (prior at t == 0)
template <bool First>
__device__ __forceinline__ void bearings_one(const BearingsConst &c,
    uint32_t seed, uint32_t i, uint32_t t, float z, int resampled,
    float Mprev, float &x, float &y, float &vx, float &vy, float &lw, float &m,
    float &s, float &s2, float &sx, float &sy, float &sw)
{
    float e[4];
    bearings_normals(t, seed, i, e);
    float lw_old = 0.0f;
    if (First) {
        bearings_prior(c, e, x, y, vx, vy);
    } else {
        lw_old = resampled ? 0.0f : lw - Mprev;
        const float wo = resampled ? 1.0f : __expf(lw_old);
        sx += wo * x;
        sy += wo * y;
        sw += wo;
        bearings_step(c, e, x, y, vx, vy);
    }
    lw = lw_old + bearings_loglik(c, z, x, y);
    lse_push(lw, m, s, s2);
}

// One global step of every running filter (bootstrap kinds).  A filter at
// t < T moves and weights its particles; at t == T it only records the
// weighted mean of its final particles.  Each block takes a contiguous run
// of tiles and records one reduction per filter it touches.
template <int kBlock, int kPPT, bool First, int Kind>
__global__ void __launch_bounds__(kBlock, 1280 / kBlock) k_batch_step(
    const BatchArgs a)
{
    constexpr uint32_t kTile = kBlock * kPPT;
    constexpr int kW = kBlock / 32;
    // tiles a block takes at a time: one tile at the default 4 x 256 shape
    // (1024 particles, whose per-tile FP32 records then group the particles
    // as the single filter's blocks do), 2048 particles for smaller tiles
    // (fewer segment records; 1024 took 231 ms per 4096-filter run, 2048
    // 225 ms, 4096 227 ms)
    constexpr uint32_t kGrab = kTile >= 1024 ? 1u : 2048u / kTile;
    const uint32_t t = *a.step;
    const uint32_t ntiles = t <= a.tmax ? a.active[t] : 0u;
    __shared__ float shm[kW];
    __shared__ float shw[5][kW];
    __shared__ bool is_last;
    __shared__ uint32_t grab;
    // the next step's counter was last used by the previous step's launch
    if (blockIdx.x == 0 && threadIdx.x == 0)
        a.work[(t + 1) & 1u] = 0;
    // Blocks take runs of kGrab tiles from a counter until none is left, so
    // a block whose tiles are slower (gathered reads after a resample, many
    // small filters) takes fewer of them.
    for (;;) {
    if (threadIdx.x == 0)
        grab = atomicAdd(a.work + (t & 1u), kGrab);
    __syncthreads();
    const uint32_t lo = grab;
    __syncthreads();
    if (lo >= ntiles)
        break;
    const uint32_t hi = min(ntiles, lo + kGrab);
    // the run is cut into segments of one filter each; a segment reads its
    // filter's description and state once, then streams its tiles
    uint32_t tile = lo;
    while (tile < hi) {
        const uint32_t f = a.tile_filter[tile];
        const BFilter F = a.flt[f];
        PfScalars &S = a.st[f];
        const bool mon = !First && t == F.T;
        const int resampled = First ? 1 : S.resampled;
        const bool gather = First ? false : (S.gather != 0);
        const float Mprev = First ? 0.0f : S.Mf;
        float ox = 0.0f, oy = 0.0f;
        if (!mon) {
            if (Kind == kKindCv) {
                ox = a.obs[2 * (F.obs_off + t) + 0];
                oy = a.obs[2 * (F.obs_off + t) + 1];
            } else {
                ox = a.obs[F.obs_off + t];
            }
        }
        const uint32_t seg = tile;
        uint32_t end = min(hi, F.tile0 + F.ntiles);
        if (end <= tile) { // a tile table that disagrees with the filters
            if (threadIdx.x == 0)
                atomicOr(&S.err, DEV_ERR_INTERNAL);
            end = tile + 1;
        }
        float m = -INFINITY, s = 0, s2 = 0, sx = 0, sy = 0, sw = 0;
        for (; tile < end; ++tile) {
            const uint32_t i0 = (tile - F.tile0) * kTile + threadIdx.x * kPPT;
            const bool full = i0 + kPPT <= F.n;
            float X[kPPT], Y[kPPT], VX[kPPT], VY[kPPT], LW[kPPT];
#pragma unroll
            for (int k = 0; k < kPPT; ++k)
                X[k] = Y[k] = VX[k] = VY[k] = LW[k] = 0.0f;
            if (!First) {
                const uint32_t g0 = F.off + i0;
                // after a resample, a group whose slots all keep their own
                // particle reads like an unresampled one
                bool own = !gather;
                if (gather && full && kPPT == 4) {
                    const int4 I = __ldcs(reinterpret_cast<const int4 *>(a.idx + g0));
                    const int b = static_cast<int>(i0);
                    own = I.x == b && I.y == b + 1 && I.z == b + 2 && I.w == b + 3;
                }
                if (own && full) {
                    load_run<kPPT>(a.ax + g0, X);
                    load_run<kPPT>(a.ay + g0, Y);
                    load_run<kPPT>(a.avx + g0, VX);
                    load_run<kPPT>(a.avy + g0, VY);
                } else {
#pragma unroll
                    for (int k = 0; k < kPPT; ++k) {
                        const uint32_t i = i0 + k;
                        if (i < F.n) {
                            const uint32_t src =
                                gather ? batch_source(a, F, S, i) : i;
                            X[k] = a.ax[F.off + src];
                            Y[k] = a.ay[F.off + src];
                            VX[k] = a.avx[F.off + src];
                            VY[k] = a.avy[F.off + src];
                        }
                    }
                }
                if (!resampled) {
                    if (full) {
                        load_run<kPPT>(a.lw + g0, LW);
                    } else {
#pragma unroll
                        for (int k = 0; k < kPPT; ++k)
                            if (i0 + k < F.n)
                                LW[k] = a.lw[g0 + k];
                    }
                }
            }
            if (mon) {
#pragma unroll
                for (int k = 0; k < kPPT; ++k)
                    if (i0 + k < F.n) {
                        const float wo = resampled ? 1.0f : __expf(LW[k] - Mprev);
                        sx += wo * X[k];
                        sy += wo * Y[k];
                        sw += wo;
                    }
            } else {
#pragma unroll
                for (int k = 0; k < kPPT; ++k)
                    if (i0 + k < F.n) {
                        if (Kind == kKindCv)
                            batch_one<First>(F.c, F.seed, i0 + k, t, ox, oy,
                                resampled, Mprev, X[k], Y[k], VX[k], VY[k], LW[k],
                                m, s, s2, sx, sy, sw);
                        else
                            bearings_one<First>(F.bc, F.seed, i0 + k, t, ox,
                                resampled, Mprev, X[k], Y[k], VX[k], VY[k], LW[k],
                                m, s, s2, sx, sy, sw);
                    }
                const uint32_t g0 = F.off + i0;
                if (full) {
                    store_run<kPPT>(a.bx + g0, X);
                    store_run<kPPT>(a.by + g0, Y);
                    store_run<kPPT>(a.bvx + g0, VX);
                    store_run<kPPT>(a.bvy + g0, VY);
                    store_run<kPPT>(a.lw + g0, LW);
                } else {
#pragma unroll
                    for (int k = 0; k < kPPT; ++k)
                        if (i0 + k < F.n) {
                            a.bx[g0 + k] = X[k];
                            a.by[g0 + k] = Y[k];
                            a.bvx[g0 + k] = VX[k];
                            a.bvy[g0 + k] = VY[k];
                            a.lw[g0 + k] = LW[k];
                        }
                }
            }
        }
        // the filter's segment ends here: record it
        tile_finish<kBlock, First>(a, seg, end - seg, f, F, S, t, mon, m, s,
            s2, sx, sy, sw, shm, shw, is_last);
        __syncthreads();
    }
    }
}

constexpr int kLearnBlock = 128;                // 4 warps
constexpr uint32_t kLearnTile = kLearnBlock;     // 32 particles a warp

// One global step of the learned-proposal filters.  Each warp evaluates the
// proposal network for 32 particles on the tensor cores (two 16-row tiles
// sharing the weight loads); lane 4g + q then moves particle g + 8q of the
// warp's 32.
template <bool First>
__global__ void __launch_bounds__(kLearnBlock) k_batch_step_learned(
    const BatchArgs a)
{
    constexpr int kW = kLearnBlock / 32;
    __shared__ __align__(16) uint32_t sp[kPackedWords];
    __shared__ float shm[kW];
    __shared__ float shw[5][kW];
    __shared__ bool is_last;
    const uint32_t t = *a.step;
    const uint32_t ntiles = t <= a.tmax ? a.active[t] : 0u;
    if (!First)
        load_packed(sp, a.packed);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int g = lane >> 2, q = lane & 3;
    // tiles a block takes at a time (1024 particles), from a per-step
    // counter; the next step's counter was last used by the previous step
    constexpr uint32_t kGrab = 1024u / kLearnTile;
    __shared__ uint32_t grab;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        a.work[(t + 1) & 1u] = 0;
    for (;;) {
    if (threadIdx.x == 0)
        grab = atomicAdd(a.work + (t & 1u), kGrab);
    __syncthreads();
    const uint32_t lo = grab;
    __syncthreads();
    if (lo >= ntiles)
        break;
    const uint32_t hi = min(ntiles, lo + kGrab);
    // one segment per filter: its description and state are read once
    uint32_t tile = lo;
    while (tile < hi) {
        const uint32_t f = a.tile_filter[tile];
        const BFilter F = a.flt[f];
        const BearingsConst &c = F.bc;
        PfScalars &S = a.st[f];
        const bool mon = !First && t == F.T;
        const int resampled = First ? 1 : S.resampled;
        const bool gather = First ? false : (S.gather != 0);
        const float Mprev = First ? 0.0f : S.Mf;
        const float z = mon ? 0.0f : a.obs[F.obs_off + t];
        const uint32_t seg = tile;
        uint32_t end = min(hi, F.tile0 + F.ntiles);
        if (end <= tile) { // a tile table that disagrees with the filters
            if (threadIdx.x == 0)
                atomicOr(&S.err, DEV_ERR_INTERNAL);
            end = tile + 1;
        }
        float m = -INFINITY, s = 0, s2 = 0, sx = 0, sy = 0, sw = 0;
        for (; tile < end; ++tile) {
            const uint32_t i =
                (tile - F.tile0) * kLearnTile + 32 * wid + g + 8 * q;
            const bool mine = i < F.n;
            float x = 0, y = 0, vx = 0, vy = 0, lw = 0;
            if (!First && mine) {
                const uint32_t src = gather ? batch_source(a, F, S, i) : i;
                x = a.ax[F.off + src];
                y = a.ay[F.off + src];
                vx = a.avx[F.off + src];
                vy = a.avy[F.off + src];
                lw = resampled ? 0.0f : a.lw[F.off + i];
            }
            if (mon) {
                if (mine) {
                    const float wo = resampled ? 1.0f : __expf(lw - Mprev);
                    sx += wo * x;
                    sy += wo * y;
                    sw += wo;
                }
            } else if (First) {
                if (mine) {
                    float e[4];
                    bearings_normals(t, F.seed, i, e);
                    bearings_prior(c, e, x, y, vx, vy);
                    lw = bearings_loglik(c, z, x, y);
                    lse_push(lw, m, s, s2);
                }
            } else {
                const float2 scz = a.obs_sc[F.obs_off + t];
                const float sz = scz.x, cz = scz.y;
                float fe[6];
                bearings_features(c, x, y, vx, vy, sz, cz, fe);
                uint32_t a0[4], b0[4];
                features_to_a2(fe, a0, b0);
                // one 16-row tile at a time keeps one tile's activations live
                float oa[4], ob[4];
#pragma unroll 1
                for (int h = 0; h < 2; ++h) {
                    uint32_t in[4];
#pragma unroll
                    for (int r = 0; r < 4; ++r)
                        in[r] = h ? b0[r] : a0[r];
                    float o[4];
                    mlp_forward_warp<false, true>(sp, in, o);
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        if (h)
                            ob[r] = o[r];
                        else
                            oa[r] = o[r];
                    }
                }
                float v[8];
                out_to_owner2(oa, ob, v);
                if (mine) {
                    const float lw_old = resampled ? 0.0f : lw - Mprev;
                    const float wo = resampled ? 1.0f : __expf(lw_old);
                    sx += wo * x;
                    sy += wo * y;
                    sw += wo;
                    float e[4], fr[4], nu[4];
                    bearings_normals(t, F.seed, i, e);
                    float lq = 0;
#pragma unroll
                    for (int d = 0; d < 4; ++d) {
                        const float l = fminf(fmaxf(v[4 + d], c.lmin), c.lmax);
                        fr[d] = v[d] + __expf(0.5f * l) * e[d];
                        lq += 0.5f * (e[d] * e[d] - fr[d] * fr[d]) + 0.5f * l;
                    }
                    frame_to_axes(sz, cz, fr, nu); // the draw, bearing frame
                    bearings_step(c, nu, x, y, vx, vy);
                    lw = lw_old + bearings_loglik(c, z, x, y) + lq;
                    lse_push(lw, m, s, s2);
                }
            }
            if (!mon && mine) {
                const uint32_t gi = F.off + i;
                a.bx[gi] = x;
                a.by[gi] = y;
                a.bvx[gi] = vx;
                a.bvy[gi] = vy;
                a.lw[gi] = lw;
            }
        }
        tile_finish<kLearnBlock, First>(a, seg, end - seg, f, F, S, t, mon, m,
            s, s2, sx, sy, sw, shm, shw, is_last);
        __syncthreads();
    }
    }
}

// ---------------------------------------------------------------- resampling
//
// The filters that resample at a step are resampled together by three
// kernels over the step's list of equal chunks: entry v of the list is chunk
// k of filter f (its particles [k c, (k + 1) c) with c = F.rs_chunk), and
// the chunks of a filter are consecutive entries, listed by the block that
// finished the filter's step (tile_finish).  The three passes are the single
// filter's k_rs32_qsum / count / assign: a fixed-point total per chunk,
// replication counts, and slot assignment with the sources of the empty
// slots.  A chunk
// takes its offsets from the per-chunk totals of the earlier chunks of its
// filter (at most kMaxRsChunks, summed by every warp on its own).  Blocks
// walk the list with a grid stride: the grids are fixed when a run is
// captured, and filters that do not resample cost nothing.

// one list entry, with its filter's sizes
struct RsChunk {
    uint32_t f, k;    // filter, chunk of the filter
    uint32_t base;    // list entry of the filter's chunk 0
    uint32_t nc;      // chunks of the filter
    uint32_t n, off, shift;
    uint32_t lo, hi;  // particles (or surplus ranks) of the chunk
};

__device__ __forceinline__ RsChunk rs_chunk_at(const BatchArgs &a, uint32_t v)
{
    const uint2 e =
        __ldcg(a.rs_list + static_cast<size_t>(a.rpar) * a.rs_cap + v);
    const BFilter &F = a.flt[e.x];
    RsChunk c;
    c.f = e.x;
    c.k = e.y;
    c.base = v - e.y;
    c.n = F.n;
    c.off = F.off;
    c.shift = F.shift;
    const uint32_t csz = F.rs_chunk;
    c.nc = (c.n + csz - 1) / csz;
    c.lo = min(c.n, c.k * csz);
    c.hi = min(c.n, c.lo + csz);
    return c;
}

// op over the per-chunk totals of the filter: of chunks j < k (before) and
// of all its chunks (all); every lane of the calling warp gets both
template <typename T, typename Op>
__device__ __forceinline__ void chunk_totals(
    const T *part, const RsChunk &c, Op op, T identity, T &before, T &all)
{
    const uint32_t lane = threadIdx.x & 31;
    const T v = lane < c.nc ? __ldcg(part + c.base + lane) : identity;
    before = warp_reduce(lane < c.k ? v : identity, op);
    all = warp_reduce(v, op);
}

// pass 1: fixed-point total of each chunk (four tiles in flight per thread).
// Block 0 also advances the step counter (every step kernel block has read
// it) and empties the next step's list.
__global__ void __launch_bounds__(kPfBlock) k_brs_qsum(const BatchArgs a)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(a.step, 1u);
        a.rs_count[a.rpar ^ 1u] = 0;
    }
    const uint32_t count = __ldcg(a.rs_count + a.rpar);
    __shared__ uint64_t sh[kPfBlock / 32 + 1];
    constexpr int kG = 4;
    for (uint32_t v = blockIdx.x; v < count; v += gridDim.x) {
        const RsChunk c = rs_chunk_at(a, v);
        const float M = a.st[c.f].Mf;
        const float *lw = a.lw + c.off;
        uint64_t acc = 0;
        for (uint32_t base = c.lo; base < c.hi; base += kG * kPfTile) {
            if (base + kG * kPfTile <= c.hi) {
                float4 x[kG];
#pragma unroll
                for (int h = 0; h < kG; ++h)
                    x[h] = __ldcg(reinterpret_cast<const float4 *>(
                        lw + base + h * kPfTile + threadIdx.x * 4));
#pragma unroll
                for (int h = 0; h < kG; ++h)
                    acc += fixed_q(x[h].x, M, c.shift) +
                        fixed_q(x[h].y, M, c.shift) +
                        fixed_q(x[h].z, M, c.shift) +
                        fixed_q(x[h].w, M, c.shift);
            } else {
                for (int h = 0; h < kG; ++h) {
                    const uint32_t i0 = base + h * kPfTile + threadIdx.x * 4;
                    for (uint32_t i = i0; i < c.hi && i < i0 + 4; ++i)
                        acc += fixed_q(lw[i], M, c.shift);
                }
            }
        }
        acc = block_reduce(acc, OpAdd(), uint64_t(0), sh);
        // the filter's last chunk to finish (a thread-fenced ticket on
        // done3; nothing waits) sets the filter's counting constants
        if (threadIdx.x == 0) {
            a.rs_q[v] = acc;
            __threadfence();
            PfScalars &S = a.st[c.f];
            if (atomicAdd(&S.done3, 1u) == c.nc - 1) {
                S.done3 = 0;
                __threadfence();
                uint64_t Q = 0;
                for (uint32_t k = 0; k < c.nc; ++k)
                    Q += __ldcg(a.rs_q + c.base + k);
                uint32_t err = 0;
                cdf_constants(S, Q, c.n, a.scheme == VSMC_CUDA_SYSTEMATIC, err);
                if (err & ~DEV_ERR_NONFINITE) // a zero total: pass 2 says so
                    atomicOr(&S.err, err & ~DEV_ERR_NONFINITE);
            }
        }
        __syncthreads(); // thread 0 done before the next chunk
    }
}

// pass 2: replication counts from the fixed-point CDF; empty and copy
// counts per chunk.  Each particle's CDF value is its exact 64-bit prefix
// sum (the chunk's offset, a block scan per tile) and F(C) comes from the
// filter's fixed-point reciprocal (cdf_floor), set by the filter's last
// chunk in pass 1.  A thread's first count needs F just before its first
// particle: lanes 1..31 take it from the lane before, lane 0 evaluates it.
// Stratified words come from the tile's block of engine words in shared
// memory.
template <bool Sys>
__global__ void __launch_bounds__(kPfBlock, 3) k_brs_count(const BatchArgs a)
{
    const uint32_t count = __ldcg(a.rs_count + a.rpar);
    constexpr bool sys = Sys; // the scheme (a.scheme) picked the instance
    __shared__ uint64_t shs[kPfBlock / 32 + 1];
    __shared__ uint32_t she[kPfBlock / 32 + 1];
    __shared__ uint4 wbuf[2 * kPfBlock];        // stratified words of a tile
    __shared__ uint32_t wsh[2 * (kPfBlock / 32)];
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t v = blockIdx.x; v < count; v += gridDim.x) {
        const RsChunk c = rs_chunk_at(a, v);
        PfScalars &S = a.st[c.f];
        uint64_t offset, Q;
        chunk_totals(a.rs_q, c, OpAdd(), uint64_t(0), offset, Q);
        if (Q == 0) { // the same for the whole block
            if (c.k == 0 && threadIdx.x == 0)
                atomicOr(&S.err, DEV_ERR_NONFINITE);
            continue;
        }
        // the engine before this resample (pass 3 advances it)
        const PfScalars &sc = S;
        const float M = sc.Mf;
        const uint32_t n = c.n;
        const float *lw = a.lw + c.off;
        int32_t *rep = a.rep + c.off;
        const CdfRcp p = load_cdf_rcp(sc, n);
        uint32_t empties = 0, copies = 0;
        // one reciprocal case per chunk (Usual: p.s > 0), chosen once
        auto run = [&](auto usual) {
            constexpr bool Usual = decltype(usual)::value;
            uint64_t carry = offset;
            // the next tile's log-weights are loaded while this one is counted
            float4 nxt = make_float4(0, 0, 0, 0);
            if (c.lo + threadIdx.x * 4 + 3 < c.hi)
                nxt = __ldcg(reinterpret_cast<const float4 *>(
                    lw + c.lo + threadIdx.x * 4));
            for (uint32_t base = c.lo; base < c.hi; base += kPfTile) {
                const uint32_t i0 = base + threadIdx.x * 4;
                const float4 x = nxt;
                if (i0 + kPfTile + 3 < c.hi)
                    nxt = __ldcg(
                        reinterpret_cast<const float4 *>(lw + i0 + kPfTile));
                uint64_t q[4];
                if (i0 + 3 < c.hi) {
                    q[0] = fixed_q(x.x, M, c.shift);
                    q[1] = fixed_q(x.y, M, c.shift);
                    q[2] = fixed_q(x.z, M, c.shift);
                    q[3] = fixed_q(x.w, M, c.shift);
                } else {
    #pragma unroll
                    for (int k = 0; k < 4; ++k)
                        q[k] = i0 + k < c.hi ? fixed_q(lw[i0 + k], M, c.shift) : 0;
                }
                uint64_t s[4];
                s[0] = q[0];
                s[1] = s[0] + q[1];
                s[2] = s[1] + q[2];
                s[3] = s[2] + q[3];
                uint64_t tile_total;
                const uint64_t incl =
                    block_inclusive_scan(s[3], OpAdd(), uint64_t(0), shs, &tile_total);
                const uint64_t cb = carry + (incl - s[3]);
                uint32_t Fv[4], Fl = 0;
                if (sys) {
    #pragma unroll
                    for (int k = 0; k < 4; ++k)
                        Fv[k] = i0 + k + 1 >= n ? n : sys_F<Usual>(cb + s[k], p);
                    if (lane == 0 && i0 != 0)
                        Fl = sys_F<Usual>(cb, p);
                } else {
                    uint32_t j[4];
                    uint64_t r[4];
    #pragma unroll
                    for (int k = 0; k < 4; ++k)
                        j[k] = strat_j<Usual>(cb + s[k], p, r[k]);
                    uint32_t jv = 0;
    #pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (j[k] < n)
                            jv = j[k];
                    const uint32_t wlo = j[0] < n ? sc.rindex + j[0] : 0xFFFFFFFFu;
                    const uint32_t whi = j[0] < n ? sc.rindex + jv : 0u;
                    const WordBuf wv =
                        fill_words<kPfBlock>(sc, wlo, whi, wbuf, 2 * kPfBlock, wsh);
    #pragma unroll
                    for (int k = 0; k < 4; ++k)
                        Fv[k] = i0 + k + 1 >= n ? n
                            : (j[k] >= n ? n
                                         : j[k] + (ceil_aq(buf_word(sc,
                                                       sc.rindex + j[k], wv), Q) <=
                                                           r[k]
                                                       ? 1u
                                                       : 0u));
                    if (lane == 0 && i0 != 0) {
                        uint64_t r0;
                        const uint32_t j0 = strat_j<Usual>(cb, p, r0);
                        Fl = j0 >= n ? n
                            : j0 + (ceil_aq(buf_word(sc, sc.rindex + j0, wv), Q) <=
                                           r0
                                       ? 1u
                                       : 0u);
                    }
                }
                // F before this thread's first particle (particle 0 has
                // nothing before it)
                const uint32_t Fup = __shfl_up_sync(0xFFFFFFFFu, Fv[3], 1);
                uint32_t Fprev = lane == 0 ? Fl : Fup;
                int32_t r[4];
    #pragma unroll
                for (int k = 0; k < 4; ++k) {
                    r[k] = static_cast<int32_t>(Fv[k] - Fprev);
                    Fprev = Fv[k];
                }
                if (i0 + 3 < c.hi) {
                    *reinterpret_cast<int4 *>(rep + i0) =
                        make_int4(r[0], r[1], r[2], r[3]);
    #pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        empties += r[k] == 0 ? 1u : 0u;
                        copies += static_cast<uint32_t>(r[k]);
                    }
                } else {
    #pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (i0 + k < c.hi) {
                            rep[i0 + k] = r[k];
                            empties += r[k] == 0 ? 1u : 0u;
                            copies += static_cast<uint32_t>(r[k]);
                        }
                }
                carry += tile_total;
            }
        };
        if (p.s != 0)
            run(std::true_type{});
        else
            run(std::false_type{});
        empties = block_reduce(empties, OpAdd(), 0u, she);
        copies = block_reduce(copies, OpAdd(), 0u, she);
        if (threadIdx.x == 0) {
            a.rs_e[v] = empties;
            a.rs_c[v] = copies;
        }
    }
}


// pass 3: slot assignment.  With c copies and e empty slots before slot i,
// the first surplus rank of i is c - (i - e); idx[i] = i for a parent,
// -(e + 1) for the e-th empty slot, and the sources of the surplus ranks of
// a parent with two or more copies are written by its warp
// (write_surplus_runs).  Chunk 0 records the filter's resample: Q, the
// empty count, the gather flag and the engine words the scheme consumed.
__global__ void __launch_bounds__(kPfBlock) k_brs_assign(const BatchArgs a)
{
    const uint32_t count = __ldcg(a.rs_count + a.rpar);
    const bool sys = a.scheme == VSMC_CUDA_SYSTEMATIC;
    __shared__ uint64_t sh64[kPfBlock / 32 + 1];
    __shared__ __align__(16) uint32_t shm[kPfBlock / 32][kRunChunk];
    for (uint32_t v = blockIdx.x; v < count; v += gridDim.x) {
        const RsChunk c = rs_chunk_at(a, v);
        PfScalars &S = a.st[c.f];
        uint64_t qb, Q;
        chunk_totals(a.rs_q, c, OpAdd(), uint64_t(0), qb, Q);
        if (Q == 0) { // counted nothing: no resample
            if (c.k == 0 && threadIdx.x == 0)
                S.nempty = 0;
            continue;
        }
        uint32_t eoff, etotal, coff, ctotal;
        chunk_totals(a.rs_e, c, OpAdd(), 0u, eoff, etotal);
        chunk_totals(a.rs_c, c, OpAdd(), 0u, coff, ctotal);
        const int32_t *rep = a.rep + c.off;
        int32_t *idx = a.idx + c.off;
        uint32_t *srcs = a.srcs + c.off;
        if (c.k == 0 && threadIdx.x == 0) {
            S.Q = Q;
            S.nempty = etotal;
            S.gather = 1;
            if (ctotal != c.n)
                atomicOr(&S.err, DEV_ERR_INTERNAL);
            // the words U01SequenceSystematic / U01SequenceStratified
            // consume (rng/u01_sequence.hpp:177-259,
            // resample/transform.hpp:61-70)
            if (sys) {
                engine_advance(S, 1);
            } else {
                const uint32_t jf =
                    c.n - static_cast<uint32_t>(rep[c.n - 1]);
                engine_advance(S, jf < c.n ? jf + 1 : c.n);
            }
        }
        uint32_t err = 0;
        int4 nxt = load_rep4(rep, c.lo + threadIdx.x * 4, c.hi);
        for (uint32_t base = c.lo; base < c.hi; base += kPfTile) {
            const uint32_t i0 = base + threadIdx.x * 4;
            const int4 cur = nxt;
            if (base + kPfTile < c.hi)
                nxt = load_rep4(rep, i0 + kPfTile, c.hi);
            const int32_t r[4] = {cur.x, cur.y, cur.z, cur.w};
            uint32_t tr = 0, te = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (r[k] >= 0) {
                    tr += static_cast<uint32_t>(r[k]);
                    te += r[k] == 0 ? 1u : 0u;
                }
            const uint64_t w = (static_cast<uint64_t>(tr) << 32) | te;
            uint64_t tot;
            const uint64_t incl =
                block_inclusive_scan(w, OpAdd(), uint64_t(0), sh64, &tot);
            const uint64_t exv = incl - w;
            uint32_t cc = coff + static_cast<uint32_t>(exv >> 32);
            uint32_t e = eoff + static_cast<uint32_t>(exv & 0xFFFFFFFFu);
            const uint32_t c0 = cc, e0 = e;
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
                        rs[k] = cc - (i - e);
                        rl[k] = static_cast<uint32_t>(r[k]) - 1;
                    }
                }
                if (r[k] > 0)
                    cc += static_cast<uint32_t>(r[k]);
            }
            // the sources of the warp's surplus ranks
            {
                const uint32_t first = c0 - (i0 - e0);
                const uint32_t W0 = __shfl_sync(0xFFFFFFFFu, first, 0);
                uint32_t Sw = rl[0] + rl[1] + rl[2] + rl[3];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                    Sw += __shfl_xor_sync(0xFFFFFFFFu, Sw, o);
                if (Sw != 0) {
                    if (Sw > etotal || W0 > etotal - Sw)
                        err |= DEV_ERR_INTERNAL;
                    else
                        write_surplus_runs(srcs, rs, rl, i0, W0, Sw,
                            shm[threadIdx.x >> 5], err);
                }
            }
            if (i0 + 3 < c.hi) {
                *reinterpret_cast<int4 *>(idx + i0) =
                    make_int4(out[0], out[1], out[2], out[3]);
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (r[k] >= 0)
                        idx[i0 + k] = out[k];
            }
            coff += static_cast<uint32_t>(tot >> 32);
            eoff += static_cast<uint32_t>(tot & 0xFFFFFFFFu);
        }
        if (err)
            atomicOr(&S.err, err);
    }
}

// the run's observations in FP32, as the step kernels use them, and for
// the bearings kinds (sc != null) the sine and cosine of each FP32 bearing
__global__ void k_obs_f32(
    const double *obs, float *out, float2 *sc, uint32_t count)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += gridDim.x * blockDim.x) {
        const float z = static_cast<float>(obs[i]);
        out[i] = z;
        if (sc)
            sc[i] = make_float2(sinf(z), cosf(z));
    }
}

__global__ void k_batch_reset(PfScalars *st, const BFilter *flt, uint32_t nf,
    uint32_t *step, uint32_t *rs_count)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f == 0) {
        *step = 0;
        // list counts, then the step kernel's tile counters
        rs_count[0] = rs_count[1] = rs_count[2] = rs_count[3] = 0;
    }
    if (f >= nf)
        return;
    PfScalars z = {};
    z.resampled = 1;
    z.rindex = 4;
    z.rkey[0] = 0;
    z.rkey[1] = flt[f].seed;
    z.rctr[2] = 1;
    st[f] = z;
}

// each filter's observations from its own model and seed (one thread each)
__global__ void k_batch_simulate(const vsmc_cuda_cv_model *models,
    const uint32_t *seeds, const uint32_t *T, const uint32_t *obs_off,
    uint32_t nf, double *truth, double *obs)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf)
        return;
    const vsmc_cuda_cv_model m = models[f];
    cv_simulate_seq(seeds[f], T[f], m.dt, m.sigma_a, m.obs_scale, m.nu,
        m.sd_pos0, m.sd_vel0, truth ? truth + 4 * obs_off[f] : nullptr,
        obs + 2 * obs_off[f]);
}

// Bearings simulation of one filter on one thread: the FP64 draws of
// vsmc_cuda_bearings_simulate (CounterEngine(seed), NormalDistribution pairs,
// one NormalDistribution(0, sigma_z) for the bearing noise).
__global__ void k_batch_simulate_bearings(
    const vsmc_cuda_bearings_model *models, const uint32_t *seeds,
    const uint32_t *T, const uint32_t *obs_off, uint32_t nf, double *truth,
    double *obs)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf)
        return;
    bearings_simulate_seq(seeds[f], T[f], models[f],
        truth ? truth + 4 * obs_off[f] : nullptr, obs + obs_off[f]);
}

constexpr uint32_t kRsMinChunk = 4 * kPfTile; // resampling chunk: 4096 or more
constexpr uint32_t kMaxRsChunks = 32;          // chunks of one filter, at most
constexpr int kRsKernels = 3;
// the scan schedules the autotuner times: the smallest chunk of a filter
constexpr uint32_t kRsSchedules[] = {4096, 8192, 16384, 32768};
constexpr int kNumSchedules = 4;

// A filter's resampling chunk: min_chunk, doubled until the filter has at
// most kMaxRsChunks chunks.  Larger chunks mean fewer list entries (and
// fewer partial records to sum) but a longer last wave.
inline uint32_t rs_chunk_for(uint32_t n, uint32_t min_chunk)
{
    uint32_t c = min_chunk;
    while ((n + c - 1) / c > kMaxRsChunks)
        c *= 2;
    return c;
}

struct Shape {
    int ppt, block;
};
constexpr Shape kShapes[] = {
    {1, 128}, {2, 128}, {4, 128}, {1, 256}, {2, 256}, {4, 256}};
constexpr int kNumShapes = 6;

template <int kBlock, int kPPT, int Kind>
static cudaError_t launch_step_k(bool first, int grid, const BatchArgs &a,
    cudaStream_t st)
{
    if (first)
        k_batch_step<kBlock, kPPT, true, Kind><<<grid, kBlock, 0, st>>>(a);
    else
        k_batch_step<kBlock, kPPT, false, Kind><<<grid, kBlock, 0, st>>>(a);
    return cudaGetLastError();
}

template <int kBlock, int kPPT>
static cudaError_t launch_step_t(int kind, bool first, int grid,
    const BatchArgs &a, cudaStream_t st)
{
    return kind == kKindCv
        ? launch_step_k<kBlock, kPPT, kKindCv>(first, grid, a, st)
        : launch_step_k<kBlock, kPPT, kKindBearings>(first, grid, a, st);
}

static cudaError_t launch_step(int kind, Shape s, bool first, int grid,
    const BatchArgs &a, cudaStream_t st)
{
    if (kind == kKindLearned) {
        if (first)
            k_batch_step_learned<true><<<grid, kLearnBlock, 0, st>>>(a);
        else
            k_batch_step_learned<false><<<grid, kLearnBlock, 0, st>>>(a);
        return cudaGetLastError();
    }
    if (s.block == 128) {
        if (s.ppt == 1)
            return launch_step_t<128, 1>(kind, first, grid, a, st);
        if (s.ppt == 2)
            return launch_step_t<128, 2>(kind, first, grid, a, st);
        return launch_step_t<128, 4>(kind, first, grid, a, st);
    }
    if (s.ppt == 1)
        return launch_step_t<256, 1>(kind, first, grid, a, st);
    if (s.ppt == 2)
        return launch_step_t<256, 2>(kind, first, grid, a, st);
    return launch_step_t<256, 4>(kind, first, grid, a, st);
}

template <typename K>
static int occupancy_of(K kernel, int block)
{
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, block, 0) !=
            cudaSuccess ||
        occ < 1)
        occ = 2;
    return occ;
}

template <int kBlock, int kPPT>
static int occupancy_t(int kind)
{
    return kind == kKindCv
        ? occupancy_of(k_batch_step<kBlock, kPPT, false, kKindCv>, kBlock)
        : occupancy_of(
              k_batch_step<kBlock, kPPT, false, kKindBearings>, kBlock);
}

static int occupancy(int kind, Shape s)
{
    if (kind == kKindLearned)
        return occupancy_of(k_batch_step_learned<false>, kLearnBlock);
    if (s.block == 128)
        return s.ppt == 1 ? occupancy_t<128, 1>(kind)
                          : (s.ppt == 2 ? occupancy_t<128, 2>(kind)
                                        : occupancy_t<128, 4>(kind));
    return s.ppt == 1 ? occupancy_t<256, 1>(kind)
                      : (s.ppt == 2 ? occupancy_t<256, 2>(kind)
                                    : occupancy_t<256, 4>(kind));
}

} // namespace vsmc_cuda

struct vsmc_cuda_batch {
    int kind = kKindCv;
    const uint32_t *packed = nullptr; // learned kind: proposal network
    std::vector<vsmc_cuda_bearings_model> bmodels;
    uint32_t nf = 0;
    uint32_t tmax = 0;
    int scheme = VSMC_CUDA_STRATIFIED;
    double threshold = 0.5;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    Shape shape = {4, 256};
    // caller order
    std::vector<uint32_t> n, T, seeds;
    std::vector<vsmc_cuda_cv_model> models;
    std::vector<uint32_t> obs_off; // prefix sums of T (caller order)
    size_t total_T = 0;
    // internal order: horizon descending
    std::vector<uint32_t> order;     // internal -> caller
    uint32_t rs_cap = 0;            // resampling chunks of all filters
    int rs_grid[kRsKernels] = {};   // persistent grids of the passes
    std::vector<BFilter> flt;        // internal order
    std::vector<uint32_t> tile_filter, active;
    size_t total_particles = 0; // with padding
    size_t max_tiles = 0;
    // device
    BFilter *d_flt = nullptr;
    PfScalars *d_st = nullptr;
    uint32_t *d_tile_filter = nullptr, *d_active = nullptr,
             *d_step = nullptr;
    uint2 *d_rs_list = nullptr;
    uint32_t *d_rs_count = nullptr;
    uint64_t *d_rs_q = nullptr;
    uint32_t *d_rs_e = nullptr, *d_rs_c = nullptr;
    float *d_state[2] = {nullptr, nullptr};
    float *d_lw = nullptr;
    int32_t *d_rep = nullptr, *d_idx = nullptr;
    uint32_t *d_srcs = nullptr;
    TileRecord *d_part = nullptr;
    float *d_obsf = nullptr; // the run's observations in FP32
    float2 *d_obs_sc = nullptr; // bearings kinds: sin, cos of each bearing
    double *d_obs = nullptr;
    double *d_mean = nullptr, *d_ess = nullptr, *d_logz = nullptr;
    int *d_res = nullptr;
    // run graph (for one observation pointer, shape and schedule)
    cudaGraphExec_t graph = nullptr;
    const double *graph_obs = nullptr;
    Shape graph_shape = {0, 0};
    uint32_t graph_chunk = 0;
    // scan schedule: the smallest resampling chunk of a filter (the list and
    // its buffers are sized for kRsMinChunk, the smallest allowed)
    uint32_t rs_min_chunk = 0;
};

namespace vsmc_cuda
{

template <typename T>
static int balloc(T **p, size_t count)
{
    void *q = nullptr;
    VSMC_CUDA_TRY(cudaMalloc(&q, sizeof(T) * (count ? count : 1)));
    *p = static_cast<T *>(q);
    return VSMC_CUDA_OK;
}

static void batch_free(vsmc_cuda_batch *b)
{
    if (b->graph)
        cudaGraphExecDestroy(b->graph);
    void *ptrs[] = {b->d_flt, b->d_st, b->d_tile_filter, b->d_active,
        b->d_step, b->d_rs_list, b->d_rs_count, b->d_rs_q, b->d_rs_e,
        b->d_rs_c, b->d_state[0], b->d_state[1], b->d_lw,
        b->d_rep, b->d_idx, b->d_srcs, b->d_part, b->d_obs, b->d_obsf, b->d_obs_sc,
        b->d_mean, b->d_ess, b->d_logz, b->d_res};
    for (void *p : ptrs)
        if (p)
            cudaFree(p);
    if (b->own_stream && b->stream)
        cudaStreamDestroy(b->stream);
}

// tile tables for a shape (host + device)
static int batch_layout(vsmc_cuda_batch *b, Shape s)
{
    const uint32_t tile = b->kind == kKindLearned
        ? kLearnTile
        : static_cast<uint32_t>(s.ppt * s.block);
    b->tile_filter.clear();
    for (uint32_t k = 0; k < b->nf; ++k) {
        BFilter &F = b->flt[k];
        F.tile0 = static_cast<uint32_t>(b->tile_filter.size());
        F.ntiles = (F.n + tile - 1) / tile;
        for (uint32_t j = 0; j < F.ntiles; ++j)
            b->tile_filter.push_back(k);
    }
    if (b->tile_filter.size() > b->max_tiles)
        return VSMC_CUDA_ERR_INTERNAL;
    // filters are sorted by T descending: those with T >= t are a prefix
    b->active.assign(b->tmax + 1, 0);
    uint32_t k = b->nf;
    for (uint32_t t = 0; t <= b->tmax; ++t) {
        while (k > 0 && b->flt[k - 1].T < t)
            --k;
        b->active[t] = k == 0 ? 0 : b->flt[k - 1].tile0 + b->flt[k - 1].ntiles;
    }
    cudaStream_t st = b->stream;
    VSMC_CUDA_TRY(cudaMemcpyAsync(b->d_flt, b->flt.data(),
        sizeof(BFilter) * b->nf, cudaMemcpyHostToDevice, st));
    VSMC_CUDA_TRY(cudaMemcpyAsync(b->d_tile_filter, b->tile_filter.data(),
        sizeof(uint32_t) * b->tile_filter.size(), cudaMemcpyHostToDevice, st));
    VSMC_CUDA_TRY(cudaMemcpyAsync(b->d_active, b->active.data(),
        sizeof(uint32_t) * b->active.size(), cudaMemcpyHostToDevice, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    b->shape = s;
    return VSMC_CUDA_OK;
}

static BatchArgs batch_args(vsmc_cuda_batch *b, const double *obs, int cur)
{
    BatchArgs a = {};
    const size_t ld = b->total_particles;
    const float *A = b->d_state[cur];
    float *B = b->d_state[1 - cur];
    a.flt = b->d_flt;
    a.st = b->d_st;
    a.tile_filter = b->d_tile_filter;
    a.active = b->d_active;
    a.ax = A;
    a.ay = A + ld;
    a.avx = A + 2 * ld;
    a.avy = A + 3 * ld;
    a.bx = B;
    a.by = B + ld;
    a.bvx = B + 2 * ld;
    a.bvy = B + 3 * ld;
    a.lw = b->d_lw;
    a.rep = b->d_rep;
    a.idx = b->d_idx;
    a.srcs = b->d_srcs;
    a.part = b->d_part;
    a.obs = b->d_obsf;
    a.obs_sc = b->d_obs_sc;
    a.h_mean = b->d_mean;
    a.h_ess = b->d_ess;
    a.h_logz = b->d_logz;
    a.h_res = b->d_res;
    a.step = b->d_step;
    a.rs_list = b->d_rs_list;
    a.rs_count = b->d_rs_count;
    a.work = b->d_rs_count + 2;
    a.rs_q = b->d_rs_q;
    a.rs_e = b->d_rs_e;
    a.rs_c = b->d_rs_c;
    a.rs_cap = b->rs_cap;
    a.rpar = static_cast<uint32_t>(cur); // step parity, as the state buffers
    a.packed = b->packed;
    a.nfilters = b->nf;
    a.tmax = b->tmax;
    a.scheme = b->scheme;
    a.threshold = b->threshold;
    return a;
}

// enqueue a whole run (reset + steps 0..nsteps-1) on the batch's stream;
// grid = the step kernel's persistent grid for the current shape
static int enqueue_run(
    vsmc_cuda_batch *b, const double *obs, int nsteps, int grid)
{
    cudaStream_t st = b->stream;
    const uint32_t nobs = static_cast<uint32_t>(
        (b->kind == kKindCv ? 2 : 1) * b->total_T);
    k_obs_f32<<<grid_for(nobs, 256, 1, 4), 256, 0, st>>>(obs, b->d_obsf,
        b->kind == kKindCv ? nullptr : b->d_obs_sc, nobs);
    VSMC_CUDA_CHECK_LAUNCH();
    k_batch_reset<<<(b->nf + 255) / 256, 256, 0, st>>>(
        b->d_st, b->d_flt, b->nf, b->d_step, b->d_rs_count);
    VSMC_CUDA_CHECK_LAUNCH();
    for (int t = 0; t < nsteps; ++t) {
        const BatchArgs a = batch_args(b, obs, t & 1);
        VSMC_CUDA_TRY(launch_step(b->kind, b->shape, t == 0, grid, a, st));
        // the filters that resample, in the chunks the step listed
        const dim3 blk(kPfBlock);
        k_brs_qsum<<<b->rs_grid[0], blk, 0, st>>>(a);
        if (a.scheme == VSMC_CUDA_SYSTEMATIC)
            k_brs_count<true><<<b->rs_grid[1], blk, 0, st>>>(a);
        else
            k_brs_count<false><<<b->rs_grid[1], blk, 0, st>>>(a);
        k_brs_assign<<<b->rs_grid[2], blk, 0, st>>>(a);
        VSMC_CUDA_CHECK_LAUNCH();
    }
    return VSMC_CUDA_OK;
}

static int check_errors(vsmc_cuda_batch *b)
{
    std::vector<PfScalars> st(b->nf);
    VSMC_CUDA_TRY(cudaMemcpyAsync(st.data(), b->d_st,
        sizeof(PfScalars) * b->nf, cudaMemcpyDeviceToHost, b->stream));
    VSMC_CUDA_TRY(cudaStreamSynchronize(b->stream));
    uint32_t err = 0;
    for (const PfScalars &s : st)
        err |= s.err;
    if (err & DEV_ERR_NONFINITE)
        return VSMC_CUDA_ERR_NONFINITE;
    if (err)
        return VSMC_CUDA_ERR_INTERNAL;
    return VSMC_CUDA_OK;
}

} // namespace vsmc_cuda

extern "C" {

} // extern "C"

namespace vsmc_cuda
{

// Shared constructor of the three kinds: cv (position model) or bm
// (bearings model) per filter; packed: the proposal network (learned kind).
static int batch_create(vsmc_cuda_batch **out, int kind, size_t nfilters,
    const uint32_t *n, const uint32_t *T, const vsmc_cuda_cv_model *cv,
    const vsmc_cuda_bearings_model *bm, const uint32_t *seeds,
    const uint32_t *packed, int scheme, double threshold, void *stream)
{
    if (out == nullptr || n == nullptr || T == nullptr || seeds == nullptr ||
        std::isnan(threshold) ||
        (scheme != VSMC_CUDA_STRATIFIED && scheme != VSMC_CUDA_SYSTEMATIC))
        return VSMC_CUDA_ERR_ARG;
    *out = nullptr;
    if (nfilters < 1 || nfilters > (size_t(1) << 24))
        return VSMC_CUDA_ERR_SIZE;
    const uint32_t min_tile = kind == kKindLearned ? kLearnTile : 128u;
    size_t total = 0, totalT = 0, tiles = 0;
    uint32_t tmax = 0;
    for (size_t f = 0; f < nfilters; ++f) {
        if (kind == kKindCv ? !valid_cv_model(&cv[f])
                            : !valid_bearings_model(&bm[f]))
            return VSMC_CUDA_ERR_ARG;
        if (n[f] < 2 || n[f] > (1u << 30) || T[f] < 1 || T[f] > (1u << 24))
            return VSMC_CUDA_ERR_SIZE;
        total += (static_cast<size_t>(n[f]) + 3) / 4 * 4;
        totalT += T[f];
        tiles += (n[f] + min_tile - 1) / min_tile; // the smallest tile
        tmax = std::max(tmax, T[f]);
    }
    if (total >= (size_t(1) << 31) || totalT >= (size_t(1) << 31))
        return VSMC_CUDA_ERR_SIZE;
    vsmc_cuda_batch *b = new (std::nothrow) vsmc_cuda_batch;
    if (b == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    b->kind = kind;
    b->packed = packed;
    b->nf = static_cast<uint32_t>(nfilters);
    b->tmax = tmax;
    b->scheme = scheme;
    b->threshold = threshold;
    b->n.assign(n, n + nfilters);
    b->T.assign(T, T + nfilters);
    b->seeds.assign(seeds, seeds + nfilters);
    if (kind == kKindCv)
        b->models.assign(cv, cv + nfilters);
    else
        b->bmodels.assign(bm, bm + nfilters);
    b->total_T = totalT;
    b->total_particles = total;
    b->max_tiles = tiles;
    b->obs_off.resize(nfilters);
    size_t acc = 0;
    for (size_t f = 0; f < nfilters; ++f) {
        b->obs_off[f] = static_cast<uint32_t>(acc);
        acc += T[f];
    }
    b->order.resize(nfilters);
    for (uint32_t f = 0; f < nfilters; ++f)
        b->order[f] = f;
    std::stable_sort(b->order.begin(), b->order.end(),
        [&](uint32_t x, uint32_t y) { return T[x] > T[y]; });
    b->flt.resize(nfilters);
    b->rs_min_chunk = kRsMinChunk;
    size_t off = 0;
    for (uint32_t k = 0; k < nfilters; ++k) {
        const uint32_t f = b->order[k];
        BFilter &F = b->flt[k];
        F = BFilter{};
        F.n = n[f];
        F.off = static_cast<uint32_t>(off);
        off += (static_cast<size_t>(n[f]) + 3) / 4 * 4;
        F.T = T[f];
        F.obs_off = b->obs_off[f];
        F.hist_off = b->obs_off[f];
        F.seed = seeds[f];
        int lg = 0;
        while ((size_t(1) << lg) < n[f])
            ++lg;
        F.shift = static_cast<uint32_t>(63 - lg);
        F.rs_chunk = rs_chunk_for(F.n, kRsMinChunk);
        b->rs_cap += (F.n + F.rs_chunk - 1) / F.rs_chunk;
        if (kind == kKindCv)
            F.c = make_cv_const<float>(cv[f]);
        else
            F.bc = make_bearings_const(bm[f]);
    }
    // the resampling passes walk the step's list with one full wave of
    // blocks each
    {
        const int sms = num_sms();
        const int occ[kRsKernels] = {occupancy_of(k_brs_qsum, kPfBlock),
            std::min(occupancy_of(k_brs_count<true>, kPfBlock),
                occupancy_of(k_brs_count<false>, kPfBlock)),
            occupancy_of(k_brs_assign, kPfBlock)};
        for (int k = 0; k < kRsKernels; ++k)
            b->rs_grid[k] = static_cast<int>(std::min<size_t>(
                static_cast<size_t>(sms) * occ[k], b->rs_cap));
    }

    b->stream = as_stream(stream);
    if (b->stream == nullptr) {
        if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) !=
            cudaSuccess) {
            delete b;
            return VSMC_CUDA_ERR_CUDA;
        }
        b->own_stream = true;
    }
    int rc = VSMC_CUDA_OK;
#define B_TRY(x)                                                              \
    do {                                                                      \
        rc = (x);                                                             \
        if (rc != VSMC_CUDA_OK) {                                             \
            batch_free(b);                                                    \
            delete b;                                                         \
            return rc;                                                        \
        }                                                                     \
    } while (0)
    B_TRY(balloc(&b->d_flt, nfilters));
    B_TRY(balloc(&b->d_st, nfilters));
    B_TRY(balloc(&b->d_tile_filter, tiles));
    B_TRY(balloc(&b->d_active, tmax + 1));
    B_TRY(balloc(&b->d_rs_list, 2 * static_cast<size_t>(b->rs_cap)));
    B_TRY(balloc(&b->d_rs_count, 4));
    B_TRY(balloc(&b->d_rs_q, b->rs_cap));
    B_TRY(balloc(&b->d_rs_e, b->rs_cap));
    B_TRY(balloc(&b->d_rs_c, b->rs_cap));
    B_TRY(balloc(&b->d_step, 1));
    B_TRY(balloc(&b->d_state[0], 4 * total));
    B_TRY(balloc(&b->d_state[1], 4 * total));
    B_TRY(balloc(&b->d_lw, total));
    B_TRY(balloc(&b->d_rep, total));
    B_TRY(balloc(&b->d_idx, total));
    B_TRY(balloc(&b->d_srcs, total));
    B_TRY(balloc(&b->d_part, tiles));
    B_TRY(balloc(&b->d_obs, 2 * totalT));
    B_TRY(balloc(&b->d_obsf, 2 * totalT));
    if (kind != kKindCv)
        B_TRY(balloc(&b->d_obs_sc, totalT));
    B_TRY(balloc(&b->d_mean, 2 * totalT));
    B_TRY(balloc(&b->d_ess, totalT));
    B_TRY(balloc(&b->d_logz, totalT));
    B_TRY(balloc(&b->d_res, totalT));
    if (cudaMemsetAsync(b->d_mean, 0, sizeof(double) * 2 * totalT,
            b->stream) != cudaSuccess)
        B_TRY(VSMC_CUDA_ERR_CUDA);
    B_TRY(batch_layout(b, b->shape));
#undef B_TRY
    *out = b;
    return VSMC_CUDA_OK;
}

} // namespace vsmc_cuda

extern "C" {

int vsmc_cuda_batch_create(vsmc_cuda_batch **out, size_t nfilters,
    const uint32_t *n, const uint32_t *T, const vsmc_cuda_cv_model *models,
    const uint32_t *seeds, int scheme, double threshold, void *stream)
{
    if (models == nullptr)
        return VSMC_CUDA_ERR_ARG;
    return batch_create(out, kKindCv, nfilters, n, T, models, nullptr, seeds,
        nullptr, scheme, threshold, stream);
}

int vsmc_cuda_batch_create_bearings(vsmc_cuda_batch **out, size_t nfilters,
    const uint32_t *n, const uint32_t *T,
    const vsmc_cuda_bearings_model *models, const uint32_t *seeds,
    const uint32_t *packed, int scheme, double threshold, void *stream)
{
    if (models == nullptr)
        return VSMC_CUDA_ERR_ARG;
    return batch_create(out, packed ? kKindLearned : kKindBearings, nfilters,
        n, T, nullptr, models, seeds, packed, scheme, threshold, stream);
}

int vsmc_cuda_batch_destroy(vsmc_cuda_batch *b)
{
    if (b == nullptr)
        return VSMC_CUDA_OK;
    cudaStreamSynchronize(b->stream);
    batch_free(b);
    delete b;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_batch_stream(vsmc_cuda_batch *b, void **stream)
{
    if (b == nullptr || stream == nullptr)
        return VSMC_CUDA_ERR_ARG;
    *stream = b->stream;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_batch_simulate(vsmc_cuda_batch *b, double *truth_dev,
    double *obs_dev)
{
    if (b == nullptr || obs_dev == nullptr)
        return VSMC_CUDA_ERR_ARG;
    uint32_t *dseed = nullptr, *dT = nullptr, *doff = nullptr;
    cudaStream_t st = b->stream;
    Scratch scratch(st);
    void *dm = b->kind == kKindCv
        ? static_cast<void *>(scratch.get<vsmc_cuda_cv_model>(b->nf))
        : static_cast<void *>(scratch.get<vsmc_cuda_bearings_model>(b->nf));
    dseed = scratch.get<uint32_t>(b->nf);
    dT = scratch.get<uint32_t>(b->nf);
    doff = scratch.get<uint32_t>(b->nf);
    if (!dm || !dseed || !dT || !doff)
        return VSMC_CUDA_ERR_ALLOC;
    if (b->kind == kKindCv)
        VSMC_CUDA_TRY(cudaMemcpyAsync(dm, b->models.data(),
            sizeof(vsmc_cuda_cv_model) * b->nf, cudaMemcpyHostToDevice, st));
    else
        VSMC_CUDA_TRY(cudaMemcpyAsync(dm, b->bmodels.data(),
            sizeof(vsmc_cuda_bearings_model) * b->nf, cudaMemcpyHostToDevice,
            st));
    VSMC_CUDA_TRY(cudaMemcpyAsync(dseed, b->seeds.data(),
        sizeof(uint32_t) * b->nf, cudaMemcpyHostToDevice, st));
    VSMC_CUDA_TRY(cudaMemcpyAsync(dT, b->T.data(), sizeof(uint32_t) * b->nf,
        cudaMemcpyHostToDevice, st));
    VSMC_CUDA_TRY(cudaMemcpyAsync(doff, b->obs_off.data(),
        sizeof(uint32_t) * b->nf, cudaMemcpyHostToDevice, st));
    if (b->kind == kKindCv)
        k_batch_simulate<<<(b->nf + 63) / 64, 64, 0, st>>>(
            static_cast<const vsmc_cuda_cv_model *>(dm), dseed, dT, doff,
            b->nf, truth_dev, obs_dev);
    else
        k_batch_simulate_bearings<<<(b->nf + 63) / 64, 64, 0, st>>>(
            static_cast<const vsmc_cuda_bearings_model *>(dm), dseed, dT,
            doff, b->nf, truth_dev, obs_dev);
    VSMC_CUDA_CHECK_LAUNCH();
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    return VSMC_CUDA_OK;
}

int vsmc_cuda_batch_run_device(vsmc_cuda_batch *b, const double *obs_dev)
{
    if (b == nullptr || obs_dev == nullptr)
        return VSMC_CUDA_ERR_ARG;
    const int nsteps = static_cast<int>(b->tmax) + 1;
    if (b->graph == nullptr || b->graph_obs != obs_dev ||
        b->graph_shape.ppt != b->shape.ppt ||
        b->graph_shape.block != b->shape.block ||
        b->graph_chunk != b->rs_min_chunk) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        const int grid = num_sms() * occupancy(b->kind, b->shape);
        VSMC_CUDA_TRY(cudaStreamBeginCapture(
            b->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_run(b, obs_dev, nsteps, grid);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (rc != VSMC_CUDA_OK) {
            if (g)
                cudaGraphDestroy(g);
            return rc;
        }
        VSMC_CUDA_TRY(e);
        const cudaError_t ei = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        VSMC_CUDA_TRY(ei);
        b->graph_obs = obs_dev;
        b->graph_shape = b->shape;
        b->graph_chunk = b->rs_min_chunk;
    }
    VSMC_CUDA_TRY(cudaGraphLaunch(b->graph, b->stream));
    return VSMC_CUDA_OK;
}

int vsmc_cuda_batch_history(vsmc_cuda_batch *b, double *mean_host,
    double *ess_host, int *resampled_host, double *logz_host)
{
    if (b == nullptr)
        return VSMC_CUDA_ERR_ARG;
    const int rc = check_errors(b);
    if (rc != VSMC_CUDA_OK)
        return rc;
    cudaStream_t st = b->stream;
    const size_t TT = b->total_T;
    if (mean_host)
        VSMC_CUDA_TRY(cudaMemcpyAsync(mean_host, b->d_mean,
            sizeof(double) * 2 * TT, cudaMemcpyDeviceToHost, st));
    if (ess_host)
        VSMC_CUDA_TRY(cudaMemcpyAsync(ess_host, b->d_ess, sizeof(double) * TT,
            cudaMemcpyDeviceToHost, st));
    if (resampled_host)
        VSMC_CUDA_TRY(cudaMemcpyAsync(resampled_host, b->d_res,
            sizeof(int) * TT, cudaMemcpyDeviceToHost, st));
    if (logz_host)
        VSMC_CUDA_TRY(cudaMemcpyAsync(logz_host, b->d_logz,
            sizeof(double) * TT, cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    return VSMC_CUDA_OK;
}

int vsmc_cuda_batch_run(vsmc_cuda_batch *b, const double *obs_host,
    double *mean_host, double *ess_host, int *resampled_host,
    double *logz_host)
{
    if (b == nullptr || obs_host == nullptr)
        return VSMC_CUDA_ERR_ARG;
    const size_t obs_dim = b->kind == kKindCv ? 2 : 1;
    VSMC_CUDA_TRY(cudaMemcpyAsync(b->d_obs, obs_host,
        sizeof(double) * obs_dim * b->total_T, cudaMemcpyHostToDevice,
        b->stream));
    const int rc = vsmc_cuda_batch_run_device(b, b->d_obs);
    if (rc != VSMC_CUDA_OK)
        return rc;
    return vsmc_cuda_batch_history(
        b, mean_host, ess_host, resampled_host, logz_host);
}

int vsmc_cuda_batch_set_shape(vsmc_cuda_batch *b, int ppt, int block)
{
    if (b == nullptr || b->kind == kKindLearned)
        return VSMC_CUDA_ERR_ARG;
    for (int k = 0; k < kNumShapes; ++k)
        if (kShapes[k].ppt == ppt && kShapes[k].block == block)
            return batch_layout(b, kShapes[k]);
    return VSMC_CUDA_ERR_ARG;
}

int vsmc_cuda_batch_get_shape(vsmc_cuda_batch *b, int *ppt, int *block)
{
    if (b == nullptr || ppt == nullptr || block == nullptr)
        return VSMC_CUDA_ERR_ARG;
    *ppt = b->shape.ppt;
    *block = b->shape.block;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_batch_set_schedule(vsmc_cuda_batch *b, uint32_t min_chunk)
{
    if (b == nullptr)
        return VSMC_CUDA_ERR_ARG;
    bool known = false;
    for (int k = 0; k < kNumSchedules; ++k)
        known = known || kRsSchedules[k] == min_chunk;
    if (!known)
        return VSMC_CUDA_ERR_ARG;
    for (uint32_t k = 0; k < b->nf; ++k) {
        BFilter &F = b->flt[k];
        F.rs_chunk = rs_chunk_for(F.n, min_chunk);
    }
    b->rs_min_chunk = min_chunk;
    // re-uploads the filter descriptions (their chunks); the list keeps the
    // capacity of the smallest chunk, which bounds every schedule
    return batch_layout(b, b->shape);
}

int vsmc_cuda_batch_get_schedule(vsmc_cuda_batch *b, uint32_t *min_chunk)
{
    if (b == nullptr || min_chunk == nullptr)
        return VSMC_CUDA_ERR_ARG;
    *min_chunk = b->rs_min_chunk;
    return VSMC_CUDA_OK;
}

// time `nsteps` steps of the batch (one warm-up run first)
static int time_steps(vsmc_cuda_batch *b, const double *obs_dev, int nsteps,
    cudaEvent_t e0, cudaEvent_t e1, float *ms)
{
    const int grid = num_sms() * occupancy(b->kind, b->shape);
    int rc = enqueue_run(b, obs_dev, nsteps, grid); // warm-up
    if (rc != VSMC_CUDA_OK)
        return rc;
    VSMC_CUDA_TRY(cudaEventRecord(e0, b->stream));
    rc = enqueue_run(b, obs_dev, nsteps, grid);
    if (rc != VSMC_CUDA_OK)
        return rc;
    VSMC_CUDA_TRY(cudaEventRecord(e1, b->stream));
    VSMC_CUDA_TRY(cudaEventSynchronize(e1));
    VSMC_CUDA_TRY(cudaEventElapsedTime(ms, e0, e1));
    return VSMC_CUDA_OK;
}

int vsmc_cuda_batch_autotune_schedule(vsmc_cuda_batch *b,
    const double *obs_dev, int steps, float *ms_host)
{
    if (b == nullptr || obs_dev == nullptr || steps < 1)
        return VSMC_CUDA_ERR_ARG;
    const int nsteps = std::min(steps, static_cast<int>(b->tmax) + 1);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    VSMC_CUDA_TRY(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return VSMC_CUDA_ERR_CUDA;
    }
    int best = -1;
    float best_ms = 0;
    int rc = VSMC_CUDA_OK;
    for (int k = 0; k < kNumSchedules && rc == VSMC_CUDA_OK; ++k) {
        rc = vsmc_cuda_batch_set_schedule(b, kRsSchedules[k]);
        float ms = 0;
        if (rc == VSMC_CUDA_OK)
            rc = time_steps(b, obs_dev, nsteps, e0, e1, &ms);
        if (rc != VSMC_CUDA_OK)
            break;
        if (ms_host)
            ms_host[k] = ms;
        if (best < 0 || ms < best_ms) {
            best = k;
            best_ms = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != VSMC_CUDA_OK)
        return rc;
    rc = check_errors(b);
    if (rc != VSMC_CUDA_OK)
        return rc;
    return vsmc_cuda_batch_set_schedule(b, kRsSchedules[best]);
}

int vsmc_cuda_batch_autotune(vsmc_cuda_batch *b, const double *obs_dev,
    int steps, float *ms_host)
{
    if (b == nullptr || obs_dev == nullptr || steps < 1 ||
        b->kind == kKindLearned)
        return VSMC_CUDA_ERR_ARG;
    const int nsteps = std::min(steps, static_cast<int>(b->tmax) + 1);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    VSMC_CUDA_TRY(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return VSMC_CUDA_ERR_CUDA;
    }
    int best = -1;
    float best_ms = 0;
    int rc = VSMC_CUDA_OK;
    for (int k = 0; k < kNumShapes && rc == VSMC_CUDA_OK; ++k) {
        rc = batch_layout(b, kShapes[k]);
        if (rc != VSMC_CUDA_OK)
            break;
        const int grid = num_sms() * occupancy(b->kind, b->shape);
        rc = enqueue_run(b, obs_dev, nsteps, grid); // warm-up
        if (rc != VSMC_CUDA_OK)
            break;
        if (cudaEventRecord(e0, b->stream) != cudaSuccess) {
            rc = VSMC_CUDA_ERR_CUDA;
            break;
        }
        rc = enqueue_run(b, obs_dev, nsteps, grid);
        if (rc != VSMC_CUDA_OK)
            break;
        float ms = 0;
        if (cudaEventRecord(e1, b->stream) != cudaSuccess ||
            cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
            rc = VSMC_CUDA_ERR_CUDA;
            break;
        }
        if (ms_host)
            ms_host[k] = ms;
        if (best < 0 || ms < best_ms) {
            best = k;
            best_ms = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != VSMC_CUDA_OK)
        return rc;
    rc = check_errors(b);
    if (rc != VSMC_CUDA_OK)
        return rc;
    rc = batch_layout(b, kShapes[best]);
    if (rc != VSMC_CUDA_OK)
        return rc;
    // then the scan schedule (the resampling chunk) for that shape
    return vsmc_cuda_batch_autotune_schedule(b, obs_dev, steps, nullptr);
}

} // extern "C"
