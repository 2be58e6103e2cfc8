// vsmc_cuda_filter.cuh - the fused FP32 particle-filter step of libvsmc_cuda
// for any user model, compiled with nvcc (sm_103a) into the user's program.
//
// In the reference a model is the user's per-particle `eval_sp` inside a
// MoveBase / MoveOMP functor: eval_pre once per step, eval_sp per particle,
// eval_post once (smp/backend_base.hpp:243-363, smp/backend_omp.hpp:93-105),
// followed by Weight::add_log (core/weight.hpp:168-173).  Here the model is a
// device functor and one kernel does all of it: it reads every particle
// (through the resampling index after a resample), moves it, evaluates its
// log-likelihood, updates its FP32 log-weight and reduces, per block,
// (max, sum exp, sum exp^2) of the new log-weights and the weighted sums of
// the first `monitor_dim` state components.  The last block to finish
// combines the blocks' records in FP64 into the ESS, the log-evidence
// increment, the monitor mean and the resampling decision.  The library
// (vsmc_cuda.h) owns the buffers and the resampling passes; this header only
// adds the model-dependent kernel.  The library's own constant-velocity
// filter is an instance of the same template.
//
// A model is a trivially copyable struct (it is a kernel argument):
//
//   struct MyModel {
//       static constexpr int dim = 4;         // state components, <= 8
//       static constexpr int monitor_dim = 2; // leading components whose
//                                             // weighted mean is recorded
//       struct step_type { ... };             // per-step constants
//       // eval_pre: once per thread and step (t = step index)
//       __device__ step_type step(uint32_t t) const;
//       // t = 0: draw the initial particle (x is uninitialized on entry)
//       __device__ void init(const step_type &, vsmc_cuda::ParticleRng &,
//           float (&x)[dim]) const;
//       // t >= 1: propagate x in place (eval_sp)
//       __device__ void move(const step_type &, vsmc_cuda::ParticleRng &,
//           float (&x)[dim]) const;
//       // log g(y_t | x) of the moved particle, added to its log-weight
//       __device__ float log_likelihood(const step_type &,
//           const float (&x)[dim]) const;
//   };
//
// and one step is
//
//   vsmc_cuda_pf_step_desc d;
//   vsmc_cuda_pf_step_desc_get(pf, &d);         // buffers of the next step
//   vsmc_cuda::pf_step_launch(d, model);        // this header's kernel
//   vsmc_cuda_pf_step_commit(pf);               // resampling, next buffers
//
// (vsmc_cuda_sampler.cuh wraps this in Sampler<T> classes).  Randomness comes
// from the ParticleRng the kernel hands the model: the Philox4x32 stream
// with key {t, seed} and counters {1.., i, 0, 0} of particle i (the slot
// index, after resampling).
#ifndef VSMC_CUDA_FILTER_CUH
#define VSMC_CUDA_FILTER_CUH

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "vsmc_cuda.h"
#include "vsmc_cuda_device.cuh"

namespace vsmc_cuda
{

constexpr int kPfBlock = 256;
constexpr int kPfTile = kPfBlock * 4; // particles per block and tile
constexpr int kMaxFilterDim = 8;
constexpr int kMaxMonitorDim = 4;

// Device-side error word bits of the filter scalars (written with atomicOr).
enum : unsigned {
    DEV_ERR_NONFINITE = 1u, // NaN / inf / negative weight where forbidden
    DEV_ERR_BOUND = 2u,     // an exactness or iteration bound was exceeded
    DEV_ERR_INTERNAL = 4u,  // an index left its range
};

// Device-resident filter scalars (one per filter; the library allocates
// them, this kernel and the library's resampling passes share the layout).
struct PfScalars {
    double M;    // max of the stored log-weights after the last weighting
    double S;    // sum exp(lw - M)
    double logz; // cumulative log-evidence
    double ess;
    double mean[kMaxMonitorDim]; // monitor: weighted mean after the step
    uint64_t Q;          // fixed-point CDF total of the pending resample
    uint64_t qrcp;       // floor((2^128 - 1) / (Q << qz)) - 2^64
    uint64_t qG;         // systematic: ceil(a Q / 2^32) for the shared word a
    uint64_t qgam;       // systematic: floor(2^64 qG / Q)
    uint64_t qm;         // floor(2^(64 + qs) n / Q) (when qs > 0)
    uint64_t qgs;        // floor(2^qs qG / Q)
    uint32_t qz;         // leading zero bits of Q
    uint32_t qs;         // fraction bits of the n / Q reciprocal (0: unused)
    uint32_t done3;      // completion counter of the resampling passes
    uint32_t step;       // next step index t
    int32_t resampled;   // last step resampled: weights equal, lw stale
    int32_t gather;      // state must be read through idx (after a resample)
    uint32_t done;       // completion counter of the fused step
    uint32_t done2;      // completion counter of the other reductions
    uint32_t err;        // DEV_ERR_* bits
    uint32_t nempty;     // empty slots of the pending resample
    uint32_t rindex;     // resampling engine: next word index in gen(rctr)
    uint32_t rkey[2];
    uint32_t rctr[4];
    float Mf; // M as a float (the batched filters' kernels read it per tile)
};

// Per-block record of the fused step: new log-weights' block max m, sum
// exp(lw - m), sum exp(2 (lw - m)), and sum exp(lw - m) x_d for the
// monitored components.
struct PfPartial {
    double m, s, s2;
    double mon[kMaxMonitorDim];
    double prev[kMaxMonitorDim]; // previous-step monitor sums (Previous)
    double prev_w;
};

// Kernel arguments (from vsmc_cuda_pf_step_desc).
struct PfStepArgs {
    const float *in; // state before the step: dim rows of `stride`
    float *out;      // state after the step
    float *lw;       // log-weights, updated in place
    const int32_t *idx;
    const uint32_t *srcs;
    PfPartial *part;
    PfScalars *sc;
    double *h_mean, *h_ess, *h_logz;
    int *h_res;
    size_t stride;
    uint32_t n, seed, max_steps;
    double threshold; // resample when ESS < threshold * n (< 0: never)
    int mon_prev;     // PfMon::Previous (the filter's own runs)
};

// ------------------------------------------------- weighted accumulation

// Running (max, sum exp, sum exp^2, monitored weighted sums) of log-weights,
// all relative to the running max, in FP32.  A plain aggregate (it also
// lives in shared memory); start from lse_empty().
template <int MD>
struct LseMon {
    float m, s, s2;
    float mon[MD > 0 ? MD : 1];

    template <int D>
    __device__ __forceinline__ void push(float v, const float (&x)[D])
    {
        if (!(v > -INFINITY)) // -inf and NaN carry no weight
            return;
        if (v > m) {
            const float e = __expf(m - v);
            s = s * e + 1.0f;
            s2 = s2 * e * e + 1.0f;
#pragma unroll
            for (int d = 0; d < MD; ++d)
                mon[d] = mon[d] * e + x[d];
            m = v;
        } else {
            const float e = __expf(v - m);
            s += e;
            s2 = fmaf(e, e, s2);
#pragma unroll
            for (int d = 0; d < MD; ++d)
                mon[d] = fmaf(e, x[d], mon[d]);
        }
    }

    __device__ __forceinline__ void merge(const LseMon &o)
    {
        if (!(o.m > -INFINITY))
            return;
        if (!(m > -INFINITY)) {
            *this = o;
            return;
        }
        if (o.m > m) {
            const float e = __expf(m - o.m);
            s = s * e + o.s;
            s2 = s2 * e * e + o.s2;
#pragma unroll
            for (int d = 0; d < MD; ++d)
                mon[d] = mon[d] * e + o.mon[d];
            m = o.m;
        } else {
            const float e = __expf(o.m - m);
            s += o.s * e;
            s2 += o.s2 * e * e;
#pragma unroll
            for (int d = 0; d < MD; ++d)
                mon[d] += o.mon[d] * e;
        }
    }

    __device__ __forceinline__ LseMon shfl_xor(int lanes) const
    {
        LseMon o = *this;
        o.m = __shfl_xor_sync(0xFFFFFFFFu, m, lanes);
        o.s = __shfl_xor_sync(0xFFFFFFFFu, s, lanes);
        o.s2 = __shfl_xor_sync(0xFFFFFFFFu, s2, lanes);
#pragma unroll
        for (int d = 0; d < MD; ++d)
            o.mon[d] = __shfl_xor_sync(0xFFFFFFFFu, mon[d], lanes);
        return o;
    }
};

template <int MD>
__device__ __forceinline__ LseMon<MD> lse_empty()
{
    LseMon<MD> a;
    a.m = -INFINITY;
    a.s = 0.0f;
    a.s2 = 0.0f;
#pragma unroll
    for (int d = 0; d < (MD > 0 ? MD : 1); ++d)
        a.mon[d] = 0.0f;
    return a;
}

// ------------------------------------------------------------ particle I/O

__device__ __forceinline__ float4 pf_ld4(const float *p)
{
    return __ldcs(reinterpret_cast<const float4 *>(p));
}

__device__ __forceinline__ void pf_st4(float *p, float4 v)
{
    __stcs(reinterpret_cast<float4 *>(p), v);
}

__device__ __forceinline__ float pf_get(const float4 &v, int k)
{
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

__device__ __forceinline__ void pf_set(float4 &v, int k, float f)
{
    if (k == 0)
        v.x = f;
    else if (k == 1)
        v.y = f;
    else if (k == 2)
        v.z = f;
    else
        v.w = f;
}

// Source slot of slot i after a resample: idx[i] >= 0 is the slot itself
// (a parent keeps its slot), idx[i] = -(e + 1) is the e-th empty slot,
// filled from srcs[e] (the layout of resample/transform.hpp:116-133).
__device__ __forceinline__ uint32_t pf_source(
    const uint32_t *srcs, int32_t v)
{
    return v >= 0 ? static_cast<uint32_t>(v) : __ldcg(srcs + (-v - 1));
}

// Rows of particles i0..i0+3, gathered through the index after a resample.
// A group of four slots that all keep their own particles takes one float4
// per row.
template <int D>
__device__ __forceinline__ void pf_load_group(
    const PfStepArgs &a, uint32_t i0, bool gather, float4 (&R)[D])
{
    if (gather) {
        const int4 I = __ldcs(reinterpret_cast<const int4 *>(a.idx + i0));
        const int b = static_cast<int>(i0);
        if (I.x == b && I.y == b + 1 && I.z == b + 2 && I.w == b + 3) {
#pragma unroll
            for (int d = 0; d < D; ++d)
                R[d] = pf_ld4(a.in + d * a.stride + i0);
        } else {
            uint32_t s0 = pf_source(a.srcs, I.x);
            uint32_t s1 = pf_source(a.srcs, I.y);
            uint32_t s2 = pf_source(a.srcs, I.z);
            uint32_t s3 = pf_source(a.srcs, I.w);
            if (max(max(s0, s1), max(s2, s3)) >= a.n) {
                // an index outside the particles: record it, read slot 0
                atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
                s0 = s0 < a.n ? s0 : 0;
                s1 = s1 < a.n ? s1 : 0;
                s2 = s2 < a.n ? s2 : 0;
                s3 = s3 < a.n ? s3 : 0;
            }
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const float *r = a.in + d * a.stride;
                R[d] = make_float4(r[s0], r[s1], r[s2], r[s3]);
            }
        }
    } else {
#pragma unroll
        for (int d = 0; d < D; ++d)
            R[d] = pf_ld4(a.in + d * a.stride + i0);
    }
}

// The monitor's place in the step.  Current: the step's own weighted mean
// of the moved particles, reduced with the evidence (a host reading the
// monitor after every step, as Sampler<T> does).  Previous: the previous
// step's monitor, from the particles this step reads (weights
// exp(lw_prev - M_prev), or equal after a resample); the filter's own runs,
// where it costs one exponential and no pass after a resample.
enum class PfMon { Current, Previous };

template <int MD>
struct PrevSums {
    float x[MD > 0 ? MD : 1];
    float w;
};

// One particle: draw or move, weight, accumulate.
template <class Model, bool First, PfMon Mon, int MD, int AMD>
__device__ __forceinline__ void pf_particle(const Model &model,
    const typename Model::step_type &ctx, uint32_t t, uint32_t seed,
    uint32_t i, int resampled, float Mprev, float (&x)[Model::dim], float &lw,
    LseMon<AMD> &acc, PrevSums<MD> &prev)
{
    ParticleRng rng(t, seed, i);
    float lw_old = 0.0f;
    if (First) {
        model.init(ctx, rng, x);
    } else {
        lw_old = resampled ? 0.0f : lw - Mprev;
        if (Mon == PfMon::Previous) {
            const float wo = resampled ? 1.0f : __expf(lw_old);
#pragma unroll
            for (int d = 0; d < MD; ++d)
                prev.x[d] = fmaf(wo, x[d], prev.x[d]);
            prev.w += wo;
        }
        model.move(ctx, rng, x);
    }
    lw = lw_old + model.log_likelihood(ctx, x);
    acc.push(lw, x);
}

// ------------------------------------------------------------ fused step

template <class Model, bool First, PfMon Mon>
__global__ void __launch_bounds__(kPfBlock, 4) k_pf_step(
    const PfStepArgs a, const Model model)
{
    constexpr int D = Model::dim;
    constexpr int MD = Model::monitor_dim;
    // the evidence sums carry the monitor only for the current-step mode
    constexpr int AMD = Mon == PfMon::Current ? MD : 0;
    const uint32_t t = a.sc->step;
    const int resampled = First ? 1 : a.sc->resampled;
    const bool gather = First ? false : (a.sc->gather != 0);
    const float Mprev = First ? 0.0f : static_cast<float>(a.sc->M);
    const typename Model::step_type ctx = model.step(t);
    const uint32_t n = a.n;
    LseMon<AMD> acc = lse_empty<AMD>();
    PrevSums<MD> prev;
#pragma unroll
    for (int d = 0; d < (MD > 0 ? MD : 1); ++d)
        prev.x[d] = 0.0f;
    prev.w = 0.0f;

    const uint32_t ntiles = (n + kPfTile - 1) / kPfTile;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint32_t i0 = tile * kPfTile + threadIdx.x * 4;
        if (i0 + 3 < n) {
            float4 R[D];
            float4 LW = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (!First) {
                pf_load_group<D>(a, i0, gather, R);
                if (!resampled)
                    LW = pf_ld4(a.lw + i0);
            } else {
#pragma unroll
                for (int d = 0; d < D; ++d)
                    R[d] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float x[D];
#pragma unroll
                for (int d = 0; d < D; ++d)
                    x[d] = pf_get(R[d], k);
                float l = pf_get(LW, k);
                pf_particle<Model, First, Mon, MD, AMD>(model, ctx, t, a.seed,
                    i0 + k, resampled, Mprev, x, l, acc, prev);
#pragma unroll
                for (int d = 0; d < D; ++d)
                    pf_set(R[d], k, x[d]);
                pf_set(LW, k, l);
            }
#pragma unroll
            for (int d = 0; d < D; ++d)
                pf_st4(a.out + d * a.stride + i0, R[d]);
            pf_st4(a.lw + i0, LW);
        } else {
            for (uint32_t i = i0; i < n && i < i0 + 4; ++i) {
                float x[D];
                float l = 0.0f;
                if (!First) {
                    uint32_t src = gather ? pf_source(a.srcs, a.idx[i]) : i;
                    if (src >= n) {
                        atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
                        src = 0;
                    }
#pragma unroll
                    for (int d = 0; d < D; ++d)
                        x[d] = a.in[d * a.stride + src];
                    l = resampled ? 0.0f : a.lw[i];
                } else {
#pragma unroll
                    for (int d = 0; d < D; ++d)
                        x[d] = 0.0f;
                }
                pf_particle<Model, First, Mon, MD, AMD>(
                    model, ctx, t, a.seed, i, resampled, Mprev, x, l, acc,
                    prev);
#pragma unroll
                for (int d = 0; d < D; ++d)
                    a.out[d * a.stride + i] = x[d];
                a.lw[i] = l;
            }
        }
    }

    // ---- warp level in FP32
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        acc.merge(acc.shfl_xor(d));
    constexpr bool prev_on = !First && Mon == PfMon::Previous;
    if (prev_on) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int d = 0; d < MD; ++d)
                prev.x[d] += __shfl_xor_sync(0xFFFFFFFFu, prev.x[d], o);
            prev.w += __shfl_xor_sync(0xFFFFFFFFu, prev.w, o);
        }
    }
    // ---- block level in FP32 (warp 0 merges the warps' records), then one
    // FP64 record per block
    constexpr int kW = kPfBlock / 32;
    __shared__ LseMon<AMD> shw[kW];
    __shared__ float shp[kMaxMonitorDim + 1][kW];
    __shared__ double shd[3 + 2 * kMaxMonitorDim + 1][kW];
    __shared__ float shmax[kW];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        shw[wid] = acc;
        if (prev_on) {
#pragma unroll
            for (int d = 0; d < MD; ++d)
                shp[d][wid] = prev.x[d];
            shp[kMaxMonitorDim][wid] = prev.w;
        }
    }
    __syncthreads();
    if (wid == 0) {
        LseMon<AMD> w = lse_empty<AMD>();
        if (lane < kW)
            w = shw[lane];
#pragma unroll
        for (int d = kW / 2; d > 0; d >>= 1)
            w.merge(w.shfl_xor(d));
        if (lane == 0) {
            PfPartial p;
            p.m = w.m;
            p.s = w.s;
            p.s2 = w.s2;
#pragma unroll
            for (int d = 0; d < kMaxMonitorDim; ++d) {
                p.mon[d] = d < AMD ? w.mon[d < AMD ? d : 0] : 0.0;
                double pv = 0;
                if (prev_on && d < MD)
                    for (int k = 0; k < kW; ++k)
                        pv += shp[d < MD ? d : 0][k];
                p.prev[d] = pv;
            }
            double pw = 0;
            if (prev_on)
                for (int k = 0; k < kW; ++k)
                    pw += shp[kMaxMonitorDim][k];
            p.prev_w = pw;
            a.part[blockIdx.x] = p;
            __threadfence();
            is_last = atomicAdd(&a.sc->done, 1u) == gridDim.x - 1;
        }
    }
    __syncthreads();
    if (!is_last)
        return;

    // ---- last block: combine every block's record in FP64
    __threadfence();
    float M = -INFINITY;
    for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x)
        M = fmaxf(M, static_cast<float>(__ldcg(&a.part[b].m)));
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        M = fmaxf(M, __shfl_xor_sync(0xFFFFFFFFu, M, d));
    if (lane == 0)
        shmax[wid] = M;
    __syncthreads();
    M = shmax[0];
#pragma unroll
    for (int w = 1; w < kW; ++w)
        M = fmaxf(M, shmax[w]);
    double v[3 + 2 * kMaxMonitorDim + 1] = {};
    for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
        const double pm = __ldcg(&a.part[b].m);
        if (pm > -INFINITY) {
            const double f = __expf(static_cast<float>(pm) - M);
            v[0] += __ldcg(&a.part[b].s) * f;
            v[1] += __ldcg(&a.part[b].s2) * f * f;
#pragma unroll
            for (int d = 0; d < AMD; ++d)
                v[3 + d] += __ldcg(&a.part[b].mon[d]) * f;
        }
        if (prev_on) {
#pragma unroll
            for (int d = 0; d < MD; ++d)
                v[3 + kMaxMonitorDim + d] += __ldcg(&a.part[b].prev[d]);
            v[3 + 2 * kMaxMonitorDim] += __ldcg(&a.part[b].prev_w);
        }
    }
#pragma unroll
    for (int k = 0; k < 3 + 2 * kMaxMonitorDim + 1; ++k) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1)
            v[k] += __shfl_xor_sync(0xFFFFFFFFu, v[k], d);
        if (lane == 0)
            shd[k][wid] = v[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0, S2 = 0, MON[kMaxMonitorDim] = {},
               PREV[kMaxMonitorDim] = {}, PW = 0;
        for (int w = 0; w < kW; ++w) {
            S += shd[0][w];
            S2 += shd[1][w];
#pragma unroll
            for (int d = 0; d < MD; ++d) {
                MON[d] += shd[3 + d][w];
                PREV[d] += shd[3 + kMaxMonitorDim + d][w];
            }
            PW += shd[3 + 2 * kMaxMonitorDim][w];
        }
        if (prev_on && t >= 1 && t - 1 < a.max_steps) {
#pragma unroll
            for (int d = 0; d < MD; ++d)
                a.h_mean[static_cast<size_t>(t - 1) * MD + d] = PREV[d] / PW;
        }
        PfScalars &sc = *a.sc;
        const double prev_mass = resampled ? static_cast<double>(n) : sc.S;
        const bool rec = t < a.max_steps;
        const double ess = S * S / S2;
        const double M1 = static_cast<double>(M);
        sc.logz += M1 + log(S) - log(prev_mass);
        if (!(S > 0) || !(ess > 0))
            sc.err |= DEV_ERR_NONFINITE;
        const int flag =
            ess < a.threshold * static_cast<double>(n) ? 1 : 0;
        if (Mon == PfMon::Current) {
#pragma unroll
            for (int d = 0; d < MD; ++d) {
                sc.mean[d] = MON[d] / S;
                if (rec)
                    a.h_mean[static_cast<size_t>(t) * MD + d] = MON[d] / S;
            }
        }
        if (rec) {
            a.h_ess[t] = ess;
            a.h_logz[t] = sc.logz;
            a.h_res[t] = flag;
        }
        sc.M = M1;
        sc.Mf = M;
        sc.S = S;
        sc.ess = ess;
        sc.resampled = flag;
        sc.gather = 0; // every block has read it; a resample sets it again
        sc.step = t + 1;
        sc.done = 0;
    }
}

// ------------------------------------------------------------ host launch

template <class Model, bool First, PfMon Mon>
inline int pf_step_occupancy()
{
    static int occ = 0;
    if (occ == 0) {
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &o, k_pf_step<Model, First, Mon>, kPfBlock, 0) !=
                cudaSuccess ||
            o < 1)
            o = 1;
        occ = o;
    }
    return occ;
}

// Launch the fused step of `model` on the buffers of d (the next step of
// the filter d came from).  Returns a vsmc_cuda_status.
template <class Model>
inline int pf_step_launch(const vsmc_cuda_pf_step_desc &d, const Model &model)
{
    static_assert(Model::dim >= 1 && Model::dim <= kMaxFilterDim,
        "a model has 1 to 8 state components");
    static_assert(Model::monitor_dim >= 0 &&
            Model::monitor_dim <= kMaxMonitorDim &&
            Model::monitor_dim <= Model::dim,
        "monitor_dim is at most 4 and at most dim");
    if (d.dim != static_cast<size_t>(Model::dim) ||
        d.monitor_dim != static_cast<size_t>(Model::monitor_dim) ||
        d.state_in == nullptr || d.state_out == nullptr ||
        d.log_weight == nullptr || d.scalars == nullptr ||
        d.partials == nullptr || d.n == 0 || d.stride % 4 != 0)
        return VSMC_CUDA_ERR_ARG;
    PfStepArgs a;
    a.in = d.state_in;
    a.out = d.state_out;
    a.lw = d.log_weight;
    a.idx = d.index;
    a.srcs = d.sources;
    a.part = static_cast<PfPartial *>(d.partials);
    a.sc = static_cast<PfScalars *>(d.scalars);
    a.h_mean = d.hist_mean;
    a.h_ess = d.hist_ess;
    a.h_logz = d.hist_logz;
    a.h_res = d.hist_resampled;
    a.stride = d.stride;
    a.n = static_cast<uint32_t>(d.n);
    a.seed = d.seed;
    a.max_steps = static_cast<uint32_t>(d.max_steps);
    a.threshold = d.threshold;
    a.mon_prev = d.record_previous_mean;
    const bool first = d.step == 0;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
            cudaSuccess)
        return VSMC_CUDA_ERR_CUDA;
    const bool prevmon = a.mon_prev != 0;
    const int occ = first
        ? (prevmon ? pf_step_occupancy<Model, true, PfMon::Previous>()
                   : pf_step_occupancy<Model, true, PfMon::Current>())
        : (prevmon ? pf_step_occupancy<Model, false, PfMon::Previous>()
                   : pf_step_occupancy<Model, false, PfMon::Current>());
    const size_t ntiles = (d.n + kPfTile - 1) / kPfTile;
    size_t grid = static_cast<size_t>(sms) * static_cast<size_t>(occ);
    if (grid > ntiles)
        grid = ntiles;
    if (grid > d.max_grid)
        grid = d.max_grid;
    if (grid < 1)
        return VSMC_CUDA_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(d.stream);
    const unsigned g = static_cast<unsigned>(grid);
    if (first && prevmon)
        k_pf_step<Model, true, PfMon::Previous><<<g, kPfBlock, 0, st>>>(a,
            model);
    else if (first)
        k_pf_step<Model, true, PfMon::Current><<<g, kPfBlock, 0, st>>>(a,
            model);
    else if (prevmon)
        k_pf_step<Model, false, PfMon::Previous><<<g, kPfBlock, 0, st>>>(a,
            model);
    else
        k_pf_step<Model, false, PfMon::Current><<<g, kPfBlock, 0, st>>>(a,
            model);
    return cudaGetLastError() == cudaSuccess ? VSMC_CUDA_OK
                                             : VSMC_CUDA_ERR_CUDA;
}

} // namespace vsmc_cuda

#endif // VSMC_CUDA_FILTER_CUH
