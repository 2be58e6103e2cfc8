// Counter-based RNG on the device: counter-addressed Philox4x32-10 /
// Threefry4x64-20 blocks, the engine's bulk word stream (bit-exact with the
// reference's CounterEngine, rng/counter.hpp:288-496), and the reference's
// batch u01 / normal layouts (rng/u01_distribution.hpp:215-233,
// rng/normal_distribution.hpp:222-267).
#include "common.cuh"
#include "rng_device.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace vsmc_cuda
{

// --------------------------------------------------- counter-addressed blocks

template <bool Aligned>
__global__ void __launch_bounds__(256) k_philox_blocks(uint32_t k0,
    uint32_t k1, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
    size_t nblocks, uint32_t *out)
{
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t b = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
         b < nblocks; b += stride) {
        uint32_t c[4] = {c0, c1, c2, c3};
        ctr32_add(c, static_cast<uint64_t>(b) + 1);
        const u32x4 r = philox4x32_10(c[0], c[1], c[2], c[3], k0, k1);
        if (Aligned) {
            __stcs(reinterpret_cast<uint4 *>(out) + b,
                make_uint4(r.x, r.y, r.z, r.w));
        } else {
            out[4 * b + 0] = r.x;
            out[4 * b + 1] = r.y;
            out[4 * b + 2] = r.z;
            out[4 * b + 3] = r.w;
        }
    }
}

template <bool Aligned>
__global__ void __launch_bounds__(256) k_threefry_blocks(uint64_t k0,
    uint64_t k1, uint64_t k2, uint64_t k3, uint64_t c0, uint64_t c1,
    uint64_t c2, uint64_t c3, size_t nblocks, uint64_t *out)
{
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t b = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
         b < nblocks; b += stride) {
        uint64_t c[4] = {c0, c1, c2, c3};
        ctr64_add(c, static_cast<uint64_t>(b) + 1);
        const u64x4 r = threefry4x64_20({c[0], c[1], c[2], c[3]}, k0, k1, k2, k3);
        if (Aligned) {
            ulonglong2 *o = reinterpret_cast<ulonglong2 *>(out) + 2 * b;
            __stcs(o, make_ulonglong2(r.x, r.y));
            __stcs(o + 1, make_ulonglong2(r.z, r.w));
        } else {
            out[4 * b + 0] = r.x;
            out[4 * b + 1] = r.y;
            out[4 * b + 2] = r.z;
            out[4 * b + 3] = r.w;
        }
    }
}

// ------------------------------------------------------------ stream plans

// Output element types the plan kernel can write.
enum class Emit { Word, U01D, U01F };

// The four outputs of one block at o[0..3]: one 16-byte streaming store per
// 16 bytes when o is 16-byte aligned, else element stores.
template <Emit E, typename Gen, typename Out>
__device__ __forceinline__ void emit4(Out *o, const typename Gen::block_t &blk)
{
    Out v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        emit<E>(v, i, Gen::word(blk, i));
    if ((reinterpret_cast<uintptr_t>(o) & 15) == 0) {
        uint4 u[sizeof(Out) / 4];
        memcpy(u, v, sizeof(v));
#pragma unroll
        for (int h = 0; h < static_cast<int>(sizeof(Out) / 4); ++h)
            __stcs(reinterpret_cast<uint4 *>(o) + h, u[h]);
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
            o[i] = v[i];
    }
}

// Writes stream positions [p_begin, p_end) of `plan` to out[p - p_begin].
template <typename Gen, Emit E, typename Out>
__global__ void __launch_bounds__(256) k_plan_stream(Gen gen, StreamPlan plan,
    uint64_t p_begin, uint64_t p_end, Out *out)
{
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    const size_t tid = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    // the partially used current block gen(C0)
    if (tid == 0 && p_begin < plan.head) {
        const typename Gen::block_t blk = gen.block_at_start(plan);
        for (uint64_t p = p_begin; p < plan.head && p < p_end; ++p)
            emit<E>(out, p - p_begin,
                Gen::word(blk, plan.x + static_cast<uint32_t>(p)));
    }
    if (p_end <= plan.head)
        return;
    const uint64_t q0 = p_begin > plan.head ? p_begin - plan.head : 0;
    const uint64_t q1 = p_end - plan.head;
    const uint64_t j0 = q0 / 4, j1 = (q1 + 3) / 4;
    for (uint64_t j = j0 + tid; j < j1; j += stride) {
        const typename Gen::block_t blk = gen.block(plan, j);
        const uint64_t p0 = plan.head + 4 * j;
        if (p0 >= p_begin && p0 + 4 <= p_end) { // an interior block
            emit4<E, Gen>(out + (p0 - p_begin), blk);
            continue;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint64_t p = p0 + i;
            if (p >= p_begin && p < p_end)
                emit<E>(out, p - p_begin, Gen::word(blk, i));
        }
    }
}

// Box-Muller over the reference's batch layout (normal_distribution.hpp:
// 222-239: per 1024-value chunk of k values, nu = k / 2 radii then nu
// angles; out[i] = s sin, out[nu + i] = s cos) in one pass: per chunk, the
// block generates the chunk's Philox / Threefry blocks once into shared
// memory (one per thread, the chunk's words in stream order), then turns
// each (radius, angle) pair into its sine and cosine values, so every value
// is written once and no word goes through memory.
template <typename Gen, typename R>
__global__ void __launch_bounds__(256) k_normal_fused(Gen gen, StreamPlan plan,
    size_t n, R *r, R mean, R sd)
{
    using W = typename Gen::word_t;
    __shared__ W words[1024];
    const size_t nchunks = (n + 1023) / 1024;
    for (size_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const uint64_t base = static_cast<uint64_t>(c) * 1024;
        const uint32_t k = static_cast<uint32_t>(
            n - base < 1024 ? n - base : 1024);
        const uint32_t nu = k / 2;
        const uint32_t used = 2 * nu; // the odd value comes from the tail
        // words of positions [base, base + used)
        if (base < plan.head && threadIdx.x == 0) {
            const typename Gen::block_t blk = gen.block_at_start(plan);
            for (uint64_t p = base; p < plan.head && p < base + used; ++p)
                words[p - base] =
                    Gen::word(blk, plan.x + static_cast<uint32_t>(p));
        }
        const uint64_t plo = base > plan.head ? base : plan.head;
        const uint64_t phi = base + used;
        if (phi > plo) {
            const uint64_t j0 = (plo - plan.head) / 4;
            const uint64_t j1 = (phi - plan.head + 3) / 4;
            for (uint64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
                const typename Gen::block_t blk = gen.block(plan, j);
                const uint64_t p0 = plan.head + 4 * j;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const uint64_t p = p0 + i;
                    if (p >= base && p < phi)
                        words[p - base] = Gen::word(blk, i);
                }
            }
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < nu; i += blockDim.x) {
            R u1, u2;
            if constexpr (sizeof(R) == 8) {
                if constexpr (sizeof(W) == 4) {
                    u1 = u01_co_d(words[i]);
                    u2 = u01_co_d(words[nu + i]);
                } else {
                    u1 = u01_co_d64(words[i]);
                    u2 = u01_co_d64(words[nu + i]);
                }
            } else {
                if constexpr (sizeof(W) == 4) {
                    u1 = u01_co_f(words[i]);
                    u2 = u01_co_f(words[nu + i]);
                } else {
                    u1 = u01_co_f64(words[i]);
                    u2 = u01_co_f64(words[nu + i]);
                }
            }
            R s, sv, cv;
            box_muller_batch(u1, u2, sd, s, sv, cv);
            __stcs(r + base + i, fma_free_add(fma_free_mul(s, sv), mean));
            __stcs(r + base + nu + i, fma_free_add(fma_free_mul(s, cv), mean));
        }
        __syncthreads(); // words[] is reused by the next chunk
    }
}

template <typename R>
__global__ void k_normal_odd_tail(size_t n, R *r, const R *extra, R mean, R sd)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const R u = extra[0], v = extra[1];
        r[n - 1] = odd_tail_value(u, v, mean, sd);
    }
}

// ------------------------------------------------------- per-stream scalar

template <typename Eng>
__global__ void __launch_bounds__(128) k_normal_streams(typename Eng::key_t key,
    size_t nstreams, size_t per, double mean, double sd, double *r)
{
    const size_t s = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= nstreams)
        return;
    Eng eng(key, s);
    NormalScalar<double> nd(mean, sd);
    for (size_t k = 0; k < per; ++k)
        r[s * per + k] = nd(eng);
}

template <typename Eng>
__global__ void __launch_bounds__(128) k_student_t_streams(
    typename Eng::key_t key, size_t nstreams, size_t per, double df, double *r)
{
    const size_t s = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= nstreams)
        return;
    Eng eng(key, s);
    StudentTScalar st(df);
    for (size_t k = 0; k < per; ++k)
        r[s * per + k] = st(eng);
}

// ------------------------------------------------------------ host helpers

static bool valid_rng(const vsmc_cuda_rng *rng)
{
    return rng != nullptr &&
        (rng->kind == VSMC_CUDA_PHILOX4X32 ||
            rng->kind == VSMC_CUDA_THREEFRY4X64) &&
        rng->index >= 1 && rng->index <= 4;
}

template <typename Gen, Emit E, typename Out>
static int launch_plan(const Gen &gen, const StreamPlan &plan,
    uint64_t p_begin, uint64_t p_end, Out *out, cudaStream_t st)
{
    if (p_end <= p_begin)
        return VSMC_CUDA_OK;
    const uint64_t nblk = (p_end - p_begin) / 4 + 2;
    const int grid = grid_for(nblk, 256, 1, 8);
    k_plan_stream<Gen, E, Out><<<grid, 256, 0, st>>>(gen, plan, p_begin, p_end, out);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

// Emit `n` stream words/reals for `rng` following `plan`; writes the engine
// state after the plan back into *rng.
template <Emit E, typename Out32, typename Out64>
static int run_plan(vsmc_cuda_rng *rng, const StreamPlan &plan, size_t n,
    void *out, cudaStream_t st)
{
    int rc;
    if (rng->kind == VSMC_CUDA_PHILOX4X32) {
        PhiloxGen gen(*rng);
        rc = launch_plan<PhiloxGen, E>(gen, plan, 0, n, static_cast<Out32 *>(out), st);
    } else {
        ThreefryGen gen(*rng);
        rc = launch_plan<ThreefryGen, E>(gen, plan, 0, n, static_cast<Out64 *>(out), st);
    }
    if (rc != VSMC_CUDA_OK)
        return rc;
    plan_final_state(*rng, plan);
    return VSMC_CUDA_OK;
}

template <typename R>
static int rng_normal_impl(
    vsmc_cuda_rng *rng, size_t n, R *r, R mean, R sd, void *stream)
{
    if (!valid_rng(rng) || (r == nullptr && n))
        return VSMC_CUDA_ERR_ARG;
    if (n == 0)
        return VSMC_CUDA_OK;
    cudaStream_t st = as_stream(stream);
    const bool odd = (n % 2) != 0;
    // the n u01 words of the chunked calls, then (odd n) two scalar words
    const StreamPlan plan = plan_chunked_calls(*rng, n, odd ? 2 : 0);
    constexpr Emit E = sizeof(R) == 8 ? Emit::U01D : Emit::U01F;
    Scratch scratch(st);
    R *extra = nullptr;
    if (odd) {
        extra = scratch.get<R>(2);
        if (extra == nullptr)
            return VSMC_CUDA_ERR_ALLOC;
    }
    int rc = VSMC_CUDA_OK;
    // the pairs of every chunk in one pass; the odd value's two words
    // (positions n, n + 1) through the stream kernel
    const size_t nchunks = (n + 1023) / 1024;
    const int grid = static_cast<int>(
        std::min<size_t>(nchunks, static_cast<size_t>(num_sms()) * 8));
    if (rng->kind == VSMC_CUDA_PHILOX4X32) {
        PhiloxGen gen(*rng);
        if (n >= 2)
            k_normal_fused<PhiloxGen, R><<<grid, 256, 0, st>>>(
                gen, plan, n, r, mean, sd);
        if (odd)
            rc = launch_plan<PhiloxGen, E>(gen, plan, n, n + 2, extra, st);
    } else {
        ThreefryGen gen(*rng);
        if (n >= 2)
            k_normal_fused<ThreefryGen, R><<<grid, 256, 0, st>>>(
                gen, plan, n, r, mean, sd);
        if (odd)
            rc = launch_plan<ThreefryGen, E>(gen, plan, n, n + 2, extra, st);
    }
    VSMC_CUDA_CHECK_LAUNCH();
    if (rc != VSMC_CUDA_OK)
        return rc;
    if (odd) {
        k_normal_odd_tail<R><<<1, 32, 0, st>>>(n, r, extra, mean, sd);
        VSMC_CUDA_CHECK_LAUNCH();
    }
    plan_final_state(*rng, plan);
    return VSMC_CUDA_OK;
}

} // namespace vsmc_cuda

using namespace vsmc_cuda;

extern "C" {

int vsmc_cuda_rng_init(vsmc_cuda_rng *rng, int kind, uint64_t seed)
{
    if (rng == nullptr ||
        (kind != VSMC_CUDA_PHILOX4X32 && kind != VSMC_CUDA_THREEFRY4X64))
        return VSMC_CUDA_ERR_ARG;
    std::memset(rng, 0, sizeof(*rng));
    rng->kind = kind;
    rng->index = 4;
    rng->key[0] = kind == VSMC_CUDA_PHILOX4X32 ? (seed & 0xFFFFFFFFull) : seed;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_rng_set_key(vsmc_cuda_rng *rng, int n, const uint64_t *key)
{
    if (rng == nullptr || key == nullptr || n < 0)
        return VSMC_CUDA_ERR_ARG;
    const int limbs = rng->kind == VSMC_CUDA_PHILOX4X32 ? 2 : 4;
    uint64_t k[4] = {0, 0, 0, 0};
    for (int i = 0; i < limbs && i < n; ++i)
        k[i] = rng->kind == VSMC_CUDA_PHILOX4X32 ? (key[i] & 0xFFFFFFFFull)
                                                  : key[i];
    std::memcpy(rng->key, k, sizeof(k));
    std::memset(rng->ctr, 0, sizeof(rng->ctr));
    rng->index = 4;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_rng_set_ctr(vsmc_cuda_rng *rng, int n, const uint64_t *ctr)
{
    if (rng == nullptr || ctr == nullptr || n < 0)
        return VSMC_CUDA_ERR_ARG;
    uint64_t c[4] = {0, 0, 0, 0};
    for (int i = 0; i < 4 && i < n; ++i)
        c[i] = rng->kind == VSMC_CUDA_PHILOX4X32 ? (ctr[i] & 0xFFFFFFFFull)
                                                  : ctr[i];
    std::memcpy(rng->ctr, c, sizeof(c));
    rng->index = 4;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_philox4x32_blocks(const uint32_t key[2], const uint32_t ctr0[4],
    size_t nblocks, uint32_t *out, void *stream)
{
    if (key == nullptr || ctr0 == nullptr || (out == nullptr && nblocks))
        return VSMC_CUDA_ERR_ARG;
    if (nblocks == 0)
        return VSMC_CUDA_OK;
    const int grid = grid_for(nblocks, 256, 1, 8);
    cudaStream_t st = as_stream(stream);
    if (reinterpret_cast<uintptr_t>(out) % 16 == 0)
        k_philox_blocks<true><<<grid, 256, 0, st>>>(key[0], key[1], ctr0[0],
            ctr0[1], ctr0[2], ctr0[3], nblocks, out);
    else
        k_philox_blocks<false><<<grid, 256, 0, st>>>(key[0], key[1], ctr0[0],
            ctr0[1], ctr0[2], ctr0[3], nblocks, out);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_threefry4x64_blocks(const uint64_t key[4],
    const uint64_t ctr0[4], size_t nblocks, uint64_t *out, void *stream)
{
    if (key == nullptr || ctr0 == nullptr || (out == nullptr && nblocks))
        return VSMC_CUDA_ERR_ARG;
    if (nblocks == 0)
        return VSMC_CUDA_OK;
    const int grid = grid_for(nblocks, 256, 1, 8);
    cudaStream_t st = as_stream(stream);
    if (reinterpret_cast<uintptr_t>(out) % 16 == 0)
        k_threefry_blocks<true><<<grid, 256, 0, st>>>(key[0], key[1], key[2],
            key[3], ctr0[0], ctr0[1], ctr0[2], ctr0[3], nblocks, out);
    else
        k_threefry_blocks<false><<<grid, 256, 0, st>>>(key[0], key[1], key[2],
            key[3], ctr0[0], ctr0[1], ctr0[2], ctr0[3], nblocks, out);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_rng_rand(vsmc_cuda_rng *rng, size_t n, void *r, void *stream)
{
    if (!valid_rng(rng) || (r == nullptr && n))
        return VSMC_CUDA_ERR_ARG;
    const StreamPlan plan = plan_single_call(*rng, n);
    return run_plan<Emit::Word, uint32_t, uint64_t>(
        rng, plan, n, r, as_stream(stream));
}

int vsmc_cuda_rng_u01(vsmc_cuda_rng *rng, size_t n, double *r, void *stream)
{
    if (!valid_rng(rng) || (r == nullptr && n))
        return VSMC_CUDA_ERR_ARG;
    const StreamPlan plan = plan_chunked_calls(*rng, n, 0);
    return run_plan<Emit::U01D, double, double>(
        rng, plan, n, r, as_stream(stream));
}

int vsmc_cuda_rng_u01_f32(vsmc_cuda_rng *rng, size_t n, float *r, void *stream)
{
    if (!valid_rng(rng) || (r == nullptr && n))
        return VSMC_CUDA_ERR_ARG;
    const StreamPlan plan = plan_chunked_calls(*rng, n, 0);
    return run_plan<Emit::U01F, float, float>(
        rng, plan, n, r, as_stream(stream));
}

int vsmc_cuda_rng_normal(vsmc_cuda_rng *rng, size_t n, double *r, double mean,
    double stddev, void *stream)
{
    return rng_normal_impl<double>(rng, n, r, mean, stddev, stream);
}

int vsmc_cuda_rng_normal_f32(vsmc_cuda_rng *rng, size_t n, float *r,
    float mean, float stddev, void *stream)
{
    return rng_normal_impl<float>(rng, n, r, mean, stddev, stream);
}

int vsmc_cuda_normal_streams(int kind, const uint64_t key[4], size_t nstreams,
    size_t per_stream, double mean, double stddev, double *r, void *stream)
{
    if (key == nullptr || (r == nullptr && nstreams && per_stream))
        return VSMC_CUDA_ERR_ARG;
    if (nstreams == 0 || per_stream == 0)
        return VSMC_CUDA_OK;
    if (nstreams > 0xFFFFFFFFull)
        return VSMC_CUDA_ERR_SIZE;
    const int grid = static_cast<int>((nstreams + 127) / 128);
    cudaStream_t st = as_stream(stream);
    if (kind == VSMC_CUDA_PHILOX4X32)
        k_normal_streams<PhiloxScalar><<<grid, 128, 0, st>>>(
            PhiloxScalar::make_key(key), nstreams, per_stream, mean, stddev, r);
    else if (kind == VSMC_CUDA_THREEFRY4X64)
        k_normal_streams<ThreefryScalar><<<grid, 128, 0, st>>>(
            ThreefryScalar::make_key(key), nstreams, per_stream, mean, stddev,
            r);
    else
        return VSMC_CUDA_ERR_ARG;
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_student_t_streams(int kind, const uint64_t key[4],
    size_t nstreams, size_t per_stream, double df, double *r, void *stream)
{
    if (key == nullptr || (r == nullptr && nstreams && per_stream) ||
        !(df > 0))
        return VSMC_CUDA_ERR_ARG;
    if (nstreams == 0 || per_stream == 0)
        return VSMC_CUDA_OK;
    if (nstreams > 0xFFFFFFFFull)
        return VSMC_CUDA_ERR_SIZE;
    const int grid = static_cast<int>((nstreams + 127) / 128);
    cudaStream_t st = as_stream(stream);
    if (kind == VSMC_CUDA_PHILOX4X32)
        k_student_t_streams<PhiloxScalar><<<grid, 128, 0, st>>>(
            PhiloxScalar::make_key(key), nstreams, per_stream, df, r);
    else if (kind == VSMC_CUDA_THREEFRY4X64)
        k_student_t_streams<ThreefryScalar><<<grid, 128, 0, st>>>(
            ThreefryScalar::make_key(key), nstreams, per_stream, df, r);
    else
        return VSMC_CUDA_ERR_ARG;
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

} // extern "C"
