// vsmc_cuda_device.cuh - device primitives for model code run by the fused
// particle-filter step of libvsmc_cuda (sm_103a).
//
// A user model (see vsmc_cuda_filter.cuh) draws its randomness from a
// ParticleRng: the per-particle Philox4x32-10 stream the filter assigns to
// particle i at step t.  The pieces here are the counter-based generator,
// the reference's integer -> real maps and an FP32 Box-Muller pair; the
// library's own kernels use the same definitions, so a model written against
// them draws exactly the words the library's built-in models draw.
//
// Generator constants are the published Random123 ones, as they appear in
// the reference (rng/philox.hpp:76-101).  The u01 maps are those of
// rng/u01.hpp:126-172; every scale is a power of two, so they are exact.
#ifndef VSMC_CUDA_DEVICE_CUH
#define VSMC_CUDA_DEVICE_CUH

#include <cstdint>
#include <cuda_runtime.h>

namespace vsmc_cuda
{

struct u32x4 {
    uint32_t x, y, z, w;
};

// Philox4x32-10 on one counter block (no pre-increment).  Ten rounds; the
// key is bumped by the Weyl constants before rounds 2..10
// (rng/philox.hpp:162-232).
__device__ __forceinline__ u32x4 philox4x32_10(
    uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
    uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        // each 32 x 32 product once, as one widening multiply
        const uint64_t pa = static_cast<uint64_t>(c2) * 0xCD9E8D57u;
        const uint64_t pb = static_cast<uint64_t>(c0) * 0xD2511F53u;
        const uint32_t hi_a = static_cast<uint32_t>(pa >> 32);
        const uint32_t lo_a = static_cast<uint32_t>(pa);
        const uint32_t hi_b = static_cast<uint32_t>(pb >> 32);
        const uint32_t lo_b = static_cast<uint32_t>(pb);
        const uint32_t n0 = hi_a ^ k0 ^ c1;
        const uint32_t n2 = hi_b ^ k1 ^ c3;
        c0 = n0;
        c1 = lo_a;
        c2 = n2;
        c3 = lo_b;
    }
    return {c0, c1, c2, c3};
}

// ---------------------------------------------------------------- u01

// [0,1) from 32 bits in double: u * 2^-32
__host__ __device__ __forceinline__ double u01_co_d(uint32_t u)
{
    return static_cast<double>(u) * 0x1p-32;
}
// [0,1) from 32 bits in float: (u >> 8) * 2^-24
__host__ __device__ __forceinline__ float u01_co_f(uint32_t u)
{
    return static_cast<float>(u >> 8) * 0x1p-24f;
}
// (0,1] from 32 bits in float: (u >> 8) * 2^-24 + 2^-24
__host__ __device__ __forceinline__ float u01_oc_f(uint32_t u)
{
    return static_cast<float>(u >> 8) * 0x1p-24f + 0x1p-24f;
}
// [0,1) from 64 bits in double: (u >> 11) * 2^-53
__host__ __device__ __forceinline__ double u01_co_d64(uint64_t u)
{
    return static_cast<double>(u >> 11) * 0x1p-53;
}
// [0,1) from 64 bits in float: (u >> 40) * 2^-24
__host__ __device__ __forceinline__ float u01_co_f64(uint64_t u)
{
    return static_cast<float>(u >> 40) * 0x1p-24f;
}

// 2*pi as the reference's const_pi_2 (math/constants.hpp:66)
constexpr double kPi2 = 6.283185307179586476925286766559005768394;
constexpr float kPi2f = 6.283185307179586476925286766559005768394f;

// FP32 standard-normal pair: Box-Muller with a (0,1] radius uniform and a
// [0,1) angle, on the SFU: the hardware log2, the reciprocal square root for
// the radius, and the hardware sine and cosine of 2 pi u in [0, 2 pi).
// The hardware log's absolute error (about 1e-7 in ln u) is not small
// against ln u itself for u near 1, so there -2 ln u1 = -2 ln(1 - e), with
// e = 1 - u1 exact in the 24-bit grid, comes from the series
// 2 (e + e^2/2 + e^3/3 + e^4/4) (relative error below e^4 / 5 < 2^-22 for
// e < 2^-5).  Elsewhere the log's error is below 4e-6 of ln u, and a normal
// differs from the one with correctly rounded functions by ~2e-6 relative.
__device__ __forceinline__ void normal_pair_f(uint32_t w0, uint32_t w1,
    float &z1, float &z2)
{
    const uint32_t m = w0 >> 8;
    const float e = static_cast<float>(0xFFFFFFu - m) * 0x1p-24f;
    const float u1 = 1.0f - e; // = u01_oc_f(w0), exactly
    const float u2 = u01_co_f(w1);
    const float ser = 2.0f * e *
        fmaf(e, fmaf(e, fmaf(e, 0.25f, 0.333333343f), 0.5f), 1.0f);
    const float l = e < 0x1p-5f ? ser : -2.0f * __logf(u1);
    const float r = l > 0.0f ? l * rsqrtf(l) : 0.0f;
    float sv, cv;
    __sincosf(6.28318530717958648f * u2, &sv, &cv);
    z1 = r * cv;
    z2 = r * sv;
}

// ------------------------------------------------------- particle stream

// The random words of particle i at step t: Philox4x32-10 with key
// {t, seed} and counters {b, i, 0, 0} for b = 1, 2, ..., i.e. the stream of
// an engine placed at counter {0, i, 0, 0} in the reference's pre-increment
// convention (rng/philox.hpp:263-269).  Words are taken in block order
// (x, y, z, w of block 1, then block 2, ...).  The object lives in registers:
// when every call is inlined the block index folds to a constant and no
// state is kept.
//
// The filter's resample-move sweeps (vsmc_cuda_pf_set_mcmc) use counters
// {2 + k, i, 0, 0}; a model that draws more than four words per step shares
// those blocks with them, which matters only if both are used.
class ParticleRng
{
    public:
    __device__ __forceinline__ ParticleRng(
        uint32_t t, uint32_t seed, uint32_t i)
        : t_(t), seed_(seed), i_(i)
    {
    }

    // the next 32-bit word
    __device__ __forceinline__ uint32_t operator()()
    {
        if (k_ == 4) {
            ++b_;
            blk_ = philox4x32_10(b_, i_, 0u, 0u, t_, seed_);
            k_ = 0;
        }
        const uint32_t w =
            k_ == 0 ? blk_.x : (k_ == 1 ? blk_.y : (k_ == 2 ? blk_.z : blk_.w));
        ++k_;
        return w;
    }

    // [0, 1) from one word, the reference's u01_co for float
    __device__ __forceinline__ float u01() { return u01_co_f((*this)()); }

    // two independent N(0, 1) from two words (normal_pair_f)
    __device__ __forceinline__ void normal_pair(float &z1, float &z2)
    {
        const uint32_t w0 = (*this)();
        const uint32_t w1 = (*this)();
        normal_pair_f(w0, w1, z1, z2);
    }

    // one N(0, 1); the pair's second value is kept for the next call, as
    // NormalDistribution caches its sine value (rng/normal_distribution.hpp:
    // 199-216)
    __device__ __forceinline__ float normal()
    {
        if (have_) {
            have_ = false;
            return cached_;
        }
        float z1, z2;
        normal_pair(z1, z2);
        cached_ = z2;
        have_ = true;
        return z1;
    }

    __device__ __forceinline__ uint32_t step() const { return t_; }
    __device__ __forceinline__ uint32_t particle() const { return i_; }

    private:
    uint32_t t_, seed_, i_;
    uint32_t b_ = 0;
    int k_ = 4;
    u32x4 blk_ = {0, 0, 0, 0};
    bool have_ = false;
    float cached_ = 0.0f;
};

} // namespace vsmc_cuda

#endif // VSMC_CUDA_DEVICE_CUH
