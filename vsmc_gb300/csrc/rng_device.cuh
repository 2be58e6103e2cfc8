// Engine stream plans and scalar distributions (device side).
//
// A CounterEngine (rng/counter.hpp:288-496) hands out words from a buffered
// block gen(ctr); its bulk path operator()(n, r) drains the buffer, then
// generates whole blocks in generator calls of at most 256 blocks
// (counter.hpp:370-386), then takes the last < 4 words through the scalar
// path.  Inside one generator call the counters of the blocks are made by
// increment(ctr, n, ctr_block) (counter.hpp:230-262): when a call reaches
// the top of the low limb, increment(ctr, nskip) (counter.hpp:78-89) also
// carries into limb 1 for the block whose low limb is exactly all ones, and
// when that block ends the call the carry stays in the engine counter.
//
// A StreamPlan lays out the stream of one sequence of such calls as global
// blocks j = 0, 1, ... after the current block gen(C0), so a kernel can
// compute any block's counter in O(1):
//   A(j) = C0 + 1 + j + 2^W * (extra carries before j, plus j's own),
// where the extra carries sit only at bulk blocks whose low limb is all ones.
#pragma once

#include "common.cuh"

#include <math_constants.h>

namespace vsmc_cuda
{

struct StreamPlan {
    uint64_t c0[4];       // engine counter at the start
    uint32_t x;           // engine index at the start (1..4)
    uint32_t head;        // words taken from the current block gen(C0)
    uint32_t periodic_x4; // periodic part: 1 = 256 bulk blocks per call,
                          //                0 = 255 bulk + 1 scalar per call
    uint32_t simple;      // no block's low counter limb reaches all ones:
                          // block j's counter is c0 + j + 1, no carry
    uint64_t first_last;  // first block of the final (or only) call
    uint64_t nb_last;     // bulk blocks in the final call
    uint64_t n_total;     // words in the whole plan
    uint64_t total_blocks;
};

__host__ __device__ inline void plan_block_type(
    const StreamPlan &p, uint64_t j, bool &bulk, bool &chunk_end)
{
    if (j < p.first_last) {
        const uint64_t loc = j % 256;
        if (p.periodic_x4) {
            bulk = true;
            chunk_end = loc == 255;
        } else {
            bulk = loc < 255;
            chunk_end = loc == 254;
        }
    } else {
        const uint64_t loc = j - p.first_last;
        bulk = loc < p.nb_last;
        chunk_end = bulk && (loc % 256 == 255 || loc + 1 == p.nb_last);
    }
}

// Number of extra limb-1 carries applying to block j (W = 32 or 64 bits in
// the low limb).
template <int W>
__host__ __device__ inline uint64_t plan_extra_carries(
    const StreamPlan &p, uint64_t j)
{
    // blocks whose low limb is all ones: j' = first + k * 2^W
    uint64_t first;
    if (W == 32)
        first = static_cast<uint32_t>(0xFFFFFFFEu - static_cast<uint32_t>(p.c0[0]));
    else
        first = 0xFFFFFFFFFFFFFFFEull - p.c0[0];
    uint64_t extra = 0;
    bool bulk, cend;
    // earlier chunk-end carries (at most a handful for any feasible length)
    for (int k = 0; k < 8; ++k) {
        const uint64_t jj = W == 32 ? first + (static_cast<uint64_t>(k) << 32)
                                    : (k == 0 ? first : ~0ull);
        if (W == 64 && k > 0)
            break;
        if (jj >= j)
            break;
        plan_block_type(p, jj, bulk, cend);
        if (bulk && cend)
            ++extra;
    }
    // own carry
    bool own_ff;
    if (W == 32)
        own_ff = static_cast<uint32_t>(p.c0[0] + 1 + j) == 0xFFFFFFFFu;
    else
        own_ff = (p.c0[0] + 1 + j) == 0xFFFFFFFFFFFFFFFFull;
    plan_block_type(p, j, bulk, cend);
    if (bulk && own_ff)
        ++extra;
    return extra;
}

__host__ __device__ inline void plan_counter32(
    const StreamPlan &p, uint64_t j, uint32_t c[4])
{
    c[0] = static_cast<uint32_t>(p.c0[0]);
    c[1] = static_cast<uint32_t>(p.c0[1]);
    c[2] = static_cast<uint32_t>(p.c0[2]);
    c[3] = static_cast<uint32_t>(p.c0[3]);
    ctr32_add(c, j + 1);
    const uint64_t extra = plan_extra_carries<32>(p, j);
    for (uint64_t e = 0; e < extra; ++e)
        ctr32_carry1(c);
}

__host__ __device__ inline void plan_counter64(
    const StreamPlan &p, uint64_t j, uint64_t c[4])
{
    for (int i = 0; i < 4; ++i)
        c[i] = p.c0[i];
    ctr64_add(c, j + 1);
    const uint64_t extra = plan_extra_carries<64>(p, j);
    for (uint64_t e = 0; e < extra; ++e)
        ctr64_carry1(c);
}

inline void plan_finish(StreamPlan &p)
{
    p.head = static_cast<uint32_t>(
        p.n_total < 4 - p.x ? p.n_total : 4 - p.x);
    p.total_blocks = p.n_total > p.head ? (p.n_total - p.head + 3) / 4 : 0;
    // low limbs c0 + 1 .. c0 + total_blocks all below 0xFFFFFFFF (for
    // either engine): no carry and no extra carry of the bulk path
    p.simple = p.total_blocks <= 0xFFFFFFFEull &&
            p.c0[0] <= 0xFFFFFFFEull - p.total_blocks
        ? 1u
        : 0u;
}

// One CounterEngine::operator()(n, r) call.
inline StreamPlan plan_single_call(const vsmc_cuda_rng &rng, size_t n)
{
    StreamPlan p = {};
    for (int i = 0; i < 4; ++i)
        p.c0[i] = rng.ctr[i];
    p.x = rng.index;
    p.periodic_x4 = 1;
    p.first_last = 0;
    const uint64_t remain = 4 - p.x;
    p.nb_last = n < remain ? 0 : (n - remain) / 4;
    p.n_total = n;
    plan_finish(p);
    return p;
}

// u01_distribution(rng, n, r): calls of 1024 words, then one of n % 1024;
// `extra` scalar words follow (the odd-n tail of normal_distribution).
inline StreamPlan plan_chunked_calls(
    const vsmc_cuda_rng &rng, size_t n, size_t extra)
{
    StreamPlan p = {};
    for (int i = 0; i < 4; ++i)
        p.c0[i] = rng.ctr[i];
    p.x = rng.index;
    const uint64_t nf = n / 1024;
    const uint64_t r = n % 1024;
    p.periodic_x4 = p.x == 4 ? 1 : 0;
    p.first_last = 256 * nf;
    const uint64_t remain = 4 - p.x;
    p.nb_last = r < remain ? 0 : (r - remain) / 4;
    p.n_total = n + extra;
    plan_finish(p);
    return p;
}

// Engine state after all words of the plan.
inline void plan_final_state(vsmc_cuda_rng &rng, const StreamPlan &p)
{
    if (p.total_blocks == 0) {
        rng.index = static_cast<uint32_t>(p.x + p.n_total);
        return;
    }
    const uint64_t J = p.total_blocks - 1;
    if (rng.kind == VSMC_CUDA_PHILOX4X32) {
        uint32_t c[4];
        plan_counter32(p, J, c);
        for (int i = 0; i < 4; ++i)
            rng.ctr[i] = c[i];
    } else {
        uint64_t c[4];
        plan_counter64(p, J, c);
        for (int i = 0; i < 4; ++i)
            rng.ctr[i] = c[i];
    }
    rng.index = static_cast<uint32_t>((p.n_total - p.head - 1) % 4 + 1);
}

// ------------------------------------------------------- block generators

struct PhiloxGen {
    using word_t = uint32_t;
    using block_t = u32x4;
    uint32_t k0, k1;

    explicit PhiloxGen(const vsmc_cuda_rng &r)
        : k0(static_cast<uint32_t>(r.key[0])),
          k1(static_cast<uint32_t>(r.key[1]))
    {
    }

    __device__ block_t block_at_start(const StreamPlan &p) const
    {
        return philox4x32_10(static_cast<uint32_t>(p.c0[0]),
            static_cast<uint32_t>(p.c0[1]), static_cast<uint32_t>(p.c0[2]),
            static_cast<uint32_t>(p.c0[3]), k0, k1);
    }

    __device__ block_t block(const StreamPlan &p, uint64_t j) const
    {
        uint32_t c[4];
        if (p.simple) {
            c[0] = static_cast<uint32_t>(p.c0[0] + 1 + j);
            c[1] = static_cast<uint32_t>(p.c0[1]);
            c[2] = static_cast<uint32_t>(p.c0[2]);
            c[3] = static_cast<uint32_t>(p.c0[3]);
        } else {
            plan_counter32(p, j, c);
        }
        return philox4x32_10(c[0], c[1], c[2], c[3], k0, k1);
    }

    __device__ static word_t word(const block_t &b, uint32_t i)
    {
        return i == 0 ? b.x : (i == 1 ? b.y : (i == 2 ? b.z : b.w));
    }
};

struct ThreefryGen {
    using word_t = uint64_t;
    using block_t = u64x4;
    uint64_t k[4];

    explicit ThreefryGen(const vsmc_cuda_rng &r)
    {
        for (int i = 0; i < 4; ++i)
            k[i] = r.key[i];
    }

    __device__ block_t block_at_start(const StreamPlan &p) const
    {
        return threefry4x64_20(
            {p.c0[0], p.c0[1], p.c0[2], p.c0[3]}, k[0], k[1], k[2], k[3]);
    }

    __device__ block_t block(const StreamPlan &p, uint64_t j) const
    {
        uint64_t c[4];
        if (p.simple) {
            c[0] = p.c0[0] + 1 + j;
            c[1] = p.c0[1];
            c[2] = p.c0[2];
            c[3] = p.c0[3];
        } else {
            plan_counter64(p, j, c);
        }
        return threefry4x64_20({c[0], c[1], c[2], c[3]}, k[0], k[1], k[2], k[3]);
    }

    __device__ static word_t word(const block_t &b, uint32_t i)
    {
        return i == 0 ? b.x : (i == 1 ? b.y : (i == 2 ? b.z : b.w));
    }
};

// ------------------------------------------------------------- emitters

template <int E>
struct EmitTag {
};

template <auto E, typename Out>
__device__ __forceinline__ void emit(Out *out, size_t p, uint32_t w)
{
    if constexpr (static_cast<int>(E) == 0)
        out[p] = static_cast<Out>(w);
    else if constexpr (static_cast<int>(E) == 1)
        out[p] = static_cast<Out>(u01_co_d(w));
    else
        out[p] = static_cast<Out>(u01_co_f(w));
}

template <auto E, typename Out>
__device__ __forceinline__ void emit(Out *out, size_t p, uint64_t w)
{
    if constexpr (static_cast<int>(E) == 0)
        out[p] = static_cast<Out>(w);
    else if constexpr (static_cast<int>(E) == 1)
        out[p] = static_cast<Out>(u01_co_d64(w));
    else
        out[p] = static_cast<Out>(u01_co_f64(w));
}

// ----------------------------------------------- contraction-free arithmetic

__device__ __forceinline__ double fma_free_mul(double a, double b)
{
    return __dmul_rn(a, b);
}
__device__ __forceinline__ double fma_free_add(double a, double b)
{
    return __dadd_rn(a, b);
}
__device__ __forceinline__ float fma_free_mul(float a, float b)
{
    return __fmul_rn(a, b);
}
__device__ __forceinline__ float fma_free_add(float a, float b)
{
    return __fadd_rn(a, b);
}

// Batch Box-Muller step for one (radius, angle) pair
// (normal_distribution.hpp:229-238): s = sd * sqrt(-2 log u1), angle 2 pi u2.
__device__ __forceinline__ void box_muller_batch(
    double u1, double u2, double sd, double &s, double &sv, double &cv)
{
    double t = log(u1);
    t = __dmul_rn(-2.0, t);
    t = sqrt(t);
    const double th = __dmul_rn(kPi2, u2);
    sincos(th, &sv, &cv);
    s = __dmul_rn(sd, t);
}

__device__ __forceinline__ void box_muller_batch(
    float u1, float u2, float sd, float &s, float &sv, float &cv)
{
    float t = logf(u1);
    t = __fmul_rn(-2.0f, t);
    t = sqrtf(t);
    const float th = __fmul_rn(kPi2f, u2);
    sincosf(th, &sv, &cv);
    s = __fmul_rn(sd, t);
}

// last value of an odd-length batch (normal_distribution.hpp:259-266)
__device__ __forceinline__ double odd_tail_value(
    double u, double v, double mean, double sd)
{
    const double a = __dmul_rn(sd, sqrt(__dmul_rn(-2.0, log(u))));
    return __dadd_rn(mean, __dmul_rn(a, cos(__dmul_rn(kPi2, v))));
}

__device__ __forceinline__ float odd_tail_value(
    float u, float v, float mean, float sd)
{
    const float a = __fmul_rn(sd, sqrtf(__fmul_rn(-2.0f, logf(u))));
    return __fadd_rn(mean, __fmul_rn(a, cosf(__fmul_rn(kPi2f, v))));
}

// ------------------------------------------------- scalar-path engines

// CounterEngine scalar operator() (counter.hpp:347-355) for one stream placed
// at counter {0, s, 0, 0}.
struct PhiloxScalar {
    struct key_t {
        uint32_t k0, k1;
    };
    static key_t make_key(const uint64_t *k)
    {
        return {static_cast<uint32_t>(k[0]), static_cast<uint32_t>(k[1])};
    }
    uint32_t k0, k1;
    uint32_t c[4];
    u32x4 buf;
    int index;

    __device__ PhiloxScalar(key_t k, uint64_t s) : k0(k.k0), k1(k.k1), index(4)
    {
        c[0] = 0;
        c[1] = static_cast<uint32_t>(s);
        c[2] = 0;
        c[3] = 0;
    }

    __device__ uint32_t next()
    {
        if (index == 4) {
            ctr32_add(c, 1);
            buf = philox4x32_10(c[0], c[1], c[2], c[3], k0, k1);
            index = 0;
        }
        const int i = index++;
        return i == 0 ? buf.x : (i == 1 ? buf.y : (i == 2 ? buf.z : buf.w));
    }

    __device__ double u01d() { return u01_co_d(next()); }
};

struct ThreefryScalar {
    struct key_t {
        uint64_t k[4];
    };
    static key_t make_key(const uint64_t *k)
    {
        return {{k[0], k[1], k[2], k[3]}};
    }
    uint64_t k[4];
    uint64_t c[4];
    u64x4 buf;
    int index;

    __device__ ThreefryScalar(key_t kk, uint64_t s) : index(4)
    {
        for (int i = 0; i < 4; ++i)
            k[i] = kk.k[i];
        c[0] = 0;
        c[1] = s;
        c[2] = 0;
        c[3] = 0;
    }

    __device__ uint64_t next()
    {
        if (index == 4) {
            ctr64_add(c, 1);
            buf = threefry4x64_20({c[0], c[1], c[2], c[3]}, k[0], k[1], k[2], k[3]);
            index = 0;
        }
        const int i = index++;
        return i == 0 ? buf.x : (i == 1 ? buf.y : (i == 2 ? buf.z : buf.w));
    }

    __device__ double u01d() { return u01_co_d64(next()); }
};

// NormalDistribution<double> scalar draws with the cached second value
// (normal_distribution.hpp:199-216).
template <typename R>
struct NormalScalar {
    R mean, sd, v;
    bool saved;

    __device__ NormalScalar(R m, R s) : mean(m), sd(s), v(0), saved(false) {}

    template <typename Eng>
    __device__ R operator()(Eng &eng)
    {
        R z;
        if (saved) {
            z = v;
            saved = false;
        } else {
            const R u1 = sqrt(__dmul_rn(-2.0, log(eng.u01d())));
            const R u2 = __dmul_rn(kPi2, eng.u01d());
            double sv, cv;
            sincos(u2, &sv, &cv);
            z = __dmul_rn(u1, cv);
            v = __dmul_rn(u1, sv);
            saved = true;
        }
        return __dadd_rn(mean, __dmul_rn(sd, z));
    }
};

// StudentTDistribution<double>: normal first, then chi-squared = Gamma(df/2,
// 2) by the reference's four gamma algorithms
// (student_t_distribution.hpp:78-91, gamma_distribution.hpp:57-216).
//
// Every rejection loop accepts with probability above 1/2 per try for any
// alpha, so a variate needing kGammaMaxTries tries means a broken engine or
// argument: the loop then stops, the variate is NaN and `err` gets
// DEV_ERR_BOUND.
constexpr int kGammaMaxTries = 1 << 16;

struct StudentTScalar {
    double df, alpha, d, c;
    int alg; // 0 T (alpha < 0.6), 1 W (alpha < 1), 2 N (alpha > 1), 3 E
    uint32_t err = 0;
    NormalScalar<double> normal;

    __device__ explicit StudentTScalar(double nu)
        : df(nu), alpha(nu / 2), d(0), c(0), normal(0, 1)
    {
        if (alpha < 0.6) {
            alg = 0;
            d = 1 - alpha;
            c = 1 / alpha;
        } else if (alpha < 1) {
            alg = 1;
            d = pow(alpha, alpha / (1 - alpha)) * (1 - alpha);
            c = 1 / alpha;
        } else if (alpha > 1) {
            alg = 2;
            d = alpha - 1.0 / 3;
            c = 1 / (3 * sqrt(d));
        } else {
            alg = 3;
        }
    }

    template <typename Eng>
    __device__ double gamma(Eng &eng)
    {
        double r = CUDART_NAN;
        int tries = 0;
        if (alg == 0) {
            for (; tries < kGammaMaxTries; ++tries) {
                double u = eng.u01d();
                double e = -log(eng.u01d());
                if (u > d) {
                    u = -log(__dmul_rn(c, 1 - u));
                    e = __dadd_rn(e, u);
                    u = __dadd_rn(d, __dmul_rn(alpha, u));
                }
                const double x = exp(__dmul_rn(c, log(u)));
                if (fabs(x) < e) {
                    r = x;
                    break;
                }
            }
        } else if (alg == 1) {
            for (; tries < kGammaMaxTries; ++tries) {
                const double u = -log(eng.u01d());
                const double e = -log(eng.u01d());
                const double x = exp(__dmul_rn(c, log(u)));
                if (!(__dadd_rn(u, e) < __dadd_rn(d, x))) {
                    r = x;
                    break;
                }
            }
        } else if (alg == 2) {
            NormalScalar<double> rnorm(0, 1);
            for (; tries < kGammaMaxTries; ++tries) {
                const double u = eng.u01d();
                double w = 0, v = 0;
                bool pos = false;
                for (; tries < kGammaMaxTries; ++tries) {
                    w = rnorm(eng);
                    v = __dadd_rn(1.0, __dmul_rn(c, w));
                    if (!(v <= 0)) {
                        pos = true;
                        break;
                    }
                }
                if (!pos)
                    break;
                v = __dmul_rn(__dmul_rn(v, v), v);
                const double w2 = __dmul_rn(w, w);
                double e = __dadd_rn(1.0, -__dmul_rn(__dmul_rn(0.0331, w2), w2));
                if (u < e) {
                    r = __dmul_rn(d, v);
                    break;
                }
                e = __dadd_rn(w2 / 2,
                    __dmul_rn(d, __dadd_rn(__dadd_rn(1.0, -v), log(v))));
                if (log(u) < e) {
                    r = __dmul_rn(d, v);
                    break;
                }
            }
        } else {
            r = -log(eng.u01d());
        }
        if (tries >= kGammaMaxTries)
            err |= DEV_ERR_BOUND;
        return __dmul_rn(2.0, r);
    }

    template <typename Eng>
    __device__ double operator()(Eng &eng)
    {
        const double z = normal(eng);
        const double u = df / gamma(eng);
        return __dmul_rn(z, sqrt(u));
    }
};

} // namespace vsmc_cuda
