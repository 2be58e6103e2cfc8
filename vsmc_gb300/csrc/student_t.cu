// Student-t variates from a vsmc_cuda_rng engine with the batch semantics of
// the reference's C ABI vsmc_rng_student_t (lib/src/vsmc_rng.cpp:41-64,
// 207), that is student_t_distribution(rng, n, r, df)
// (rng/student_t_distribution.hpp:97-128):
//
//   for each chunk of at most 1024 variates, in order:
//     r <- chi-squared(df) = Gamma(df / 2, 2) by the batch gamma
//          (rng/gamma_distribution.hpp:230-410): one vectorised attempt of
//          the whole chunk (algorithm T, W, N or E by alpha), the accepted
//          values packed first in index order, then one scalar
//          GammaDistribution draw for each rejected slot;
//     r <- sqrt(r * (1 / df));
//     z <- a batch of N(0, 1) (rng/normal_distribution.hpp:222-267);
//     r <- z / r.
//
// Every engine call is reproduced word for word: a batch of n <= 1024 words
// is the engine's bulk path (counter.hpp:357-390: drain the buffered block,
// one generator call of whole blocks whose counters follow increment(ctr,
// n, ctr_block), counter.hpp:230-262, including its extra limb-1 carry at
// an all-ones low limb, then scalar draws for the last < 4 words), a scalar
// draw is the engine's operator() (counter.hpp:347-355).  The stream is
// sequential by construction -- how many words a chunk consumes depends on
// its own values -- so one block of 1024 threads walks the chunks in order:
// thread 0 plans each engine call and runs the scalar draws, and the block
// evaluates every batch in parallel (each thread computes its own words from
// their counters).  FP64 arithmetic follows the reference's operation order
// without contraction; log / exp / sqrt / sincos are CUDA's, within an ulp or
// two of the host libm, so a variate agrees to about 1e-15 relative and a
// value that lands within an ulp of an accept / reject boundary can take the
// other branch (and shift the rest of the stream).
#include "common.cuh"
#include "rng_device.cuh"

#include <cstring>

using namespace vsmc_cuda;

namespace vsmc_cuda
{

namespace
{

constexpr int kStBlock = 1024; // threads; one variate of a chunk each

// The engine's counter and buffer position: the buffered block is gen(c),
// index its next word (4: exhausted).
template <typename W>
struct EngPos {
    W c[4];
    uint32_t index;
};

struct PhiloxT {
    using W = uint32_t;
    static constexpr W kMax = 0xFFFFFFFFu;
    uint32_t k0, k1;
    __device__ W word(const W (&c)[4], uint32_t lane) const
    {
        const u32x4 b = philox4x32_10(c[0], c[1], c[2], c[3], k0, k1);
        return lane == 0 ? b.x : (lane == 1 ? b.y : (lane == 2 ? b.z : b.w));
    }
    __device__ static double u01(W w) { return u01_co_d(w); }
    __device__ static void inc(W (&c)[4]) { ctr32_add(c, 1); }
    __device__ static void carry1(W (&c)[4]) { ctr32_carry1(c); }
};

struct ThreefryT {
    using W = uint64_t;
    static constexpr W kMax = 0xFFFFFFFFFFFFFFFFull;
    uint64_t k[4];
    __device__ W word(const W (&c)[4], uint32_t lane) const
    {
        const u64x4 b = threefry4x64_20({c[0], c[1], c[2], c[3]}, k[0], k[1],
            k[2], k[3]);
        return lane == 0 ? b.x : (lane == 1 ? b.y : (lane == 2 ? b.z : b.w));
    }
    __device__ static double u01(W w) { return u01_co_d64(w); }
    __device__ static void inc(W (&c)[4]) { ctr64_add(c, 1); }
    __device__ static void carry1(W (&c)[4]) { ctr64_carry1(c); }
};

// One bulk call of n <= 1024 words: `head` words from the buffered block
// (hc, lanes hlane..), `nblk` blocks of one generator call starting at
// counter c1, then `tail` words of block tc.
template <typename W>
struct Bulk {
    W hc[4];
    W c1[4];
    W tc[4];
    uint32_t hlane, head, nblk, tail;
    int quirk; // the call's counters carry past an all-ones low limb
};

template <class G>
__device__ void copy4(typename G::W (&d)[4], const typename G::W (&s)[4])
{
#pragma unroll
    for (int i = 0; i < 4; ++i)
        d[i] = s[i];
}

// counter of block i of the generator call (increment(ctr, n, ctr_block))
template <class G>
__device__ void bulk_block_ctr(const Bulk<typename G::W> &b, uint32_t i,
    typename G::W (&c)[4])
{
    copy4<G>(c, b.c1);
    if (!b.quirk) {
        c[0] += i;
    } else {
        // increment(ctr, nskip): the low limb adds; a limb at or past the
        // top carries into limb 1 (also when it lands exactly on all ones)
        const bool carry = !(c[0] < G::kMax - i);
        c[0] += i;
        if (carry)
            G::carry1(c);
    }
}

// Plan a bulk call of n <= 1024 words and advance the engine (one thread).
template <class G>
__device__ void bulk_plan(EngPos<typename G::W> &s, uint32_t n,
    Bulk<typename G::W> &b)
{
    copy4<G>(b.hc, s.c);
    b.hlane = s.index;
    b.nblk = 0;
    b.tail = 0;
    b.quirk = 0;
    const uint32_t remain = 4 - s.index;
    if (n < remain) {
        b.head = n;
        s.index += n;
        return;
    }
    b.head = remain;
    const uint32_t np = n - remain;
    s.index = 4;
    b.nblk = np / 4;
    if (b.nblk != 0) {
        copy4<G>(b.c1, s.c);
        G::inc(b.c1);
        b.quirk = (b.c1[0] < G::kMax - b.nblk) ? 0 : 1;
        typename G::W last[4];
        bulk_block_ctr<G>(b, b.nblk - 1, last);
        copy4<G>(s.c, last); // the engine counter is the call's last block
    }
    b.tail = np % 4;
    if (b.tail != 0) { // scalar draws: a fresh block after the call
        G::inc(s.c);
        copy4<G>(b.tc, s.c);
        s.index = b.tail;
    }
}

template <class G>
__device__ typename G::W bulk_word(
    const G &g, const Bulk<typename G::W> &b, uint32_t p)
{
    if (p < b.head)
        return g.word(b.hc, b.hlane + p);
    const uint32_t q = p - b.head;
    if (q < 4 * b.nblk) {
        typename G::W c[4];
        bulk_block_ctr<G>(b, q / 4, c);
        return g.word(c, q % 4);
    }
    return g.word(b.tc, q - 4 * b.nblk);
}

// The engine's scalar operator() as a StudentTScalar / NormalScalar engine
// (thread 0 only).
template <class G>
struct ScalarEng {
    const G &g;
    EngPos<typename G::W> &s;
    __device__ typename G::W next()
    {
        if (s.index == 4) {
            G::inc(s.c);
            s.index = 0;
        }
        return g.word(s.c, s.index++);
    }
    __device__ double u01d() { return G::u01(next()); }
};

struct StShared {
    double a[2 * kStBlock]; // u (and e for T / W): 2 n uniforms
    double w[kStBlock];     // normals
    double x[kStBlock];     // candidate values
    int acc[kStBlock];
};

// A batch of n <= 2048 uniforms into out[0..n): u01_distribution's calls of
// at most 1024 words (rng/u01_distribution.hpp:215-233).  Every thread.
template <class G>
__device__ void u01_batch(const G &g, EngPos<typename G::W> &s,
    Bulk<typename G::W> &b, uint32_t n, double *out)
{
    for (uint32_t off = 0; off < n; off += 1024) {
        const uint32_t k = n - off < 1024 ? n - off : 1024;
        __syncthreads();
        if (threadIdx.x == 0)
            bulk_plan<G>(s, k, b);
        __syncthreads();
        for (uint32_t p = threadIdx.x; p < k; p += blockDim.x)
            out[off + p] = G::u01(bulk_word<G>(g, b, p));
    }
    __syncthreads();
}

// normal_distribution(rng, n, out, 0, 1) for n <= 1024: the batch layout
// (radii then angles; sine branch first) and, for odd n, two scalar
// uniforms for the last value.  `tmp` holds the n uniforms.  Every thread.
template <class G>
__device__ void normal_batch(const G &g, EngPos<typename G::W> &s,
    Bulk<typename G::W> &b, uint32_t n, double *tmp, double *out)
{
    u01_batch<G>(g, s, b, n, tmp);
    const uint32_t nu = n / 2;
    for (uint32_t i = threadIdx.x; i < nu; i += blockDim.x) {
        double sc, sv, cv;
        box_muller_batch(tmp[i], tmp[nu + i], 1.0, sc, sv, cv);
        out[i] = fma_free_add(fma_free_mul(sc, sv), 0.0);
        out[nu + i] = fma_free_add(fma_free_mul(sc, cv), 0.0);
    }
    if (n % 2 != 0 && threadIdx.x == 0) {
        ScalarEng<G> e{g, s};
        const double u = e.u01d();
        const double v = e.u01d();
        out[n - 1] = odd_tail_value(u, v, 0.0, 1.0);
    }
    __syncthreads();
}

template <class G>
__global__ void __launch_bounds__(kStBlock) k_student_t_engine(G g,
    EngPos<typename G::W> start, size_t n, double df, double *r,
    EngPos<typename G::W> *end, uint32_t *err)
{
    __shared__ EngPos<typename G::W> s;
    __shared__ Bulk<typename G::W> b;
    __shared__ StShared sh;
    __shared__ uint32_t nacc;
    const uint32_t t = threadIdx.x;
    if (t == 0)
        s = start;
    StudentTScalar st(df); // alpha = df / 2; gamma() draws Gamma(alpha, 2)
    const double alpha = st.alpha, c = st.c, d = st.d, beta = 2.0;
    uint32_t e_bits = 0;
    for (size_t base = 0; base < n; base += kStBlock) {
        const uint32_t k = static_cast<uint32_t>(
            n - base < static_cast<size_t>(kStBlock) ? n - base : kStBlock);
        double *rr = r + base;
        // ---- one vectorised gamma attempt over the chunk
        bool accept = false;
        double xv = 0;
        if (st.alg == 0 || st.alg == 1) { // T / W: 2 k uniforms
            u01_batch<G>(g, s, b, 2 * k, sh.a);
            if (t < k) {
                double u = sh.a[t];
                double e = -1.0 * log(sh.a[k + t]);
                if (st.alg == 0) {
                    if (u > d) {
                        u = -log(fma_free_mul(c, fma_free_add(1.0, -u)));
                        e = fma_free_add(e, u);
                        u = fma_free_add(d, fma_free_mul(alpha, u));
                    }
                    const double x = exp(fma_free_mul(c, log(u)));
                    xv = fma_free_mul(beta, x);
                    accept = fabs(x) < e;
                } else {
                    u = -1.0 * log(u);
                    const double x = exp(fma_free_mul(c, log(u)));
                    xv = fma_free_mul(beta, x);
                    accept = fma_free_add(u, e) > fma_free_add(d, x);
                }
            }
        } else if (st.alg == 2) { // N
            u01_batch<G>(g, s, b, k, sh.a);
            normal_batch<G>(g, s, b, k, sh.x, sh.w);
            bool neg = false;
            if (t < k)
                neg = fma_free_add(fma_free_mul(c, sh.w[t]), 1.0) <= 0;
            if (__syncthreads_or(neg) && t == 0) {
                // v <= 0: redraw w with one scalar NormalDistribution, in
                // index order
                ScalarEng<G> e{g, s};
                NormalScalar<double> rnorm(0, 1);
                for (uint32_t i = 0; i < k; ++i) {
                    if (!(fma_free_add(fma_free_mul(c, sh.w[i]), 1.0) <= 0))
                        continue;
                    int guard = 0;
                    double w, v;
                    do {
                        w = rnorm(e);
                        v = fma_free_add(1.0, fma_free_mul(c, w));
                    } while (v <= 0 && ++guard < kGammaMaxTries);
                    if (guard >= kGammaMaxTries)
                        e_bits |= DEV_ERR_BOUND;
                    sh.w[i] = w;
                }
            }
            __syncthreads();
            if (t < k) {
                const double u = sh.a[t];
                const double w = sh.w[t];
                double v = fma_free_add(fma_free_mul(c, w), 1.0);
                v = fma_free_mul(v, fma_free_mul(v, v));
                double e = fma_free_mul(w, w);
                e = fma_free_mul(e, e);
                e = fma_free_add(fma_free_mul(-0.0331, e), 1.0);
                xv = fma_free_mul(fma_free_mul(d, beta), v);
                if (u < e) {
                    accept = true;
                } else {
                    const double e2 = fma_free_add(
                        fma_free_mul(w, w) / 2,
                        fma_free_mul(d, fma_free_add(fma_free_add(1.0, -v),
                                            log(v))));
                    accept = log(u) < e2;
                }
            }
        } else { // E
            u01_batch<G>(g, s, b, k, sh.a);
            if (t < k) {
                xv = fma_free_mul(-beta, log(sh.a[t]));
                accept = true;
            }
        }
        // ---- pack the accepted values in index order
        sh.acc[t] = accept ? 1 : 0;
        __syncthreads();
        if (t == 0) {
            uint32_t m = 0;
            for (uint32_t i = 0; i < k; ++i) {
                const int a = sh.acc[i];
                sh.acc[i] = static_cast<int>(m);
                m += a;
            }
            nacc = m;
        }
        __syncthreads();
        if (t < k && accept)
            rr[sh.acc[t]] = xv;
        __syncthreads();
        // ---- scalar GammaDistribution draws for the rejected slots
        if (t == 0) {
            ScalarEng<G> e{g, s};
            for (uint32_t i = nacc; i < k; ++i)
                rr[i] = st.gamma(e);
            e_bits |= st.err;
        }
        __syncthreads();
        // ---- r = sqrt(r * (1 / df)); z; r = z / r
        const double inv = 1 / df;
        double rv = 0;
        if (t < k)
            rv = sqrt(fma_free_mul(inv, rr[t]));
        normal_batch<G>(g, s, b, k, sh.a, sh.w);
        if (t < k)
            rr[t] = sh.w[t] / rv;
        __syncthreads();
    }
    if (t == 0) {
        *end = s;
        if (e_bits)
            atomicOr(err, e_bits);
    }
}

} // namespace

} // namespace vsmc_cuda

extern "C" int vsmc_cuda_rng_student_t(vsmc_cuda_rng *rng, size_t n,
    double *r, double df, void *stream)
{
    if (rng == nullptr ||
        (rng->kind != VSMC_CUDA_PHILOX4X32 &&
            rng->kind != VSMC_CUDA_THREEFRY4X64) ||
        rng->index < 1 || rng->index > 4 || (r == nullptr && n) || !(df > 0))
        return VSMC_CUDA_ERR_ARG;
    if (n == 0)
        return VSMC_CUDA_OK;
    cudaStream_t st = as_stream(stream);
    Scratch scratch(st);
    // the engine state after the call, and the error word
    unsigned char *dev = scratch.get<unsigned char>(256);
    if (dev == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    uint32_t *err = reinterpret_cast<uint32_t *>(dev + 128);
    VSMC_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    unsigned char host[256];
    if (rng->kind == VSMC_CUDA_PHILOX4X32) {
        PhiloxT g{static_cast<uint32_t>(rng->key[0]),
            static_cast<uint32_t>(rng->key[1])};
        EngPos<uint32_t> s0;
        for (int i = 0; i < 4; ++i)
            s0.c[i] = static_cast<uint32_t>(rng->ctr[i]);
        s0.index = rng->index;
        auto *end = reinterpret_cast<EngPos<uint32_t> *>(dev);
        k_student_t_engine<PhiloxT><<<1, kStBlock, 0, st>>>(
            g, s0, n, df, r, end, err);
    } else {
        ThreefryT g{{rng->key[0], rng->key[1], rng->key[2], rng->key[3]}};
        EngPos<uint64_t> s0;
        for (int i = 0; i < 4; ++i)
            s0.c[i] = rng->ctr[i];
        s0.index = rng->index;
        auto *end = reinterpret_cast<EngPos<uint64_t> *>(dev);
        k_student_t_engine<ThreefryT><<<1, kStBlock, 0, st>>>(
            g, s0, n, df, r, end, err);
    }
    VSMC_CUDA_CHECK_LAUNCH();
    VSMC_CUDA_TRY(cudaMemcpyAsync(host, dev, sizeof(host),
        cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    uint32_t e = 0;
    std::memcpy(&e, host + 128, sizeof(e));
    if (rng->kind == VSMC_CUDA_PHILOX4X32) {
        EngPos<uint32_t> s;
        std::memcpy(&s, host, sizeof(s));
        for (int i = 0; i < 4; ++i)
            rng->ctr[i] = s.c[i];
        rng->index = s.index;
    } else {
        EngPos<uint64_t> s;
        std::memcpy(&s, host, sizeof(s));
        for (int i = 0; i < 4; ++i)
            rng->ctr[i] = s.c[i];
        rng->index = s.index;
    }
    return e ? VSMC_CUDA_ERR_TIMEOUT : VSMC_CUDA_OK;
}
