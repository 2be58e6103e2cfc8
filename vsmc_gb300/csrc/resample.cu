// Resampling transforms, schemes, particle copy, weights and the monitor mean
// on the device, with the reference's arithmetic.
//
// Cumulative weights and normalizing sums are the reference's left-to-right
// sums bit for bit (seqsum.cu).  Counting uniforms against the CDF follows the
// two-pointer loop of resample/transform.hpp:43-71: after particle i the loop
// has consumed every uniform before the first one above cdf_i, so with the
// prefix maximum pm_j of the uniforms, F(cdf_i) = #{j : pm_j <= cdf_i} and
// rep_i = F(cdf_i) - F(cdf_{i-1}); the last particle takes the rest.
#include "common.cuh"
#include "rng_device.cuh"
#include "scan.cuh"
#include "seqsum.cuh"
#include "resample_internal.cuh"

#include <climits>
#include <cmath>
#include <cstring>

namespace vsmc_cuda
{

namespace
{

constexpr int kB = 256;

int grid1(size_t n) { return grid_for(n ? n : 1, kB, 4, 8); }

#define GRID_LOOP(i, n)                                                       \
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; \
         i < (n); i += static_cast<size_t>(gridDim.x) * blockDim.x)

// ------------------------------------------------------------ elementwise

__global__ void k_fill_i32(size_t n, int *p, int v)
{
    GRID_LOOP(i, n) p[i] = v;
}

__global__ void k_set_one(int *p, int v)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        *p = v;
}

// max-scan key: NaN compares as "above everything", as the reference's
// `u <= accw` test is false for NaN
__device__ __forceinline__ double key_of(double u)
{
    return isnan(u) ? INFINITY : u;
}

struct LoadKey {
    const double *u;
    __device__ double operator()(size_t i) const { return key_of(u[i]); }
};

struct StoreD {
    double *p;
    __device__ void operator()(size_t i, double v) const { p[i] = v; }
};

// #{j < n : pm_j <= x} (pm non-decreasing)
__device__ __forceinline__ size_t upper_count(
    const double *pm, size_t n, double x)
{
    size_t lo = 0, hi = n;
    while (lo < hi) {
        const size_t mid = lo + (hi - lo) / 2;
        if (pm[mid] <= x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// #{i < m : s_i < x} (s non-decreasing): the first i with s_i >= x
__device__ __forceinline__ size_t lower_count(
    const double *s, size_t m, double x)
{
    size_t lo = 0, hi = m;
    while (lo < hi) {
        const size_t mid = lo + (hi - lo) / 2;
        if (s[mid] < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Order-preserving integer key of a double, so the running maximum of the
// uniforms and the counting compare integers (GB300's FP64 rate is a small
// fraction of its integer rate): keys order as the doubles do, -0 equals +0,
// and a NaN uniform sits above everything, as the two-pointer test
// `u <= accw` is false for it.
__device__ __forceinline__ long long okey(double u)
{
    const long long b = __double_as_longlong(u);
    const unsigned long long a =
        static_cast<unsigned long long>(b) & 0x7FFFFFFFFFFFFFFFull;
    if (a == 0)
        return 0; // +0 and -0
    if (a > 0x7FF0000000000000ull)
        return LLONG_MAX; // NaN
    return b >= 0 ? b : (b ^ LLONG_MAX);
}

// the key a CDF value is compared with: a NaN CDF value counts no uniform
__device__ __forceinline__ long long okey_cdf(double x)
{
    const unsigned long long a =
        static_cast<unsigned long long>(__double_as_longlong(x)) &
        0x7FFFFFFFFFFFFFFFull;
    return a > 0x7FF0000000000000ull ? LLONG_MIN : okey(x);
}

struct LoadOKey {
    const double *u;
    __device__ long long operator()(size_t i) const { return okey(u[i]); }
};

struct StoreK {
    long long *p;
    __device__ void operator()(size_t i, long long v) const { p[i] = v; }
};

struct OpMaxK {
    __device__ __forceinline__ long long operator()(long long a,
        long long b) const
    {
        return a < b ? b : a;
    }
};

// Keys of the uniforms for counting: the running maximum's keys (KeysMax),
// or, for uniforms known to be non-decreasing, non-negative and free of NaN,
// each uniform's own key (KeysOwn; the running maximum is then the sequence
// itself).
struct KeysMax {
    const long long *pmk;
    __device__ __forceinline__ long long operator[](size_t j) const
    {
        return pmk[j];
    }
};

struct KeysOwn {
    const double *u;
    __device__ __forceinline__ long long operator[](size_t j) const
    {
        // okey of a non-negative, non-NaN double is its bit pattern
        return __double_as_longlong(u[j]);
    }
};

// The first index j >= lo with pmk_j > x (hi if none), given that every
// j < lo has pmk_j <= x and pmk_hi > x or hi == n.
template <class Keys>
__device__ __forceinline__ size_t first_above(
    const Keys &pmk, size_t lo, size_t hi, long long x)
{
    while (lo < hi) {
        const size_t mid = lo + (hi - lo) / 2;
        if (pmk[mid] <= x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// #{j < n : pmk_j <= x} by exponential search from a guess g <= n.
template <class Keys>
__device__ __forceinline__ size_t count_from(
    const Keys &pmk, size_t n, long long x, size_t g)
{
    size_t lo, hi;
    size_t step = 1;
    if (g < n && pmk[g] <= x) { // the answer is above g
        lo = g + 1;
        hi = n;
        while (lo < n) {
            const size_t probe = lo + step - 1;
            if (probe >= n)
                break;
            if (pmk[probe] > x) {
                hi = probe;
                break;
            }
            lo = probe + 1;
            step <<= 1;
        }
    } else { // the answer is at most g
        lo = 0;
        hi = g;
        while (step <= hi) {
            const size_t probe = hi - step;
            if (pmk[probe] <= x) {
                lo = probe + 1;
                break;
            }
            hi = probe;
            step <<= 1;
        }
    }
    return first_above(pmk, lo, hi, x);
}

// floor(c n) for c in [0, 1) from the bits of c (integer operations; only a
// starting guess, so the low bits of c are dropped); n for c >= 1, 0 for a
// negative c
__device__ __forceinline__ size_t guess_cn(double c, size_t n)
{
    const unsigned long long b =
        static_cast<unsigned long long>(__double_as_longlong(c));
    if (b >> 63)
        return 0;
    const int e = static_cast<int>(b >> 52) - 1023;
    if (e >= 0)
        return n;
    const int sh = 31 - e; // c n = (mant >> 21) n 2^(e - 31)
    if (sh >= 64)
        return 0;
    const unsigned long long m32 = ((b & ((1ull << 52) - 1)) | (1ull << 52)) >> 21;
    const unsigned long long g = (m32 * static_cast<unsigned long long>(n)) >> sh;
    return g < n ? static_cast<size_t>(g) : n;
}

// F[i] = #{j < n : pmk_j <= key(cdf_i)} for i < m - 1, both sequences
// non-decreasing.  Every scheme spreads its uniforms over [0, 1), so the
// answer is near n cdf_i: an exponential search from that guess needs a few
// loads, and consecutive lanes touch neighbouring addresses.  A weight that
// takes many copies costs a logarithmic number of loads.
template <class Keys>
__global__ void __launch_bounds__(kB) k_counts(size_t m, size_t n,
    const double *cdf, const Keys pmk, uint32_t *F)
{
    GRID_LOOP(i, m - 1)
    {
        const double c = cdf[i];
        F[i] = static_cast<uint32_t>(
            count_from(pmk, n, okey_cdf(c), guess_cn(c, n)));
    }
}

__global__ void k_rep_from_counts(size_t m, size_t n, const uint32_t *F,
    int *rep, const int *integ)
{
    GRID_LOOP(i, m)
    {
        const uint32_t hi = i + 1 < m ? F[i] : static_cast<uint32_t>(n);
        const uint32_t lo = i > 0 ? F[i - 1] : 0u;
        int r = static_cast<int>(hi - lo);
        if (integ)
            r += integ[i];
        rep[i] = r;
    }
}

__global__ void k_index_from_cdf(size_t m, size_t n, const double *cdf,
    const double *pm, int *idx)
{
    GRID_LOOP(j, n)
    idx[j] = static_cast<int>(lower_count(cdf, m - 1, pm[j]));
}

// ---------------------------------------------- uniforms from the engine
// word k of the scalar stream of (key, ctr, index): gen(ctr + (index+k)/4)
struct EngineState {
    uint32_t k0, k1;
    uint32_t c[4];
    uint32_t index;
};

__device__ __forceinline__ uint32_t stream_word(const EngineState &e, size_t k)
{
    const uint64_t pos = static_cast<uint64_t>(e.index) + k;
    uint32_t c[4] = {e.c[0], e.c[1], e.c[2], e.c[3]};
    ctr32_add(c, pos / 4);
    const u32x4 b = philox4x32_10(c[0], c[1], c[2], c[3], e.k0, e.k1);
    const uint32_t i = static_cast<uint32_t>(pos % 4);
    return i == 0 ? b.x : (i == 1 ? b.y : (i == 2 ? b.z : b.w));
}

// x * 2^-e rounded to the nearest double, ties to even, for 0 <= x < 2^63
// and a result in the normal range: the rounding of an exact value to 53
// significant bits done on the integer (IEEE 754 round-to-nearest-even),
// and the double assembled from its bits, so no FP64 instruction runs.
__device__ __forceinline__ double rne_scaled(uint64_t x, int e)
{
    if (x == 0)
        return 0.0;
    int b = 64 - __clzll(static_cast<long long>(x)); // significant bits
    uint64_t m = x;
    int sh = 0;
    if (b > 53) {
        sh = b - 53;
        const uint64_t rest = x & ((1ull << sh) - 1);
        const uint64_t half = 1ull << (sh - 1);
        m = x >> sh;
        if (rest > half || (rest == half && (m & 1)))
            ++m;
        if (m >> 53) { // rounded up to 2^53
            m >>= 1;
            ++sh;
        }
        b = 53;
    }
    // value = m * 2^(sh - e), m < 2^53 with b significant bits
    const int exp2 = b - 1 + sh - e; // unbiased exponent of the result
    const uint64_t frac = (m << (53 - b)) & ((1ull << 52) - 1);
    const uint64_t bits =
        (static_cast<uint64_t>(exp2 + 1023) << 52) | frac;
    return __longlong_as_double(static_cast<long long>(bits));
}

// U01SequenceStratified: u_j = U_j * delta + j * delta.  Word j is at
// stream position index + j; one Philox block gives the four words of
// positions 4b .. 4b + 3.  For n = 2^k (log2n = k, else -1) delta is exact,
// both products are exact scalings of U_j = w 2^-32 and j, and the one
// rounding is that of the sum: u_j = RNE(j 2^32 + w) 2^-(32 + k), formed in
// integers (rne_scaled).  Otherwise the FP64 arithmetic of the reference.
__global__ void k_stratified_seq(EngineState e, size_t n, int log2n, double *u)
{
    const double delta = 1.0 / static_cast<double>(n);
    const uint64_t first = e.index;
    const uint64_t nblk = (first + n + 3) / 4;
    GRID_LOOP(b, nblk)
    {
        uint32_t c[4] = {e.c[0], e.c[1], e.c[2], e.c[3]};
        ctr32_add(c, b);
        const u32x4 w = philox4x32_10(c[0], c[1], c[2], c[3], e.k0, e.k1);
        const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint64_t pos = 4 * static_cast<uint64_t>(b) + k;
            if (pos < first || pos - first >= n)
                continue;
            const size_t j = static_cast<size_t>(pos - first);
            if (log2n >= 0) {
                u[j] = rne_scaled((static_cast<uint64_t>(j) << 32) | ws[k],
                    32 + log2n);
            } else {
                const double U = u01_co_d(ws[k]);
                u[j] = __dadd_rn(__dmul_rn(U, delta),
                    __dmul_rn(static_cast<double>(j), delta));
            }
        }
    }
}

// U01SequenceSystematic: u0 = U * delta, u_j = u0 + j * delta (for n = 2^k
// the same integer rounding with one word for every j)
__global__ void k_systematic_seq(EngineState e, size_t n, int log2n, double *u)
{
    const uint32_t w0 = stream_word(e, 0);
    if (log2n >= 0) {
        GRID_LOOP(j, n)
        u[j] = rne_scaled((static_cast<uint64_t>(j) << 32) | w0, 32 + log2n);
        return;
    }
    const double delta = 1.0 / static_cast<double>(n);
    const double u0 = __dmul_rn(u01_co_d(w0), delta);
    GRID_LOOP(j, n)
    u[j] = __dadd_rn(u0, __dmul_rn(static_cast<double>(j), delta));
}

// U01SequenceSorted terms: -log(U_j) / (n - j), summed left to right below
__global__ void k_sorted_terms(EngineState e, size_t n, double *t)
{
    GRID_LOOP(j, n)
    {
        const double U = u01_co_d(stream_word(e, j));
        t[j] = -(log(U) / static_cast<double>(n - j));
    }
}

__global__ void k_sorted_terms_arr(size_t n, const double *u01, double *t)
{
    GRID_LOOP(j, n) t[j] = -(log(u01[j]) / static_cast<double>(n - j));
}

// u_j = 1 - exp(lmax_j), lmax_j = -prefix_j
__global__ void k_sorted_finish(size_t n, const double *neg_lmax, double *u)
{
    GRID_LOOP(j, n) u[j] = 1.0 - exp(-neg_lmax[j]);
}

__global__ void k_stratified_arr(size_t n, const double *u01, double *out)
{
    const double delta = 1.0 / static_cast<double>(n);
    GRID_LOOP(i, n)
    out[i] = __dadd_rn(__dmul_rn(u01[i], delta),
        __dmul_rn(static_cast<double>(i), delta));
}

__global__ void k_systematic_terms(size_t n, double u01, double *t)
{
    const double delta = 1.0 / static_cast<double>(n);
    GRID_LOOP(i, n) t[i] = i == 0 ? __dmul_rn(u01, delta) : delta;
}

// --------------------------------------------------------------- residual

// A NaN, infinite or negative weight is reported and split as zero, so the
// integer parts stay a valid count.
__global__ void k_residual_split(size_t m, size_t n, const double *w,
    double *resid, int *integ, uint32_t *err)
{
    const double coeff = static_cast<double>(n);
    GRID_LOOP(i, m)
    {
        const double wi = w[i];
        if (!(wi >= 0.0) || isinf(wi)) {
            atomicOr(err, DEV_ERR_NONFINITE);
            resid[i] = 0.0;
            integ[i] = 0;
            continue;
        }
        const double x = __dmul_rn(coeff, wi);
        const double ip = trunc(fmin(x, 2147483647.0));
        resid[i] = x - ip; // modf: exact
        integ[i] = static_cast<int>(ip);
    }
}

__global__ void k_scale(size_t m, const double *total, double *v)
{
    const double inv = 1.0 / *total;
    GRID_LOOP(i, m) v[i] = __dmul_rn(inv, v[i]);
}

// ------------------------------------------------------------ rep -> index

struct I2 {
    int32_t a, b;
};

struct OpI2 {
    __device__ __forceinline__ I2 operator()(const I2 &x, const I2 &y) const
    {
        return {x.a + y.a, x.b + y.b};
    }
};

struct OpMaxI {
    __device__ __forceinline__ int32_t operator()(int32_t x, int32_t y) const
    {
        return x < y ? y : x;
    }
};

// (empty flag, surplus) for m == n; (rep, 0) for m != n
struct LoadES {
    const int *rep;
    bool square;
    __device__ I2 operator()(size_t i) const
    {
        const int r = rep[i];
        if (square)
            return {r == 0 ? 1 : 0, r > 1 ? r - 1 : 0};
        return {r, 0};
    }
};

struct StoreI2 {
    I2 *p;
    __device__ void operator()(size_t i, I2 v) const { p[i] = v; }
};

// marks: rank of the first surplus copy of p (m == n), or first output slot
// of p (m != n), gets p + 1
__global__ void k_marks(size_t m, bool square, const int *rep, const I2 *incl,
    int *marks, size_t nmarks, uint32_t *err)
{
    GRID_LOOP(p, m)
    {
        const int r = rep[p];
        if (r < 0) {
            atomicOr(err, DEV_ERR_INTERNAL);
            continue;
        }
        if (square) {
            if (r > 1) {
                const int first = incl[p].b - (r - 1); // exclusive surplus
                if (first >= 0 && static_cast<size_t>(first) < nmarks)
                    marks[first] = static_cast<int>(p) + 1;
                else
                    atomicOr(err, DEV_ERR_INTERNAL);
            }
        } else if (r > 0) {
            const int first = incl[p].a - r;
            if (first >= 0 && static_cast<size_t>(first) < nmarks)
                marks[first] = static_cast<int>(p) + 1;
            else
                atomicOr(err, DEV_ERR_INTERNAL);
        }
    }
}

struct LoadI {
    const int *p;
    __device__ int32_t operator()(size_t i) const { return p[i]; }
};

struct StoreI {
    int *p;
    __device__ void operator()(size_t i, int32_t v) const { p[i] = v; }
};

// int entries widened to 64 bits (sums of up to 2^31 counts of up to 2^31)
struct LoadIW {
    const int *p;
    __device__ long long operator()(size_t i) const { return p[i]; }
};

// keeps only the last value of a scan (the total)
struct StoreLastW {
    long long *p;
    size_t last;
    __device__ void operator()(size_t i, long long v) const
    {
        if (i == last)
            *p = v;
    }
};

__global__ void k_index_square(size_t n, const int *rep, const I2 *incl,
    const int *src_of_rank, size_t nrank, int *idx, uint32_t *err)
{
    GRID_LOOP(d, n)
    {
        if (rep[d] != 0) {
            idx[d] = static_cast<int>(d);
        } else {
            const int k = incl[d].a - 1; // exclusive empty rank
            if (k >= 0 && static_cast<size_t>(k) < nrank && src_of_rank[k] > 0)
                idx[d] = src_of_rank[k] - 1;
            else
                atomicOr(err, DEV_ERR_INTERNAL);
        }
    }
}

__global__ void k_index_flat(size_t total, const int *src, int *idx)
{
    GRID_LOOP(d, total) idx[d] = src[d] - 1;
}

__global__ void k_hist(size_t m, size_t n, const int *idx, int *rep,
    uint32_t *err)
{
    GRID_LOOP(i, n)
    {
        const int p = idx[i];
        if (p < 0 || static_cast<size_t>(p) >= m)
            atomicOr(err, DEV_ERR_INTERNAL);
        else
            atomicAdd(rep + p, 1);
    }
}

// --------------------------------------------------------------- copying

__global__ void k_check_fixed_points(size_t n, const int *idx, uint32_t *err)
{
    GRID_LOOP(d, n)
    {
        const int s = idx[d];
        if (s < 0 || static_cast<size_t>(s) >= n || idx[s] != s)
            atomicOr(err, DEV_ERR_INTERNAL);
    }
}

template <typename T>
__global__ void k_copy_state(size_t n, size_t dim, size_t ld, const int *idx,
    T *state, const uint32_t *err)
{
    if (*err)
        return;
    GRID_LOOP(d, n)
    {
        const size_t s = static_cast<size_t>(idx[d]);
        if (s != d)
            for (size_t r = 0; r < dim; ++r)
                state[r * ld + d] = state[r * ld + s];
    }
}

// ---------------------------------------------------------------- weights

struct OpMaxD {
    __device__ __forceinline__ double operator()(double a, double b) const
    {
        return a < b ? b : a;
    }
};

__global__ void k_reduce_max(size_t n, const double *v, double *part)
{
    double m = -INFINITY;
    GRID_LOOP(i, n) m = fmax(m, v[i]);
    __shared__ double sh[kB / 32 + 1];
    m = block_reduce(m, OpMaxD(), -static_cast<double>(INFINITY), sh);
    if (threadIdx.x == 0)
        part[blockIdx.x] = m;
}

__global__ void k_max_parts(int nb, double *part)
{
    double m = -INFINITY;
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        m = fmax(m, part[b]);
    __shared__ double sh[kB / 32 + 1];
    m = block_reduce(m, OpMaxD(), -static_cast<double>(INFINITY), sh);
    if (threadIdx.x == 0)
        part[0] = m;
}

// W = exp(lw - max)  (post_set_log -> normalize(true), weight.hpp:202-229)
__global__ void k_exp_shift(size_t n, const double *lw, const double *mx,
    double *W)
{
    const double m = *mx;
    GRID_LOOP(i, n) W[i] = exp(lw[i] - m);
}

// W = log(W) + l  (add_log, weight.hpp:168-173)
__global__ void k_log_add(size_t n, const double *l, double *W)
{
    GRID_LOOP(i, n) W[i] = __dadd_rn(log(W[i]), l[i]);
}

__global__ void k_square(size_t n, const double *W, double *sq)
{
    GRID_LOOP(i, n) sq[i] = __dmul_rn(W[i], W[i]);
}

__global__ void k_inv_total(const double *total, double *ess)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        *ess = 1.0 / *total;
}

__global__ void k_fill_d(size_t n, double *p, double v)
{
    GRID_LOOP(i, n) p[i] = v;
}

// ---------------------------------------------------------------- monitor

template <typename T>
__global__ void k_wsum(size_t n, size_t dim, size_t ld, const T *state,
    const double *W, double *part)
{
    __shared__ double sh[kB / 32 + 1];
    for (size_t d = 0; d < dim; ++d) {
        double s = 0;
        GRID_LOOP(i, n) s += W[i] * static_cast<double>(state[d * ld + i]);
        s = block_reduce(s, OpAdd(), 0.0, sh);
        if (threadIdx.x == 0)
            part[d * gridDim.x + blockIdx.x] = s;
    }
}

__global__ void k_wsum_final(size_t dim, int nb, const double *part,
    double *out)
{
    if (threadIdx.x < dim && blockIdx.x == 0) {
        double s = 0;
        for (int b = 0; b < nb; ++b)
            s += part[threadIdx.x * nb + b];
        out[threadIdx.x] = s;
    }
}

EngineState engine_state(const vsmc_cuda_rng &r)
{
    EngineState e;
    e.k0 = static_cast<uint32_t>(r.key[0]);
    e.k1 = static_cast<uint32_t>(r.key[1]);
    for (int i = 0; i < 4; ++i)
        e.c[i] = static_cast<uint32_t>(r.ctr[i]);
    e.index = r.index;
    return e;
}

// advance the host engine by k words of the scalar stream
void engine_advance_host(vsmc_cuda_rng &r, uint64_t k)
{
    if (k == 0)
        return;
    const uint64_t last = static_cast<uint64_t>(r.index) + k - 1;
    uint32_t c[4] = {static_cast<uint32_t>(r.ctr[0]),
        static_cast<uint32_t>(r.ctr[1]), static_cast<uint32_t>(r.ctr[2]),
        static_cast<uint32_t>(r.ctr[3])};
    ctr32_add(c, last / 4);
    for (int i = 0; i < 4; ++i)
        r.ctr[i] = c[i];
    r.index = static_cast<uint32_t>(last % 4) + 1;
}

bool size_ok(size_t n) { return n < (size_t(1) << 31); }

} // namespace

// ------------------------------------------------------- internal entries

// rep for m weights against n uniforms u (device); integ added if non-null.
// sorted: the caller knows u is non-decreasing, non-negative and free of
// NaN (the integer stratified / systematic sequences for N = 2^k), so its
// running maximum is u itself and is not formed.
int u01_rep_device(size_t m, size_t n, const double *w, const double *u,
    int *rep, const int *integ, uint32_t *err, Scratch &scratch,
    cudaStream_t st, bool sorted)
{
    if (m == 0)
        return VSMC_CUDA_OK;
    if (m == 1 || n == 0) {
        if (m == 1) {
            k_set_one<<<1, 32, 0, st>>>(rep, static_cast<int>(n));
            VSMC_CUDA_CHECK_LAUNCH();
            if (integ)
                k_rep_from_counts<<<1, 32, 0, st>>>(1, n, nullptr, rep, integ);
        } else {
            k_fill_i32<<<grid1(m), kB, 0, st>>>(m, rep, 0);
            VSMC_CUDA_CHECK_LAUNCH();
            if (integ) {
                uint32_t *F = scratch.get<uint32_t>(m);
                if (F == nullptr)
                    return VSMC_CUDA_ERR_ALLOC;
                VSMC_CUDA_TRY(cudaMemsetAsync(F, 0, sizeof(uint32_t) * m, st));
                k_rep_from_counts<<<grid1(m), kB, 0, st>>>(m, 0, F, rep, integ);
            }
        }
        VSMC_CUDA_CHECK_LAUNCH();
        return VSMC_CUDA_OK;
    }
    double *cdf = scratch.get<double>(m - 1);
    uint32_t *F = scratch.get<uint32_t>(m);
    if (!cdf || !F)
        return VSMC_CUDA_ERR_ALLOC;
    int rc = seqsum_device(m - 1, w, cdf, nullptr, err, scratch, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    if (sorted) {
        k_counts<<<grid1(m), kB, 0, st>>>(m, n, cdf, KeysOwn{u}, F);
    } else {
        long long *pmk = scratch.get<long long>(n);
        long long *pp = scratch.get<long long>(scan_parts(n));
        if (!pmk || !pp)
            return VSMC_CUDA_ERR_ALLOC;
        rc = device_scan(
            n, LoadOKey{u}, StoreK{pmk}, OpMaxK(), LLONG_MIN, pp, st);
        if (rc != VSMC_CUDA_OK)
            return rc;
        k_counts<<<grid1(m), kB, 0, st>>>(m, n, cdf, KeysMax{pmk}, F);
    }
    k_rep_from_counts<<<grid1(m), kB, 0, st>>>(m, n, F, rep, integ);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int rep_index_device(size_t m, size_t n, const int *rep, int *idx,
    uint32_t *err, Scratch &scratch, cudaStream_t st)
{
    if (m == 0 || n == 0)
        return VSMC_CUDA_OK;
    const bool square = m == n;
    I2 *incl = scratch.get<I2>(m);
    I2 *pp = scratch.get<I2>(scan_parts(m));
    if (!incl || !pp)
        return VSMC_CUDA_ERR_ALLOC;
    int rc = device_scan(m, LoadES{rep, square}, StoreI2{incl}, OpI2(),
        I2{0, 0}, pp, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    // the number of ranks / slots is needed on the host to size the scan
    I2 tot;
    VSMC_CUDA_TRY(cudaMemcpyAsync(
        &tot, incl + (m - 1), sizeof(I2), cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    size_t nmarks;
    if (square) {
        if (tot.a != tot.b || tot.a < 0)
            return VSMC_CUDA_ERR_ARG; // counts do not sum to n
        nmarks = static_cast<size_t>(tot.a);
    } else {
        if (tot.a < 0 || static_cast<size_t>(tot.a) > n)
            return VSMC_CUDA_ERR_ARG;
        nmarks = static_cast<size_t>(tot.a);
    }
    if (nmarks == 0) {
        if (square)
            k_index_square<<<grid1(n), kB, 0, st>>>(
                n, rep, incl, nullptr, 0, idx, err);
        VSMC_CUDA_CHECK_LAUNCH();
        return VSMC_CUDA_OK;
    }
    int *marks = scratch.get<int>(nmarks);
    int *srcs = scratch.get<int>(nmarks);
    int *pm = scratch.get<int>(scan_parts(nmarks));
    if (!marks || !srcs || !pm)
        return VSMC_CUDA_ERR_ALLOC;
    VSMC_CUDA_TRY(cudaMemsetAsync(marks, 0, sizeof(int) * nmarks, st));
    k_marks<<<grid1(m), kB, 0, st>>>(m, square, rep, incl, marks, nmarks, err);
    VSMC_CUDA_CHECK_LAUNCH();
    rc = device_scan(nmarks, LoadI{marks}, StoreI{srcs}, OpMaxI(), 0, pm, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    if (square)
        k_index_square<<<grid1(n), kB, 0, st>>>(
            n, rep, incl, srcs, nmarks, idx, err);
    else
        k_index_flat<<<grid1(nmarks), kB, 0, st>>>(nmarks, srcs, idx);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

// residual split; *R_dev receives n - sum(integ) (device size_t)
int residual_device(size_t m, size_t n, const double *w, double *resid,
    int *integ, size_t *R_host, uint32_t *err, Scratch &scratch,
    cudaStream_t st)
{
    if (m == 0) {
        *R_host = n;
        return VSMC_CUDA_OK;
    }
    k_residual_split<<<grid1(m), kB, 0, st>>>(m, n, w, resid, integ, err);
    VSMC_CUDA_CHECK_LAUNCH();
    double *total = scratch.get<double>(1);
    long long *isum = scratch.get<long long>(1);
    long long *pp = scratch.get<long long>(scan_parts(m));
    if (!total || !isum || !pp)
        return VSMC_CUDA_ERR_ALLOC;
    int rc = seqsum_device(m, resid, nullptr, total, err, scratch, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    k_scale<<<grid1(m), kB, 0, st>>>(m, total, resid);
    VSMC_CUDA_CHECK_LAUNCH();
    // the integer parts summed in 64 bits: unnormalized weights can push
    // the sum past 2^31, and a wrapped 32-bit sum could land back in [0, n]
    rc = device_scan(m, LoadIW{integ}, StoreLastW{isum, m - 1}, OpAdd(),
        0LL, pp, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    long long R = 0;
    uint32_t e = 0;
    VSMC_CUDA_TRY(cudaMemcpyAsync(
        &R, isum, sizeof(R), cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(
        cudaMemcpyAsync(&e, err, sizeof(e), cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    if (e & DEV_ERR_NONFINITE)
        return VSMC_CUDA_ERR_NONFINITE;
    // normalised weights give integer parts summing to at most n
    if (R < 0 || static_cast<unsigned long long>(R) > n)
        return VSMC_CUDA_ERR_ARG;
    *R_host = n - static_cast<size_t>(R);
    return VSMC_CUDA_OK;
}

// words a lazily read uniform sequence of length n consumed, given the counts
// (the loop reads up to the first uniform above the second-to-last CDF value)
int consumed_words(size_t m, size_t n, const int *rep_dev, const int *integ_dev,
    cudaStream_t st, uint64_t *words)
{
    *words = 0;
    if (m < 2 || n == 0)
        return VSMC_CUDA_OK;
    int last = 0, ilast = 0;
    VSMC_CUDA_TRY(cudaMemcpyAsync(
        &last, rep_dev + (m - 1), sizeof(int), cudaMemcpyDeviceToHost, st));
    if (integ_dev)
        VSMC_CUDA_TRY(cudaMemcpyAsync(&ilast, integ_dev + (m - 1),
            sizeof(int), cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    const size_t tail = static_cast<size_t>(last - ilast);
    const size_t jf = n - tail;
    *words = jf < n ? jf + 1 : n;
    return VSMC_CUDA_OK;
}

int scheme_device(size_t m, size_t n, vsmc_cuda_rng *rng, const double *w,
    int *rep, int scheme, Scratch &scratch, cudaStream_t st)
{
    uint32_t *err = scratch.get<uint32_t>(1);
    if (err == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    VSMC_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    const bool residual = scheme >= VSMC_CUDA_RESIDUAL;
    const int base = residual ? scheme - VSMC_CUDA_RESIDUAL : scheme;
    const double *wt = w;
    int *integ = nullptr;
    size_t N = n;
    int rc;
    if (residual) {
        double *resid = scratch.get<double>(m);
        integ = scratch.get<int>(m);
        if (!resid || !integ)
            return VSMC_CUDA_ERR_ALLOC;
        rc = residual_device(m, n, w, resid, integ, &N, err, scratch, st);
        if (rc != VSMC_CUDA_OK)
            return rc;
        wt = resid;
    }
    const EngineState es = engine_state(*rng);
    double *u = scratch.get<double>(N);
    if (u == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    // N = 2^k: the uniforms are formed in integers (exact, no FP64)
    int log2n = -1;
    if (N > 0 && (N & (N - 1)) == 0 && N <= (size_t(1) << 31)) {
        log2n = 0;
        while ((size_t(1) << log2n) < N)
            ++log2n;
    }
    if (N > 0) {
        if (base == VSMC_CUDA_STRATIFIED) {
            k_stratified_seq<<<grid1(N), kB, 0, st>>>(es, N, log2n, u);
        } else if (base == VSMC_CUDA_SYSTEMATIC) {
            k_systematic_seq<<<grid1(N), kB, 0, st>>>(es, N, log2n, u);
        } else {
            double *t = scratch.get<double>(N);
            if (t == nullptr)
                return VSMC_CUDA_ERR_ALLOC;
            k_sorted_terms<<<grid1(N), kB, 0, st>>>(es, N, t);
            VSMC_CUDA_CHECK_LAUNCH();
            rc = seqsum_device(N, t, t, nullptr, err, scratch, st, true);
            if (rc != VSMC_CUDA_OK)
                return rc;
            k_sorted_finish<<<grid1(N), kB, 0, st>>>(N, t, u);
        }
        VSMC_CUDA_CHECK_LAUNCH();
    }
    // the integer sequences (N = 2^k) round a non-decreasing sequence of
    // integers to nearest, so they are non-decreasing themselves
    const bool sorted = log2n >= 0 &&
        (base == VSMC_CUDA_STRATIFIED || base == VSMC_CUDA_SYSTEMATIC);
    rc = u01_rep_device(m, N, wt, u, rep, integ, err, scratch, st, sorted);
    if (rc != VSMC_CUDA_OK)
        return rc;
    uint64_t words = 0;
    if (base == VSMC_CUDA_SYSTEMATIC) {
        words = 1; // the sequence constructor draws once
    } else if (m >= 1) {
        rc = consumed_words(m, N, rep, integ, st, &words);
        if (rc != VSMC_CUDA_OK)
            return rc;
    }
    int status = VSMC_CUDA_OK;
    rc = read_err(err, st, &status);
    if (rc != VSMC_CUDA_OK)
        return rc;
    if (status != VSMC_CUDA_OK)
        return status;
    engine_advance_host(*rng, words);
    return VSMC_CUDA_OK;
}

// Weight::normalize(use_log) on W in place: sum, scale, ESS (weight.hpp:208-229)
int weight_normalize_device(size_t n, double *W, double *ess_dev,
    uint32_t *err, Scratch &scratch, cudaStream_t st)
{
    double *total = scratch.get<double>(1);
    double *sq = scratch.get<double>(n);
    double *tsq = scratch.get<double>(1);
    if (!total || !sq || !tsq)
        return VSMC_CUDA_ERR_ALLOC;
    int rc = seqsum_device(n, W, nullptr, total, err, scratch, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    k_scale<<<grid1(n), kB, 0, st>>>(n, total, W);
    k_square<<<grid1(n), kB, 0, st>>>(n, W, sq);
    VSMC_CUDA_CHECK_LAUNCH();
    rc = seqsum_device(n, sq, nullptr, tsq, err, scratch, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    if (ess_dev) {
        k_inv_total<<<1, 32, 0, st>>>(tsq, ess_dev);
        VSMC_CUDA_CHECK_LAUNCH();
    }
    return VSMC_CUDA_OK;
}

// post_set_log: subtract the max, exponentiate, normalize
int weight_post_set_log_device(size_t n, double *W, double *ess_dev,
    uint32_t *err, Scratch &scratch, cudaStream_t st)
{
    const int nb = grid1(n);
    double *part = scratch.get<double>(nb);
    if (part == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    k_reduce_max<<<nb, kB, 0, st>>>(n, W, part);
    k_max_parts<<<1, kB, 0, st>>>(nb, part);
    k_exp_shift<<<grid1(n), kB, 0, st>>>(n, W, part, W);
    VSMC_CUDA_CHECK_LAUNCH();
    return weight_normalize_device(n, W, ess_dev, err, scratch, st);
}

int weight_set_equal_device(size_t n, double *W, double *ess_dev,
    uint32_t *err, Scratch &scratch, cudaStream_t st)
{
    k_fill_d<<<grid1(n), kB, 0, st>>>(n, W, 1.0 / static_cast<double>(n));
    VSMC_CUDA_CHECK_LAUNCH();
    return weight_normalize_device(n, W, ess_dev, err, scratch, st);
}

int weight_add_log_device(size_t n, const double *l, double *W,
    double *ess_dev, uint32_t *err, Scratch &scratch, cudaStream_t st)
{
    k_log_add<<<grid1(n), kB, 0, st>>>(n, l, W);
    VSMC_CUDA_CHECK_LAUNCH();
    return weight_post_set_log_device(n, W, ess_dev, err, scratch, st);
}

template <typename T>
int monitor_mean_device(size_t n, size_t dim, size_t ld, const T *state,
    const double *W, double *out, Scratch &scratch, cudaStream_t st)
{
    const int nb = grid_for(n, kB, 8, 2);
    double *part = scratch.get<double>(dim * nb);
    if (part == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    k_wsum<T><<<nb, kB, 0, st>>>(n, dim, ld, state, W, part);
    k_wsum_final<<<1, 32, 0, st>>>(dim, nb, part, out);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

template int monitor_mean_device<float>(size_t, size_t, size_t, const float *,
    const double *, double *, Scratch &, cudaStream_t);
template int monitor_mean_device<double>(size_t, size_t, size_t,
    const double *, const double *, double *, Scratch &, cudaStream_t);

template <typename T>
int state_copy_device(size_t n, size_t dim, size_t ld, const int *idx,
    T *state, uint32_t *err, cudaStream_t st)
{
    k_check_fixed_points<<<grid1(n), kB, 0, st>>>(n, idx, err);
    k_copy_state<T><<<grid1(n), kB, 0, st>>>(n, dim, ld, idx, state, err);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

template int state_copy_device<float>(
    size_t, size_t, size_t, const int *, float *, uint32_t *, cudaStream_t);
template int state_copy_device<double>(
    size_t, size_t, size_t, const int *, double *, uint32_t *, cudaStream_t);

} // namespace vsmc_cuda

using namespace vsmc_cuda;

namespace
{

// run `body(err, scratch)` with a fresh error word, then report it
template <typename F>
int with_err(void *stream, F body)
{
    cudaStream_t st = as_stream(stream);
    Scratch scratch(st);
    uint32_t *err = scratch.get<uint32_t>(1);
    if (err == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    VSMC_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    int rc = body(err, scratch, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    int status = VSMC_CUDA_OK;
    rc = read_err(err, st, &status);
    return rc != VSMC_CUDA_OK ? rc : status;
}

bool valid_philox(const vsmc_cuda_rng *r)
{
    return r != nullptr && r->kind == VSMC_CUDA_PHILOX4X32 && r->index >= 1 &&
        r->index <= 4;
}

} // namespace

extern "C" {

int vsmc_cuda_u01_sorted(size_t n, const double *u01, double *u01seq,
    void *stream)
{
    if ((u01 == nullptr || u01seq == nullptr) && n)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    if (n == 0)
        return VSMC_CUDA_OK;
    return with_err(stream, [&](uint32_t *err, Scratch &sc, cudaStream_t st) -> int {
        double *t = sc.get<double>(n);
        if (t == nullptr)
            return static_cast<int>(VSMC_CUDA_ERR_ALLOC);
        k_sorted_terms_arr<<<grid1(n), kB, 0, st>>>(n, u01, t);
        VSMC_CUDA_CHECK_LAUNCH();
        int rc = seqsum_device(n, t, t, nullptr, err, sc, st, true);
        if (rc != VSMC_CUDA_OK)
            return rc;
        k_sorted_finish<<<grid1(n), kB, 0, st>>>(n, t, u01seq);
        VSMC_CUDA_CHECK_LAUNCH();
        return static_cast<int>(VSMC_CUDA_OK);
    });
}

int vsmc_cuda_u01_stratified(size_t n, const double *u01, double *u01seq,
    void *stream)
{
    if ((u01 == nullptr || u01seq == nullptr) && n)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    if (n == 0)
        return VSMC_CUDA_OK;
    k_stratified_arr<<<grid1(n), kB, 0, as_stream(stream)>>>(n, u01, u01seq);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_u01_systematic(size_t n, double u01, double *u01seq,
    void *stream)
{
    if (u01seq == nullptr && n)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    if (n == 0)
        return VSMC_CUDA_OK;
    return with_err(stream, [&](uint32_t *err, Scratch &sc, cudaStream_t st) -> int {
        double *t = sc.get<double>(n);
        if (t == nullptr)
            return static_cast<int>(VSMC_CUDA_ERR_ALLOC);
        k_systematic_terms<<<grid1(n), kB, 0, st>>>(n, u01, t);
        VSMC_CUDA_CHECK_LAUNCH();
        return seqsum_device(n, t, u01seq, nullptr, err, sc, st);
    });
}

int vsmc_cuda_resample_trans_u01_rep(size_t m, size_t n, const double *weight,
    const double *u01, int *replication, void *stream)
{
    if ((m && (weight == nullptr || replication == nullptr)) ||
        (n && m > 1 && u01 == nullptr))
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(m) || !size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    return with_err(stream, [&](uint32_t *err, Scratch &sc, cudaStream_t st) -> int {
        return u01_rep_device(m, n, weight, u01, replication, nullptr, err,
            sc, st);
    });
}

int vsmc_cuda_resample_trans_u01_index(size_t m, size_t n,
    const double *weight, const double *u01, int *index, void *stream)
{
    if (m == 0 || n == 0)
        return VSMC_CUDA_OK;
    if (weight == nullptr || u01 == nullptr || index == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(m) || !size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    return with_err(stream, [&](uint32_t *err, Scratch &sc, cudaStream_t st) -> int {
        if (m == 1) {
            k_fill_i32<<<grid1(n), kB, 0, st>>>(n, index, 0);
            VSMC_CUDA_CHECK_LAUNCH();
            return static_cast<int>(VSMC_CUDA_OK);
        }
        double *cdf = sc.get<double>(m - 1);
        double *pm = sc.get<double>(n);
        double *pp = sc.get<double>(scan_parts(n));
        if (!cdf || !pm || !pp)
            return static_cast<int>(VSMC_CUDA_ERR_ALLOC);
        int rc = seqsum_device(m - 1, weight, cdf, nullptr, err, sc, st);
        if (rc != VSMC_CUDA_OK)
            return rc;
        rc = device_scan(
            n, LoadKey{u01}, StoreD{pm}, OpMaxD(), -static_cast<double>(INFINITY), pp, st);
        if (rc != VSMC_CUDA_OK)
            return rc;
        k_index_from_cdf<<<grid1(n), kB, 0, st>>>(m, n, cdf, pm, index);
        VSMC_CUDA_CHECK_LAUNCH();
        return static_cast<int>(VSMC_CUDA_OK);
    });
}

int vsmc_cuda_resample_trans_rep_index(size_t m, size_t n,
    const int *replication, int *index, void *stream)
{
    if (m == 0 || n == 0)
        return VSMC_CUDA_OK;
    if (replication == nullptr || index == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(m) || !size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    return with_err(stream, [&](uint32_t *err, Scratch &sc, cudaStream_t st) -> int {
        return rep_index_device(m, n, replication, index, err, sc, st);
    });
}

int vsmc_cuda_resample_trans_index_rep(size_t m, size_t n, const int *index,
    int *replication, void *stream)
{
    if (m == 0 || n == 0)
        return VSMC_CUDA_OK;
    if (replication == nullptr || index == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(m) || !size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    return with_err(stream, [&](uint32_t *err, Scratch &sc, cudaStream_t st) -> int {
        (void)sc;
        VSMC_CUDA_TRY(cudaMemsetAsync(replication, 0, sizeof(int) * m, st));
        k_hist<<<grid1(n), kB, 0, st>>>(m, n, index, replication, err);
        VSMC_CUDA_CHECK_LAUNCH();
        return static_cast<int>(VSMC_CUDA_OK);
    });
}

int vsmc_cuda_resample_trans_residual(size_t m, size_t n,
    const double *weight, double *resid, int *integ, size_t *r_host,
    void *stream)
{
    if (r_host == nullptr ||
        (m && (weight == nullptr || resid == nullptr || integ == nullptr)))
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(m) || !size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    return with_err(stream, [&](uint32_t *err, Scratch &sc, cudaStream_t st) -> int {
        return residual_device(m, n, weight, resid, integ, r_host, err, sc, st);
    });
}

int vsmc_cuda_resample(size_t m, size_t n, vsmc_cuda_rng *rng,
    const double *weight, int *replication, int scheme, void *stream)
{
    if (!valid_philox(rng) || scheme < VSMC_CUDA_MULTINOMIAL ||
        scheme > VSMC_CUDA_RESIDUAL_SYSTEMATIC ||
        (m && (weight == nullptr || replication == nullptr)))
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(m) || !size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    cudaStream_t st = as_stream(stream);
    Scratch scratch(st);
    return scheme_device(m, n, rng, weight, replication, scheme, scratch, st);
}

#define VSMC_CUDA_SCHEME_ENTRY(name, id)                                      \
    int vsmc_cuda_resample_##name(size_t m, size_t n, vsmc_cuda_rng *rng,     \
        const double *weight, int *replication, void *stream)                 \
    {                                                                         \
        return vsmc_cuda_resample(m, n, rng, weight, replication, id, stream); \
    }

VSMC_CUDA_SCHEME_ENTRY(multinomial, VSMC_CUDA_MULTINOMIAL)
VSMC_CUDA_SCHEME_ENTRY(stratified, VSMC_CUDA_STRATIFIED)
VSMC_CUDA_SCHEME_ENTRY(systematic, VSMC_CUDA_SYSTEMATIC)
VSMC_CUDA_SCHEME_ENTRY(residual, VSMC_CUDA_RESIDUAL)
VSMC_CUDA_SCHEME_ENTRY(residual_stratified, VSMC_CUDA_RESIDUAL_STRATIFIED)
VSMC_CUDA_SCHEME_ENTRY(residual_systematic, VSMC_CUDA_RESIDUAL_SYSTEMATIC)

int vsmc_cuda_state_copy_f32(size_t n, size_t dim, const int *index,
    float *state, void *stream)
{
    if (n && (index == nullptr || state == nullptr))
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    if (n == 0 || dim == 0)
        return VSMC_CUDA_OK;
    const int rc = with_err(stream, [&](uint32_t *err, Scratch &, cudaStream_t st) -> int {
        return state_copy_device<float>(n, dim, n, index, state, err, st);
    });
    return rc == VSMC_CUDA_ERR_INTERNAL ? VSMC_CUDA_ERR_ARG : rc;
}

int vsmc_cuda_state_copy_f64(size_t n, size_t dim, const int *index,
    double *state, void *stream)
{
    if (n && (index == nullptr || state == nullptr))
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    if (n == 0 || dim == 0)
        return VSMC_CUDA_OK;
    const int rc = with_err(stream, [&](uint32_t *err, Scratch &, cudaStream_t st) -> int {
        return state_copy_device<double>(n, dim, n, index, state, err, st);
    });
    return rc == VSMC_CUDA_ERR_INTERNAL ? VSMC_CUDA_ERR_ARG : rc;
}

int vsmc_cuda_weight_set(size_t n, const double *w, double *W,
    double *ess_dev, void *stream)
{
    if (n == 0)
        return VSMC_CUDA_OK;
    if (w == nullptr || W == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    return with_err(stream, [&](uint32_t *err, Scratch &sc, cudaStream_t st) -> int {
        if (W != w)
            VSMC_CUDA_TRY(cudaMemcpyAsync(W, w, sizeof(double) * n,
                cudaMemcpyDeviceToDevice, st));
        return weight_normalize_device(n, W, ess_dev, err, sc, st);
    });
}

int vsmc_cuda_weight_set_log(size_t n, const double *lw, double *W,
    double *ess_dev, void *stream)
{
    if (n == 0)
        return VSMC_CUDA_OK;
    if (lw == nullptr || W == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    return with_err(stream, [&](uint32_t *err, Scratch &sc, cudaStream_t st) -> int {
        if (W != lw)
            VSMC_CUDA_TRY(cudaMemcpyAsync(W, lw, sizeof(double) * n,
                cudaMemcpyDeviceToDevice, st));
        return weight_post_set_log_device(n, W, ess_dev, err, sc, st);
    });
}

int vsmc_cuda_weight_add_log(size_t n, const double *l, double *W,
    double *ess_dev, void *stream)
{
    if (n == 0)
        return VSMC_CUDA_OK;
    if (l == nullptr || W == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    return with_err(stream, [&](uint32_t *err, Scratch &sc, cudaStream_t st) -> int {
        return weight_add_log_device(n, l, W, ess_dev, err, sc, st);
    });
}

int vsmc_cuda_weight_set_equal(size_t n, double *W, double *ess_dev,
    void *stream)
{
    if (n == 0)
        return VSMC_CUDA_OK;
    if (W == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(n))
        return VSMC_CUDA_ERR_SIZE;
    return with_err(stream, [&](uint32_t *err, Scratch &sc, cudaStream_t st) -> int {
        return weight_set_equal_device(n, W, ess_dev, err, sc, st);
    });
}

int vsmc_cuda_monitor_mean_f64(size_t n, size_t dim, const double *state,
    const double *W, double *out_dev, void *stream)
{
    if (state == nullptr || W == nullptr || out_dev == nullptr || dim > 32)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(n) || n == 0)
        return VSMC_CUDA_ERR_SIZE;
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    return monitor_mean_device<double>(n, dim, n, state, W, out_dev, sc, st);
}

int vsmc_cuda_monitor_mean_f32(size_t n, size_t dim, const float *state,
    const double *W, double *out_dev, void *stream)
{
    if (state == nullptr || W == nullptr || out_dev == nullptr || dim > 32)
        return VSMC_CUDA_ERR_ARG;
    if (!size_ok(n) || n == 0)
        return VSMC_CUDA_ERR_SIZE;
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    return monitor_mean_device<float>(n, dim, n, state, W, out_dev, sc, st);
}

} // extern "C"
