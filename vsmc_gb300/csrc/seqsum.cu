// Left-to-right double summation, bit-identical to a sequential loop, in
// parallel.
//
// The reference accumulates its resampling CDF and its normalizing sums one
// element at a time (resample/transform.hpp:61-69, core/weight.hpp:224-229,
// resample/transform.hpp:164).  For non-negative terms the running sum s is
// non-decreasing, and while s_{i-1} and s_i stay in one binade [2^e, 2^(e+1))
// every partial sum is a multiple of u = 2^(e-52), so
//     s_i = fl(s_{i-1} + x_i) = s_{i-1} + rint(x_i / u) * u
// whenever x_i / u is not exactly half-way (a tie rounds to even, which
// depends on s_{i-1}).  The increment rint(x_i / u) is an exact integer that
// does not depend on s_{i-1}, so runs of such elements are an exact integer
// prefix sum.  What is left -- the first element, elements whose running sum
// may cross a power of two, ties, and sums too small for the relative
// bounds -- is a short list of breakpoints, evaluated in order by one thread
// with real IEEE additions.  The binade of every running sum is taken from an
// approximate parallel prefix P with the margin 2^-19 relative, far above
// both |P - exact| and |sequential - exact| <= (n - 1) 2^-53 (n < 2^31).
//
// The classification works on the doubles' bit patterns with integer
// operations (GB300's FP64 rate is a small fraction of its integer rate),
// and runs once per element inside the scan that counts breakpoints; the
// later passes read breakpoints and increments back from the scan's output.
// Between breakpoints every running sum lies in one binade, so
// s_i = s_b + (r_b+1 + ... + r_i) u is the bit pattern of s_b plus that
// integer.
#include "common.cuh"
#include "scan.cuh"
#include "seqsum.cuh"

#include <cmath>

namespace vsmc_cuda
{

namespace
{

struct RF {
    uint64_t r;   // integer increment in units of the element's binade ulp
    uint32_t f;   // 1 = breakpoint
    uint32_t own; // the right operand's own flag (the element's, in a scan)
};

// Sums (r, f); `own` takes the right operand's, which is associative, so
// an inclusive scan leaves each element's own breakpoint flag in it.
struct OpRF {
    __device__ __forceinline__ RF operator()(const RF &a, const RF &b) const
    {
        return {a.r + b.r, a.f + b.f, b.own};
    }
};

// The margin tests on the fraction field f (units of 2^-52) of P, for
// m = 2^-19:
//   P (1 - m) >= 2^e       holds when f >= 2^33 + 2^14 + 1 (> 2^52 m / (1 - m))
//   P (1 + m) <  2^(e + 1) holds when f <  2^52 - 2^34     (< 2^52 (1 - m) / (1 + m))
constexpr uint64_t kFracMask = (1ull << 52) - 1;
constexpr uint64_t kFracLo = (1ull << 33) + (1ull << 14) + 1;
constexpr uint64_t kFracHi = (1ull << 52) - (1ull << 34);
constexpr uint32_t kExpMin = 1023 - 1000; // running sums below 2^-1000 are breakpoints

// exact power of two (ldexp scales without rounding)
__device__ __forceinline__ double pow2(int k) { return ldexp(1.0, k); }

__device__ __forceinline__ uint64_t dbits(double v)
{
    return static_cast<uint64_t>(__double_as_longlong(v));
}

// classification of element i from the approximate prefix P
struct Class {
    bool regular;
    int e;      // binade of s_{i-1} and s_i (regular only)
    uint64_t r; // rint(x_i / 2^(e-52)) (regular only)
};

__device__ __forceinline__ Class classify(size_t i, const double *x,
    const double *P, uint32_t *err, bool allow_inf)
{
    // every load up front and every test as a flag (no early return), so
    // the loads of a thread's elements can all be in flight together
    const uint64_t xb = dbits(x[i]);
    const uint64_t pa = dbits(P[i > 0 ? i - 1 : 0]);
    const uint64_t pb = dbits(P[i]);
    const uint32_t xe = static_cast<uint32_t>(xb >> 52) & 0x7FFu;
    const uint64_t xf = xb & kFracMask;
    // x >= 0 fails for NaN and for negatives other than -0
    const bool bad = (xe == 0x7FFu && xf != 0) || ((xb >> 63) && (xb << 1));
    const bool inf = xe == 0x7FFu && xf == 0;
    if (bad || (inf && !allow_inf)) {
        if (err)
            atomicOr(err, DEV_ERR_NONFINITE);
    }
    const uint32_t ea = static_cast<uint32_t>(pa >> 52); // sign bit included
    bool ok = !bad & !inf & (i != 0);
    ok &= (ea >= kExpMin) & (ea <= 2046u) & ((pa & kFracMask) >= kFracLo);
    ok &= (static_cast<uint32_t>(pb >> 52) == ea) & ((pb & kFracMask) < kFracHi);
    const int e = static_cast<int>(ea) - 1023;
    // x = mant 2^q; x / 2^(e-52) = mant / 2^k with k = e - 52 - q; k < 0
    // (x above the running sum's binade) is left to the fix-up
    const uint64_t mant = xe ? (xf | (1ull << 52)) : xf;
    const int q = (xe ? static_cast<int>(xe) : 1) - 1075;
    const int k = e - 52 - q;
    ok &= k >= 0;
    // k >= 64: mant < 2^53 <= 2^(k-1), below half a unit and no tie
    const int kk = k < 1 ? 1 : (k > 63 ? 63 : k);
    const uint64_t rem = mant & ((1ull << kk) - 1);
    const uint64_t half = 1ull << (kk - 1);
    const bool mid = k >= 1 && k <= 63;
    ok &= !(mid && rem == half); // a tie: rounding depends on the sum's parity
    const uint64_t r = k == 0 ? mant
        : (k > 63 ? 0ull : (mant >> kk) + (rem > half ? 1ull : 0ull));
    Class c;
    c.regular = ok;
    c.e = e;
    c.r = ok ? r : 0ull;
    return c;
}

struct LoadX {
    const double *x;
    __device__ double operator()(size_t i) const { return x[i]; }
};

struct StoreD {
    double *p;
    __device__ void operator()(size_t i, double v) const { p[i] = v; }
};

struct LoadRF {
    const double *x;
    const double *P;
    uint32_t *err;
    bool allow_inf;
    __device__ RF operator()(size_t i) const
    {
        const Class c = classify(i, x, P, err, allow_inf);
        const uint32_t f = c.regular ? 0u : 1u;
        return {c.regular ? c.r : 0ull, f, f};
    }
};

// The scan's output, and the breakpoint records in order: breakpoint k
// (the element whose inclusive count f steps to k + 1) is at bidx[k], with
// the increments through it (its own r is 0) in bcr[k].
struct StoreRF {
    RF *p;
    uint32_t *bidx;
    uint64_t *bcr;
    __device__ void operator()(size_t i, RF v) const
    {
        p[i] = v;
        if (v.own) {
            bidx[v.f - 1] = static_cast<uint32_t>(i);
            bcr[v.f - 1] = v.r;
        }
    }
};

// One block walks the breakpoints in order with real additions.
__global__ void __launch_bounds__(256) k_fixup(size_t n, const double *x,
    const double *P, const RF *C, const uint32_t *bidx, const uint64_t *bcr,
    double *sb, double *total, uint32_t *err, bool allow_inf)
{
    __shared__ double s_xb[256];
    __shared__ uint32_t s_b[256];
    __shared__ uint64_t s_crm1[256];
    __shared__ int s_em1[256];
    __shared__ int s_reg_m1[256];
    const uint32_t nbk = C[n - 1].f;
    double S = 0.0;          // value at the previous breakpoint
    uint32_t bprev = 0;
    uint64_t crprev = 0;
    for (uint32_t c0 = 0; c0 < nbk; c0 += 256) {
        const uint32_t k = c0 + threadIdx.x;
        if (k < nbk) {
            const uint32_t b = bidx[k];
            s_b[threadIdx.x] = b;
            s_xb[threadIdx.x] = x[b];
            if (b > 0) {
                const Class cm = classify(b - 1, x, P, nullptr, allow_inf);
                s_reg_m1[threadIdx.x] = cm.regular ? 1 : 0;
                s_em1[threadIdx.x] = cm.e;
                s_crm1[threadIdx.x] = C[b - 1].r;
            } else {
                s_reg_m1[threadIdx.x] = 0;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t m = nbk - c0 < 256 ? nbk - c0 : 256;
            for (uint32_t j = 0; j < m; ++j) {
                const uint32_t b = s_b[j];
                double sp;
                if (c0 + j == 0) {
                    sp = 0.0;
                    if (b != 0)
                        atomicOr(err, DEV_ERR_INTERNAL);
                } else if (!s_reg_m1[j]) {
                    sp = S; // b - 1 is the previous breakpoint
                    if (b - 1 != bprev)
                        atomicOr(err, DEV_ERR_INTERNAL);
                } else {
                    sp = S + static_cast<double>(s_crm1[j] - crprev) *
                            pow2(s_em1[j] - 52);
                }
                S = __dadd_rn(sp, s_xb[j]);
                sb[c0 + j] = S;
                bprev = b;
                crprev = bcr[c0 + j];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && total != nullptr) {
        const Class cl = classify(n - 1, x, P, nullptr, allow_inf);
        if (cl.regular)
            *total = S + static_cast<double>(C[n - 1].r - crprev) *
                    pow2(cl.e - 52);
        else
            *total = S;
    }
}

// s_i from its breakpoint: the breakpoint's own sum, or that sum's bit
// pattern plus the integer increments since (one binade, one ulp grid)
__global__ void __launch_bounds__(256) k_prefix_out(size_t n, const RF *C,
    const uint64_t *bcr, const double *sb, double *out, uint32_t *err)
{
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
         i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const RF ci = C[i];
        const uint32_t k = ci.f - 1;
        double s;
        if (ci.own) {
            s = sb[k];
        } else {
            const uint64_t b = dbits(sb[k]);
            const uint64_t v = b + (ci.r - bcr[k]);
            // the sum must stay in the breakpoint's binade (sign included)
            if ((v >> 52) != (b >> 52))
                atomicOr(err, DEV_ERR_BOUND);
            s = __longlong_as_double(static_cast<long long>(v));
        }
        out[i] = s;
    }
}

} // namespace

int seqsum_device(size_t n, const double *x, double *prefix, double *total,
    uint32_t *err, Scratch &scratch, cudaStream_t st, bool allow_inf)
{
    if (n == 0) {
        if (total)
            VSMC_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(double), st));
        return VSMC_CUDA_OK;
    }
    if (n >= (size_t(1) << 31))
        return VSMC_CUDA_ERR_SIZE;
    const size_t nb = scan_parts(n);
    double *P = scratch.get<double>(n);
    double *pd = scratch.get<double>(nb);
    RF *C = scratch.get<RF>(n);
    RF *pr = scratch.get<RF>(nb);
    uint32_t *bidx = scratch.get<uint32_t>(n);
    uint64_t *bcr = scratch.get<uint64_t>(n);
    double *sb = scratch.get<double>(n);
    if (!P || !pd || !C || !pr || !bidx || !bcr || !sb)
        return VSMC_CUDA_ERR_ALLOC;
    int rc = device_scan(n, LoadX{x}, StoreD{P}, OpAdd(), 0.0, pd, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    rc = device_scan(n, LoadRF{x, P, err, allow_inf}, StoreRF{C, bidx, bcr},
        OpRF(), RF{0, 0, 0}, pr, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    const int grid = grid_for(n, 256, 4, 8);
    k_fixup<<<1, 256, 0, st>>>(
        n, x, P, C, bidx, bcr, sb, total, err, allow_inf);
    if (prefix)
        k_prefix_out<<<grid, 256, 0, st>>>(n, C, bcr, sb, prefix, err);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int read_err(uint32_t *err_dev, cudaStream_t st, int *status)
{
    uint32_t e = 0;
    VSMC_CUDA_TRY(cudaMemcpyAsync(
        &e, err_dev, sizeof(e), cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    if (e & DEV_ERR_NONFINITE)
        *status = VSMC_CUDA_ERR_NONFINITE;
    else if (e)
        *status = VSMC_CUDA_ERR_INTERNAL;
    else
        *status = VSMC_CUDA_OK;
    return VSMC_CUDA_OK;
}

} // namespace vsmc_cuda

using namespace vsmc_cuda;

extern "C" int vsmc_cuda_sequential_sum(size_t n, const double *x,
    double *prefix, double *total_dev, void *stream)
{
    if ((x == nullptr && n) || (prefix == nullptr && total_dev == nullptr))
        return VSMC_CUDA_ERR_ARG;
    cudaStream_t st = as_stream(stream);
    Scratch scratch(st);
    uint32_t *err = scratch.get<uint32_t>(1);
    if (err == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    VSMC_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    int rc = seqsum_device(n, x, prefix, total_dev, err, scratch, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    int status = VSMC_CUDA_OK;
    rc = read_err(err, st, &status);
    return rc != VSMC_CUDA_OK ? rc : status;
}
