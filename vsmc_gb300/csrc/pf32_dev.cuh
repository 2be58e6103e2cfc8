// Device helpers of the FP32 filters (single and batched): log-sum-exp
// accumulation, the resampling engine's word stream, and exact counting of
// systematic / stratified uniforms against a 64-bit fixed-point CDF.
#pragma once

#include "common.cuh"
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

// merge (m2, t, t2) into (m, s, s2): max, sum exp(v - m), sum exp(2(v - m))
__device__ __forceinline__ void lse_merge_f(
    float &m, float &s, float &s2, float m2, float t, float t2)
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
        const float e = __expf(m - m2);
        s = s * e + t;
        s2 = s2 * e * e + t2;
        m = m2;
    } else {
        const float e = __expf(m2 - m);
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

// Counting uniforms against the fixed-point CDF.
//
// Uniform j is u_j = (j + a_j 2^-32) / N with a 32-bit word a_j.  With the
// integer CDF C_i and total Q, u_j <= C / Q  <=>  (j 2^32 + a_j) Q <= C N 2^32
// <=>  j Q + G_j <= C N  with G_j = ceil(a_j Q / 2^32) < Q, since both sides
// are integers.  The counts follow from one exact floor(C N / Q) with its
// remainder per CDF value.
struct CountP {
    uint64_t Q;     // CDF total
    uint64_t G;     // systematic: ceil(a Q / 2^32) (one word for every j)
    uint32_t n;
    double dscale;  // n / Q
};

__device__ __forceinline__ uint64_t ceil_aq(uint32_t a, uint64_t Q)
{
    const uint64_t hi = __umul64hi(static_cast<uint64_t>(a), Q); // < 2^32
    const uint64_t lo = static_cast<uint64_t>(a) * Q;
    return ((hi << 32) | (lo >> 32)) + ((lo & 0xFFFFFFFFull) != 0 ? 1 : 0);
}

__device__ __forceinline__ CountP make_count_params(
    uint64_t Q, uint32_t n, uint32_t a_sys)
{
    CountP p;
    p.Q = Q;
    p.G = ceil_aq(a_sys, Q);
    p.n = n;
    p.dscale = static_cast<double>(n) / static_cast<double>(Q);
    return p;
}

// j = floor((C n - G) / Q) and r = (C n - G) - j Q; false if C n < G
__device__ __forceinline__ bool cn_divmod(uint64_t C, uint64_t G,
    const CountP &p, long long &j, uint64_t &r, uint32_t &err)
{
    uint64_t xh = __umul64hi(C, static_cast<uint64_t>(p.n));
    uint64_t xl = C * static_cast<uint64_t>(p.n);
    if (xl < G) {
        if (xh == 0)
            return false;
        --xh;
    }
    xl -= G;
    // estimate within a unit or two of the answer: C n / Q in FP64 is off
    // by at most n 2^-51 + 1 (three roundings), below 2 for any n < 2^31
    // (one FP64 product per call; callers make one per block or fewer)
    const double f = static_cast<double>(C) * p.dscale;
    long long jj = static_cast<long long>(f) - 2;
    if (jj < 0)
        jj = 0;
    if (jj > static_cast<long long>(p.n))
        jj = static_cast<long long>(p.n);
    // R = X - jj Q, 128-bit; walk down while negative, up while >= Q
    const uint64_t ph = __umul64hi(static_cast<uint64_t>(jj), p.Q);
    const uint64_t pl = static_cast<uint64_t>(jj) * p.Q;
    uint64_t rl = xl - pl;
    uint64_t rh = xh - ph - (xl < pl ? 1 : 0);
    int guard = 0;
    while (static_cast<long long>(rh) < 0) { // X < jj Q
        --jj;
        const uint64_t t = rl + p.Q;
        rh += (t < rl ? 1 : 0);
        rl = t;
        if (++guard > 64) {
            err |= DEV_ERR_BOUND;
            break;
        }
    }
    guard = 0;
    while (rh != 0 || rl >= p.Q) {
        ++jj;
        rh -= (rl < p.Q ? 1 : 0);
        rl -= p.Q;
        if (++guard > 64) {
            err |= DEV_ERR_BOUND;
            break;
        }
    }
    j = jj;
    r = rl;
    return true;
}

// floor(w * 2^shift) for w = exp(lw - M) in (0, 1], by integer operations on
// the float's bits (no 64-bit conversion instruction)
__device__ __forceinline__ uint64_t fixed_q(float lw, float M, uint32_t shift)
{
    if (!(lw > -INFINITY))
        return 0;
    const float w = fminf(__expf(lw - M), 1.0f);
    const uint32_t bits = __float_as_uint(w);
    const int e = static_cast<int>(bits >> 23); // biased exponent
    if (e == 0)
        return 0; // below 2^-126: floor(w 2^shift) == 0 for shift <= 63
    const uint64_t mant = (bits & 0x7FFFFFu) | 0x800000u;
    const int sh = e - 150 + static_cast<int>(shift); // w = mant * 2^(e-150)
    if (sh >= 0)
        return mant << sh;
    if (sh <= -64)
        return 0;
    return mant >> (-sh);
}

// A CDF value's position against the uniforms, X = C n - G (G = 0 for
// stratified), kept as X = (j - 1) Q + r with 0 <= r < Q.  Then F(C) = j
// (systematic, clamped to n), or j - 1 plus one if uniform j - 1 lies at or
// below C / Q (stratified).  A step of the CDF adds q n to X, so positions
// follow from one 128-bit division per block, then only additions.
struct QR {
    uint32_t j;
    uint64_t r;
};

__device__ __forceinline__ QR qr_add(const QR &a, const QR &b, uint64_t Q)
{
    QR c;
    c.j = a.j + b.j;
    c.r = a.r + b.r; // both below Q < 2^63: no wrap
    if (c.r >= Q) {
        c.r -= Q;
        ++c.j;
    }
    return c;
}

// A quotient estimate of r / Q that never exceeds the true quotient.  The
// conversion of r (toward zero, then one rounding) is within 1.5 2^-23 of
// r, invQ = rcp(float(Q)) within 2^-23 of 1 / Q, and the two products add
// 2^-23: est <= (r / Q)(1 + 3.5 2^-23)(1 - 2^-20) < r / Q.  Its floor is at
// most the quotient, and at least the quotient minus (r / Q) 1.4e-6 + 1.
__device__ __forceinline__ uint32_t quot_below(uint64_t r, float invQ)
{
    const float est = fmaf(__uint2float_rz(static_cast<uint32_t>(r >> 32)),
                          4294967296.0f,
                          __uint2float_rz(static_cast<uint32_t>(r))) *
        invQ * (1.0f - 0x1p-20f);
    return __float2uint_rz(est);
}

// Bring r below Q, adding the quotient to j.  Every lane takes the same
// path: one estimate from below (quot_below; 0 when r < Q), which leaves at
// most (r / Q) 1.4e-6 + 1 (below 2 for fewer than 7e5 copies), then two
// conditional steps, so the warp does not split on how many copies its
// lanes' particles take.  Only a position advanced by 7e5 or more copies
// needs the second estimate (a quotient below 2^31 always leaves less than
// 2 after it), and one more step.
__device__ __forceinline__ void qr_reduce(
    uint64_t &r, uint32_t &j, uint64_t Q, float invQ, uint32_t &err)
{
    uint32_t d = quot_below(r, invQ);
    r -= static_cast<uint64_t>(d) * Q; // d Q <= r: no wrap
    j += d;
    if (r >= Q) {
        r -= Q;
        ++j;
    }
    if (r >= Q) {
        r -= Q;
        ++j;
    }
    if (r >= Q) { // 7e5 or more copies: a second estimate
        d = quot_below(r, invQ);
        r -= static_cast<uint64_t>(d) * Q;
        j += d;
        if (r >= Q) {
            r -= Q;
            ++j;
        }
        if (r >= Q) {
            r -= Q;
            ++j;
        }
        if (r >= Q) // unreachable by the bounds above; recorded if ever
            err |= DEV_ERR_BOUND;
    }
}

// q n added to a position.  Filter weights satisfy q <= 2^K and
// n <= 2^(63 - K), so q n <= 2^63 and r + q n < 2^64; integer weights given
// by a caller are checked and take the 128-bit division when they do not.
__device__ __forceinline__ void qr_push(QR &acc, uint64_t q, uint32_t n,
    bool checked, uint64_t Q, float invQ, const CountP &cp, uint32_t &err)
{
    if (checked) {
        const uint64_t plo = static_cast<uint64_t>(static_cast<uint32_t>(q)) * n;
        const uint64_t phi = (q >> 32) * n;
        const uint64_t lo = plo + (phi << 32);
        const uint64_t hi = (phi >> 32) + (lo < plo ? 1 : 0);
        const uint64_t s = acc.r + lo;
        if (hi != 0 || s < lo) {
            long long jj;
            uint64_t rr;
            cn_divmod(q, 0, cp, jj, rr, err);
            acc = qr_add(acc, QR{static_cast<uint32_t>(jj), rr}, Q);
            return;
        }
        acc.r = s;
    } else {
        acc.r += q * n;
    }
    qr_reduce(acc.r, acc.j, Q, invQ, err);
}

// Stratified counting needs, for each CDF position X = (j - 1) Q + r, the
// engine word of uniform j - 1.  A tile's positions are nondecreasing, so
// the words it needs lie in one range of the engine stream; the block
// generates that range's Philox blocks once into shared memory (one or two
// per thread) instead of each thread generating the blocks its own
// positions fall in.  Block b of the stream is at wb[b - b0] for
// b0 <= b < b0 + nb; a block beyond the buffer (a tile whose positions
// span more than it) is generated where it is needed.
struct WordBuf {
    const uint4 *wb;
    uint32_t b0, nb;
};

// block b of the engine stream, for the rare word outside the buffer (not
// inlined: it stays off the register budget of the common path)
static __device__ __noinline__ uint4 engine_block_at(
    const PfScalars &sc, uint32_t b)
{
    uint32_t c[4] = {sc.rctr[0], sc.rctr[1], sc.rctr[2], sc.rctr[3]};
    ctr32_add(c, b);
    const u32x4 p =
        philox4x32_10(c[0], c[1], c[2], c[3], sc.rkey[0], sc.rkey[1]);
    return make_uint4(p.x, p.y, p.z, p.w);
}

// word `pos` (rindex + j) of the engine stream
__device__ __forceinline__ uint32_t buf_word(
    const PfScalars &sc, uint32_t pos, const WordBuf &w)
{
    const uint32_t b = pos >> 2;
    const uint32_t d = b - w.b0;
    const uint4 v = d < w.nb ? w.wb[d] : engine_block_at(sc, b);
    const uint32_t r = pos & 3u;
    return r == 0 ? v.x : (r == 1 ? v.y : (r == 2 ? v.z : v.w));
}

// F from a position (see QR), the stratified words from the tile's buffer
__device__ __forceinline__ uint32_t f_of_buf(const QR &x, bool sys,
    uint32_t n, uint64_t Q, const PfScalars &sc, const WordBuf &w)
{
    if (sys)
        return x.j < n ? x.j : n;
    if (x.j == 0)
        return 0;
    const uint32_t j0 = x.j - 1;
    if (j0 >= n)
        return n;
    return j0 + (ceil_aq(buf_word(sc, sc.rindex + j0, w), Q) <= x.r ? 1u
                                                                     : 0u);
}

// The engine words [wlo, whi] (empty when wlo > whi) a thread may need:
// from its start position st to the position after its last particle,
// last = st + loc (a superset of what f_of_buf reads).
__device__ __forceinline__ void words_span(const QR &st, const QR &last,
    uint32_t n, const PfScalars &sc, uint32_t &wlo, uint32_t &whi)
{
    const uint32_t jl = st.j >= 1 ? st.j - 1 : 0;
    const uint32_t jh = (last.j < n ? last.j : n);
    if (jh == 0 || jl > jh - 1) {
        wlo = 0xFFFFFFFFu;
        whi = 0;
    } else {
        wlo = sc.rindex + jl;
        whi = sc.rindex + (jh - 1);
    }
}

// Generates the Philox blocks covering every thread's [wlo, whi] into wb
// (cap blocks) and returns the buffer view.  sh holds 2 * kBlock / 32
// entries.  Call with the whole block; it has two barriers.
template <int kBlock>
__device__ __forceinline__ WordBuf fill_words(const PfScalars &sc,
    uint32_t wlo, uint32_t whi, uint4 *wb, uint32_t cap, uint32_t *sh)
{
    constexpr int kW = kBlock / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t lo = __reduce_min_sync(0xFFFFFFFFu, wlo);
    const uint32_t hi = __reduce_max_sync(0xFFFFFFFFu, whi);
    if (lane == 0) {
        sh[wid] = lo;
        sh[kW + wid] = hi;
    }
    __syncthreads();
    uint32_t blo = 0xFFFFFFFFu, bhi = 0;
#pragma unroll
    for (int k = 0; k < kW; ++k) {
        blo = min(blo, sh[k]);
        bhi = max(bhi, sh[kW + k]);
    }
    WordBuf w;
    w.wb = wb;
    w.b0 = 0;
    w.nb = 0;
    if (blo <= bhi) {
        w.b0 = blo >> 2;
        const uint32_t nb = (bhi >> 2) - w.b0 + 1;
        w.nb = nb < cap ? nb : cap;
        for (uint32_t d = threadIdx.x; d < w.nb; d += kBlock) {
            uint32_t c[4] = {sc.rctr[0], sc.rctr[1], sc.rctr[2], sc.rctr[3]};
            ctr32_add(c, w.b0 + d);
            const u32x4 p =
                philox4x32_10(c[0], c[1], c[2], c[3], sc.rkey[0], sc.rkey[1]);
            wb[d] = make_uint4(p.x, p.y, p.z, p.w);
        }
    }
    __syncthreads();
    return w;
}

// Block-wide exclusive scan of positions over kBlock threads; *total gets
// the block's sum; sh holds kBlock / 32 entries.
template <int kBlock = kPfBlock>
__device__ __forceinline__ QR block_exclusive_qr(
    QR v, uint64_t Q, QR *sh, QR *total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int nw = kBlock / 32;
    QR x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        QR o;
        o.j = __shfl_up_sync(0xFFFFFFFFu, x.j, d);
        o.r = __shfl_up_sync(0xFFFFFFFFu, x.r, d);
        if (lane >= d)
            x = qr_add(o, x, Q);
    }
    if (lane == 31)
        sh[wid] = x;
    __syncthreads();
    if (wid == 0) {
        QR w = lane < nw ? sh[lane] : QR{0, 0};
#pragma unroll
        for (int d = 1; d < nw; d <<= 1) {
            QR o;
            o.j = __shfl_up_sync(0xFFFFFFFFu, w.j, d);
            o.r = __shfl_up_sync(0xFFFFFFFFu, w.r, d);
            if (lane >= d)
                w = qr_add(o, w, Q);
        }
        if (lane < nw)
            sh[lane] = w;
    }
    __syncthreads();
    QR ex;
    ex.j = __shfl_up_sync(0xFFFFFFFFu, x.j, 1);
    ex.r = __shfl_up_sync(0xFFFFFFFFu, x.r, 1);
    if (lane == 0)
        ex = QR{0, 0};
    if (wid > 0)
        ex = qr_add(sh[wid - 1], ex, Q);
    *total = sh[nw - 1];
    __syncthreads();
    return ex;
}

// counts of slots i0..i0+3 below hi (-1 past hi)
__device__ __forceinline__ int4 load_rep4(
    const int32_t *rep, uint32_t i0, uint32_t hi)
{
    if (i0 + 3 < hi)
        return __ldcg(reinterpret_cast<const int4 *>(rep + i0));
    int4 v;
    v.x = i0 + 0 < hi ? rep[i0 + 0] : -1;
    v.y = i0 + 1 < hi ? rep[i0 + 1] : -1;
    v.z = i0 + 2 < hi ? rep[i0 + 2] : -1;
    v.w = i0 + 3 < hi ? rep[i0 + 3] : -1;
    return v;
}

// row values i0..i0+3 below hi (0 past hi); i0 is a multiple of 4
__device__ __forceinline__ float4 load_row4(
    const float *row, uint32_t i0, uint32_t hi)
{
    if (i0 + 3 < hi)
        return __ldcs(reinterpret_cast<const float4 *>(row + i0));
    float4 v;
    v.x = i0 + 0 < hi ? row[i0 + 0] : 0.0f;
    v.y = i0 + 1 < hi ? row[i0 + 1] : 0.0f;
    v.z = i0 + 2 < hi ? row[i0 + 2] : 0.0f;
    v.w = i0 + 3 < hi ? row[i0 + 3] : 0.0f;
    return v;
}

// Surplus runs of one warp's 128 particles.  A parent with r >= 2 copies
// keeps one in its own slot and its other r - 1 fill the next r - 1 empty
// slots in order, so the warp's parents own consecutive runs that together
// cover the warp's surplus ranks [W0, W0 + S) exactly.  The sources
// srcs[W0 .. W0 + S) are written in order from position p:
//   * when the run holding p goes on for at least a chunk (kRunChunk ranks),
//     the warp stores its parent up to the run's end directly (32
//     consecutive ranks per store), so a parent with a huge copy count costs
//     its ranks' stores and nothing more;
//   * otherwise each parent marks the first rank of its run inside the
//     chunk [p, p + kRunChunk) in the warp's shared-memory row, a warp
//     max-scan over the chunk gives every rank its parent, and the warp
//     stores the chunk (coalesced).
// Warp-synchronous: called by every lane with warp-uniform W0 and S; rs / rl:
// the lane's runs (start rank, length; 0 for none).
constexpr uint32_t kRunChunk = 128;

__device__ __forceinline__ void write_surplus_runs(uint32_t *srcs,
    const uint32_t (&rs)[4], const uint32_t (&rl)[4], uint32_t i0,
    uint32_t W0, uint32_t S, uint32_t *shm, uint32_t &err)
{
    const uint32_t lane = threadIdx.x & 31;
    uint32_t p0 = 0;
    while (p0 < S) {
        // the run holding p0 (exactly one lane has it)
        uint32_t own_end = 0, own_par = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t b0 = rs[k] - W0;
            if (rl[k] != 0 && b0 <= p0 && p0 < b0 + rl[k]) {
                own_end = b0 + rl[k];
                own_par = i0 + k;
            }
        }
        const unsigned who = __ballot_sync(0xFFFFFFFFu, own_end != 0);
        if (who == 0) {
            err |= DEV_ERR_INTERNAL; // a rank no run covers
            return;
        }
        const int src = __ffs(who) - 1;
        const uint32_t end = __shfl_sync(0xFFFFFFFFu, own_end, src);
        const uint32_t par = __shfl_sync(0xFFFFFFFFu, own_par, src);
        const uint32_t stop = end < S ? end : S;
        if (stop - p0 >= kRunChunk) {
            for (uint32_t q = p0 + lane; q < stop; q += 32)
                srcs[W0 + q] = par;
            p0 = stop;
            continue;
        }
        reinterpret_cast<uint4 *>(shm)[lane] = make_uint4(0, 0, 0, 0);
        __syncwarp();
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (rl[k] == 0)
                continue;
            const uint32_t b0 = rs[k] - W0, b1 = b0 + rl[k];
            if (b1 > p0 && b0 < p0 + kRunChunk)
                shm[(b0 > p0 ? b0 : p0) - p0] = i0 + k + 1;
        }
        __syncwarp();
        const uint4 m = reinterpret_cast<const uint4 *>(shm)[lane];
        uint32_t run[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
        for (int j = 1; j < 4; ++j)
            run[j] = max(run[j], run[j - 1]);
        uint32_t incl = run[3];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<uint32_t>(o))
                incl = max(incl, y);
        }
        uint32_t before = __shfl_up_sync(0xFFFFFFFFu, incl, 1);
        if (lane == 0)
            before = 0;
        const uint32_t lim = S - p0 < kRunChunk ? S - p0 : kRunChunk;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t pos = 4 * lane + j;
            if (pos < lim) {
                const uint32_t o = max(run[j], before);
                if (o == 0)
                    err |= DEV_ERR_INTERNAL; // a rank no run covers
                srcs[W0 + p0 + pos] = o - 1;
            }
        }
        __syncwarp(); // the row is reused by the next chunk
        p0 += kRunChunk;
    }
}

} // namespace vsmc_cuda
