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
// <=>  j Q + G_j <= C N  with G_j = ceil(a_j Q / 2^32) <= Q, since both sides
// are integers.  The counts follow from one exact floor((C N - G) / Q) per
// CDF value (below).
__device__ __forceinline__ uint64_t ceil_aq(uint32_t a, uint64_t Q)
{
    const uint64_t hi = __umul64hi(static_cast<uint64_t>(a), Q); // < 2^32
    const uint64_t lo = static_cast<uint64_t>(a) * Q;
    return ((hi << 32) | (lo >> 32)) + ((lo & 0xFFFFFFFFull) != 0 ? 1 : 0);
}

__device__ __forceinline__ U128 sub_u128(const U128 &a, const U128 &b)
{
    return {a.hi - b.hi - (a.lo < b.lo ? 1ull : 0ull), a.lo - b.lo};
}

// floor((hi 2^64 + lo) / d) for hi < d (the quotient fits 64 bits).  Two
// FP64 estimates from below, each followed by the exact 128-bit remainder:
// the first is within 2^-47 of the quotient (relative), which leaves a
// remainder below (2^17 + 1) d; the second leaves less than 2 d; then at
// most two unit steps (bounded; DEV_ERR_BOUND if ever exceeded).  One
// thread calls it twice per resampling event.
__device__ __forceinline__ uint64_t div_u128_u64(
    uint64_t hi, uint64_t lo, uint64_t d, uint32_t &err)
{
    const double dd = static_cast<double>(d);
    U128 R = {hi, lo};
    uint64_t quo = 0;
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
        const double x =
            fma(static_cast<double>(R.hi), 0x1p64, static_cast<double>(R.lo));
        const double e = x / dd * (1.0 - 0x1p-48);
        const uint64_t t = e < 0x1p64 ? static_cast<uint64_t>(e) : 0ull;
        R = sub_u128(R, mul_u64(t, d));
        quo += t;
    }
    for (int s = 0; s < 4 && (R.hi != 0 || R.lo >= d); ++s) {
        R = sub_u128(R, U128{0, d});
        ++quo;
    }
    if (R.hi != 0 || R.lo >= d)
        err |= DEV_ERR_BOUND;
    return quo;
}

// Counting by a fixed-point reciprocal (no division per particle).
//
// Usual case (qs > 0, totals Q >= 2^20 n): with s fraction bits chosen so
// that 2^s n < Q <= 2^(s+1) n (s at most 32), m = floor(2^(64+s) n / Q) and
// gs = floor(2^s G / Q).  H, the high half of C m from three 32 x 32-bit
// products (the low x low product and the carries of the dropped halves
// left out), is 0 to 3 below C m / 2^64, and C m / 2^64 is within 0.5 below
// 2^s C n / Q (C < 2^63); so B = H - gs lies in (V - 4.5, V + 1) for
// V = 2^s (C n - G) / Q.  floor((C n - G) / Q) is then B >> s unless B's low
// s bits are below 2 or within 6 of 2^s; there one exact test settles it.
//
// Any other total: z = clz(Q), rcp = floor((2^128 - 1) / (Q << z)) - 2^64,
// gam = floor(2^64 G / Q) (2^64 - 1 when G = Q).  For C < Q, with
// C' = C << z, H = C' + umulhi(C', rcp) lies in (T - 2, T] for
// T = 2^64 C / Q, so B = n H - gam lies in (V - 2n, V + 1] for
// V = 2^64 (C n - G) / Q, and floor(V / 2^64) is B's high word unless B's
// low word is 0 or within 4n + 8 of 2^64.
//
// G = ceil(a Q / 2^32) for the systematic word a; stratified: G = 0.  The
// exact test for a candidate m is m Q + G <= C n in 128 bits.
struct CdfRcp {
    uint64_t Q, G;
    uint64_t m, gs; // usual case
    uint64_t rcp, gam;
    uint64_t wlim; // 2^64 - (4 n + 8): low words at or above it are checked
    uint32_t s, fmask, z, n; // fmask = 2^s - 1 (32 bits)
};

__device__ __forceinline__ CdfRcp load_cdf_rcp(const PfScalars &sc, uint32_t n)
{
    CdfRcp p;
    p.Q = sc.Q;
    p.G = sc.qG;
    p.m = sc.qm;
    p.gs = sc.qgs;
    p.s = sc.qs;
    p.fmask = static_cast<uint32_t>((1ull << sc.qs) - 1ull);
    p.rcp = sc.qrcp;
    p.gam = sc.qgam;
    p.z = sc.qz;
    p.n = n;
    p.wlim = 0ull - (4ull * n + 8ull);
    return p;
}

// floor((C n - G) / Q) when the estimate k may be one off: low means the
// answer is k or k - 1, otherwise k or k + 1
static __device__ __noinline__ int64_t cdf_floor_near(
    uint64_t C, int64_t k, bool low, uint64_t Q, uint64_t G, uint32_t n)
{
    const int64_t m = low ? k : k + 1;
    bool ok = true; // m <= floor((C n - G) / Q), i.e. m Q + G <= C n
    if (m >= 0) {
        const U128 cn = mul_u64(C, static_cast<uint64_t>(n));
        U128 mq = mul_u64(static_cast<uint64_t>(m), Q);
        const uint64_t l = mq.lo + G;
        mq.hi += l < mq.lo ? 1ull : 0ull;
        mq.lo = l;
        ok = le_u128(mq, cn);
    }
    if (low)
        return ok ? k : k - 1;
    return ok ? k + 1 : k;
}

// floor((C n - G) / Q) for C < Q (at least -1, below n).  Usual: the
// usual case's reciprocal (p.s > 0) is known to apply, so the loop that
// calls this holds one path only (the choice is made once per pass).
template <bool Usual>
__device__ __forceinline__ int64_t cdf_floor(uint64_t C, const CdfRcp &p)
{
    if (Usual) {
        const uint32_t c1 = static_cast<uint32_t>(C >> 32);
        const uint32_t c0 = static_cast<uint32_t>(C);
        const uint32_t m1 = static_cast<uint32_t>(p.m >> 32);
        const uint32_t m0 = static_cast<uint32_t>(p.m);
        const uint64_t H = static_cast<uint64_t>(c1) * m1 +
            __umulhi(c1, m0) + __umulhi(c0, m1);
        const uint64_t B = H - p.gs; // two's complement: -2^s <= B < 2^63
        const uint32_t bl = static_cast<uint32_t>(B);
        // B >> s (20 <= s <= 32): its low 32 bits are the signed answer
        const int32_t k = static_cast<int32_t>(
            __funnelshift_rc(bl, static_cast<uint32_t>(B >> 32), p.s));
        if (((bl + 6u) & p.fmask) < 8u)
            return cdf_floor_near(C, k, (bl & p.fmask) < 2u, p.Q, p.G, p.n);
        return k;
    }
    const uint64_t Cs = C << p.z;
    const uint64_t H = Cs + __umul64hi(Cs, p.rcp);
    const uint64_t al = H * static_cast<uint64_t>(p.n);
    const uint64_t ah = __umul64hi(H, static_cast<uint64_t>(p.n));
    const uint64_t f = al - p.gam;
    int64_t k = static_cast<int64_t>(ah - (al < p.gam ? 1ull : 0ull));
    if (f == 0 || f >= p.wlim)
        k = cdf_floor_near(C, k, f == 0, p.Q, p.G, p.n);
    return k;
}

// F(C): the systematic uniforms at or below C / Q, clamped to n
template <bool Usual>
__device__ __forceinline__ uint32_t sys_F(uint64_t C, const CdfRcp &p)
{
    if (C >= p.Q)
        return p.n;
    const int64_t F = cdf_floor<Usual>(C, p) + 1;
    return F < static_cast<int64_t>(p.n) ? static_cast<uint32_t>(F) : p.n;
}

// The resampling engine's position (the words the stratified uniforms use).
struct EnginePos {
    uint32_t key[2], ctr[4], index;
};

__device__ __forceinline__ EnginePos engine_pos(const PfScalars &sc)
{
    return {{sc.rkey[0], sc.rkey[1]},
        {sc.rctr[0], sc.rctr[1], sc.rctr[2], sc.rctr[3]}, sc.rindex};
}

// Philox block b of the engine's stream (word rindex + j is in block
// (rindex + j) / 4)
__device__ __forceinline__ uint4 engine_block(const EnginePos &e, uint32_t b)
{
    uint32_t c[4] = {e.ctr[0], e.ctr[1], e.ctr[2], e.ctr[3]};
    ctr32_add(c, b);
    const u32x4 v = philox4x32_10(c[0], c[1], c[2], c[3], e.key[0], e.key[1]);
    return make_uint4(v.x, v.y, v.z, v.w);
}

// the rare block past a warp's row (not inlined: off the common path's
// register budget)
static __device__ __noinline__ uint4 engine_block_far(
    const EnginePos &e, uint32_t b)
{
    return engine_block(e, b);
}

// Stratified: uniform j lies in [j / n, (j + 1) / n), so the uniforms at or
// below C / Q are every j < j* = floor(C n / Q), and j* itself when its own
// word passes, G_{j*} = ceil(a_{j*} Q / 2^32) <= r = C n - j* Q.  r < Q, so
// 64-bit wrapping arithmetic gives it exactly.  j and r for one CDF value
// (j = n when C >= Q).
template <bool Usual>
__device__ __forceinline__ uint32_t strat_j(
    uint64_t C, const CdfRcp &p, uint64_t &r)
{
    if (C >= p.Q) {
        r = 0;
        return p.n;
    }
    const uint32_t j = static_cast<uint32_t>(cdf_floor<Usual>(C, p));
    r = C * static_cast<uint64_t>(p.n) - static_cast<uint64_t>(j) * p.Q;
    return j;
}

// F from (j, r), word j taken from the warp's row of Philox blocks
// [b0, b0 + nb) or generated when past it
__device__ __forceinline__ uint32_t strat_F(uint32_t j, uint64_t r,
    const CdfRcp &p, const EnginePos &e, const uint4 *row, uint32_t b0,
    uint32_t nb)
{
    if (j >= p.n)
        return p.n;
    const uint32_t pos = e.index + j;
    const uint32_t b = pos >> 2;
    const uint32_t d = b - b0;
    const uint4 v = d < nb ? row[d] : engine_block_far(e, b);
    const uint32_t k = pos & 3u;
    const uint32_t a = k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
    return j + (ceil_aq(a, p.Q) <= r ? 1u : 0u);
}

// The per-event constants above, from the total Q (one thread).  A total of
// 0 or of 2^63 and more is not a valid integer CDF: DEV_ERR_NONFINITE, with
// constants that keep every later pass in range.
__device__ __forceinline__ void cdf_constants(
    PfScalars &sc, uint64_t Q, uint32_t n, bool sys, uint32_t &err)
{
    sc.Q = Q;
    sc.qs = 0;
    sc.qm = 0;
    sc.qgs = 0;
    sc.qz = 0;
    sc.qrcp = 0;
    sc.qG = 0;
    sc.qgam = 0;
    if (Q == 0 || (Q >> 63) != 0) {
        err |= DEV_ERR_NONFINITE;
        return;
    }
    const uint64_t G = sys ? ceil_aq(engine_word(sc, 0), Q) : 0ull;
    sc.qG = G;
    // the usual case's s: the largest s <= 32 with 2^s n < Q, if s >= 20;
    // the general reciprocal otherwise
    uint32_t s = 32;
    while (s > 0 && (static_cast<uint64_t>(n) << s) >= Q)
        --s;
    if (s >= 20) {
        sc.qs = s;
        sc.qm = div_u128_u64(static_cast<uint64_t>(n) << s, 0, Q, err);
        sc.qgs = div_u128_u64(G >> (64 - s), G << s, Q, err);
        return;
    }
    const uint32_t z = static_cast<uint32_t>(__clzll(static_cast<long long>(Q)));
    const uint64_t Qs = Q << z;
    sc.qz = z;
    sc.qrcp = div_u128_u64(~Qs, ~0ull, Qs, err);
    sc.qgam = G >= Q ? ~0ull : div_u128_u64(G, 0, Q, err);
}

// floor(w * 2^shift) for w = exp(lw - M) in [0, 1] and shift <= 63, in two
// 32-bit halves by float operations that are all exact: x = w 2^shift is
// w with its exponent moved; h = trunc(x 2^-32) is the high half; and
// x - h 2^32 (one fma) is the low half exactly, because it is x mod 2^32,
// which keeps at most x's 24 significant bits (or is x itself, below 2^32).
// Both halves then convert by truncation.  -inf and NaN give 0.
__device__ __forceinline__ uint64_t fixed_q(float lw, float M, uint32_t shift)
{
    const float w = fminf(__expf(lw - M), 1.0f);
    const float x = w * __uint_as_float((127u + shift) << 23);
    const float h = truncf(x * 0x1p-32f);
    const uint32_t hi = __float2uint_rz(h);
    const uint32_t lo = __float2uint_rz(fmaf(-h, 0x1p32f, x));
    const uint64_t q = (static_cast<uint64_t>(hi) << 32) | lo;
    return lw > -INFINITY ? q : 0ull;
}

// Stratified counting in the batched filters' block-wide tiles needs, for
// each CDF value, the engine word of its uniform j* (strat_j).  A tile's CDF
// values are nondecreasing, so the words it needs lie in one range of the
// engine stream; the block generates that range's Philox blocks once into
// shared memory (one or two per thread) instead of each thread generating
// the blocks its own words fall in.  Block b of the stream is at
// wb[b - b0] for b0 <= b < b0 + nb; a block beyond the buffer (a tile whose
// words span more than it) is generated where it is needed.
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
//   * when more than a chunk (kRunChunk ranks) is left and the run holding p
//     goes on for at least a chunk, the warp stores its parent up to the
//     run's end directly (32 consecutive ranks per store), so a parent with
//     a huge copy count costs its ranks' stores and nothing more;
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
        // a run can cover a whole chunk only when more than a chunk is left
        // (the usual group, whose ranks fit one chunk, skips the search)
        if (S - p0 > kRunChunk) {
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
