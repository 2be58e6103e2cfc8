// The proposal network: a 6 -> 64 -> 64 -> 8 MLP with GELU (tanh form)
// hidden layers, BF16 weights and activations into the tensor cores, FP32
// accumulation.  One warp evaluates 16 rows at a time with mma.m16n8k16; a
// layer's FP32 accumulator fragments are turned into the next layer's BF16
// operand fragments in registers (the accumulator layout of two adjacent
// 8-column tiles is the operand layout of one 16-column tile), so the
// activations never leave the warp.
//
// Parameters (FP32 master copy, row-major, out x in):
//   W1 [64][6], b1 [64], W2 [64][64], b2 [64], W3 [8][64], b3 [8].
// The packed copy holds the BF16 operand fragments in the order the warps
// read them (one 8-byte load per lane per fragment) and the FP32 biases.
//
// No reference counterpart (the reference has no learned proposal).
#pragma once

#include "common.cuh"

#include <cuda_bf16.h>

#include <cstring>

namespace vsmc_cuda
{

constexpr int kIn = 6;      // network inputs
constexpr int kHid = 64;    // hidden width
constexpr int kOut = 8;     // 4 mean offsets + 4 log-variance offsets
constexpr int kInPad = 16;  // inputs padded to one k-tile

// master parameter offsets (floats)
constexpr int kW1 = 0;
constexpr int kB1 = kW1 + kHid * kIn;
constexpr int kW2 = kB1 + kHid;
constexpr int kB2 = kW2 + kHid * kHid;
constexpr int kW3 = kB2 + kHid;
constexpr int kB3 = kW3 + kOut * kHid;
constexpr int kNumParams = kB3 + kOut; // 5128

// packed operand fragments: [tiles][32 lanes][2 x b32]
constexpr int kFragWords = 64;                       // b32 words per tile
constexpr int kF1 = 0;                               // W1^T: 1 k x 8 n
constexpr int kF2 = kF1 + 8 * kFragWords;            // W2^T: 4 k x 8 n
constexpr int kF3 = kF2 + 32 * kFragWords;           // W3^T: 4 k x 1 n
constexpr int kF3b = kF3 + 4 * kFragWords;           // W3 (backward): 1 k x 8 n
constexpr int kF2b = kF3b + 8 * kFragWords;          // W2 (backward): 4 k x 8 n
constexpr int kFragTotal = kF2b + 32 * kFragWords;   // b32 words
constexpr int kPackedBias = kFragTotal;              // b1, b2, b3 (FP32 bits)
constexpr int kPackedWords = kPackedBias + kHid + kHid + kOut;

__host__ __device__ inline float gelu_k0() { return -1.5957691216057308f; }
__host__ __device__ inline float gelu_k1() { return -0.0713548162726009f; }

// GELU, tanh form: x * sigmoid(2 sqrt(2/pi) (x + 0.044715 x^3))
__device__ __forceinline__ float gelu_f(float x)
{
    const float x2 = x * x;
    const float e = __expf(x * fmaf(gelu_k1(), x2, gelu_k0()));
    return __fdividef(x, 1.0f + e);
}

// derivative of gelu_f
__device__ __forceinline__ float gelu_grad_f(float x)
{
    const float x2 = x * x;
    const float e = __expf(x * fmaf(gelu_k1(), x2, gelu_k0()));
    const float s = __fdividef(1.0f, 1.0f + e); // sigmoid(2u)
    // d/dx [x s(2u)] = s + x s (1 - s) 2u'(x), 2u'(x) = -(k0 + 3 k1 x^2)
    return s - x * s * (1.0f - s) * fmaf(3.0f * gelu_k1(), x2, gelu_k0());
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// GELU (tanh form) of two pre-activations in packed BF16 arithmetic, the
// way the filters evaluate the network: x rounded to BF16, then
// 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))) with BF16 multiplies and
// the hardware tanh approximation (tanh.approx.bf16x2, sm_90 and later).
// One SFU operation per pair instead of two per value; the result is the
// BF16 operand the next layer takes.  Training keeps gelu_f in FP32.
__device__ __forceinline__ uint32_t gelu2_bf16(float lo, float hi)
{
    const __nv_bfloat162 x = __floats2bfloat162_rn(lo, hi);
    const __nv_bfloat162 c0 = __float2bfloat162_rn(0.7978845608028654f);
    const __nv_bfloat162 c1 = __float2bfloat162_rn(0.0356774081363001f);
    const __nv_bfloat162 half = __float2bfloat162_rn(0.5f);
    const __nv_bfloat162 u = __hmul2(x, __hfma2(__hmul2(x, x), c1, c0));
    uint32_t ub, tb;
    memcpy(&ub, &u, 4);
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(tb) : "r"(ub));
    __nv_bfloat162 t;
    memcpy(&t, &tb, 4);
    const __nv_bfloat162 h = __hmul2(x, half);
    const __nv_bfloat162 r = __hfma2(h, t, h);
    uint32_t out;
    memcpy(&out, &r, 4);
    return out;
}

// the BF16 operand pair GELU(lo), GELU(hi): packed BF16 (Fast) or FP32
template <bool Fast>
__device__ __forceinline__ uint32_t gelu_pair(float lo, float hi)
{
    if constexpr (Fast)
        return gelu2_bf16(lo, hi);
    else
        return pack_bf16(gelu_f(lo), gelu_f(hi));
}

__device__ __forceinline__ float bf16_round(float x)
{
    return __bfloat162float(__float2bfloat16_rn(x));
}

// D = A (16x16 bf16, row) * B (16x8 bf16, col) + C, FP32 accumulate
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4],
    uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// the packed fragment of tile `tile` at `base` for this lane
__device__ __forceinline__ uint2 frag(
    const uint32_t *packed, int base, int tile, int lane)
{
    return *reinterpret_cast<const uint2 *>(
        packed + base + tile * kFragWords + 2 * lane);
}

// Forward pass of one warp over 16 rows.  a0 holds the input operand
// fragment (16 x 16, inputs in columns 0..5).  Outputs: out (accumulator
// fragment of the 16 x 8 result, biases added); if pre1 / pre2 are given,
// the hidden pre-activations (accumulator fragments of 8 n-tiles) and the
// BF16 operand fragments of the hidden activations are kept for the
// backward pass.  packed: the packed parameters (shared memory).
template <bool Keep, bool Fast = false>
__device__ __forceinline__ void mlp_forward_warp(const uint32_t *packed,
    const uint32_t (&a0)[4], float (&out)[4], float (*pre1)[4] = nullptr,
    float (*pre2)[4] = nullptr, uint32_t (*act1)[4] = nullptr,
    uint32_t (*act2)[4] = nullptr)
{
    const int lane = threadIdx.x & 31;
    const int tig = lane & 3;
    const float *bias = reinterpret_cast<const float *>(packed + kPackedBias);
    // ---- layer 1: 8 n-tiles, one k-tile
    float h[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float bl = bias[8 * nt + 2 * tig];
        const float bh = bias[8 * nt + 2 * tig + 1];
        h[nt][0] = bl;
        h[nt][1] = bh;
        h[nt][2] = bl;
        h[nt][3] = bh;
        const uint2 b = frag(packed, kF1, nt, lane);
        mma_bf16(h[nt], a0, b.x, b.y);
    }
    uint32_t a[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        if (Keep) {
#pragma unroll
            for (int r = 0; r < 4; ++r)
                pre1[nt][r] = h[nt][r];
        }
        const int kt = nt >> 1, hi = nt & 1;
        a[kt][0 + 2 * hi] = gelu_pair<Fast>(h[nt][0], h[nt][1]);
        a[kt][1 + 2 * hi] = gelu_pair<Fast>(h[nt][2], h[nt][3]);
    }
    if (Keep) {
#pragma unroll
        for (int kt = 0; kt < 4; ++kt)
#pragma unroll
            for (int r = 0; r < 4; ++r)
                act1[kt][r] = a[kt][r];
    }
    // ---- layer 2: 4 k-tiles x 8 n-tiles
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float bl = bias[kHid + 8 * nt + 2 * tig];
        const float bh = bias[kHid + 8 * nt + 2 * tig + 1];
        h[nt][0] = bl;
        h[nt][1] = bh;
        h[nt][2] = bl;
        h[nt][3] = bh;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const uint2 b = frag(packed, kF2, kt * 8 + nt, lane);
            mma_bf16(h[nt], a[kt], b.x, b.y);
        }
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        if (Keep) {
#pragma unroll
            for (int r = 0; r < 4; ++r)
                pre2[nt][r] = h[nt][r];
        }
        const int kt = nt >> 1, hi = nt & 1;
        a[kt][0 + 2 * hi] = gelu_pair<Fast>(h[nt][0], h[nt][1]);
        a[kt][1 + 2 * hi] = gelu_pair<Fast>(h[nt][2], h[nt][3]);
    }
    if (Keep) {
#pragma unroll
        for (int kt = 0; kt < 4; ++kt)
#pragma unroll
            for (int r = 0; r < 4; ++r)
                act2[kt][r] = a[kt][r];
    }
    // ---- layer 3: 4 k-tiles, one n-tile
    {
        const float bl = bias[2 * kHid + 2 * tig];
        const float bh = bias[2 * kHid + 2 * tig + 1];
        out[0] = bl;
        out[1] = bh;
        out[2] = bl;
        out[3] = bh;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const uint2 b = frag(packed, kF3, kt, lane);
            mma_bf16(out, a[kt], b.x, b.y);
        }
    }
}

// Forward pass of one warp over 32 rows as two 16-row tiles (a, b) that
// share every weight fragment load.  Accumulator outputs oa, ob.
template <bool Fast = false>
__device__ __forceinline__ void mlp_forward_warp2(const uint32_t *packed,
    const uint32_t (&a0)[4], const uint32_t (&b0)[4], float (&oa)[4],
    float (&ob)[4])
{
    const int lane = threadIdx.x & 31;
    const int tig = lane & 3;
    const float *bias = reinterpret_cast<const float *>(packed + kPackedBias);
    float ha[8][4], hb[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float bl = bias[8 * nt + 2 * tig];
        const float bh = bias[8 * nt + 2 * tig + 1];
        ha[nt][0] = hb[nt][0] = bl;
        ha[nt][1] = hb[nt][1] = bh;
        ha[nt][2] = hb[nt][2] = bl;
        ha[nt][3] = hb[nt][3] = bh;
        const uint2 w = frag(packed, kF1, nt, lane);
        mma_bf16(ha[nt], a0, w.x, w.y);
        mma_bf16(hb[nt], b0, w.x, w.y);
    }
    uint32_t xa[4][4], xb[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int kt = nt >> 1, hi = nt & 1;
        xa[kt][0 + 2 * hi] = gelu_pair<Fast>(ha[nt][0], ha[nt][1]);
        xa[kt][1 + 2 * hi] = gelu_pair<Fast>(ha[nt][2], ha[nt][3]);
        xb[kt][0 + 2 * hi] = gelu_pair<Fast>(hb[nt][0], hb[nt][1]);
        xb[kt][1 + 2 * hi] = gelu_pair<Fast>(hb[nt][2], hb[nt][3]);
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float bl = bias[kHid + 8 * nt + 2 * tig];
        const float bh = bias[kHid + 8 * nt + 2 * tig + 1];
        ha[nt][0] = hb[nt][0] = bl;
        ha[nt][1] = hb[nt][1] = bh;
        ha[nt][2] = hb[nt][2] = bl;
        ha[nt][3] = hb[nt][3] = bh;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const uint2 w = frag(packed, kF2, kt * 8 + nt, lane);
            mma_bf16(ha[nt], xa[kt], w.x, w.y);
            mma_bf16(hb[nt], xb[kt], w.x, w.y);
        }
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int kt = nt >> 1, hi = nt & 1;
        xa[kt][0 + 2 * hi] = gelu_pair<Fast>(ha[nt][0], ha[nt][1]);
        xa[kt][1 + 2 * hi] = gelu_pair<Fast>(ha[nt][2], ha[nt][3]);
        xb[kt][0 + 2 * hi] = gelu_pair<Fast>(hb[nt][0], hb[nt][1]);
        xb[kt][1 + 2 * hi] = gelu_pair<Fast>(hb[nt][2], hb[nt][3]);
    }
    {
        const float bl = bias[2 * kHid + 2 * tig];
        const float bh = bias[2 * kHid + 2 * tig + 1];
        oa[0] = ob[0] = bl;
        oa[1] = ob[1] = bh;
        oa[2] = ob[2] = bl;
        oa[3] = ob[3] = bh;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const uint2 w = frag(packed, kF3, kt, lane);
            mma_bf16(oa, xa[kt], w.x, w.y);
            mma_bf16(ob, xb[kt], w.x, w.y);
        }
    }
}

// copy the packed parameters into shared memory (all threads of the block)
__device__ __forceinline__ void load_packed(
    uint32_t *dst, const uint32_t *src)
{
    for (int i = threadIdx.x; i < kPackedWords / 4; i += blockDim.x)
        reinterpret_cast<uint4 *>(dst)[i] =
            __ldg(reinterpret_cast<const uint4 *>(src) + i);
    for (int i = kPackedWords / 4 * 4 + threadIdx.x; i < kPackedWords;
         i += blockDim.x)
        dst[i] = src[i];
    __syncthreads();
}

// ------------------------------------------------- warp-level plumbing

// Input operand fragment from the 6 features held by the owners of the
// quad's two rows (lane 4g holds row g, lane 4g + 1 holds row g + 8).
__device__ __forceinline__ void features_to_a(
    const float (&f)[6], uint32_t (&a)[4])
{
    const int lane = threadIdx.x & 31;
    const int t = lane & 3;
    const int src0 = lane & ~3, src1 = src0 + 1;
    float r0lo = 0, r0hi = 0, r1lo = 0, r1hi = 0;
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        const float x0 = __shfl_sync(0xFFFFFFFFu, f[2 * p], src0);
        const float y0 = __shfl_sync(0xFFFFFFFFu, f[2 * p + 1], src0);
        const float x1 = __shfl_sync(0xFFFFFFFFu, f[2 * p], src1);
        const float y1 = __shfl_sync(0xFFFFFFFFu, f[2 * p + 1], src1);
        if (t == p) {
            r0lo = x0;
            r0hi = y0;
            r1lo = x1;
            r1hi = y1;
        }
    }
    a[0] = pack_bf16(r0lo, r0hi);
    a[1] = pack_bf16(r1lo, r1hi);
    a[2] = 0;
    a[3] = 0;
}

// The 8 outputs of the owner's row from the quad's accumulator fragment.
__device__ __forceinline__ void out_to_owner(
    const float (&o)[4], float (&v)[8])
{
    const int lane = threadIdx.x & 31;
    const int base = lane & ~3;
    const bool second = (lane & 3) == 1; // owner of row g + 8
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float c0 = __shfl_sync(0xFFFFFFFFu, o[0], base + j);
        const float c1 = __shfl_sync(0xFFFFFFFFu, o[1], base + j);
        const float c2 = __shfl_sync(0xFFFFFFFFu, o[2], base + j);
        const float c3 = __shfl_sync(0xFFFFFFFFu, o[3], base + j);
        v[2 * j] = second ? c2 : c0;
        v[2 * j + 1] = second ? c3 : c1;
    }
}

// Operand fragment (16 x 16, columns 8..15 zero) of an 8-wide per-row
// vector held by the owners.
__device__ __forceinline__ void owner8_to_a(
    const float (&v)[8], uint32_t (&a)[4])
{
    const int lane = threadIdx.x & 31;
    const int t = lane & 3;
    const int src0 = lane & ~3, src1 = src0 + 1;
    float r0lo = 0, r0hi = 0, r1lo = 0, r1hi = 0;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        const float x0 = __shfl_sync(0xFFFFFFFFu, v[2 * p], src0);
        const float y0 = __shfl_sync(0xFFFFFFFFu, v[2 * p + 1], src0);
        const float x1 = __shfl_sync(0xFFFFFFFFu, v[2 * p], src1);
        const float y1 = __shfl_sync(0xFFFFFFFFu, v[2 * p + 1], src1);
        if (t == p) {
            r0lo = x0;
            r0hi = y0;
            r1lo = x1;
            r1hi = y1;
        }
    }
    a[0] = pack_bf16(r0lo, r0hi);
    a[1] = pack_bf16(r1lo, r1hi);
    a[2] = 0;
    a[3] = 0;
}


// 32-row plumbing: lane 4g + q owns row g + 8q of the warp's 32 (tile a
// holds rows 0..15, tile b rows 16..31).
__device__ __forceinline__ void features_to_a2(
    const float (&f)[6], uint32_t (&a)[4], uint32_t (&b)[4])
{
    const int lane = threadIdx.x & 31;
    const int t = lane & 3;
    const int base = lane & ~3;
    float v[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
#pragma unroll
    for (int p = 0; p < 3; ++p) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float x = __shfl_sync(0xFFFFFFFFu, f[2 * p], base + q);
            const float y = __shfl_sync(0xFFFFFFFFu, f[2 * p + 1], base + q);
            if (t == p) {
                v[q][0] = x;
                v[q][1] = y;
            }
        }
    }
    a[0] = pack_bf16(v[0][0], v[0][1]);
    a[1] = pack_bf16(v[1][0], v[1][1]);
    a[2] = a[3] = 0;
    b[0] = pack_bf16(v[2][0], v[2][1]);
    b[1] = pack_bf16(v[3][0], v[3][1]);
    b[2] = b[3] = 0;
}

__device__ __forceinline__ void out_to_owner2(
    const float (&oa)[4], const float (&ob)[4], float (&v)[8])
{
    const int lane = threadIdx.x & 31;
    const int base = lane & ~3;
    const int q = lane & 3;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float a0 = __shfl_sync(0xFFFFFFFFu, oa[0], base + j);
        const float a1 = __shfl_sync(0xFFFFFFFFu, oa[1], base + j);
        const float a2 = __shfl_sync(0xFFFFFFFFu, oa[2], base + j);
        const float a3 = __shfl_sync(0xFFFFFFFFu, oa[3], base + j);
        const float b0 = __shfl_sync(0xFFFFFFFFu, ob[0], base + j);
        const float b1 = __shfl_sync(0xFFFFFFFFu, ob[1], base + j);
        const float b2 = __shfl_sync(0xFFFFFFFFu, ob[2], base + j);
        const float b3 = __shfl_sync(0xFFFFFFFFu, ob[3], base + j);
        v[2 * j] = q == 0 ? a0 : (q == 1 ? a2 : (q == 2 ? b0 : b2));
        v[2 * j + 1] = q == 0 ? a1 : (q == 1 ? a3 : (q == 2 ? b1 : b3));
    }
}

} // namespace vsmc_cuda
