// Learned proposal for the bearings-only model: the simulator, the
// kernel-level move / weight entry, the network's packing, forward pass and
// loss gradient, Adam, and a trainer that learns from simulated
// trajectories -- all on the device.
//
// Training data: (x_{t-1}, z_t, nu_t) triples with nu_t ~ N(0, I) the
// whitened transition noise of x_t = F x_{t-1} + L nu_t and z_t the bearing
// of x_t; the loss is the negative log density of nu_t under the proposal,
//   0.5 sum_d [(nu_d - m_d)^2 exp(-l_d) + l_d],
// whose minimiser is the locally optimal proposal p(x_t | x_{t-1}, z_t)
// within the Gaussian family.
//
// No reference counterpart (the reference has no learned proposal).
#include "bearings.cuh"
#include "mlp.cuh"
#include "tc05.cuh"
#include "rng_device.cuh"

#include <cmath>
#include <new>
#include <vector>

using namespace vsmc_cuda;

namespace vsmc_cuda
{

// ------------------------------------------------------------ simulation

// Sequential FP64 simulation on one thread (bearings_simulate_seq).
__global__ void k_bearings_simulate(uint32_t seed, uint32_t T,
    vsmc_cuda_bearings_model m, double *truth, double *obs)
{
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    bearings_simulate_seq(seed, T, m, truth, obs);
}

// ------------------------------------------------------------- packing

__device__ __forceinline__ float pw(const float *p, int off, int row,
    int ncol, int col, int nrow)
{
    return (row < nrow && col < ncol) ? p[off + row * ncol + col] : 0.0f;
}

// one b32 word of the packed parameters per thread
__global__ void k_mlp_pack(const float *p, uint32_t *packed)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= kPackedWords)
        return;
    if (w >= kPackedBias) {
        const int i = w - kPackedBias;
        const float v = i < kHid ? p[kB1 + i]
                                 : (i < 2 * kHid ? p[kB2 + i - kHid]
                                                 : p[kB3 + i - 2 * kHid]);
        packed[w] = __float_as_uint(v);
        return;
    }
    int sec, base;
    if (w < kF2) {
        sec = 0;
        base = kF1;
    } else if (w < kF3) {
        sec = 1;
        base = kF2;
    } else if (w < kF3b) {
        sec = 2;
        base = kF3;
    } else if (w < kF2b) {
        sec = 3;
        base = kF3b;
    } else {
        sec = 4;
        base = kF2b;
    }
    const int r = w - base;
    const int tile = r / kFragWords;
    const int lane = (r % kFragWords) / 2;
    const int which = r % 2; // b0 (k rows 2t, 2t+1) or b1 (2t+8, 2t+9)
    const int g = lane >> 2, t = lane & 3;
    const int k0 = 2 * t + 8 * which; // k row inside the 16-row tile
    float lo = 0, hi = 0;
    switch (sec) {
        case 0: { // B[k][n] = W1[n][k], k < 6
            const int n = 8 * tile + g;
            lo = pw(p, kW1, n, kIn, k0, kHid);
            hi = pw(p, kW1, n, kIn, k0 + 1, kHid);
            break;
        }
        case 1: { // tile = kt * 8 + nt: B[k][n] = W2[n][k]
            const int kt = tile / 8, nt = tile % 8;
            const int n = 8 * nt + g, k = 16 * kt + k0;
            lo = p[kW2 + n * kHid + k];
            hi = p[kW2 + n * kHid + k + 1];
            break;
        }
        case 2: { // tile = kt: B[k][n] = W3[n][k]
            const int k = 16 * tile + k0;
            lo = p[kW3 + g * kHid + k];
            hi = p[kW3 + g * kHid + k + 1];
            break;
        }
        case 3: { // tile = nt: B[k = d][n = j] = W3[d][j], d < 8
            const int j = 8 * tile + g;
            lo = pw(p, kW3, k0, kHid, j, kOut);
            hi = pw(p, kW3, k0 + 1, kHid, j, kOut);
            break;
        }
        default: { // tile = kt * 8 + nt: B[k = j][n = k'] = W2[j][k']
            const int kt = tile / 8, nt = tile % 8;
            const int kk = 8 * nt + g, j = 16 * kt + k0;
            lo = p[kW2 + j * kHid + kk];
            hi = p[kW2 + (j + 1) * kHid + kk];
            break;
        }
    }
    packed[w] = pack_bf16(lo, hi);
}

// ------------------------------------------------------- kernel-level move

// One move + weight increment per particle on caller-owned SoA state.
// t == 0 draws the prior; the bootstrap draws nu ~ N(0, I); the learned
// proposal (packed != null) evaluates the network per 16 particles per warp.
template <bool Learned>
__global__ void __launch_bounds__(128) k_bearings_move(uint32_t n, uint32_t t,
    uint32_t seed, BearingsConst c, float z, const uint32_t *packed,
    float *sx, float *sy, float *svx, float *svy, float *lw_inc)
{
    __shared__ __align__(16) uint32_t sp[Learned ? kPackedWords : 1];
    if (Learned)
        load_packed(sp, packed);
    const float sz = sinf(z), cz = cosf(z);
    if (!Learned || t == 0) {
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
             i += gridDim.x * blockDim.x) {
            float e[4];
            bearings_normals(t, seed, i, e);
            float x = sx[i], y = sy[i], vx = svx[i], vy = svy[i];
            if (t == 0)
                bearings_prior(c, e, x, y, vx, vy);
            else
                bearings_step(c, e, x, y, vx, vy);
            sx[i] = x;
            sy[i] = y;
            svx[i] = vx;
            svy[i] = vy;
            lw_inc[i] = bearings_loglik(c, z, x, y);
        }
        return;
    }
    const int lane = threadIdx.x & 31;
    const int wglobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int g = lane >> 2, q = lane & 3;
    for (uint32_t p0 = 32u * wglobal; p0 < n; p0 += 32u * nwarps) {
        const uint32_t i = p0 + g + 8u * q;
        const bool mine = i < n;
        float x = 0, y = 0, vx = 0, vy = 0;
        if (mine) {
            x = sx[i];
            y = sy[i];
            vx = svx[i];
            vy = svy[i];
        }
        float f[6];
        bearings_features(c, x, y, vx, vy, sz, cz, f);
        uint32_t a0[4], b0[4];
        features_to_a2(f, a0, b0);
        float oa[4], ob[4];
        mlp_forward_warp2<true>(sp, a0, b0, oa, ob);
        float v[8];
        out_to_owner2(oa, ob, v);
        if (mine) {
            float e[4], fr[4], nu[4];
            bearings_normals(t, seed, i, e);
            float lq = 0;
#pragma unroll
            for (int d = 0; d < 4; ++d) {
                const float l = fminf(fmaxf(v[4 + d], c.lmin), c.lmax);
                fr[d] = v[d] + __expf(0.5f * l) * e[d];
                lq += 0.5f * (e[d] * e[d] - fr[d] * fr[d]) + 0.5f * l;
            }
            frame_to_axes(sz, cz, fr, nu); // the draw, bearing frame
            bearings_step(c, nu, x, y, vx, vy);
            sx[i] = x;
            sy[i] = y;
            svx[i] = vx;
            svy[i] = vy;
            lw_inc[i] = bearings_loglik(c, z, x, y) + lq;
        }
    }
}

// ------------------------------------------------------- forward (parity)

__global__ void __launch_bounds__(128) k_mlp_forward(
    const uint32_t *packed, uint32_t B, const float *feat, float *out)
{
    __shared__ __align__(16) uint32_t sp[kPackedWords];
    load_packed(sp, packed);
    const int lane = threadIdx.x & 31;
    const int wglobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int g = lane >> 2, q = lane & 3;
    for (uint32_t p0 = 32u * wglobal; p0 < B; p0 += 32u * nwarps) {
        const uint32_t i = p0 + g + 8u * q;
        const bool mine = i < B;
        float f[6];
#pragma unroll
        for (int k = 0; k < 6; ++k)
            f[k] = mine ? feat[6 * i + k] : 0.0f;
        uint32_t a0[4], b0[4];
        features_to_a2(f, a0, b0);
        float oa[4], ob[4];
        mlp_forward_warp2(sp, a0, b0, oa, ob);
        float v[8];
        out_to_owner2(oa, ob, v);
        if (mine)
#pragma unroll
            for (int k = 0; k < 8; ++k)
                out[8 * i + k] = v[k];
    }
}

// ------------------------------------------------------------ gradient
//
// Loss and gradient partials of one block over its samples.  The forward
// pass and the backward data path (deltas through W3 and W2) run per warp
// on 16 rows with mma.sync, as in the filters.  The weight gradients are
// contractions over the samples, dW = delta^T a, and run on the Blackwell
// tensor core: every round of 64 samples the block writes its activations
// and deltas into shared memory as K-major BF16 operands (K = the samples)
// and one thread issues tcgen05.mma into FP32 accumulators in tensor memory
// that live for the whole kernel.  Two products cover every weight:
//
//   D1 (128 x 80) = [a1 | a2]^T [dp2 | dout | 0]:
//       D1[k][j] = dW2[j][k] (k, j < 64), D1[64 + k][64 + d] = dW3[d][k]
//   D2 (128 x 16) = [dp1 | dp2]^T [a0 | 1 | 0]:
//       D2[j][c] = dW1[j][c] (c < 6), D2[j][6] = db1[j], D2[64 + j][6] = db2[j]
//
// The activations are BF16 already (the forward's operands); each FP32
// delta is split into BF16 hi + lo parts (v = hi + lo to about 2^-17
// relative) and both are multiplied, so the sums keep the deltas' FP32
// precision.  Stage buffers alternate, and an mbarrier per buffer
// (tcgen05.commit) says when the tensor core has finished reading one, so
// a round's contraction overlaps the next round's forward and backward
// passes.  db3 and the loss are register sums.  part: [grid][kNumParams + 1]
// (the last entry is the block's loss sum); a block whose tensor-core wait
// ran out writes NaN there and in its gradient entries.

constexpr int kGradWarps = 4;
constexpr int kGradRows = 16 * kGradWarps; // samples per round (the K tile)

// operands inside one stage buffer: K-major, no swizzle, rows of 64 samples
// (8 core matrices of 128 B along K, 8-row groups 1024 B apart)
constexpr uint32_t kTcLbo = 128;
constexpr uint32_t kTcSbo = 1024;
constexpr uint32_t kOpA1 = 0;                   // 128 rows: a1, a2
constexpr uint32_t kOpB1h = kOpA1 + 128 * 128;  // 80 rows: dp2, dout, 0 (hi)
constexpr uint32_t kOpB1l = kOpB1h + 80 * 128;  // (lo)
constexpr uint32_t kOpA2h = kOpB1l + 80 * 128;  // 128 rows: dp1, dp2 (hi)
constexpr uint32_t kOpA2l = kOpA2h + 128 * 128; // (lo)
constexpr uint32_t kOpB2 = kOpA2l + 128 * 128;  // 16 rows: a0, 1, 0
constexpr uint32_t kStageBytes = kOpB2 + 16 * 128;
constexpr uint32_t kTmemCols = 128;
constexpr uint32_t kD1Col = 0, kD2Col = 96;
constexpr uint32_t kPackedBytes = (sizeof(uint32_t) * kPackedWords + 1023) / 1024 * 1024;
constexpr size_t kGradSmem = 1024 /* alignment slack */ + kPackedBytes +
    2 * kStageBytes + 64 /* mbarriers, TMEM address */;
constexpr uint64_t kTcWaitNs = 1000000000ull; // 1 s

// byte offset of (operand row, sample s) in a K-major no-swizzle operand
__device__ __forceinline__ uint32_t op_off(uint32_t row, uint32_t s)
{
    return (row >> 3) * kTcSbo + (s >> 3) * kTcLbo + (row & 7) * 16u +
        (s & 7) * 2u;
}

__device__ __forceinline__ void st16(unsigned char *buf, uint32_t off,
    uint32_t v)
{
    *reinterpret_cast<uint16_t *>(buf + off) = static_cast<uint16_t>(v);
}

// the two BF16 halves of a packed operand word at rows r, r + 1
__device__ __forceinline__ void st_pair(unsigned char *buf, uint32_t op,
    uint32_t row, uint32_t s, uint32_t w)
{
    st16(buf, op + op_off(row, s), w & 0xFFFFu);
    st16(buf, op + op_off(row + 1, s), w >> 16);
}

// an FP32 delta as BF16 hi and lo parts into two operands
__device__ __forceinline__ void st_split(unsigned char *buf, uint32_t oph,
    uint32_t opl, uint32_t row, uint32_t s, float v)
{
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
    const uint32_t o = op_off(row, s);
    *reinterpret_cast<__nv_bfloat16 *>(buf + oph + o) = h;
    *reinterpret_cast<__nv_bfloat16 *>(buf + opl + o) = l;
}

// the round's contraction, issued by one thread on stage buffer `sb`
__device__ __forceinline__ void grad_mma_round(
    uint32_t sb, uint32_t tmem, bool accumulate)
{
    constexpr uint32_t id1 = tc05::idesc_bf16(128, 80);
    constexpr uint32_t id2 = tc05::idesc_bf16(128, 16);
#pragma unroll
    for (uint32_t kk = 0; kk < kGradRows / 16; ++kk) {
        const uint32_t ko = kk * 2 * kTcLbo; // 16 samples = 2 core matrices
        const uint32_t acc = (accumulate || kk > 0) ? 1u : 0u;
        const uint64_t a1 = tc05::desc_kmajor(sb + kOpA1 + ko, kTcLbo, kTcSbo);
        tc05::mma_bf16(tmem + kD1Col, a1,
            tc05::desc_kmajor(sb + kOpB1h + ko, kTcLbo, kTcSbo), id1, acc);
        tc05::mma_bf16(tmem + kD1Col, a1,
            tc05::desc_kmajor(sb + kOpB1l + ko, kTcLbo, kTcSbo), id1, 1u);
        const uint64_t b2 = tc05::desc_kmajor(sb + kOpB2 + ko, kTcLbo, kTcSbo);
        tc05::mma_bf16(tmem + kD2Col,
            tc05::desc_kmajor(sb + kOpA2h + ko, kTcLbo, kTcSbo), b2, id2, acc);
        tc05::mma_bf16(tmem + kD2Col,
            tc05::desc_kmajor(sb + kOpA2l + ko, kTcLbo, kTcSbo), b2, id2, 1u);
    }
}

__global__ void __launch_bounds__(128, 1) k_mlp_grad(const uint32_t *packed,
    uint32_t B, const float *feat, const float *nu_in, float inv_b,
    double *part)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned carve-up (the descriptors need 16)
    const uint32_t raw = tc05::smem_addr(smem_raw);
    unsigned char *smem = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
    uint32_t *sp = reinterpret_cast<uint32_t *>(smem);
    unsigned char *stage[2] = {smem + kPackedBytes,
        smem + kPackedBytes + kStageBytes};
    uint64_t *mbar = reinterpret_cast<uint64_t *>(
        smem + kPackedBytes + 2 * kStageBytes);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 2);
    __shared__ double shl[128 / 32 + 1];
    __shared__ float shb3[kGradWarps][kOut];

    const int tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    const int g = lane >> 2, q = lane & 3;

    // constant operand rows: dout padding (B1 rows 72..79), the ones row
    // and padding of B2 (rows 6..15), in both buffers
    for (int b = 0; b < 2; ++b) {
        for (uint32_t w = tid; w < 8 * 64; w += 128) {
            const uint32_t row = 72 + w / 64, s = w % 64;
            st16(stage[b], kOpB1h + op_off(row, s), 0);
            st16(stage[b], kOpB1l + op_off(row, s), 0);
        }
        for (uint32_t w = tid; w < 10 * 64; w += 128) {
            const uint32_t row = 6 + w / 64, s = w % 64;
            st16(stage[b], kOpB2 + op_off(row, s), row == 6 ? 0x3F80u : 0u);
        }
    }
    if (tid == 0) {
        tc05::mbar_init(&mbar[0], 1);
        tc05::mbar_init(&mbar[1], 1);
    }
    if (wid == 0)
        tc05::tmem_alloc(tmem_slot, kTmemCols);
    tc05::fence_before_sync();
    load_packed(sp, packed); // ends with __syncthreads
    tc05::fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    float gb3[kOut];
#pragma unroll
    for (int d = 0; d < kOut; ++d)
        gb3[d] = 0;
    float loss = 0;
    bool timed_out = false;
    const uint32_t rounds = (B + kGradRows - 1) / kGradRows;
    uint32_t it = 0;
    for (uint32_t rd = blockIdx.x; rd < rounds; rd += gridDim.x, ++it) {
        const uint32_t p0 = rd * kGradRows + 16 * wid;
        const uint32_t i = p0 + g + (q == 1 ? 8u : 0u);
        const bool mine = q < 2 && i < B;
        float f[6];
#pragma unroll
        for (int k = 0; k < 6; ++k)
            f[k] = mine ? feat[6 * i + k] : 0.0f;
        uint32_t a0[4];
        features_to_a(f, a0);
        float o[4];
        float pre1[8][4], pre2[8][4];
        uint32_t act1[4][4], act2[4][4];
        mlp_forward_warp<true>(sp, a0, o, pre1, pre2, act1, act2);
        float v[8];
        out_to_owner(o, v);
        // d loss / d output of the owner's row (rows past B contribute 0)
        float dv[8];
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            float target = mine ? nu_in[4 * i + d] : 0.0f;
            const float r = target - v[d];
            const float el = __expf(-v[4 + d]);
            dv[d] = mine ? -r * el * inv_b : 0.0f;
            dv[4 + d] = mine ? 0.5f * (1.0f - r * r * el) * inv_b : 0.0f;
            if (mine)
                loss += 0.5f * (r * r * el + v[4 + d]);
        }
#pragma unroll
        for (int d = 0; d < kOut; ++d)
            gb3[d] += dv[d];
        // dh2 = dout W3 (8 n-tiles), dpre2 = dh2 * gelu'(pre2)
        uint32_t ad[4];
        owner8_to_a(dv, ad);
        float dp2[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            dp2[nt][0] = dp2[nt][1] = dp2[nt][2] = dp2[nt][3] = 0;
            const uint2 b = frag(sp, kF3b, nt, lane);
            mma_bf16(dp2[nt], ad, b.x, b.y);
#pragma unroll
            for (int r = 0; r < 4; ++r)
                dp2[nt][r] *= gelu_grad_f(pre2[nt][r]);
        }
        // dh1 = dpre2 W2, dpre1 = dh1 * gelu'(pre1)
        uint32_t a2[4][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int kt = nt >> 1, hi = nt & 1;
            a2[kt][0 + 2 * hi] = pack_bf16(dp2[nt][0], dp2[nt][1]);
            a2[kt][1 + 2 * hi] = pack_bf16(dp2[nt][2], dp2[nt][3]);
        }
        float dp1[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            dp1[nt][0] = dp1[nt][1] = dp1[nt][2] = dp1[nt][3] = 0;
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) {
                const uint2 b = frag(sp, kF2b, kt * 8 + nt, lane);
                mma_bf16(dp1[nt], a2[kt], b.x, b.y);
            }
#pragma unroll
            for (int r = 0; r < 4; ++r)
                dp1[nt][r] *= gelu_grad_f(pre1[nt][r]);
        }
        // ---- the stage buffer is free once the contraction that last
        // read it (two rounds ago) has finished
        const int sbi = static_cast<int>(it & 1);
        bool ok = true;
        if (it >= 2)
            ok = tc05::mbar_wait(&mbar[sbi], ((it >> 1) - 1) & 1, kTcWaitNs);
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        unsigned char *buf = stage[sbi];
        const uint32_t s0 = 16 * wid + g, s1 = s0 + 8;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const uint32_t c = 16 * kt + 2 * q;
            st_pair(buf, kOpA1, c, s0, act1[kt][0]);
            st_pair(buf, kOpA1, c, s1, act1[kt][1]);
            st_pair(buf, kOpA1, c + 8, s0, act1[kt][2]);
            st_pair(buf, kOpA1, c + 8, s1, act1[kt][3]);
            st_pair(buf, kOpA1, 64 + c, s0, act2[kt][0]);
            st_pair(buf, kOpA1, 64 + c, s1, act2[kt][1]);
            st_pair(buf, kOpA1, 64 + c + 8, s0, act2[kt][2]);
            st_pair(buf, kOpA1, 64 + c + 8, s1, act2[kt][3]);
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const uint32_t c = 8 * nt + 2 * q;
            st_split(buf, kOpB1h, kOpB1l, c, s0, dp2[nt][0]);
            st_split(buf, kOpB1h, kOpB1l, c + 1, s0, dp2[nt][1]);
            st_split(buf, kOpB1h, kOpB1l, c, s1, dp2[nt][2]);
            st_split(buf, kOpB1h, kOpB1l, c + 1, s1, dp2[nt][3]);
            st_split(buf, kOpA2h, kOpA2l, 64 + c, s0, dp2[nt][0]);
            st_split(buf, kOpA2h, kOpA2l, 64 + c + 1, s0, dp2[nt][1]);
            st_split(buf, kOpA2h, kOpA2l, 64 + c, s1, dp2[nt][2]);
            st_split(buf, kOpA2h, kOpA2l, 64 + c + 1, s1, dp2[nt][3]);
            st_split(buf, kOpA2h, kOpA2l, c, s0, dp1[nt][0]);
            st_split(buf, kOpA2h, kOpA2l, c + 1, s0, dp1[nt][1]);
            st_split(buf, kOpA2h, kOpA2l, c, s1, dp1[nt][2]);
            st_split(buf, kOpA2h, kOpA2l, c + 1, s1, dp1[nt][3]);
        }
        if (q < 2) {
            const uint32_t s = q == 0 ? s0 : s1;
#pragma unroll
            for (int d = 0; d < kOut; ++d)
                st_split(buf, kOpB1h, kOpB1l, 64 + d, s, dv[d]);
        }
        if (q < 3) { // inputs 2q, 2q + 1 of rows s0 (a0[0]) and s1 (a0[1])
            st_pair(buf, kOpB2, 2 * q, s0, a0[0]);
            st_pair(buf, kOpB2, 2 * q, s1, a0[1]);
        }
        tc05::fence_async_shared();
        __syncthreads();
        if (tid == 0) {
            tc05::fence_after_sync();
            grad_mma_round(tc05::smem_addr(buf), tmem, it > 0);
            tc05::commit(&mbar[sbi]);
        }
    }
    // ---- every contraction finished: the last commit covers the earlier
    if (it > 0) {
        const uint32_t last = it - 1;
        const bool ok = tc05::mbar_wait(
            &mbar[last & 1], (last >> 1) & 1, kTcWaitNs);
        if (__syncthreads_or(!ok))
            timed_out = true;
    }
    tc05::fence_after_sync();
    double *out = part + static_cast<size_t>(blockIdx.x) * (kNumParams + 1);
    if (timed_out) {
        // record it; give the tensor core one more bounded wait before the
        // accumulators are released
        if (it > 0)
            tc05::mbar_wait(&mbar[(it - 1) & 1], ((it - 1) >> 1) & 1,
                kTcWaitNs);
        for (int k = tid; k <= kNumParams; k += 128)
            out[k] = __longlong_as_double(0x7FF8000000000000ll);
    } else if (it == 0) {
        for (int k = tid; k <= kNumParams; k += 128)
            out[k] = 0.0;
    } else {
        // ---- accumulators -> block partials (warp w reads TMEM lanes
        // 32w .. 32w + 31: row m = 32w + lane)
        const uint32_t m = 32 * wid + lane;
        const uint32_t tw = tmem + ((32u * wid) << 16);
        float vv[16];
        if (wid < 2) {
#pragma unroll
            for (int c0 = 0; c0 < 64; c0 += 16) {
                tc05::ld16(tw + kD1Col + c0, vv);
#pragma unroll
                for (int c = 0; c < 16; ++c) // dW2[j = c0 + c][k = m]
                    out[kW2 + (c0 + c) * kHid + m] = vv[c];
            }
            tc05::ld16(tw + kD2Col, vv);
#pragma unroll
            for (int c = 0; c < kIn; ++c)
                out[kW1 + m * kIn + c] = vv[c];
            out[kB1 + m] = vv[kIn];
        } else {
            const uint32_t k = m - 64;
            tc05::ld16(tw + kD1Col + 64, vv);
#pragma unroll
            for (int d = 0; d < kOut; ++d) // dW3[d][k]
                out[kW3 + d * kHid + k] = vv[d];
            tc05::ld16(tw + kD2Col, vv);
            out[kB2 + k] = vv[kIn];
        }
        // db3 and the loss: register sums over the block
#pragma unroll
        for (int d = 0; d < kOut; ++d) {
            float s = gb3[d];
#pragma unroll
            for (int o2 = 16; o2 > 0; o2 >>= 1)
                s += __shfl_xor_sync(0xFFFFFFFFu, s, o2);
            if (lane == 0)
                shb3[wid][d] = s;
        }
        __syncthreads();
        if (tid < kOut) {
            float s = 0;
            for (int w = 0; w < kGradWarps; ++w)
                s += shb3[w][tid];
            out[kB3 + tid] = s;
        }
        const double lb = block_reduce(static_cast<double>(loss), OpAdd(),
            0.0, shl);
        if (tid == 0)
            out[kNumParams] = lb;
    }
    // ---- release the tensor memory (after every warp's reads)
    tc05::fence_before_sync();
    __syncthreads();
    if (wid == 0) {
        tc05::fence_after_sync();
        tc05::tmem_free(tmem, kTmemCols);
    }
}

// ------------------------------------------- forward on tcgen05 (128 rows)
//
// The same network on the Blackwell tensor core, 128 rows per tile: one
// thread per row.  Each layer is one tcgen05.mma chain (M = 128; N = 64,
// 64, 16) from K-major BF16 operands in shared memory into FP32 tensor
// memory; the row's thread reads its accumulators back (tcgen05.ld), adds
// the bias, applies GELU and writes the row of the next layer's operand.
// The weights come from the packed mma.sync fragments, decoded once per
// block into K-major operands.  A block whose tensor-core wait runs out
// writes NaN outputs for its rows and stops.

constexpr uint32_t kFwK16Sbo = 256;   // K = 16 operands: 2 core matrices per group
constexpr uint32_t kFwK64Sbo = 1024;  // K = 64 operands: 8 per group
constexpr uint32_t kFwW1 = 0;                         // 64 x 16
constexpr uint32_t kFwW2 = kFwW1 + 64 * 32;           // 64 x 64
constexpr uint32_t kFwW3 = kFwW2 + 64 * 128;          // 16 x 64 (rows 8..15 zero)
constexpr uint32_t kFwX = kFwW3 + 16 * 128;           // 128 x 16
constexpr uint32_t kFwH1 = kFwX + 128 * 32;           // 128 x 64
constexpr uint32_t kFwH2 = kFwH1 + 128 * 128;         // 128 x 64
constexpr uint32_t kFwBias = kFwH2 + 128 * 128;       // b1, b2, b3 (FP32)
constexpr uint32_t kFwBar = kFwBias + 4 * (kHid + kHid + kOut);
constexpr size_t kFwSmem = 1024 + kFwBar + 16;
constexpr uint32_t kFwTmemCols = 128; // D1 / D3 at column 0, D2 at 64

__device__ __forceinline__ uint32_t kmaj_off(uint32_t row, uint32_t k,
    uint32_t sbo)
{
    return (row >> 3) * sbo + (k >> 3) * 128u + (row & 7) * 16u + (k & 7) * 2u;
}

// packed fragment word -> its two BF16 elements (k, n), (k + 1, n) of the
// B operand it belongs to: tile `tile` of a region with `ntn` n-tiles
__device__ __forceinline__ void frag_word_kn(uint32_t w, uint32_t ntn,
    uint32_t &k, uint32_t &n)
{
    const uint32_t tile = w / 64, within = w % 64;
    const uint32_t ln = within / 2, hi = within % 2;
    const uint32_t kt = tile / ntn, nt = tile % ntn;
    k = 16 * kt + 2 * (ln & 3) + 8 * hi;
    n = 8 * nt + (ln >> 2);
}

__global__ void __launch_bounds__(128, 4) k_mlp_forward_tc(
    const uint32_t *packed, uint32_t B, const float *feat, float *out)
{
    extern __shared__ __align__(1024) unsigned char fsm_raw[];
    const uint32_t raw = tc05::smem_addr(fsm_raw);
    unsigned char *sm = fsm_raw + ((1024u - (raw & 1023u)) & 1023u);
    float *bias = reinterpret_cast<float *>(sm + kFwBias);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + kFwBar);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + kFwBar + 8);
    const int tid = threadIdx.x, wid = tid >> 5;

    // weights: W1^T fragments (1 k-tile x 8 n-tiles), W2^T (4 x 8), W3^T
    // (4 x 1) -> K-major operands with rows = output units
    for (uint32_t w = tid; w < 8 * 64; w += 128) {
        uint32_t k, n;
        frag_word_kn(w, 8, k, n);
        const uint32_t v = packed[kF1 + w];
        st16(sm, kFwW1 + kmaj_off(n, k, kFwK16Sbo), v & 0xFFFFu);
        st16(sm, kFwW1 + kmaj_off(n, k + 1, kFwK16Sbo), v >> 16);
    }
    for (uint32_t w = tid; w < 32 * 64; w += 128) {
        uint32_t k, n;
        frag_word_kn(w, 8, k, n);
        const uint32_t v = packed[kF2 + w];
        st16(sm, kFwW2 + kmaj_off(n, k, kFwK64Sbo), v & 0xFFFFu);
        st16(sm, kFwW2 + kmaj_off(n, k + 1, kFwK64Sbo), v >> 16);
    }
    for (uint32_t w = tid; w < 4 * 64; w += 128) {
        uint32_t k, n;
        frag_word_kn(w, 1, k, n);
        const uint32_t v = packed[kF3 + w];
        st16(sm, kFwW3 + kmaj_off(n, k, kFwK64Sbo), v & 0xFFFFu);
        st16(sm, kFwW3 + kmaj_off(n, k + 1, kFwK64Sbo), v >> 16);
        st16(sm, kFwW3 + kmaj_off(n + 8, k, kFwK64Sbo), 0);
        st16(sm, kFwW3 + kmaj_off(n + 8, k + 1, kFwK64Sbo), 0);
    }
    for (int i = tid; i < kHid + kHid + kOut; i += 128)
        bias[i] = __uint_as_float(packed[kPackedBias + i]);
    if (tid == 0)
        tc05::mbar_init(mbar, 1);
    if (wid == 0)
        tc05::tmem_alloc(tmem_slot, kFwTmemCols);
    tc05::fence_before_sync();
    __syncthreads();
    tc05::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t tw = tmem + ((32u * wid) << 16); // this warp's lanes
    const uint32_t sbase = tc05::smem_addr(sm);
    const uint32_t r = tid; // the thread's row of the tile
    uint32_t phase = 0;
    bool bad = false;
    const uint32_t ntiles = (B + 127) / 128;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint32_t i = tile * 128 + r;
        const bool mine = i < B;
        // ---- input row: 6 features (BF16), zeros to 16
        {
            float f[6];
#pragma unroll
            for (int k = 0; k < 6; ++k)
                f[k] = mine ? feat[6 * i + k] : 0.0f;
            uint4 lo;
            lo.x = pack_bf16(f[0], f[1]);
            lo.y = pack_bf16(f[2], f[3]);
            lo.z = pack_bf16(f[4], f[5]);
            lo.w = 0;
            *reinterpret_cast<uint4 *>(sm + kFwX + kmaj_off(r, 0, kFwK16Sbo)) = lo;
            *reinterpret_cast<uint4 *>(sm + kFwX + kmaj_off(r, 8, kFwK16Sbo)) =
                make_uint4(0, 0, 0, 0);
        }
        // three layers: MMA chain, then the rows' epilogue
#pragma unroll 1
        for (int layer = 0; layer < 3; ++layer) {
            tc05::fence_async_shared();
            tc05::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc05::fence_after_sync();
                if (layer == 0) {
                    tc05::mma_bf16(tmem,
                        tc05::desc_kmajor(sbase + kFwX, 128, kFwK16Sbo),
                        tc05::desc_kmajor(sbase + kFwW1, 128, kFwK16Sbo),
                        tc05::idesc_bf16(128, 64), 0u);
                } else {
                    const uint32_t a = sbase + (layer == 1 ? kFwH1 : kFwH2);
                    const uint32_t b = sbase + (layer == 1 ? kFwW2 : kFwW3);
                    const uint32_t d = tmem + (layer == 1 ? 64u : 0u);
                    const uint32_t id = layer == 1 ? tc05::idesc_bf16(128, 64)
                                                   : tc05::idesc_bf16(128, 16);
#pragma unroll
                    for (uint32_t kk = 0; kk < 4; ++kk)
                        tc05::mma_bf16(d,
                            tc05::desc_kmajor(a + kk * 256, 128, kFwK64Sbo),
                            tc05::desc_kmajor(b + kk * 256, 128, kFwK64Sbo),
                            id, kk > 0 ? 1u : 0u);
                }
                tc05::commit(mbar);
            }
            const bool ok = tc05::mbar_wait(mbar, phase & 1, kTcWaitNs);
            ++phase;
            if (__syncthreads_or(!ok)) {
                bad = true;
                break;
            }
            tc05::fence_after_sync();
            if (layer < 2) {
                const uint32_t col = layer == 0 ? 0u : 64u;
                const float *bl = bias + (layer == 0 ? 0 : kHid);
                unsigned char *h = sm + (layer == 0 ? kFwH1 : kFwH2);
#pragma unroll
                for (int c0 = 0; c0 < 64; c0 += 16) {
                    float v[16];
                    tc05::ld16(tw + col + c0, v);
                    uint32_t pk[8];
#pragma unroll
                    for (int c = 0; c < 16; c += 2)
                        pk[c / 2] = pack_bf16(gelu_f(v[c] + bl[c0 + c]),
                            gelu_f(v[c + 1] + bl[c0 + c + 1]));
                    *reinterpret_cast<uint4 *>(
                        h + kmaj_off(r, c0, kFwK64Sbo)) =
                        make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    *reinterpret_cast<uint4 *>(
                        h + kmaj_off(r, c0 + 8, kFwK64Sbo)) =
                        make_uint4(pk[4], pk[5], pk[6], pk[7]);
                }
            } else {
                float v[16];
                tc05::ld16(tw, v);
                if (mine) {
                    const float *b3 = bias + 2 * kHid;
#pragma unroll
                    for (int k = 0; k < kOut; ++k)
                        out[8 * i + k] = v[k] + b3[k];
                }
            }
        }
        if (bad)
            break;
    }
    if (bad) {
        // one more bounded wait for the tensor core, then mark the rows
        tc05::mbar_wait(mbar, (phase - 1) & 1, kTcWaitNs);
        for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const uint32_t i = tile * 128 + r;
            if (i < B)
                for (int k = 0; k < 8; ++k)
                    out[8 * i + k] = __int_as_float(0x7FC00000);
        }
    }
    tc05::fence_before_sync();
    __syncthreads();
    if (wid == 0) {
        tc05::fence_after_sync();
        tc05::tmem_free(tmem, kFwTmemCols);
    }
}

// sum of the block partials (fixed order); grad = mean gradient
__global__ void k_mlp_grad_reduce(const double *part, int nblocks,
    float inv_b, float *grad, double *loss)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > kNumParams)
        return;
    double s = 0;
    for (int b = 0; b < nblocks; ++b)
        s += part[static_cast<size_t>(b) * (kNumParams + 1) + i];
    if (i < kNumParams)
        grad[i] = static_cast<float>(s);
    else if (loss)
        *loss = s * inv_b;
}

// Adam on the master parameters, then the packed copy is rebuilt
__global__ void k_adam(float *p, const float *grad, float *m1, float *m2,
    float lr, float b1, float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNumParams)
        return;
    const float gi = grad[i];
    const float a = b1 * m1[i] + (1 - b1) * gi;
    const float b = b2 * m2[i] + (1 - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    p[i] -= lr * (a * c1) / (sqrtf(b * c2) + eps);
}

// ------------------------------------------------------------- trainer

// One step of every training trajectory: t == 0 draws the prior; t > 0
// writes sample (t - 1) * M + i (features of x_{t-1} and z_t, and nu_t) and
// advances.
__global__ void k_traj_step(uint32_t M, uint32_t t, uint32_t seed,
    BearingsConst c, float sigma_z, float *tx, float *ty, float *tvx,
    float *tvy, float *feat, float *nu_out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < M;
         i += gridDim.x * blockDim.x) {
        float e[4];
        bearings_normals(t, seed, i, e);
        float x = tx[i], y = ty[i], vx = tvx[i], vy = tvy[i];
        if (t == 0) {
            bearings_prior(c, e, x, y, vx, vy);
        } else {
            const float px = x, py = y, pvx = vx, pvy = vy;
            bearings_step(c, e, x, y, vx, vy);
            // bearing noise from a second block of the trajectory's stream
            const u32x4 w2 = philox4x32_10(2u, i, 0u, 0u, t, seed);
            float zn1, zn2;
            normal_pair_f(w2.x, w2.y, zn1, zn2);
            const float z = atan2f(y, x) + sigma_z * zn1;
            const float sz = sinf(z), cz = cosf(z);
            float f[6], fr[4];
            bearings_features(c, px, py, pvx, pvy, sz, cz, f);
            axes_to_frame(sz, cz, e, fr); // the target, bearing frame
            const size_t row = static_cast<size_t>(t - 1) * M + i;
#pragma unroll
            for (int k = 0; k < 6; ++k)
                feat[6 * row + k] = f[k];
#pragma unroll
            for (int d = 0; d < 4; ++d)
                nu_out[4 * row + d] = fr[d];
        }
        tx[i] = x;
        ty[i] = y;
        tvx[i] = vx;
        tvy[i] = vy;
    }
}

// Training rows from the particle clouds of a bootstrap filter.  Block k
// simulates track k of the model (FP32; Philox4x32 key {t, seed}, counter
// {4, k, 0, 0} for the transition noise and {5, k, 0, 0} for the bearing
// noise) and runs a bootstrap filter of P = blockDim.x particles on its
// bearings, resampling every step (stratified, one uniform per particle).
// At step t >= 1 the cloud before the move is the filter's particle
// approximation of p(x_{t-1} | z_{0:t-1}); each of its particles x' gives
// one row: its network inputs for z_t, and a noise nu* chosen among K draws
// nu_k ~ N(0, I) with probability proportional to g(z_t | F x' + L nu_k)
// (sampling-importance-resampling toward the locally optimal proposal
// p(nu | x', z_t), the minimiser of the training loss), in the bearing frame.
// The K weights are combined in one pass: candidate k replaces the choice
// with probability w_k / (w_0 + ... + w_k).  Row ((k (T - 1)) + t - 1) P + j.
// Particle j's streams: key {t, seed}, counters {6, k P + j, kk, 0} (the
// candidates), {7, ...} (the replacement uniforms), {8, k P + j, 0, 0} (the
// move), {9, ...} (the resampling uniform), {10, ...} (the prior at t = 0).
constexpr int kCloudMaxP = 1024;
constexpr int kCloudMaxT = 1024;

__global__ void __launch_bounds__(kCloudMaxP) k_cloud_rows(BearingsConst c,
    float sigma_z, uint32_t seed, uint32_t T, uint32_t K, float *feat,
    float *nu_out)
{
    __shared__ float zs[kCloudMaxT];
    __shared__ float cx[kCloudMaxP], cy[kCloudMaxP], cvx[kCloudMaxP],
        cvy[kCloudMaxP];
    __shared__ float mx[kCloudMaxP], my[kCloudMaxP], mvx[kCloudMaxP],
        mvy[kCloudMaxP];
    __shared__ float cdf[kCloudMaxP];
    __shared__ float red[kCloudMaxP / 32 + 1];
    const uint32_t k = blockIdx.x, j = threadIdx.x, P = blockDim.x;
    const uint32_t pid = k * P + j;
    if (j == 0) { // the track and its bearings, one thread
        float e[4];
        const u32x4 w0 = philox4x32_10(4u, k, 0u, 0u, 0u, seed);
        normal_pair_f(w0.x, w0.y, e[0], e[1]);
        normal_pair_f(w0.z, w0.w, e[2], e[3]);
        float x, y, vx, vy;
        bearings_prior(c, e, x, y, vx, vy);
        for (uint32_t t = 0; t < T; ++t) {
            if (t > 0) {
                const u32x4 w = philox4x32_10(4u, k, 0u, 0u, t, seed);
                normal_pair_f(w.x, w.y, e[0], e[1]);
                normal_pair_f(w.z, w.w, e[2], e[3]);
                bearings_step(c, e, x, y, vx, vy);
            }
            const u32x4 w2 = philox4x32_10(5u, k, 0u, 0u, t, seed);
            float zn1, zn2;
            normal_pair_f(w2.x, w2.y, zn1, zn2);
            zs[t] = atan2f(y, x) + sigma_z * zn1;
        }
    }
    __syncthreads();
    // prior cloud, weighted by z_0 below
    float x, y, vx, vy;
    {
        float e[4];
        const u32x4 w = philox4x32_10(10u, pid, 0u, 0u, 0u, seed);
        normal_pair_f(w.x, w.y, e[0], e[1]);
        normal_pair_f(w.z, w.w, e[2], e[3]);
        bearings_prior(c, e, x, y, vx, vy);
    }
    for (uint32_t t = 0; t < T; ++t) {
        const float z = zs[t];
        if (t > 0) {
            const float sz = sinf(z), cz = cosf(z);
            const size_t row =
                (static_cast<size_t>(k) * (T - 1) + (t - 1)) * P + j;
            float f[6];
            bearings_features(c, x, y, vx, vy, sz, cz, f);
#pragma unroll
            for (int d = 0; d < 6; ++d)
                feat[6 * row + d] = f[d];
            // one pass over the K candidates
            float m = -INFINITY, sum = 0.0f;
            float pick[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            for (uint32_t kk = 0; kk < K; ++kk) {
                const u32x4 w = philox4x32_10(6u, pid, kk, 0u, t, seed);
                float e[4];
                normal_pair_f(w.x, w.y, e[0], e[1]);
                normal_pair_f(w.z, w.w, e[2], e[3]);
                float px = x, py = y, pvx = vx, pvy = vy;
                bearings_step(c, e, px, py, pvx, pvy);
                const float l = bearings_loglik(c, z, px, py);
                if (l > m) {
                    sum = sum * __expf(m - l) + 1.0f;
                    m = l;
                } else {
                    sum += __expf(l - m);
                }
                const u32x4 a = philox4x32_10(7u, pid, kk, 0u, t, seed);
                if (u01_co_f(a.x) * sum < __expf(l - m)) {
#pragma unroll
                    for (int d = 0; d < 4; ++d)
                        pick[d] = e[d];
                }
            }
            float fr[4];
            axes_to_frame(sz, cz, pick, fr);
#pragma unroll
            for (int d = 0; d < 4; ++d)
                nu_out[4 * row + d] = fr[d];
            // the bootstrap move
            float e[4];
            const u32x4 w = philox4x32_10(8u, pid, 0u, 0u, t, seed);
            normal_pair_f(w.x, w.y, e[0], e[1]);
            normal_pair_f(w.z, w.w, e[2], e[3]);
            bearings_step(c, e, x, y, vx, vy);
        }
        // weight by z_t and resample (stratified over the block's CDF)
        const float lw = bearings_loglik(c, z, x, y);
        mx[j] = x;
        my[j] = y;
        mvx[j] = vx;
        mvy[j] = vy;
        const float M = block_reduce(lw, OpMax(), -INFINITY, red);
        float total;
        const float incl =
            block_inclusive_scan(__expf(lw - M), OpAdd(), 0.0f, red, &total);
        cdf[j] = incl;
        __syncthreads();
        const u32x4 w = philox4x32_10(9u, pid, 0u, 0u, t, seed);
        const float u =
            (static_cast<float>(j) + u01_co_f(w.x)) / static_cast<float>(P) *
            total;
        uint32_t lo = 0, hi = P - 1; // the first slot with cdf > u
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (cdf[mid] > u)
                hi = mid;
            else
                lo = mid + 1;
        }
        x = mx[lo];
        y = my[lo];
        vx = mvx[lo];
        vy = mvy[lo];
        __syncthreads();
    }
}

// A minibatch of `batch` rows drawn uniformly with replacement from the
// `total` stored samples (Philox4x32 key {step, seed}, counter
// {3, row, 0, 0}; index = floor(word * total / 2^32)).
// Rows at index total and above come from the extra rows (xfeat, xnu).
__global__ void k_minibatch(uint64_t total, uint64_t nx, uint32_t batch,
    uint32_t step, uint32_t seed, const float *feat, const float *nu,
    const float *xfeat, const float *xnu, float *mf, float *mn)
{
    const uint64_t all = total + nx;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < batch;
         r += gridDim.x * blockDim.x) {
        const u32x4 w = philox4x32_10(3u, r, 0u, 0u, step, seed);
        uint64_t j = (static_cast<uint64_t>(w.x) * all) >> 32;
        const float *fs = feat, *ns = nu;
        if (j >= total) {
            j -= total;
            fs = xfeat;
            ns = xnu;
        }
#pragma unroll
        for (int k = 0; k < 6; ++k)
            mf[6 * r + k] = fs[6 * j + k];
#pragma unroll
        for (int d = 0; d < 4; ++d)
            mn[4 * r + d] = ns[4 * j + d];
    }
}

static int grad_blocks(uint32_t B)
{
    const int rounds = static_cast<int>((B + kGradRows - 1) / kGradRows);
    const int cap = num_sms(); // one block per SM (shared memory)
    return rounds < cap ? rounds : cap;
}

static bool grad_smem_ready()
{
    static bool ok = cudaFuncSetAttribute(k_mlp_grad,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(kGradSmem)) == cudaSuccess;
    return ok;
}

// enqueue loss + gradient of B samples (part: [grid][kNumParams + 1])
static int enqueue_grad(const uint32_t *packed, uint32_t B, const float *feat,
    const float *nu, double *part, float *grad, double *loss,
    cudaStream_t st)
{
    if (!grad_smem_ready())
        return VSMC_CUDA_ERR_CUDA;
    const int grid = grad_blocks(B);
    const float inv_b = 1.0f / static_cast<float>(B);
    k_mlp_grad<<<grid, 128, kGradSmem, st>>>(packed, B, feat, nu, inv_b, part);
    k_mlp_grad_reduce<<<(kNumParams + 1 + 255) / 256, 256, 0, st>>>(
        part, grid, inv_b, grad, loss);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

} // namespace vsmc_cuda

extern "C" {

int vsmc_cuda_bearings_simulate(uint32_t seed, size_t T,
    const vsmc_cuda_bearings_model *model, double *truth, double *obs,
    void *stream)
{
    if (!valid_bearings_model(model) || obs == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (T == 0)
        return VSMC_CUDA_OK;
    if (T > 0xFFFFFFFFull)
        return VSMC_CUDA_ERR_SIZE;
    k_bearings_simulate<<<1, 32, 0, as_stream(stream)>>>(seed,
        static_cast<uint32_t>(T), *model, truth, obs);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_mlp_pack(const float *params, uint32_t *packed, void *stream)
{
    if (params == nullptr || packed == nullptr)
        return VSMC_CUDA_ERR_ARG;
    k_mlp_pack<<<(kPackedWords + 255) / 256, 256, 0, as_stream(stream)>>>(
        params, packed);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_mlp_sizes(size_t *nparams, size_t *npacked)
{
    if (nparams)
        *nparams = kNumParams;
    if (npacked)
        *npacked = kPackedWords;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_mlp_forward(const uint32_t *packed, size_t B, const float *feat,
    float *out, void *stream)
{
    if (packed == nullptr || (B && (feat == nullptr || out == nullptr)))
        return VSMC_CUDA_ERR_ARG;
    if (B >= (size_t(1) << 31))
        return VSMC_CUDA_ERR_SIZE;
    if (B == 0)
        return VSMC_CUDA_OK;
    const int grid = grid_for((B + 31) / 32 * 32, 128, 1, 8);
    k_mlp_forward<<<grid, 128, 0, as_stream(stream)>>>(
        packed, static_cast<uint32_t>(B), feat, out);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_mlp_forward_tc(const uint32_t *packed, size_t B,
    const float *feat, float *out, void *stream)
{
    if (packed == nullptr || (B && (feat == nullptr || out == nullptr)))
        return VSMC_CUDA_ERR_ARG;
    if (B >= (size_t(1) << 31))
        return VSMC_CUDA_ERR_SIZE;
    if (B == 0)
        return VSMC_CUDA_OK;
    static const bool ready = cudaFuncSetAttribute(k_mlp_forward_tc,
        cudaFuncAttributeMaxDynamicSharedMemorySize,
        static_cast<int>(kFwSmem)) == cudaSuccess;
    if (!ready)
        return VSMC_CUDA_ERR_CUDA;
    const size_t tiles = (B + 127) / 128;
    const size_t cap = static_cast<size_t>(num_sms()) * 4;
    const int grid = static_cast<int>(tiles < cap ? tiles : cap);
    k_mlp_forward_tc<<<grid, 128, kFwSmem, as_stream(stream)>>>(
        packed, static_cast<uint32_t>(B), feat, out);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_mlp_loss_grad(const uint32_t *packed, size_t B,
    const float *feat, const float *nu, double *loss_dev, float *grad_dev,
    void *stream)
{
    if (packed == nullptr || feat == nullptr || nu == nullptr ||
        grad_dev == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (B < 1 || B >= (size_t(1) << 31))
        return VSMC_CUDA_ERR_SIZE;
    cudaStream_t st = as_stream(stream);
    Scratch scratch(st);
    double *part = scratch.get<double>(
        static_cast<size_t>(grad_blocks(static_cast<uint32_t>(B))) *
        (kNumParams + 1));
    if (part == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    return enqueue_grad(packed, static_cast<uint32_t>(B), feat, nu, part,
        grad_dev, loss_dev, st);
}

int vsmc_cuda_bearings_move_f32(size_t n, size_t t, uint32_t seed,
    const vsmc_cuda_bearings_model *model, double z, const uint32_t *packed,
    float *state, float *lw_inc, void *stream)
{
    if (!valid_bearings_model(model) || ((state == nullptr || lw_inc == nullptr) && n))
        return VSMC_CUDA_ERR_ARG;
    if (n >= (size_t(1) << 31) || t > 0xFFFFFFFFull)
        return VSMC_CUDA_ERR_SIZE;
    if (n == 0)
        return VSMC_CUDA_OK;
    const BearingsConst c = make_bearings_const(*model);
    const uint32_t nn = static_cast<uint32_t>(n);
    cudaStream_t st = as_stream(stream);
    if (packed != nullptr && t > 0) {
        const int grid = grid_for((n + 31) / 32 * 32, 128, 1, 8);
        k_bearings_move<true><<<grid, 128, 0, st>>>(nn,
            static_cast<uint32_t>(t), seed, c, static_cast<float>(z), packed,
            state, state + n, state + 2 * n, state + 3 * n, lw_inc);
    } else {
        const int grid = grid_for(n, 128, 1, 8);
        k_bearings_move<false><<<grid, 128, 0, st>>>(nn,
            static_cast<uint32_t>(t), seed, c, static_cast<float>(z), nullptr,
            state, state + n, state + 2 * n, state + 3 * n, lw_inc);
    }
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_mlp_init(uint32_t seed, float *params, void *stream)
{
    if (params == nullptr)
        return VSMC_CUDA_ERR_ARG;
    // Hidden layers uniform in +-sqrt(6 / fan_in) from a 32-bit linear
    // congruential sequence seeded by `seed` (initial values only; no
    // parity contract); the output layer starts at zero, so the untrained
    // proposal is the bootstrap.
    std::vector<float> h(kNumParams, 0.0f);
    uint32_t state = seed * 2654435761u + 12345u;
    auto u01 = [&]() {
        state = state * 1664525u + 1013904223u;
        return static_cast<float>(state >> 8) * (1.0f / 16777216.0f);
    };
    const float s1 = std::sqrt(6.0f / kIn), s2 = std::sqrt(6.0f / kHid);
    for (int i = 0; i < kHid * kIn; ++i)
        h[kW1 + i] = (2 * u01() - 1) * s1;
    for (int i = 0; i < kHid * kHid; ++i)
        h[kW2 + i] = (2 * u01() - 1) * s2;
    VSMC_CUDA_TRY(cudaMemcpyAsync(params, h.data(), sizeof(float) * kNumParams,
        cudaMemcpyHostToDevice, as_stream(stream)));
    VSMC_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
    return VSMC_CUDA_OK;
}

// Train the proposal network in place on `params` (device, kNumParams
// floats): ntraj trajectories from the model's prior are simulated for T
// steps and their ntraj * (T - 1) samples stored; then `steps` Adam steps,
// each on `batch` samples drawn uniformly with replacement.  loss_host (may
// be NULL) receives the mean loss of every minibatch.
int vsmc_cuda_mlp_train(const vsmc_cuda_bearings_model *model, uint32_t seed,
    size_t ntraj, size_t T, size_t batch, size_t steps, double lr,
    float *params, double *loss_host, void *stream)
{
    return vsmc_cuda_mlp_train_rows(model, seed, ntraj, T, nullptr, nullptr,
        0, batch, steps, lr, params, loss_host, stream);
}

int vsmc_cuda_mlp_cloud_rows(const vsmc_cuda_bearings_model *model,
    uint32_t seed, size_t ntracks, size_t P, size_t T, size_t K, float *feat,
    float *nu, void *stream)
{
    if (!valid_bearings_model(model) || feat == nullptr || nu == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (ntracks < 1 || ntracks > 0x7FFFFFFFull || P < 32 || P % 32 != 0 ||
        P > static_cast<size_t>(kCloudMaxP) || T < 2 ||
        T > static_cast<size_t>(kCloudMaxT) || K < 1 || K > 0xFFFFFFFFull ||
        ntracks * P > 0xFFFFFFFFull)
        return VSMC_CUDA_ERR_SIZE;
    cudaStream_t st = as_stream(stream);
    k_cloud_rows<<<static_cast<unsigned>(ntracks), static_cast<unsigned>(P),
        0, st>>>(make_bearings_const(*model),
        static_cast<float>(model->sigma_z), seed, static_cast<uint32_t>(T),
        static_cast<uint32_t>(K), feat, nu);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_mlp_train_rows(const vsmc_cuda_bearings_model *model,
    uint32_t seed, size_t ntraj, size_t T, const float *xfeat,
    const float *xnu, size_t nx, size_t batch, size_t steps, double lr,
    float *params, double *loss_host, void *stream)
{
    if (!valid_bearings_model(model) || params == nullptr || !(lr > 0) ||
        (nx > 0 && (xfeat == nullptr || xnu == nullptr)))
        return VSMC_CUDA_ERR_ARG;
    if (nx >= (size_t(1) << 32))
        return VSMC_CUDA_ERR_SIZE;
    if (ntraj < 1 || ntraj >= (size_t(1) << 28) || T < 2 ||
        T > 0xFFFFFFFFull || batch < 16 || batch >= (size_t(1) << 24) ||
        steps < 1 || steps > 0xFFFFFFFFull ||
        ntraj * (T - 1) >= (size_t(1) << 40))
        return VSMC_CUDA_ERR_SIZE;
    cudaStream_t st = as_stream(stream);
    Scratch scratch(st);
    const size_t M = ntraj;
    const size_t total = M * (T - 1);
    float *tx = scratch.get<float>(M), *ty = scratch.get<float>(M);
    float *tvx = scratch.get<float>(M), *tvy = scratch.get<float>(M);
    float *feat = scratch.get<float>(6 * total);
    float *nu = scratch.get<float>(4 * total);
    float *mf = scratch.get<float>(6 * batch);
    float *mn = scratch.get<float>(4 * batch);
    float *grad = scratch.get<float>(kNumParams);
    float *m1 = scratch.get<float>(kNumParams);
    float *m2 = scratch.get<float>(kNumParams);
    uint32_t *packed = scratch.get<uint32_t>(kPackedWords);
    double *losses = scratch.get<double>(steps);
    double *part = scratch.get<double>(
        static_cast<size_t>(grad_blocks(static_cast<uint32_t>(batch))) *
        (kNumParams + 1));
    if (!tx || !ty || !tvx || !tvy || !feat || !nu || !mf || !mn || !grad ||
        !m1 || !m2 || !packed || !losses || !part)
        return VSMC_CUDA_ERR_ALLOC;
    VSMC_CUDA_TRY(cudaMemsetAsync(m1, 0, sizeof(float) * kNumParams, st));
    VSMC_CUDA_TRY(cudaMemsetAsync(m2, 0, sizeof(float) * kNumParams, st));
    const BearingsConst c = make_bearings_const(*model);
    const int tgrid = grid_for(M, 256, 1, 8);
    for (size_t t = 0; t < T; ++t) {
        k_traj_step<<<tgrid, 256, 0, st>>>(static_cast<uint32_t>(M),
            static_cast<uint32_t>(t), seed, c,
            static_cast<float>(model->sigma_z), tx, ty, tvx, tvy, feat, nu);
        VSMC_CUDA_CHECK_LAUNCH();
    }
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    double p1 = 1, p2 = 1;
    const int mgrid = grid_for(batch, 256, 1, 8);
    for (size_t k = 0; k < steps; ++k) {
        k_minibatch<<<mgrid, 256, 0, st>>>(total, nx,
            static_cast<uint32_t>(batch), static_cast<uint32_t>(k), seed, feat,
            nu, xfeat, xnu, mf, mn);
        k_mlp_pack<<<(kPackedWords + 255) / 256, 256, 0, st>>>(params, packed);
        const int rc = enqueue_grad(packed, static_cast<uint32_t>(batch), mf,
            mn, part, grad, losses + k, st);
        if (rc != VSMC_CUDA_OK)
            return rc;
        p1 *= b1;
        p2 *= b2;
        k_adam<<<(kNumParams + 255) / 256, 256, 0, st>>>(params, grad, m1, m2,
            static_cast<float>(lr), b1, b2, eps,
            static_cast<float>(1 / (1 - p1)), static_cast<float>(1 / (1 - p2)));
        VSMC_CUDA_CHECK_LAUNCH();
    }
    if (loss_host)
        VSMC_CUDA_TRY(cudaMemcpyAsync(loss_host, losses,
            sizeof(double) * steps, cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    return VSMC_CUDA_OK;
}

} // extern "C"
