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

constexpr int kGradWarps = 4;
constexpr int kGradRows = 16 * kGradWarps; // samples per block round
constexpr int kLd = 68;                    // staging row stride (floats)

// staging: a0 [rows][8], a1 / a2 / dp1 / dp2 [rows][kLd], dout [rows][8]
constexpr int kStA0 = 0;
constexpr int kStA1 = kStA0 + kGradRows * 8;
constexpr int kStA2 = kStA1 + kGradRows * kLd;
constexpr int kStD1 = kStA2 + kGradRows * kLd;
constexpr int kStD2 = kStD1 + kGradRows * kLd;
constexpr int kStDo = kStD2 + kGradRows * kLd;
constexpr int kStTotal = kStDo + kGradRows * 8;
constexpr size_t kGradSmem =
    sizeof(uint32_t) * kPackedWords + sizeof(float) * kStTotal;

// accumulator fragment (rows g, g + 8 of 16) -> staging rows
__device__ __forceinline__ void stage_c(
    float *st, int ld, int row0, int col0, const float (&c)[4])
{
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    st[(row0 + g) * ld + col0 + 2 * t] = c[0];
    st[(row0 + g) * ld + col0 + 2 * t + 1] = c[1];
    st[(row0 + g + 8) * ld + col0 + 2 * t] = c[2];
    st[(row0 + g + 8) * ld + col0 + 2 * t + 1] = c[3];
}

__device__ __forceinline__ float2 unpack_bf16(uint32_t w)
{
    return make_float2(__uint_as_float(w << 16), __uint_as_float(w & 0xFFFF0000u));
}

// operand fragment (16 x 16 bf16) -> staging rows, columns col0..col0+15
__device__ __forceinline__ void stage_a(
    float *st, int ld, int row0, int col0, const uint32_t (&a)[4])
{
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const float2 v0 = unpack_bf16(a[0]), v1 = unpack_bf16(a[1]);
    const float2 v2 = unpack_bf16(a[2]), v3 = unpack_bf16(a[3]);
    st[(row0 + g) * ld + col0 + 2 * t] = v0.x;
    st[(row0 + g) * ld + col0 + 2 * t + 1] = v0.y;
    st[(row0 + g + 8) * ld + col0 + 2 * t] = v1.x;
    st[(row0 + g + 8) * ld + col0 + 2 * t + 1] = v1.y;
    st[(row0 + g) * ld + col0 + 2 * t + 8] = v2.x;
    st[(row0 + g) * ld + col0 + 2 * t + 9] = v2.y;
    st[(row0 + g + 8) * ld + col0 + 2 * t + 8] = v3.x;
    st[(row0 + g + 8) * ld + col0 + 2 * t + 9] = v3.y;
}

// Loss and gradient partials of one block over its samples.  Forward and
// the backward data path on the tensor cores; the weight gradients as
// register-blocked FP32 sums over staged rows.  part: [grid][kNumParams + 1]
// (the last entry is the block's loss sum).
__global__ void __launch_bounds__(128) k_mlp_grad(const uint32_t *packed,
    uint32_t B, const float *feat, const float *nu_in, float inv_b,
    double *part)
{
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t *sp = smem;
    float *st = reinterpret_cast<float *>(smem + kPackedWords);
    load_packed(sp, packed);
    const int tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    const int g = lane >> 2, q = lane & 3;
    // weight-gradient accumulators
    const int j2 = (tid >> 3) * 4, k2 = (tid & 7) * 8; // dW2 block 4 x 8
    const int d3 = tid >> 4, k3 = (tid & 15) * 4;       // dW3 1 x 4
    const int j1 = tid >> 1, k1 = (tid & 1) * 3;        // dW1 1 x 3
    float gw2[4][8], gw3[4], gw1[3], gb = 0, gb3 = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int s = 0; s < 8; ++s)
            gw2[r][s] = 0;
#pragma unroll
    for (int s = 0; s < 4; ++s)
        gw3[s] = 0;
#pragma unroll
    for (int s = 0; s < 3; ++s)
        gw1[s] = 0;
    double loss = 0;
    const uint32_t rounds = (B + kGradRows - 1) / kGradRows;
    for (uint32_t rd = blockIdx.x; rd < rounds; rd += gridDim.x) {
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
                loss += 0.5 * (static_cast<double>(r) * r * el + v[4 + d]);
        }
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
        // ---- stage this warp's 16 rows
        const int row0 = 16 * wid;
        {
            // input rows: columns 0..7 only (inputs 0..5, 6..7 zero)
            const float2 v0 = unpack_bf16(a0[0]), v1 = unpack_bf16(a0[1]);
            float *s0 = st + kStA0 + (row0 + g) * 8 + 2 * q;
            float *s1 = st + kStA0 + (row0 + g + 8) * 8 + 2 * q;
            s0[0] = v0.x;
            s0[1] = v0.y;
            s1[0] = v1.x;
            s1[1] = v1.y;
        }
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            stage_a(st + kStA1, kLd, row0, 16 * kt, act1[kt]);
            stage_a(st + kStA2, kLd, row0, 16 * kt, act2[kt]);
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            stage_c(st + kStD1, kLd, row0, 8 * nt, dp1[nt]);
            stage_c(st + kStD2, kLd, row0, 8 * nt, dp2[nt]);
        }
        if (q < 2) {
            const int row = row0 + g + (q == 1 ? 8 : 0);
#pragma unroll
            for (int d = 0; d < 8; ++d)
                st[kStDo + row * 8 + d] = dv[d];
        }
        __syncthreads();
        // ---- weight gradients over the block's rows
        for (int s = 0; s < kGradRows; ++s) {
            const float *a1r = st + kStA1 + s * kLd;
            const float *d2r = st + kStD2 + s * kLd;
            float av[8], dvv[4];
#pragma unroll
            for (int c8 = 0; c8 < 8; ++c8)
                av[c8] = a1r[k2 + c8];
#pragma unroll
            for (int r = 0; r < 4; ++r)
                dvv[r] = d2r[j2 + r];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c8 = 0; c8 < 8; ++c8)
                    gw2[r][c8] = fmaf(dvv[r], av[c8], gw2[r][c8]);
            const float *a2r = st + kStA2 + s * kLd;
            const float dd = st[kStDo + s * 8 + d3];
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4)
                gw3[c4] = fmaf(dd, a2r[k3 + c4], gw3[c4]);
            const float d1 = st[kStD1 + s * kLd + j1];
#pragma unroll
            for (int c3 = 0; c3 < 3; ++c3)
                gw1[c3] = fmaf(d1, st[kStA0 + s * 8 + k1 + c3], gw1[c3]);
            // biases: b1 (threads 0..63), b2 (64..127), b3 (0..7)
            gb += tid < kHid ? st[kStD1 + s * kLd + tid]
                             : st[kStD2 + s * kLd + tid - kHid];
            if (tid < kOut)
                gb3 += st[kStDo + s * 8 + tid];
        }
        __syncthreads();
    }
    // ---- block partials
    double *out = part + static_cast<size_t>(blockIdx.x) * (kNumParams + 1);
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c8 = 0; c8 < 8; ++c8)
            out[kW2 + (j2 + r) * kHid + k2 + c8] = gw2[r][c8];
#pragma unroll
    for (int c4 = 0; c4 < 4; ++c4)
        out[kW3 + d3 * kHid + k3 + c4] = gw3[c4];
#pragma unroll
    for (int c3 = 0; c3 < 3; ++c3)
        out[kW1 + j1 * kIn + k1 + c3] = gw1[c3];
    if (tid < kHid)
        out[kB1 + tid] = gb;
    else
        out[kB2 + tid - kHid] = gb;
    if (tid < kOut)
        out[kB3 + tid] = gb3;
    // loss: owners' sums over the block
    __shared__ double shl[128 / 32 + 1];
    loss = block_reduce(loss, OpAdd(), 0.0, shl);
    if (tid == 0)
        out[kNumParams] = loss;
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
    const int cap = num_sms() * 2;
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
