// Model entry points: one move / log-likelihood step on caller-owned state
// (the kernel-level parity hook) and the observation simulator.
#include "common.cuh"
#include "pf_model.cuh"
#include "rng_device.cuh"
#include "cv_sim.cuh"

using namespace vsmc_cuda;

namespace vsmc_cuda
{

template <typename T>
__global__ void __launch_bounds__(256) k_cv_move(uint32_t n, uint32_t t,
    uint32_t seed, CvConst<T> c, T ox, T oy, T *x, T *y, T *vx, T *vy, T *ll)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const u32x4 w = particle_block(t, seed, i);
        T X, Y, VX, VY;
        if (t == 0) {
            T z1, z2, z3, z4;
            if constexpr (sizeof(T) == 4) {
                normal_pair_f(w.x, w.y, z1, z2);
                normal_pair_f(w.z, w.w, z3, z4);
            } else {
                normal_pair_d(w.x, w.y, z1, z2);
                normal_pair_d(w.z, w.w, z3, z4);
            }
            X = c.sd_pos0 * z1;
            Y = c.sd_pos0 * z2;
            VX = c.sd_vel0 * z3;
            VY = c.sd_vel0 * z4;
        } else {
            X = x[i];
            Y = y[i];
            VX = vx[i];
            VY = vy[i];
            T z1, z2;
            if constexpr (sizeof(T) == 4)
                normal_pair_f(w.x, w.y, z1, z2);
            else
                normal_pair_d(w.x, w.y, z1, z2);
            cv_move(c, c.sigma_a * z1, c.sigma_a * z2, X, Y, VX, VY);
        }
        x[i] = X;
        y[i] = Y;
        vx[i] = VX;
        vy[i] = VY;
        ll[i] = cv_loglik(c, ox, oy, X, Y);
    }
}

// Sequential simulation on one thread (T is small); see cv_sim.cuh.
__global__ void k_cv_simulate(uint32_t seed, uint32_t T, double dt,
    double sigma_a, double obs_scale, double nu, double sd_pos0,
    double sd_vel0, double *truth, double *obs)
{
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    cv_simulate_seq(seed, T, dt, sigma_a, obs_scale, nu, sd_pos0, sd_vel0,
        truth, obs);
}

// Kernel-level resample-move steps (cv_mcmc_step) on caller-owned state.
__global__ void __launch_bounds__(256) k_cv_mcmc(uint32_t n, uint32_t t,
    uint32_t sweeps, uint32_t seed, CvConst<float> c, float ox, float oy,
    float s_rw, float inv_var, const int *parent, float *sx, float *sy,
    float *svx, float *svy, uint32_t *accepted)
{
    uint32_t acc = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const uint32_t j = parent ? static_cast<uint32_t>(parent[i]) : i;
        float x = sx[i], y = sy[i], vx = svx[i], vy = svy[i];
        float ax, ay;
        cv_innovation(c, t, seed, j, ax, ay);
        float lt =
            -0.5f * inv_var * (ax * ax + ay * ay) + cv_loglik(c, ox, oy, x, y);
        for (uint32_t k = 0; k < sweeps; ++k)
            acc += cv_mcmc_step(
                c, ox, oy, s_rw, inv_var, t, seed, i, k, x, y, vx, vy, ax, ay, lt);
        sx[i] = x;
        sy[i] = y;
        svx[i] = vx;
        svy[i] = vy;
    }
    __shared__ uint32_t sh[256 / 32 + 1];
    acc = block_reduce(acc, OpAdd(), 0u, sh);
    if (threadIdx.x == 0 && acc)
        atomicAdd(accepted, acc);
}

template <typename T>
static int cv_move_impl(size_t n, size_t t, uint32_t seed,
    const vsmc_cuda_cv_model *model, const double obs[2], T *state, T *ll,
    void *stream)
{
    if (!valid_cv_model(model) || obs == nullptr ||
        ((state == nullptr || ll == nullptr) && n))
        return VSMC_CUDA_ERR_ARG;
    if (n >= (size_t(1) << 31) || t > 0xFFFFFFFFull)
        return VSMC_CUDA_ERR_SIZE;
    if (n == 0)
        return VSMC_CUDA_OK;
    const CvConst<T> c = make_cv_const<T>(*model);
    const int grid = grid_for(n, 256, 1, 8);
    k_cv_move<T><<<grid, 256, 0, as_stream(stream)>>>(static_cast<uint32_t>(n),
        static_cast<uint32_t>(t), seed, c, static_cast<T>(obs[0]),
        static_cast<T>(obs[1]), state, state + n, state + 2 * n,
        state + 3 * n, ll);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

} // namespace vsmc_cuda

extern "C" {

int vsmc_cuda_cv_move_f64(size_t n, size_t t, uint32_t seed,
    const vsmc_cuda_cv_model *model, const double obs[2], double *state,
    double *ll, void *stream)
{
    return cv_move_impl<double>(n, t, seed, model, obs, state, ll, stream);
}

int vsmc_cuda_cv_move_f32(size_t n, size_t t, uint32_t seed,
    const vsmc_cuda_cv_model *model, const double obs[2], float *state,
    float *ll, void *stream)
{
    return cv_move_impl<float>(n, t, seed, model, obs, state, ll, stream);
}

int vsmc_cuda_cv_mcmc_f32(size_t n, size_t t, size_t sweeps, uint32_t seed,
    const vsmc_cuda_cv_model *model, const double obs[2], double scale,
    const int *parent, float *state, uint32_t *accepted, void *stream)
{
    if (!valid_cv_model(model) || obs == nullptr || accepted == nullptr ||
        !(scale >= 0) || !(model->sigma_a > 0) || (state == nullptr && n))
        return VSMC_CUDA_ERR_ARG;
    if (n >= (size_t(1) << 31) || t < 1 || t > 0xFFFFFFFFull ||
        sweeps > 1024)
        return t < 1 ? VSMC_CUDA_ERR_ARG : VSMC_CUDA_ERR_SIZE;
    if (n == 0 || sweeps == 0)
        return VSMC_CUDA_OK;
    const CvConst<float> c = make_cv_const<float>(*model);
    const float sa = static_cast<float>(model->sigma_a);
    k_cv_mcmc<<<grid_for(n, 256, 1, 8), 256, 0, as_stream(stream)>>>(
        static_cast<uint32_t>(n), static_cast<uint32_t>(t),
        static_cast<uint32_t>(sweeps), seed, c, static_cast<float>(obs[0]),
        static_cast<float>(obs[1]), static_cast<float>(scale),
        1.0f / (sa * sa), parent, state, state + n, state + 2 * n,
        state + 3 * n, accepted);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_cv_simulate(uint32_t seed, size_t T,
    const vsmc_cuda_cv_model *model, double *truth, double *obs, void *stream)
{
    if (!valid_cv_model(model) || truth == nullptr || obs == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (T == 0)
        return VSMC_CUDA_OK;
    if (T > 0xFFFFFFFFull)
        return VSMC_CUDA_ERR_SIZE;
    k_cv_simulate<<<1, 32, 0, as_stream(stream)>>>(seed,
        static_cast<uint32_t>(T), model->dt, model->sigma_a, model->obs_scale,
        model->nu, model->sd_pos0, model->sd_vel0, truth, obs);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

} // extern "C"
