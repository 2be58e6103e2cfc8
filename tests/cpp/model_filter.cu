// User models run through the fused FP32 filter: the public step-kernel
// template (include/vsmc_cuda_filter.cuh) instantiated in this translation
// unit, the filter's buffers and resampling passes from libvsmc_cuda through
// its C ABI.  Built as a shared library by tests/test_model_filter_gpu.py and
// called through ctypes.
//
//   model 0  the benchmark's constant-velocity / Student-t model, written
//            here from its definition as a user would (not the library's
//            built-in instance)
//   model 1  a 2-D Gaussian random walk x_t = x_{t-1} + s e, observed as
//            y_t = x_t + r eta per component, monitoring the first component
#include <vsmc_cuda_filter.cuh>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

namespace
{

struct UserCv {
    static constexpr int dim = 4;
    static constexpr int monitor_dim = 2;
    struct step_type {
        float ox, oy;
    };

    float dt, h, sigma_a, sd_pos0, sd_vel0;
    float lconst2, inv_s, inv_nu, half_nu1;
    const double *obs;
    uint32_t T;

    __device__ step_type step(uint32_t t) const
    {
        const uint32_t k = t < T ? t : T - 1;
        return {static_cast<float>(obs[2 * k]),
            static_cast<float>(obs[2 * k + 1])};
    }

    __device__ void init(
        const step_type &, vsmc_cuda::ParticleRng &rng, float (&x)[4]) const
    {
        float a, b, c, d;
        rng.normal_pair(a, b);
        rng.normal_pair(c, d);
        x[0] = sd_pos0 * a;
        x[1] = sd_pos0 * b;
        x[2] = sd_vel0 * c;
        x[3] = sd_vel0 * d;
    }

    __device__ void move(
        const step_type &, vsmc_cuda::ParticleRng &rng, float (&x)[4]) const
    {
        float e1, e2;
        rng.normal_pair(e1, e2);
        const float ax = sigma_a * e1, ay = sigma_a * e2;
        x[0] = x[0] + dt * x[2] + h * ax;
        x[1] = x[1] + dt * x[3] + h * ay;
        x[2] = x[2] + dt * ax;
        x[3] = x[3] + dt * ay;
    }

    // Student-t(nu, scale s) density of both coordinates, normalized:
    // 2 log C - (nu + 1) / 2 log((1 + qx)(1 + qy))
    __device__ float log_likelihood(
        const step_type &s, const float (&x)[4]) const
    {
        const float zx = (s.ox - x[0]) * inv_s;
        const float zy = (s.oy - x[1]) * inv_s;
        const float qx = zx * zx * inv_nu;
        const float qy = zy * zy * inv_nu;
        return lconst2 - half_nu1 * __logf(1.0f + fmaf(qx, qy, qx + qy));
    }
};

struct Walk2 {
    static constexpr int dim = 2;
    static constexpr int monitor_dim = 1;
    struct step_type {
        float y0, y1;
    };

    float sd0, s, inv_r, lconst;
    const double *obs;
    uint32_t T;

    __device__ step_type step(uint32_t t) const
    {
        const uint32_t k = t < T ? t : T - 1;
        return {static_cast<float>(obs[2 * k]),
            static_cast<float>(obs[2 * k + 1])};
    }

    __device__ void init(
        const step_type &, vsmc_cuda::ParticleRng &rng, float (&x)[2]) const
    {
        float a, b;
        rng.normal_pair(a, b);
        x[0] = sd0 * a;
        x[1] = sd0 * b;
    }

    __device__ void move(
        const step_type &, vsmc_cuda::ParticleRng &rng, float (&x)[2]) const
    {
        float a, b;
        rng.normal_pair(a, b);
        x[0] += s * a;
        x[1] += s * b;
    }

    __device__ float log_likelihood(
        const step_type &o, const float (&x)[2]) const
    {
        const float u = (o.y0 - x[0]) * inv_r, v = (o.y1 - x[1]) * inv_r;
        return lconst - 0.5f * (u * u + v * v);
    }
};

template <typename Model>
int run(Model m, size_t n, size_t T, uint32_t seed, int scheme,
    double threshold, int host_decides, const double *obs_host, double *mean,
    double *ess, int *res, double *logz)
{
    vsmc_cuda_pf *pf = nullptr;
    int rc = vsmc_cuda_pf_create_model(&pf, n, Model::dim, Model::monitor_dim,
        scheme, host_decides ? -1.0 : threshold, seed, T, nullptr);
    if (rc != VSMC_CUDA_OK)
        return rc;
    double *obs = nullptr;
    if (cudaMalloc(&obs, sizeof(double) * 2 * T) != cudaSuccess ||
        cudaMemcpy(obs, obs_host, sizeof(double) * 2 * T,
            cudaMemcpyHostToDevice) != cudaSuccess) {
        vsmc_cuda_pf_destroy(pf);
        cudaFree(obs);
        return VSMC_CUDA_ERR_CUDA;
    }
    m.obs = obs;
    m.T = static_cast<uint32_t>(T);
    for (size_t t = 0; rc == VSMC_CUDA_OK && t < T; ++t) {
        vsmc_cuda_pf_step_desc d;
        rc = vsmc_cuda_pf_step_desc_get(pf, &d);
        if (rc == VSMC_CUDA_OK)
            rc = vsmc_cuda::pf_step_launch(d, m);
        if (rc == VSMC_CUDA_OK)
            rc = vsmc_cuda_pf_step_commit(pf);
        if (rc == VSMC_CUDA_OK && host_decides) {
            // Particle::resample: ESS < threshold * N on the host
            vsmc_cuda_pf_status st;
            rc = vsmc_cuda_pf_get_status(pf, &st);
            if (rc == VSMC_CUDA_OK &&
                st.ess < threshold * static_cast<double>(n)) {
                rc = vsmc_cuda_pf_resample_now(pf);
                if (rc == VSMC_CUDA_OK)
                    rc = vsmc_cuda_pf_set_equal(pf);
            }
        }
    }
    if (rc == VSMC_CUDA_OK)
        rc = vsmc_cuda_pf_history(pf, T, mean, ess, res, logz);
    vsmc_cuda_pf_destroy(pf);
    cudaFree(obs);
    return rc;
}

double student_t_lconst(double nu, double s)
{
    return std::lgamma(0.5 * (nu + 1)) - std::lgamma(0.5 * nu) -
        0.5 * std::log(nu * 3.14159265358979323846) - std::log(s);
}

} // namespace

// model 0: p = {dt, sigma_a, obs_scale, nu, sd_pos0, sd_vel0}
// model 1: p = {sd0, s, r}
extern "C" int model_filter_run(int model, const double *p, size_t n,
    size_t T, uint32_t seed, int scheme, double threshold, int host_decides,
    const double *obs_host, double *mean, double *ess, int *res, double *logz)
{
    if (model == 0) {
        UserCv m{};
        m.dt = static_cast<float>(p[0]);
        m.h = static_cast<float>(0.5 * p[0] * p[0]);
        m.sigma_a = static_cast<float>(p[1]);
        m.sd_pos0 = static_cast<float>(p[4]);
        m.sd_vel0 = static_cast<float>(p[5]);
        m.lconst2 = static_cast<float>(2 * student_t_lconst(p[3], p[2]));
        m.inv_s = static_cast<float>(1 / p[2]);
        m.inv_nu = static_cast<float>(1 / p[3]);
        m.half_nu1 = static_cast<float>(0.5 * (p[3] + 1));
        return run(m, n, T, seed, scheme, threshold, host_decides, obs_host,
            mean, ess, res, logz);
    }
    if (model == 1) {
        Walk2 m{};
        m.sd0 = static_cast<float>(p[0]);
        m.s = static_cast<float>(p[1]);
        m.inv_r = static_cast<float>(1 / p[2]);
        m.lconst = static_cast<float>(
            -std::log(2 * 3.14159265358979323846) - 2 * std::log(p[2]));
        return run(m, n, T, seed, scheme, threshold, host_decides, obs_host,
            mean, ess, res, logz);
    }
    return VSMC_CUDA_ERR_ARG;
}
