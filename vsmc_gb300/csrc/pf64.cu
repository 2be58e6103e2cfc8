// FP64 bootstrap filter with the reference's arithmetic step for step: the
// Weight class's normalized doubles and left-to-right sums
// (core/weight.hpp:145-230), the scheme functors with the sequential
// resampling engine (core/particle.hpp:170-197), rep -> index with the
// reference slot layout and the in-place copy, then the Monitor's weighted
// mean (core/monitor.hpp:242-268).  Only libm (exp / log / sincos / log1p)
// differs from the reference, so a run tracks the oracle closely.  The step
// reads the ESS back to decide on resampling, as Particle::resample does.
#include "pf_internal.cuh"
#include "pf_model.cuh"
#include "resample_internal.cuh"
#include "seqsum.cuh"

#include <cmath>
#include <new>

namespace vsmc_cuda
{

struct Pf64State {
    double *ll = nullptr;   // log-likelihoods of the step
    int *rep = nullptr;
    int *idx = nullptr;
    double *scal = nullptr; // [0] ess, [1] logz, [2] evidence max, [3] sum
    double *part = nullptr; // reduction partials
    vsmc_cuda_rng reng = {};
    double logz = 0;
};

namespace
{

constexpr int kB = 256;

__global__ void __launch_bounds__(256) k_move64(uint32_t n, uint32_t ld,
    uint32_t t, uint32_t seed, CvConst<double> c, const double *obs,
    double *s, double *ll)
{
    const double ox = obs[2 * t + 0], oy = obs[2 * t + 1];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        const u32x4 w = particle_block(t, seed, i);
        double X, Y, VX, VY;
        if (t == 0) {
            double z1, z2, z3, z4;
            normal_pair_d(w.x, w.y, z1, z2);
            normal_pair_d(w.z, w.w, z3, z4);
            X = __dmul_rn(c.sd_pos0, z1);
            Y = __dmul_rn(c.sd_pos0, z2);
            VX = __dmul_rn(c.sd_vel0, z3);
            VY = __dmul_rn(c.sd_vel0, z4);
        } else {
            X = s[i];
            Y = s[ld + i];
            VX = s[2 * ld + i];
            VY = s[3 * ld + i];
            double z1, z2;
            normal_pair_d(w.x, w.y, z1, z2);
            cv_move(c, __dmul_rn(c.sigma_a, z1), __dmul_rn(c.sigma_a, z2), X,
                Y, VX, VY);
        }
        s[i] = X;
        s[ld + i] = Y;
        s[2 * ld + i] = VX;
        s[3 * ld + i] = VY;
        ll[i] = cv_loglik(c, ox, oy, X, Y);
    }
}

struct OpMaxD {
    __device__ double operator()(double a, double b) const
    {
        return a < b ? b : a;
    }
};

// evidence increment log sum_i W_i exp(ll_i - m) + m (W == null: 1/N each)
__global__ void __launch_bounds__(256) k_ev_max(uint32_t n, const double *ll,
    double *part)
{
    double m = -INFINITY;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x)
        m = fmax(m, ll[i]);
    __shared__ double sh[kB / 32 + 1];
    m = block_reduce(m, OpMaxD(), -static_cast<double>(INFINITY), sh);
    if (threadIdx.x == 0)
        part[blockIdx.x] = m;
}

__global__ void __launch_bounds__(256) k_ev_sum(uint32_t n, const double *ll,
    const double *W, const double *part, int nb, double *part2)
{
    __shared__ double sh[kB / 32 + 1];
    double m = -INFINITY;
    for (int b = 0; b < nb; ++b)
        m = fmax(m, part[b]);
    double s = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x)
        s += (W ? W[i] : 1.0) * exp(ll[i] - m);
    s = block_reduce(s, OpAdd(), 0.0, sh);
    if (threadIdx.x == 0)
        part2[blockIdx.x] = s;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        part2[nb] = m;
}

__global__ void k_ev_final(int nb, uint32_t n, bool first,
    const double *part2, double *scal, double *h_logz, uint32_t t,
    const double *ess, double *h_ess)
{
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    double s = 0;
    for (int b = 0; b < nb; ++b)
        s += part2[b];
    if (first)
        s /= static_cast<double>(n);
    scal[1] += part2[nb] + log(s);
    h_logz[t] = scal[1];
    (void)ess;
    (void)h_ess;
}

__global__ void k_copy1(const double *src, double *dst)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        *dst = *src;
}

__global__ void k_set_int(int *p, int v)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        *p = v;
}

__global__ void k_zero_d(double *p)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        *p = 0.0;
}

} // namespace

int pf64_create(vsmc_cuda_pf *pf)
{
    Pf64State *p = new (std::nothrow) Pf64State;
    if (p == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    pf->p64 = p;
    const size_t n = pf->n;
    const int nb = grid_for(n, kB, 4, 8);
    if (cudaMalloc(&p->ll, sizeof(double) * n) != cudaSuccess ||
        cudaMalloc(&p->rep, sizeof(int) * n) != cudaSuccess ||
        cudaMalloc(&p->idx, sizeof(int) * n) != cudaSuccess ||
        cudaMalloc(&p->scal, sizeof(double) * 8) != cudaSuccess ||
        cudaMalloc(&p->part, sizeof(double) * (2 * nb + 8)) != cudaSuccess)
        return VSMC_CUDA_ERR_ALLOC;
    return VSMC_CUDA_OK;
}

void pf64_destroy(vsmc_cuda_pf *pf)
{
    Pf64State *p = pf->p64;
    if (p == nullptr)
        return;
    cudaFree(p->ll);
    cudaFree(p->rep);
    cudaFree(p->idx);
    cudaFree(p->scal);
    cudaFree(p->part);
    delete p;
    pf->p64 = nullptr;
}

int pf64_step(vsmc_cuda_pf *pf, bool first)
{
    Pf64State *p = pf->p64;
    cudaStream_t st = pf->stream;
    const size_t n = pf->n;
    const uint32_t t = static_cast<uint32_t>(pf->t);
    double *W = static_cast<double *>(pf->weight);
    double *S = static_cast<double *>(pf->state);
    Scratch scratch(st);
    uint32_t *err = scratch.get<uint32_t>(1);
    if (err == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    VSMC_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(uint32_t), st));
    if (first) {
        // Sampler::initialize: resampling engine key {0, seed}, counter
        // {0, 0, 1, 0}; log-evidence 0
        vsmc_cuda_rng_init(&p->reng, VSMC_CUDA_PHILOX4X32, 0);
        const uint64_t key[2] = {0, pf->seed};
        vsmc_cuda_rng_set_key(&p->reng, 2, key);
        const uint64_t ctr[4] = {0, 0, 1, 0};
        vsmc_cuda_rng_set_ctr(&p->reng, 4, ctr);
        k_zero_d<<<1, 1, 0, st>>>(p->scal + 1);
    }
    const CvConst<double> c = make_cv_const<double>(pf->model);
    const int grid = grid_for(n, kB, 1, 8);
    k_move64<<<grid, kB, 0, st>>>(static_cast<uint32_t>(n),
        static_cast<uint32_t>(pf->stride), t, pf->seed, c, pf->obs, S, p->ll);
    VSMC_CUDA_CHECK_LAUNCH();
    // evidence increment from the weights before they are updated
    const int nb = grid_for(n, kB, 4, 8);
    k_ev_max<<<nb, kB, 0, st>>>(static_cast<uint32_t>(n), p->ll, p->part);
    k_ev_sum<<<nb, kB, 0, st>>>(static_cast<uint32_t>(n), p->ll,
        first ? nullptr : W, p->part, nb, p->part + nb);
    k_ev_final<<<1, 32, 0, st>>>(nb, static_cast<uint32_t>(n), first,
        p->part + nb, p->scal, pf->h_logz, t, nullptr, nullptr);
    VSMC_CUDA_CHECK_LAUNCH();
    int rc;
    if (first) {
        VSMC_CUDA_TRY(cudaMemcpyAsync(W, p->ll, sizeof(double) * n,
            cudaMemcpyDeviceToDevice, st));
        rc = weight_post_set_log_device(n, W, p->scal, err, scratch, st);
    } else {
        rc = weight_add_log_device(n, p->ll, W, p->scal, err, scratch, st);
    }
    if (rc != VSMC_CUDA_OK)
        return rc;
    k_copy1<<<1, 1, 0, st>>>(p->scal, pf->h_ess + t);
    VSMC_CUDA_CHECK_LAUNCH();
    double ess = 0;
    VSMC_CUDA_TRY(cudaMemcpyAsync(
        &ess, p->scal, sizeof(double), cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    const bool resample = ess < pf->threshold * static_cast<double>(n);
    if (resample) {
        rc = scheme_device(n, n, &p->reng, W, p->rep, pf->scheme, scratch, st);
        if (rc != VSMC_CUDA_OK)
            return rc;
        rc = rep_index_device(n, n, p->rep, p->idx, err, scratch, st);
        if (rc != VSMC_CUDA_OK)
            return rc;
        rc = state_copy_device<double>(n, 4, pf->stride, p->idx, S, err, st);
        if (rc != VSMC_CUDA_OK)
            return rc;
        rc = weight_set_equal_device(n, W, p->scal, err, scratch, st);
        if (rc != VSMC_CUDA_OK)
            return rc;
    }
    k_set_int<<<1, 1, 0, st>>>(pf->h_res + t, resample ? 1 : 0);
    VSMC_CUDA_CHECK_LAUNCH();
    rc = monitor_mean_device<double>(
        n, 2, pf->stride, S, W, pf->h_mean + 2 * t, scratch, st);
    if (rc != VSMC_CUDA_OK)
        return rc;
    int status = VSMC_CUDA_OK;
    rc = read_err(err, st, &status);
    return rc != VSMC_CUDA_OK ? rc : status;
}

int pf64_final_mean(vsmc_cuda_pf *) { return VSMC_CUDA_OK; }

} // namespace vsmc_cuda
