// Particle-filter driver and the model entry points of the C ABI.
//
// The filter is the reference's Sampler<T> loop (core/sampler.hpp:443-476,
// 735-785) for the bootstrap filter of the pf example: weight by the
// observation, record ESS, resample when ESS < threshold * N
// (core/particle.hpp:170-197), record the weighted position mean
// (core/monitor.hpp:242-268) and the log-evidence increment
// log sum_i W_{t-1,i} exp(l_{t,i}) (user_guide/tex/smc.tex:176-182).
#include "pf_internal.cuh"
#include "pf32.cuh"

#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

using namespace vsmc_cuda;

namespace vsmc_cuda
{

static float *buf32(vsmc_cuda_pf *pf, int which)
{
    return static_cast<float *>(which == 0 ? pf->state : pf->state2);
}

// Descriptor of the next step: it reads buffer cur and writes the other.
static void step_desc(vsmc_cuda_pf *pf, vsmc_cuda_pf_step_desc *d)
{
    *d = vsmc_cuda_pf_step_desc{};
    d->state_in = buf32(pf, pf->cur);
    d->state_out = buf32(pf, 1 - pf->cur);
    d->log_weight = static_cast<float *>(pf->weight);
    d->index = pf->idx;
    d->sources = pf->empties;
    d->partials = pf->part;
    d->scalars = pf->sc;
    d->hist_mean = pf->h_mean;
    d->hist_ess = pf->h_ess;
    d->hist_logz = pf->h_logz;
    d->hist_resampled = pf->h_res;
    d->n = pf->n;
    d->stride = pf->stride;
    d->dim = pf->dim;
    d->monitor_dim = pf->mon_dim;
    d->max_steps = pf->max_steps;
    d->max_grid = pf->max_grid;
    d->step = pf->t;
    d->seed = pf->seed;
    d->threshold = pf->threshold;
    d->stream = pf->stream;
}

// Kernel arguments of the library's per-step kernels (genealogy record,
// resample-move, materialize) with explicit input and output buffers.
static PfStepArgs step_args(vsmc_cuda_pf *pf, const float *in, float *out)
{
    PfStepArgs a = {};
    a.in = in;
    a.out = out;
    a.lw = static_cast<float *>(pf->weight);
    a.idx = pf->idx;
    a.srcs = pf->empties;
    a.part = pf->part;
    a.sc = pf->sc;
    a.h_mean = pf->h_mean;
    a.h_ess = pf->h_ess;
    a.h_logz = pf->h_logz;
    a.h_res = pf->h_res;
    a.stride = pf->stride;
    a.n = static_cast<uint32_t>(pf->n);
    a.seed = pf->seed;
    a.max_steps = static_cast<uint32_t>(pf->max_steps);
    a.threshold = pf->threshold;
    return a;
}

static CvModel cv_model(vsmc_cuda_pf *pf)
{
    CvModel m;
    m.c = make_cv_const<float>(pf->model);
    m.obs = pf->obs;
    m.max_steps = static_cast<uint32_t>(pf->max_steps);
    return m;
}

// Resampling arguments; mon_state is the state the resample draws from
// (the last step's output), whose resampled mean becomes the monitor.
static Rs32Args make_rs_args32(
    vsmc_cuda_pf *pf, const float *mon_state, int force, bool with_mon)
{
    Rs32Args r = {};
    r.lw = static_cast<const float *>(pf->weight);
    r.q = nullptr; // the log-weights are the input
    r.n = static_cast<uint32_t>(pf->n);
    r.shift = pf->shift;
    r.chunk = pf->chunk_rs;
    r.scheme = pf->scheme;
    r.force = force;
    r.qpart = pf->qpart;
    r.epart = pf->epart;
    r.cpart = pf->cpart;
    r.rep = pf->rep;
    r.idx = pf->idx;
    r.srcs = pf->empties;
    r.sc = pf->sc;
    r.mon_state = mon_state;
    r.stride = pf->stride;
    r.mon_dim = with_mon ? static_cast<uint32_t>(pf->mon_dim) : 0u;
    r.max_steps = static_cast<uint32_t>(pf->max_steps);
    r.mon_part = pf->part;
    r.h_mean = pf->h_mean;
    r.h_res = pf->h_res;
    return r;
}

// The resampling passes.  with_mon: the assign pass also records the mean
// of the resampled particles (for a host that reads the monitor right after
// resampling); the filter's own runs leave it to the next step's kernel.
static void launch_resample32(
    vsmc_cuda_pf *pf, const float *mon_state, int force, bool with_mon)
{
    const Rs32Args r = make_rs_args32(pf, mon_state, force, with_mon);
    cudaStream_t st = pf->stream;
    k_rs32_qsum<<<pf->grid_rs, kPfBlock, 0, st>>>(r);
    launch_rs32_count(pf->grid_rs, st, r);
    launch_rs32_assign(pf->grid_rs, st, r);
}

// the fused step kernel of the built-in model (reads buffer cur, writes the
// other)
static int launch_step_kernel32(vsmc_cuda_pf *pf, bool first)
{
    vsmc_cuda_pf_step_desc d;
    step_desc(pf, &d);
    d.step = first ? 0 : (pf->t > 0 ? pf->t : 1);
    // the previous step's post-resample mean from this step's input (a
    // resample-move sweep records its own)
    d.record_previous_mean = pf->mcmc_sweeps == 0 ? 1 : 0;
    const int rc = pf_step_launch(d, cv_model(pf));
    if (rc == VSMC_CUDA_ERR_CUDA)
        set_last_cuda_error(cudaGetLastError());
    return rc;
}

// the kernels that follow resampling every step: genealogy row, and the
// resample-move sweeps (whose output goes back to buffer cur)
static void launch_post32(vsmc_cuda_pf *pf)
{
    const PfStepArgs a =
        step_args(pf, buf32(pf, 1 - pf->cur), buf32(pf, pf->cur));
    if (pf->record_gen)
        k_pf32_record<<<grid_for(pf->n, kPfBlock, 4, 8), kPfBlock, 0,
            pf->stream>>>(a, pf->gen);
    if (pf->mcmc_sweeps > 0) {
        const float sa = static_cast<float>(pf->model.sigma_a);
        k_pf32_mcmc<<<grid_for(pf->n, kPfBlock, 1, 8), kPfBlock, 0,
            pf->stream>>>(a, make_cv_const<float>(pf->model), pf->obs,
            pf->mcmc_sweeps, pf->mcmc_scale, 1.0f / (sa * sa), pf->h_acc);
        k_pf32_clear_gather<<<1, 1, 0, pf->stream>>>(pf->sc);
    }
}

// the kernels of one FP32 step of the built-in model, launched on the
// stream
static int launch_step32(vsmc_cuda_pf *pf, bool first)
{
    const int rc = launch_step_kernel32(pf, first);
    if (rc != VSMC_CUDA_OK)
        return rc;
    // the filter's own runs take a resampled step's monitor from the next
    // step (resample-move sweeps replace it from t = 1; the assign pass
    // covers a resampled t = 0 then)
    launch_resample32(pf, buf32(pf, 1 - pf->cur), 0, pf->mcmc_sweeps > 0);
    launch_post32(pf);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

// the buffer holding the state after a step
static void advance_buffer(vsmc_cuda_pf *pf)
{
    if (pf->mcmc_sweeps == 0)
        pf->cur = 1 - pf->cur;
}

static int launch_first32(vsmc_cuda_pf *pf)
{
    const int rc = launch_step32(pf, true);
    if (rc == VSMC_CUDA_OK)
        advance_buffer(pf);
    return rc;
}

static int step32(vsmc_cuda_pf *pf)
{
    if (!pf->use_graph) {
        const int rc = launch_step32(pf, false);
        if (rc == VSMC_CUDA_OK)
            advance_buffer(pf);
        return rc;
    }
    const int par = pf->cur;
    if (pf->graph_exec[par] == nullptr) {
        VSMC_CUDA_TRY(cudaStreamBeginCapture(
            pf->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = launch_step32(pf, false);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(pf->stream, &g);
        if (rc != VSMC_CUDA_OK) {
            if (g)
                cudaGraphDestroy(g);
            return rc;
        }
        VSMC_CUDA_TRY(e);
        pf->graph[par] = g;
        VSMC_CUDA_TRY(cudaGraphInstantiate(&pf->graph_exec[par], g, 0));
    }
    VSMC_CUDA_TRY(cudaGraphLaunch(pf->graph_exec[par], pf->stream));
    advance_buffer(pf);
    return VSMC_CUDA_OK;
}

// apply a pending resampling gather to the stored state (host-side views)
static int materialize32(vsmc_cuda_pf *pf)
{
    int32_t gather = 0;
    VSMC_CUDA_TRY(cudaMemcpyAsync(&gather, &pf->sc->gather, sizeof(gather),
        cudaMemcpyDeviceToHost, pf->stream));
    VSMC_CUDA_TRY(cudaStreamSynchronize(pf->stream));
    if (!gather)
        return VSMC_CUDA_OK;
    const PfStepArgs a =
        step_args(pf, buf32(pf, pf->cur), buf32(pf, 1 - pf->cur));
    k_pf32_materialize<<<grid_for(pf->n, kPfBlock, 4, 8), kPfBlock, 0,
        pf->stream>>>(a, static_cast<uint32_t>(pf->dim));
    k_pf32_clear_gather<<<1, 1, 0, pf->stream>>>(pf->sc);
    VSMC_CUDA_CHECK_LAUNCH();
    pf->cur = 1 - pf->cur;
    return VSMC_CUDA_OK;
}

__global__ void k_reset_scalars(PfScalars *sc, uint32_t seed)
{
    PfScalars z = {};
    z.resampled = 1;
    z.rindex = 4;
    // resampling engine: key {0, seed}, counter {0, 0, 1, 0}
    z.rkey[0] = 0;
    z.rkey[1] = seed;
    z.rctr[0] = 0;
    z.rctr[1] = 0;
    z.rctr[2] = 1;
    z.rctr[3] = 0;
    *sc = z;
}

static int reset_scalars(vsmc_cuda_pf *pf)
{
    k_reset_scalars<<<1, 1, 0, pf->stream>>>(pf->sc, pf->seed);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

// The scalars copied into the pinned host copy by the GPU itself (32-bit
// words; the host copy is mapped): a kernel node behind the step's kernels
// instead of a copy-engine transfer.
__global__ void k_pf32_status_out(const PfScalars *sc, PfScalars *host)
{
    static_assert(sizeof(PfScalars) % 4 == 0, "whole words");
    const uint32_t *s = reinterpret_cast<const uint32_t *>(sc);
    uint32_t *d = reinterpret_cast<uint32_t *>(host);
    for (uint32_t i = threadIdx.x; i < sizeof(PfScalars) / 4; i += blockDim.x)
        d[i] = s[i];
}

// Weight::set_equal: every weight equal, the stored log-weights stale
__global__ void k_pf32_set_equal(PfScalars *sc, uint32_t n)
{
    sc->resampled = 1;
    sc->M = 0;
    sc->Mf = 0;
    sc->S = static_cast<double>(n);
    sc->ess = static_cast<double>(n);
}

// Equal weights written out (lw = 0, max 0), for a resample the host asks
// for while the weights are equal; the state keeps any pending gather.
__global__ void __launch_bounds__(kPfBlock) k_pf32_lw_zero(
    float *lw, uint32_t n, PfScalars *sc)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x)
        lw[i] = 0.0f;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc->resampled = 0;
        sc->M = 0;
        sc->Mf = 0;
        sc->S = static_cast<double>(n);
        sc->ess = static_cast<double>(n);
    }
}

// Weight::set_log / add_log from n doubles (v): lw = v (+ the current
// lw - M unless the weights are equal), then the step kernel's reduction:
// (max, sum exp, sum exp^2) and the monitor's weighted sums over the
// current particles (read through a pending gather); the last block sets
// M, S, ESS, the monitor mean and, for add, the log-evidence increment.
__global__ void __launch_bounds__(kPfBlock) k_pf32_weight_log(
    const PfStepArgs a, const double *v, int add, uint32_t mon_dim)
{
    const bool equal = a.sc->resampled != 0;
    const bool gather = a.sc->gather != 0;
    const float Mprev = static_cast<float>(a.sc->M);
    LseMon<kMaxMonitorDim> acc = lse_empty<kMaxMonitorDim>();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
         i += gridDim.x * blockDim.x) {
        float l = static_cast<float>(v[i]);
        if (add && !equal)
            l += a.lw[i] - Mprev;
        a.lw[i] = l;
        uint32_t src = gather ? pf_source(a.srcs, a.idx[i]) : i;
        if (src >= a.n) {
            atomicOr(&a.sc->err, DEV_ERR_INTERNAL);
            src = 0;
        }
        float x[kMaxMonitorDim];
#pragma unroll
        for (int d = 0; d < kMaxMonitorDim; ++d)
            x[d] = static_cast<uint32_t>(d) < mon_dim
                ? a.in[d * a.stride + src]
                : 0.0f;
        acc.push(l, x);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        acc.merge(acc.shfl_xor(d));
    constexpr int kW = kPfBlock / 32;
    __shared__ LseMon<kMaxMonitorDim> shw[kW];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        shw[wid] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        LseMon<kMaxMonitorDim> w = shw[0];
        for (int k = 1; k < kW; ++k)
            w.merge(shw[k]);
        PfPartial p;
        p.m = w.m;
        p.s = w.s;
        p.s2 = w.s2;
#pragma unroll
        for (int d = 0; d < kMaxMonitorDim; ++d)
            p.mon[d] = w.mon[d];
        a.part[blockIdx.x] = p;
        __threadfence();
        is_last = atomicAdd(&a.sc->done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last || threadIdx.x != 0)
        return;
    __threadfence();
    double M = -INFINITY;
    for (uint32_t b = 0; b < gridDim.x; ++b)
        M = fmax(M, __ldcg(&a.part[b].m));
    double S = 0, S2 = 0, MON[kMaxMonitorDim] = {};
    for (uint32_t b = 0; b < gridDim.x; ++b) {
        const double pm = __ldcg(&a.part[b].m);
        if (!(pm > -INFINITY))
            continue;
        const double f = exp(pm - M);
        S += __ldcg(&a.part[b].s) * f;
        S2 += __ldcg(&a.part[b].s2) * f * f;
#pragma unroll
        for (int d = 0; d < kMaxMonitorDim; ++d)
            MON[d] += __ldcg(&a.part[b].mon[d]) * f;
    }
    PfScalars &sc = *a.sc;
    if (!(S > 0))
        sc.err |= DEV_ERR_NONFINITE;
    if (add) {
        const double prev_mass = equal ? static_cast<double>(a.n) : sc.S;
        sc.logz += M + log(S) - log(prev_mass);
    }
#pragma unroll
    for (int d = 0; d < kMaxMonitorDim; ++d)
        if (static_cast<uint32_t>(d) < mon_dim)
            sc.mean[d] = MON[d] / S;
    sc.M = M;
    sc.Mf = static_cast<float>(M);
    sc.S = S;
    sc.ess = S * S / S2;
    sc.resampled = 0;
    sc.done = 0;
}

static void free_all(vsmc_cuda_pf *pf)
{
    for (int k = 0; k < 2; ++k) {
        if (pf->graph_exec[k])
            cudaGraphExecDestroy(pf->graph_exec[k]);
        if (pf->graph[k])
            cudaGraphDestroy(pf->graph[k]);
    }
    void *ptrs[] = {pf->h_acc, pf->gen, pf->state, pf->state2, pf->weight,
        pf->obs,
        pf->h_mean,
        pf->h_ess, pf->h_logz, pf->h_res, pf->sc, pf->part, pf->qpart,
        pf->epart, pf->cpart, pf->rep, pf->idx, pf->empties};
    for (void *p : ptrs)
        if (p)
            cudaFree(p);
    if (pf->sc_host)
        cudaFreeHost(pf->sc_host);
    if (pf->p64)
        pf64_destroy(pf);
    if (pf->own_stream && pf->stream)
        cudaStreamDestroy(pf->stream);
    pf->stream = nullptr;
}

template <typename T>
static int dalloc(T **p, size_t count)
{
    void *q = nullptr;
    VSMC_CUDA_TRY(cudaMalloc(&q, sizeof(T) * (count ? count : 1)));
    *p = static_cast<T *>(q);
    return VSMC_CUDA_OK;
}

static int sync_and_check(vsmc_cuda_pf *pf)
{
    VSMC_CUDA_TRY(cudaStreamSynchronize(pf->stream));
    uint32_t err = 0;
    VSMC_CUDA_TRY(cudaMemcpy(&err, &pf->sc->err, sizeof(err),
        cudaMemcpyDeviceToHost));
    if (err & DEV_ERR_NONFINITE)
        return VSMC_CUDA_ERR_NONFINITE;
    if (err)
        return VSMC_CUDA_ERR_INTERNAL;
    return VSMC_CUDA_OK;
}

// Shared constructor of the built-in (model != null) and the user-model
// filters.
static int pf_create(vsmc_cuda_pf **out, size_t n, size_t dim,
    size_t mon_dim, int precision, int scheme, double threshold,
    uint32_t seed, const vsmc_cuda_cv_model *model, size_t max_steps,
    void *stream)
{
    *out = nullptr;
    if (n < 1 || n >= (size_t(1) << 31) || max_steps < 1 ||
        max_steps > (size_t(1) << 31))
        return VSMC_CUDA_ERR_SIZE;
    if (scheme < VSMC_CUDA_MULTINOMIAL || scheme > VSMC_CUDA_RESIDUAL_SYSTEMATIC)
        return VSMC_CUDA_ERR_ARG;
    if (precision == 32 && scheme != VSMC_CUDA_STRATIFIED &&
        scheme != VSMC_CUDA_SYSTEMATIC)
        return VSMC_CUDA_ERR_ARG;
    vsmc_cuda_pf *pf = new (std::nothrow) vsmc_cuda_pf;
    if (pf == nullptr)
        return VSMC_CUDA_ERR_ALLOC;
    pf->n = n;
    pf->stride = (n + 255) / 256 * 256;
    pf->dim = dim;
    pf->mon_dim = mon_dim;
    pf->custom = model == nullptr;
    pf->precision = precision;
    pf->scheme = scheme;
    pf->threshold = threshold;
    pf->seed = seed;
    if (model)
        pf->model = *model;
    pf->max_steps = max_steps;
    pf->stream = as_stream(stream);
    if (pf->stream == nullptr) {
        // the legacy stream cannot be captured into a graph: use a private one
        if (cudaStreamCreateWithFlags(&pf->stream, cudaStreamNonBlocking) !=
            cudaSuccess) {
            delete pf;
            return VSMC_CUDA_ERR_CUDA;
        }
        pf->own_stream = true;
    }
    int rc = VSMC_CUDA_OK;
    const size_t esz = precision == 32 ? sizeof(float) : sizeof(double);
#define PF_TRY(x)                                                             \
    do {                                                                      \
        rc = (x);                                                             \
        if (rc != VSMC_CUDA_OK) {                                             \
            free_all(pf);                                                     \
            delete pf;                                                        \
            return rc;                                                        \
        }                                                                     \
    } while (0)
    PF_TRY(dalloc(reinterpret_cast<char **>(&pf->state),
        esz * dim * pf->stride));
    PF_TRY(dalloc(reinterpret_cast<char **>(&pf->weight), esz * pf->stride));
    if (model)
        PF_TRY(dalloc(&pf->obs, 2 * max_steps));
    PF_TRY(dalloc(&pf->h_mean, (mon_dim ? mon_dim : 1) * max_steps));
    PF_TRY(dalloc(&pf->h_ess, max_steps));
    PF_TRY(dalloc(&pf->h_logz, max_steps));
    PF_TRY(dalloc(&pf->h_res, max_steps));
    PF_TRY(dalloc(&pf->sc, 1));
    if (cudaHostAlloc(reinterpret_cast<void **>(&pf->sc_host),
            sizeof(PfScalars), cudaHostAllocMapped) != cudaSuccess) {
        pf->sc_host = nullptr;
        PF_TRY(VSMC_CUDA_ERR_ALLOC);
    }
    if (cudaHostGetDevicePointer(reinterpret_cast<void **>(&pf->sc_host_dev),
            pf->sc_host, 0) != cudaSuccess)
        PF_TRY(VSMC_CUDA_ERR_CUDA);
    if (precision == 32) {
        if (model) {
            // looked up here, outside any stream capture of a step
            pf_step_occupancy<CvModel, true, PfMon::Previous>();
            pf_step_occupancy<CvModel, false, PfMon::Previous>();
            pf_step_occupancy<CvModel, true, PfMon::Current>();
            pf_step_occupancy<CvModel, false, PfMon::Current>();
        }
        const size_t sms = static_cast<size_t>(num_sms());
        pf->max_grid = sms * 16;
        size_t grs = sms * kRsBlocksPerSm;
        size_t chunk = (n + grs - 1) / grs;
        chunk = (chunk + kPfTile - 1) / kPfTile * kPfTile;
        pf->chunk_rs = static_cast<uint32_t>(chunk);
        pf->grid_rs = static_cast<int>((n + chunk - 1) / chunk);
        int lg = 0;
        while ((size_t(1) << lg) < n)
            ++lg;
        pf->shift = static_cast<uint32_t>(63 - lg);
        PF_TRY(dalloc(&pf->part, pf->max_grid));
        PF_TRY(dalloc(&pf->qpart, pf->grid_rs * (kRsWarps + 1)));
        PF_TRY(dalloc(&pf->epart, pf->grid_rs * (kRsWarps + 1)));
        PF_TRY(dalloc(&pf->cpart, pf->grid_rs * (kRsWarps + 1)));
        PF_TRY(dalloc(reinterpret_cast<char **>(&pf->state2),
            esz * dim * pf->stride));
        PF_TRY(dalloc(&pf->rep, n + 4));
        PF_TRY(dalloc(&pf->idx, pf->stride));
        PF_TRY(dalloc(&pf->empties, n));
    } else {
        PF_TRY(pf64_create(pf));
    }
    PF_TRY(reset_scalars(pf));
#undef PF_TRY
    *out = pf;
    return VSMC_CUDA_OK;
}

} // namespace vsmc_cuda

extern "C" {

int vsmc_cuda_pf_create(vsmc_cuda_pf **out, size_t n, int precision,
    int scheme, double threshold, uint32_t seed,
    const vsmc_cuda_cv_model *model, size_t max_steps, void *stream)
{
    if (out == nullptr || !valid_cv_model(model) ||
        (precision != 32 && precision != 64) || std::isnan(threshold))
        return VSMC_CUDA_ERR_ARG;
    return pf_create(out, n, 4, 2, precision, scheme, threshold, seed, model,
        max_steps, stream);
}

int vsmc_cuda_pf_create_model(vsmc_cuda_pf **out, size_t n, size_t dim,
    size_t monitor_dim, int scheme, double threshold, uint32_t seed,
    size_t max_steps, void *stream)
{
    if (out == nullptr || std::isnan(threshold) || dim < 1 ||
        dim > static_cast<size_t>(kMaxFilterDim) ||
        monitor_dim > static_cast<size_t>(kMaxMonitorDim) ||
        monitor_dim > dim)
        return VSMC_CUDA_ERR_ARG;
    return pf_create(out, n, dim, monitor_dim, 32, scheme, threshold, seed,
        nullptr, max_steps, stream);
}

int vsmc_cuda_pf_destroy(vsmc_cuda_pf *pf)
{
    if (pf == nullptr)
        return VSMC_CUDA_OK;
    cudaStreamSynchronize(pf->stream);
    free_all(pf);
    delete pf;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_launch_step_kernel(vsmc_cuda_pf *pf)
{
    if (pf == nullptr || pf->precision != 32 || pf->custom || pf->t == 0)
        return VSMC_CUDA_ERR_ARG;
    const int rc = launch_step_kernel32(pf, false);
    if (rc != VSMC_CUDA_OK)
        return rc;
    pf->cur = 1 - pf->cur;
    ++pf->t;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_step_desc_get(vsmc_cuda_pf *pf, vsmc_cuda_pf_step_desc *d)
{
    if (pf == nullptr || d == nullptr || pf->precision != 32)
        return VSMC_CUDA_ERR_ARG;
    if (pf->t >= (size_t(1) << 32) - 1)
        return VSMC_CUDA_ERR_SIZE;
    if (pf->t == 0) {
        const int rc = reset_scalars(pf);
        if (rc != VSMC_CUDA_OK)
            return rc;
    }
    step_desc(pf, d);
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_step_commit(vsmc_cuda_pf *pf)
{
    if (pf == nullptr || pf->precision != 32)
        return VSMC_CUDA_ERR_ARG;
    pf->cur = 1 - pf->cur;
    if (pf->threshold >= 0)
        launch_resample32(pf, buf32(pf, pf->cur), 0, true);
    VSMC_CUDA_CHECK_LAUNCH();
    ++pf->t;
    pf->host_equal = false;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_step_advance(vsmc_cuda_pf *pf)
{
    if (pf == nullptr || pf->precision != 32 || pf->t == 0)
        return VSMC_CUDA_ERR_ARG;
    pf->cur = 1 - pf->cur;
    ++pf->t;
    pf->host_equal = false;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_reset(vsmc_cuda_pf *pf)
{
    if (pf == nullptr || pf->precision != 32 || !pf->custom)
        return VSMC_CUDA_ERR_ARG;
    pf->t = 0;
    pf->host_equal = false;
    return reset_scalars(pf);
}

int vsmc_cuda_pf_resample_now(vsmc_cuda_pf *pf)
{
    if (pf == nullptr || pf->precision != 32 || pf->t == 0)
        return VSMC_CUDA_ERR_ARG;
    if (pf->host_equal) {
        // equal weights: resample on them, not on the stale log-weights
        k_pf32_lw_zero<<<grid_for(pf->n, kPfBlock, 4, 4), kPfBlock, 0,
            pf->stream>>>(static_cast<float *>(pf->weight),
            static_cast<uint32_t>(pf->n), pf->sc);
    }
    launch_resample32(pf, buf32(pf, pf->cur), 1, true);
    VSMC_CUDA_CHECK_LAUNCH();
    pf->host_equal = true;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_set_equal(vsmc_cuda_pf *pf)
{
    if (pf == nullptr || pf->precision != 32)
        return VSMC_CUDA_ERR_ARG;
    if (pf->host_equal)
        return VSMC_CUDA_OK;
    k_pf32_set_equal<<<1, 1, 0, pf->stream>>>(
        pf->sc, static_cast<uint32_t>(pf->n));
    VSMC_CUDA_CHECK_LAUNCH();
    pf->host_equal = true;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_weight_log(vsmc_cuda_pf *pf, const double *lw_dev, int add)
{
    if (pf == nullptr || lw_dev == nullptr || pf->precision != 32)
        return VSMC_CUDA_ERR_ARG;
    const PfStepArgs a =
        step_args(pf, buf32(pf, pf->cur), buf32(pf, 1 - pf->cur));
    int grid = grid_for(pf->n, kPfBlock, 4, 4);
    if (static_cast<size_t>(grid) > pf->max_grid)
        grid = static_cast<int>(pf->max_grid);
    k_pf32_weight_log<<<grid, kPfBlock, 0, pf->stream>>>(
        a, lw_dev, add != 0, static_cast<uint32_t>(pf->mon_dim));
    VSMC_CUDA_CHECK_LAUNCH();
    pf->host_equal = false;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_status_enqueue(vsmc_cuda_pf *pf)
{
    if (pf == nullptr || pf->precision != 32)
        return VSMC_CUDA_ERR_ARG;
    k_pf32_status_out<<<1, 32, 0, pf->stream>>>(pf->sc, pf->sc_host_dev);
    VSMC_CUDA_CHECK_LAUNCH();
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_get_status(vsmc_cuda_pf *pf, vsmc_cuda_pf_status *out)
{
    if (pf == nullptr || out == nullptr || pf->precision != 32)
        return VSMC_CUDA_ERR_ARG;
    const int rc = vsmc_cuda_pf_status_enqueue(pf);
    if (rc != VSMC_CUDA_OK)
        return rc;
    return vsmc_cuda_pf_status_read(pf, out);
}

int vsmc_cuda_pf_status_read(vsmc_cuda_pf *pf, vsmc_cuda_pf_status *out)
{
    if (pf == nullptr || out == nullptr || pf->precision != 32)
        return VSMC_CUDA_ERR_ARG;
    VSMC_CUDA_TRY(cudaStreamSynchronize(pf->stream));
    const PfScalars &sc = *pf->sc_host;
    *out = vsmc_cuda_pf_status{};
    out->ess = sc.ess;
    out->log_evidence = sc.logz;
    out->max_log_weight = sc.M;
    out->sum_weight = sc.S;
    for (size_t d = 0; d < pf->mon_dim; ++d)
        out->mean[d] = sc.mean[d];
    out->step = pf->t;
    out->resampled = sc.resampled;
    out->monitor_dim = static_cast<int>(pf->mon_dim);
    if (sc.err & DEV_ERR_NONFINITE)
        return VSMC_CUDA_ERR_NONFINITE;
    if (sc.err)
        return VSMC_CUDA_ERR_INTERNAL;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_resample_fixed(size_t n, const uint64_t *q, int scheme,
    vsmc_cuda_rng *rng, int *replication, int *index, void *stream)
{
    if (q == nullptr || reinterpret_cast<uintptr_t>(q) % alignof(uint64_t) ||
        rng == nullptr || rng->kind != VSMC_CUDA_PHILOX4X32 ||
        rng->index < 1 || rng->index > 4 ||
        (scheme != VSMC_CUDA_STRATIFIED && scheme != VSMC_CUDA_SYSTEMATIC))
        return VSMC_CUDA_ERR_ARG;
    if (n < 2 || n >= (size_t(1) << 31))
        return VSMC_CUDA_ERR_SIZE;
    cudaStream_t st = as_stream(stream);
    Scratch scratch(st);
    const size_t grs0 = static_cast<size_t>(num_sms()) * kRsBlocksPerSm;
    size_t chunk = (n + grs0 - 1) / grs0;
    chunk = (chunk + kPfTile - 1) / kPfTile * kPfTile;
    const int grid = static_cast<int>((n + chunk - 1) / chunk);
    Rs32Args r = {};
    r.q = q;
    r.n = static_cast<uint32_t>(n);
    r.chunk = static_cast<uint32_t>(chunk);
    r.scheme = scheme;
    r.qpart = scratch.get<uint64_t>(static_cast<size_t>(grid) * (kRsWarps + 1));
    r.epart = scratch.get<uint32_t>(static_cast<size_t>(grid) * (kRsWarps + 1));
    r.cpart = scratch.get<uint32_t>(static_cast<size_t>(grid) * (kRsWarps + 1));
    r.rep = scratch.get<int32_t>(n + 4);
    r.idx = scratch.get<int32_t>(n + 4);
    r.srcs = scratch.get<uint32_t>(n);
    r.sc = scratch.get<PfScalars>(1);
    if (!r.qpart || !r.epart || !r.cpart || !r.rep || !r.idx || !r.srcs ||
        !r.sc)
        return VSMC_CUDA_ERR_ALLOC;
    k_rs32_setup<<<1, 1, 0, st>>>(r.sc, static_cast<uint32_t>(rng->key[0]),
        static_cast<uint32_t>(rng->key[1]), static_cast<uint32_t>(rng->ctr[0]),
        static_cast<uint32_t>(rng->ctr[1]), static_cast<uint32_t>(rng->ctr[2]),
        static_cast<uint32_t>(rng->ctr[3]), rng->index);
    k_rs32_qsum<<<grid, kPfBlock, 0, st>>>(r);
    launch_rs32_count(grid, st, r);
    launch_rs32_assign(grid, st, r);
    VSMC_CUDA_CHECK_LAUNCH();
    if (index)
        k_rs32_decode<<<grid_for(n, kPfBlock, 4, 8), kPfBlock, 0, st>>>(r, index);
    if (replication)
        VSMC_CUDA_TRY(cudaMemcpyAsync(replication, r.rep, sizeof(int) * n,
            cudaMemcpyDeviceToDevice, st));
    VSMC_CUDA_CHECK_LAUNCH();
    PfScalars sc;
    VSMC_CUDA_TRY(cudaMemcpyAsync(
        &sc, r.sc, sizeof(sc), cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    if (sc.err & DEV_ERR_NONFINITE)
        return VSMC_CUDA_ERR_NONFINITE;
    if (sc.err)
        return VSMC_CUDA_ERR_INTERNAL;
    for (int i = 0; i < 4; ++i)
        rng->ctr[i] = sc.rctr[i];
    rng->index = sc.rindex;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_use_graph(vsmc_cuda_pf *pf, int on)
{
    if (pf == nullptr)
        return VSMC_CUDA_ERR_ARG;
    pf->use_graph = on != 0;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_stream(vsmc_cuda_pf *pf, void **stream)
{
    if (pf == nullptr || stream == nullptr)
        return VSMC_CUDA_ERR_ARG;
    *stream = pf->stream;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_state(vsmc_cuda_pf *pf, void **state_dev, void **weight_dev)
{
    if (pf == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (pf->precision == 32) {
        const int rc = materialize32(pf);
        if (rc != VSMC_CUDA_OK)
            return rc;
    }
    if (state_dev)
        *state_dev = pf->precision == 32 ? buf32(pf, pf->cur) : pf->state;
    if (weight_dev)
        *weight_dev = pf->weight;
    return VSMC_CUDA_OK;
}

static int pf_begin(vsmc_cuda_pf *pf)
{
    int rc = reset_scalars(pf);
    if (rc != VSMC_CUDA_OK)
        return rc;
    if (pf->h_acc)
        VSMC_CUDA_TRY(cudaMemsetAsync(pf->h_acc, 0,
            sizeof(uint32_t) * pf->max_steps, pf->stream));
    pf->t = 0;
    pf->mean_pending = false;
    rc = pf->precision == 32 ? launch_first32(pf) : pf64_step(pf, true);
    if (rc != VSMC_CUDA_OK)
        return rc;
    pf->t = 1;
    pf->mean_pending = true;
    return VSMC_CUDA_OK;
}

static int pf_next(vsmc_cuda_pf *pf)
{
    const int rc = pf->precision == 32 ? step32(pf) : pf64_step(pf, false);
    if (rc != VSMC_CUDA_OK)
        return rc;
    ++pf->t;
    pf->mean_pending = true;
    return VSMC_CUDA_OK;
}

// Both filters record step t's monitor inside step t + 1 (from the
// particles that step reads); the last step needs one more kernel.  With
// resample-move sweeps the FP32 steps record their own (and the sweeps
// replace a resampled step's).
static int pf_flush_mean(vsmc_cuda_pf *pf)
{
    if (!pf->mean_pending || pf->t == 0)
        return VSMC_CUDA_OK;
    int rc = VSMC_CUDA_OK;
    if (pf->precision == 32) {
        if (!pf->custom && pf->mcmc_sweeps == 0) {
            const PfStepArgs a =
                step_args(pf, buf32(pf, pf->cur), buf32(pf, 1 - pf->cur));
            int grid = grid_for(pf->n, kPfBlock, 4, 4);
            if (static_cast<size_t>(grid) > pf->max_grid)
                grid = static_cast<int>(pf->max_grid);
            k_pf32_final_mean<<<grid, kPfBlock, 0, pf->stream>>>(
                a, static_cast<uint32_t>(pf->mon_dim));
            VSMC_CUDA_CHECK_LAUNCH();
        }
    } else {
        rc = pf64_final_mean(pf);
    }
    if (rc == VSMC_CUDA_OK)
        pf->mean_pending = false;
    return rc;
}

int vsmc_cuda_pf_initialize(vsmc_cuda_pf *pf, const double *obs_dev)
{
    if (pf == nullptr || obs_dev == nullptr || pf->custom)
        return VSMC_CUDA_ERR_ARG;
    VSMC_CUDA_TRY(cudaMemcpyAsync(pf->obs, obs_dev, 2 * sizeof(double),
        cudaMemcpyDeviceToDevice, pf->stream));
    return pf_begin(pf);
}

int vsmc_cuda_pf_iterate(vsmc_cuda_pf *pf, const double *obs_dev)
{
    if (pf == nullptr || obs_dev == nullptr || pf->custom)
        return VSMC_CUDA_ERR_ARG;
    if (pf->t == 0)
        return VSMC_CUDA_ERR_ARG;
    if (pf->t >= pf->max_steps)
        return VSMC_CUDA_ERR_SIZE;
    VSMC_CUDA_TRY(cudaMemcpyAsync(pf->obs + 2 * pf->t, obs_dev,
        2 * sizeof(double), cudaMemcpyDeviceToDevice, pf->stream));
    return pf_next(pf);
}

int vsmc_cuda_pf_run_device(vsmc_cuda_pf *pf, size_t T, const double *obs_dev)
{
    if (pf == nullptr || obs_dev == nullptr || T == 0 || pf->custom)
        return VSMC_CUDA_ERR_ARG;
    if (T > pf->max_steps)
        return VSMC_CUDA_ERR_SIZE;
    if (obs_dev != pf->obs)
        VSMC_CUDA_TRY(cudaMemcpyAsync(pf->obs, obs_dev, 2 * T * sizeof(double),
            cudaMemcpyDeviceToDevice, pf->stream));
    int rc = pf_begin(pf);
    for (size_t t = 1; rc == VSMC_CUDA_OK && t < T; ++t)
        rc = pf_next(pf);
    if (rc == VSMC_CUDA_OK)
        rc = pf_flush_mean(pf);
    return rc;
}

int vsmc_cuda_pf_history(vsmc_cuda_pf *pf, size_t T, double *mean_host,
    double *ess_host, int *resampled_host, double *logz_host)
{
    if (pf == nullptr)
        return VSMC_CUDA_ERR_ARG;
    if (T > pf->t || T > pf->max_steps)
        return VSMC_CUDA_ERR_SIZE;
    int rc = pf_flush_mean(pf);
    if (rc != VSMC_CUDA_OK)
        return rc;
    cudaStream_t st = pf->stream;
    if (mean_host && pf->mon_dim > 0)
        VSMC_CUDA_TRY(cudaMemcpyAsync(mean_host, pf->h_mean,
            pf->mon_dim * T * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (ess_host)
        VSMC_CUDA_TRY(cudaMemcpyAsync(ess_host, pf->h_ess, T * sizeof(double),
            cudaMemcpyDeviceToHost, st));
    if (resampled_host)
        VSMC_CUDA_TRY(cudaMemcpyAsync(resampled_host, pf->h_res,
            T * sizeof(int), cudaMemcpyDeviceToHost, st));
    if (logz_host)
        VSMC_CUDA_TRY(cudaMemcpyAsync(logz_host, pf->h_logz,
            T * sizeof(double), cudaMemcpyDeviceToHost, st));
    return sync_and_check(pf);
}

static void drop_graphs(vsmc_cuda_pf *pf)
{
    for (int k = 0; k < 2; ++k) {
        if (pf->graph_exec[k])
            cudaGraphExecDestroy(pf->graph_exec[k]);
        if (pf->graph[k])
            cudaGraphDestroy(pf->graph[k]);
        pf->graph_exec[k] = nullptr;
        pf->graph[k] = nullptr;
    }
}

int vsmc_cuda_pf_record_genealogy(vsmc_cuda_pf *pf, int on)
{
    if (pf == nullptr || pf->precision != 32 || pf->custom)
        return VSMC_CUDA_ERR_ARG;
    if (on && pf->gen == nullptr) {
        void *p = nullptr;
        VSMC_CUDA_TRY(cudaMalloc(&p, sizeof(int32_t) * pf->n * pf->max_steps));
        pf->gen = static_cast<int32_t *>(p);
    }
    if ((on != 0) != pf->record_gen)
        drop_graphs(pf); // captured with or without the record kernel
    pf->record_gen = on != 0;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_set_mcmc(vsmc_cuda_pf *pf, size_t sweeps, double scale)
{
    if (pf == nullptr || pf->precision != 32 || pf->custom || !(scale >= 0) ||
        !(pf->model.sigma_a > 0) || pf->t != 0)
        return VSMC_CUDA_ERR_ARG;
    if (sweeps > 1024)
        return VSMC_CUDA_ERR_SIZE;
    if (sweeps > 0 && pf->h_acc == nullptr) {
        void *p = nullptr;
        VSMC_CUDA_TRY(cudaMalloc(&p, sizeof(uint32_t) * pf->max_steps));
        pf->h_acc = static_cast<uint32_t *>(p);
        VSMC_CUDA_TRY(cudaMemset(pf->h_acc, 0, sizeof(uint32_t) * pf->max_steps));
    }
    if (static_cast<uint32_t>(sweeps) != pf->mcmc_sweeps)
        drop_graphs(pf);
    pf->mcmc_sweeps = static_cast<uint32_t>(sweeps);
    pf->mcmc_scale = static_cast<float>(scale);
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_mcmc_accepts(vsmc_cuda_pf *pf, size_t T, uint32_t *host)
{
    if (pf == nullptr || host == nullptr || pf->h_acc == nullptr ||
        T > pf->max_steps)
        return VSMC_CUDA_ERR_ARG;
    VSMC_CUDA_TRY(cudaMemcpyAsync(host, pf->h_acc, sizeof(uint32_t) * T,
        cudaMemcpyDeviceToHost, pf->stream));
    VSMC_CUDA_TRY(cudaStreamSynchronize(pf->stream));
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_genealogy(vsmc_cuda_pf *pf, const int **rows_dev)
{
    if (pf == nullptr || rows_dev == nullptr || pf->gen == nullptr)
        return VSMC_CUDA_ERR_ARG;
    *rows_dev = pf->gen;
    return VSMC_CUDA_OK;
}

int vsmc_cuda_pf_print(vsmc_cuda_pf *pf, size_t T, char sep, char *buf,
    size_t cap, size_t *len)
{
    if (pf == nullptr || len == nullptr || T > pf->max_steps)
        return VSMC_CUDA_ERR_ARG;
    const size_t md = pf->mon_dim;
    std::vector<double> mean(md * T + 1), ess(T), logz(T);
    std::vector<int> res(T);
    if (T > 0) {
        const int rc = vsmc_cuda_pf_history(
            pf, T, mean.data(), ess.data(), res.data(), logz.data());
        if (rc != VSMC_CUDA_OK)
            return rc;
    }
    if (pf->mcmc_sweeps == 0)
        return vsmc_cuda_sampler_print(T, pf->n, res.data(), ess.data(), md,
            "pos", mean.data(), 0, nullptr, sep, buf, cap, len);
    // the move accepts every particle; the MCMC column is the accept count
    std::vector<uint32_t> acc(T);
    VSMC_CUDA_TRY(cudaMemcpyAsync(acc.data(), pf->h_acc,
        sizeof(uint32_t) * T, cudaMemcpyDeviceToHost, pf->stream));
    VSMC_CUDA_TRY(cudaStreamSynchronize(pf->stream));
    std::vector<size_t> a2(2 * T);
    for (size_t t = 0; t < T; ++t) {
        a2[2 * t] = pf->n;
        a2[2 * t + 1] = acc[t];
    }
    return vsmc_cuda_sampler_print(T, pf->n, res.data(), ess.data(), 2, "pos",
        mean.data(), 2, a2.data(), sep, buf, cap, len);
}

int vsmc_cuda_pf_run(vsmc_cuda_pf *pf, size_t T, const double *obs_host,
    double *mean_host, double *ess_host, int *resampled_host,
    double *logz_host)
{
    if (pf == nullptr || obs_host == nullptr || T == 0 || pf->custom)
        return VSMC_CUDA_ERR_ARG;
    if (T > pf->max_steps)
        return VSMC_CUDA_ERR_SIZE;
    VSMC_CUDA_TRY(cudaMemcpyAsync(pf->obs, obs_host, 2 * T * sizeof(double),
        cudaMemcpyHostToDevice, pf->stream));
    int rc = vsmc_cuda_pf_run_device(pf, T, pf->obs);
    if (rc != VSMC_CUDA_OK)
        return rc;
    return vsmc_cuda_pf_history(
        pf, T, mean_host, ess_host, resampled_host, logz_host);
}

} // extern "C"

// ------------------------------------------------------------------------
// Integer-CDF resampling that allocates nothing.
//
// vsmc_cuda_resample_fixed takes its scratch (partial sums, replication
// counts, slot indices, empty-slot sources, engine scalars) from
// cudaMallocAsync on every call.  Some callers cannot allocate at call time:
// code that runs inside a memory-pool or allocator callback (allocating
// there re-enters the allocator), loops that have reserved all device memory
// up front or must keep allocator calls out of a latency budget, and hosts
// whose allocator is locked while they run.  The variant below takes the same
// scratch from one fixed array in the library's device image instead.
//
// Limits and rules for its users:
//   * n <= VSMC_CUDA_RESAMPLE_FIXED_NOALLOC_MAX_N (2^18 particles); larger n
//     is rejected with VSMC_CUDA_ERR_SIZE before any device work.  The array
//     is about 3 MiB, present on every device the library is loaded on.
//   * The first call on each device (with that device current) looks up the
//     array's address with cudaGetSymbolAddress, which may load the
//     library's device code; make that first call before any stream capture.
//   * The array is shared by all callers on a device: two calls whose work
//     overlaps in time race on it and give wrong results.  Callers serialize
//     on the host, one call at a time per device.  Each call synchronizes
//     its stream before returning, so one host thread calling in turn is
//     safe; several host threads need a lock of their own even on one
//     stream, since a call queues several launches.
//   * The address is looked up once per device and kept for the life of the
//     process; a device reset between calls is not supported.
//   * Nothing in the array needs clearing: every piece a call reads was
//     written earlier in the same call.
namespace vsmc_cuda
{

constexpr size_t kNoAllocMaxN = VSMC_CUDA_RESAMPLE_FIXED_NOALLOC_MAX_N;
// chunk >= kPfTile particles per block, so at most this many blocks
constexpr size_t kNoAllocMaxBlocks = (kNoAllocMaxN + kPfTile - 1) / kPfTile;

constexpr size_t na_align(size_t b) { return (b + 255) / 256 * 256; }

// byte offsets of the pieces inside the array, each on a 256-byte boundary
constexpr size_t kNaSc = 0;
constexpr size_t kNaQpart = kNaSc + na_align(sizeof(PfScalars));
constexpr size_t kNaEpart =
    kNaQpart + na_align(sizeof(uint64_t) * kNoAllocMaxBlocks * (kRsWarps + 1));
constexpr size_t kNaCpart =
    kNaEpart + na_align(sizeof(uint32_t) * kNoAllocMaxBlocks * (kRsWarps + 1));
constexpr size_t kNaRep =
    kNaCpart + na_align(sizeof(uint32_t) * kNoAllocMaxBlocks * (kRsWarps + 1));
constexpr size_t kNaIdx = kNaRep + na_align(sizeof(int32_t) * (kNoAllocMaxN + 4));
constexpr size_t kNaSrcs =
    kNaIdx + na_align(sizeof(int32_t) * (kNoAllocMaxN + 4));
constexpr size_t kNaBytes = kNaSrcs + na_align(sizeof(uint32_t) * kNoAllocMaxN);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

constexpr int kNaMaxDevices = 64;
static std::mutex g_noalloc_mutex;
static unsigned char *g_noalloc_ptr[kNaMaxDevices] = {};

// Address of the array on the current device (looked up once per device).
static int noalloc_scratch(unsigned char **out)
{
    int dev = -1;
    VSMC_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNaMaxDevices)
        return VSMC_CUDA_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (g_noalloc_ptr[dev] == nullptr) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_last_cuda_error(e);
            return VSMC_CUDA_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return VSMC_CUDA_OK;
}

} // namespace vsmc_cuda

extern "C" int vsmc_cuda_resample_fixed_noalloc(size_t n, const uint64_t *q,
    int scheme, vsmc_cuda_rng *rng, int *replication, int *index,
    void *stream)
{
    if (q == nullptr || reinterpret_cast<uintptr_t>(q) % alignof(uint64_t) ||
        rng == nullptr || rng->kind != VSMC_CUDA_PHILOX4X32 ||
        rng->index < 1 || rng->index > 4 ||
        (scheme != VSMC_CUDA_STRATIFIED && scheme != VSMC_CUDA_SYSTEMATIC))
        return VSMC_CUDA_ERR_ARG;
    if (n < 2 || n > kNoAllocMaxN)
        return VSMC_CUDA_ERR_SIZE;
    unsigned char *base = nullptr;
    const int rc = noalloc_scratch(&base);
    if (rc != VSMC_CUDA_OK)
        return rc;
    cudaStream_t st = as_stream(stream);
    const size_t grs0 = static_cast<size_t>(num_sms()) * kRsBlocksPerSm;
    size_t chunk = (n + grs0 - 1) / grs0;
    chunk = (chunk + kPfTile - 1) / kPfTile * kPfTile;
    const size_t grid = (n + chunk - 1) / chunk;
    if (grid > kNoAllocMaxBlocks)
        return VSMC_CUDA_ERR_INTERNAL;
    Rs32Args r = {};
    r.q = q;
    r.n = static_cast<uint32_t>(n);
    r.chunk = static_cast<uint32_t>(chunk);
    r.scheme = scheme;
    r.sc = reinterpret_cast<PfScalars *>(base + kNaSc);
    r.qpart = reinterpret_cast<uint64_t *>(base + kNaQpart);
    r.epart = reinterpret_cast<uint32_t *>(base + kNaEpart);
    r.cpart = reinterpret_cast<uint32_t *>(base + kNaCpart);
    r.rep = reinterpret_cast<int32_t *>(base + kNaRep);
    r.idx = reinterpret_cast<int32_t *>(base + kNaIdx);
    r.srcs = reinterpret_cast<uint32_t *>(base + kNaSrcs);
    k_rs32_setup<<<1, 1, 0, st>>>(r.sc, static_cast<uint32_t>(rng->key[0]),
        static_cast<uint32_t>(rng->key[1]), static_cast<uint32_t>(rng->ctr[0]),
        static_cast<uint32_t>(rng->ctr[1]), static_cast<uint32_t>(rng->ctr[2]),
        static_cast<uint32_t>(rng->ctr[3]), rng->index);
    const int g = static_cast<int>(grid);
    k_rs32_qsum<<<g, kPfBlock, 0, st>>>(r);
    launch_rs32_count(g, st, r);
    launch_rs32_assign(g, st, r);
    VSMC_CUDA_CHECK_LAUNCH();
    if (index)
        k_rs32_decode<<<grid_for(n, kPfBlock, 4, 8), kPfBlock, 0, st>>>(
            r, index);
    if (replication)
        VSMC_CUDA_TRY(cudaMemcpyAsync(replication, r.rep, sizeof(int) * n,
            cudaMemcpyDeviceToDevice, st));
    VSMC_CUDA_CHECK_LAUNCH();
    PfScalars sc;
    VSMC_CUDA_TRY(cudaMemcpyAsync(
        &sc, r.sc, sizeof(sc), cudaMemcpyDeviceToHost, st));
    VSMC_CUDA_TRY(cudaStreamSynchronize(st));
    if (sc.err & DEV_ERR_NONFINITE)
        return VSMC_CUDA_ERR_NONFINITE;
    if (sc.err)
        return VSMC_CUDA_ERR_INTERNAL;
    for (int i = 0; i < 4; ++i)
        rng->ctr[i] = sc.rctr[i];
    rng->index = sc.rindex;
    return VSMC_CUDA_OK;
}
