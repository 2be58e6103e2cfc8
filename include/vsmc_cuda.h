/* vsmc_cuda.h - C ABI of libvsmc_cuda, the GB300 (sm_103a) backend for the
 * vSMC particle-filter step.
 *
 * Conventions (every entry point):
 *   - returns an int status: VSMC_CUDA_OK (0) or a negative vsmc_cuda_status;
 *   - array arguments are DEVICE pointers unless the comment says "host";
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy stream); work
 *     is enqueued on it and the call returns without waiting, except where a
 *     comment says the call synchronizes;
 *   - lengths are size_t and must be below 2^31 (int32 replication / index
 *     arrays, as the reference's C ABI uses int);
 *   - index arrays are int32, weights double, states SoA ([dim][N]).
 *
 * Each declaration names the reference interface it replaces (path inside the
 * vSMC source tree, file:line).  The reference's own C ABI is
 * include/vsmc/vsmc.h; its C++ API is the Sampler / Particle / Weight /
 * StateMatrix / Monitor templates in include/vsmc/core/. */
#ifndef VSMC_CUDA_H
#define VSMC_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------- status */

typedef enum {
    VSMC_CUDA_OK = 0,
    VSMC_CUDA_ERR_ARG = -1,       /* null pointer / bad enum / bad argument */
    VSMC_CUDA_ERR_SIZE = -2,      /* length out of the supported range */
    VSMC_CUDA_ERR_NONFINITE = -3, /* NaN, inf or negative weight */
    VSMC_CUDA_ERR_TIMEOUT = -4,   /* a bounded device wait gave up */
    VSMC_CUDA_ERR_CUDA = -5,      /* CUDA runtime error (see last_cuda_error) */
    VSMC_CUDA_ERR_ALLOC = -6,     /* device allocation failed */
    VSMC_CUDA_ERR_INTERNAL = -7   /* an internal consistency check failed */
} vsmc_cuda_status;

const char *vsmc_cuda_status_string(int status);
/* cudaError_t value of the last CUDA failure seen by the library (0 = none) */
int vsmc_cuda_last_cuda_error(void);
int vsmc_cuda_version(void); /* major * 10000 + minor * 100 + patch */

/* --------------------------------------------------------- RNG engines */

typedef enum {
    VSMC_CUDA_PHILOX4X32 = 0,  /* vsmc::Philox4x32   (rng/philox.hpp:309) */
    VSMC_CUDA_THREEFRY4X64 = 1 /* vsmc::Threefry4x64 (rng/threefry.hpp:389) */
} vsmc_cuda_rng_kind;

/* Host-side engine state: the CounterEngine<Gen> state of
 * rng/counter.hpp:288-496 made explicit.  Philox4x32 uses the low 32 bits of
 * key[0..1] and ctr[0..3]; Threefry4x64 uses all four 64-bit limbs.
 * index is the next word of the current block (4 = block exhausted); the
 * current block itself is gen(ctr), so it is not stored.
 * Replaces the opaque `vsmc_rng` of include/vsmc/vsmc.h:48-50. */
typedef struct {
    int32_t kind;
    uint32_t index;
    uint64_t key[4];
    uint64_t ctr[4];
} vsmc_cuda_rng;

/* CounterEngine(seed): key = {seed, 0, ...}, ctr = 0 (rng/counter.hpp:309-314).
 * Replaces vsmc_rng_init / vsmc_rng_seed (vsmc.h:55-58, lib/src/vsmc_rng.cpp:68-78). */
int vsmc_cuda_rng_init(vsmc_cuda_rng *rng, int kind, uint64_t seed);
/* CounterEngine::key(k): sets the key and resets ctr to 0
 * (rng/counter.hpp:341-345); n = number of limbs given.
 * Replaces vsmc_rng_set_key (vsmc.h:64, lib/src/vsmc_rng.cpp:89-98). */
int vsmc_cuda_rng_set_key(vsmc_cuda_rng *rng, int n, const uint64_t *key);
/* CounterEngine::ctr(c): sets the counter, drops the buffered block
 * (rng/counter.hpp:335-339).  Replaces vsmc_rng_set_ctr (vsmc.h:70). */
int vsmc_cuda_rng_set_ctr(vsmc_cuda_rng *rng, int n, const uint64_t *ctr);

/* Counter-addressed blocks: block b (0-based) = gen(ctr0 + b + 1, key), the
 * reference's pre-increment convention (rng/philox.hpp:263-269), so
 * ctr0 = engine.ctr() reproduces the engine's scalar stream.  out receives
 * 4 * nblocks words.  Replaces PhiloxGenerator::operator() /
 * ThreefryGenerator::operator() (rng/philox.hpp:263-294,
 * rng/threefry.hpp:329-366) applied over a range of counters. */
int vsmc_cuda_philox4x32_blocks(const uint32_t key[2], const uint32_t ctr0[4],
    size_t nblocks, uint32_t *out, void *stream);
int vsmc_cuda_threefry4x64_blocks(const uint64_t key[4],
    const uint64_t ctr0[4], size_t nblocks, uint64_t *out, void *stream);

/* n raw words through the engine's bulk path, bit-exact with
 * CounterEngine::operator()(n, r) (rng/counter.hpp:357-390), including its
 * counter handling for blocks whose low limb is all ones
 * (rng/counter.hpp:78-89, 230-262).  r is uint32_t* (Philox) or uint64_t*
 * (Threefry).  `rng` (host) is advanced.  Replaces vsmc_rng_rand
 * (vsmc.h:74, lib/src/vsmc_rng.cpp:124-129) and rng_rand
 * (rng/counter.hpp:499-504). */
int vsmc_cuda_rng_rand(vsmc_cuda_rng *rng, size_t n, void *r, void *stream);

/* u01_distribution: n reals in [0,1), same words and values as the
 * reference batch path (rng/u01_distribution.hpp:215-233).  `rng` advanced.
 * Replaces vsmc_rng_u01 (vsmc.h:161, lib/src/vsmc_rng.cpp:203). */
int vsmc_cuda_rng_u01(vsmc_cuda_rng *rng, size_t n, double *r, void *stream);
int vsmc_cuda_rng_u01_f32(vsmc_cuda_rng *rng, size_t n, float *r, void *stream);

/* normal_distribution: n normals, the reference batch layout (per 1024
 * chunk: first half sine branch, second half cosine branch; an odd n takes
 * two more words for the last value) (rng/normal_distribution.hpp:222-267).
 * Values agree with the reference within libm accuracy.  `rng` advanced.
 * Replaces vsmc_rng_normal (vsmc.h:147, lib/src/vsmc_rng.cpp:213). */
int vsmc_cuda_rng_normal(vsmc_cuda_rng *rng, size_t n, double *r, double mean,
    double stddev, void *stream);
int vsmc_cuda_rng_normal_f32(vsmc_cuda_rng *rng, size_t n, float *r,
    float mean, float stddev, void *stream);

/* student_t_distribution: n Student-t(df) variates with the reference's
 * batch semantics (rng/student_t_distribution.hpp:97-128): per chunk of at
 * most 1024, chi-squared by the batch gamma (one vectorised attempt, the
 * accepted values packed first, a scalar GammaDistribution draw for each
 * rejected slot; rng/gamma_distribution.hpp:230-410), then a batch of
 * normals divided by sqrt(chi2 / df).  The engine is advanced by exactly the
 * words the reference consumes.  Values agree within libm accuracy (a value
 * within an ulp of an accept / reject boundary can take the other branch).
 * The chunks are sequential in the engine stream, so one block of the GPU
 * walks them.  Synchronizes the stream; VSMC_CUDA_ERR_TIMEOUT if a rejection
 * loop reached its bound of 65536 tries (the variate is NaN).
 * Replaces vsmc_rng_student_t (vsmc.h:162, lib/src/vsmc_rng.cpp:207). */
int vsmc_cuda_rng_student_t(vsmc_cuda_rng *rng, size_t n, double *r,
    double df, void *stream);

/* Independent streams with the scalar distribution semantics: stream s is
 * the engine (kind, key) placed at counter {0, s, 0, 0}; it yields
 * per_stream variates into r[s * per_stream + k] exactly as successive
 * calls of NormalDistribution<double>(mean, sd) (rng/normal_distribution.hpp:
 * 199-216) or StudentTDistribution<double>(df) (rng/student_t_distribution.hpp:
 * 78-91, gamma by rng/gamma_distribution.hpp:132-216) on that engine.
 * The gamma rejection loops stop after 65536 tries (each accepts with
 * probability above 1/2); a variate that reaches the bound is NaN. */
int vsmc_cuda_normal_streams(int kind, const uint64_t key[4], size_t nstreams,
    size_t per_stream, double mean, double stddev, double *r, void *stream);
int vsmc_cuda_student_t_streams(int kind, const uint64_t key[4],
    size_t nstreams, size_t per_stream, double df, double *r, void *stream);

/* u01 sequence array forms (rng/u01_sequence.hpp:53-89).  Replace
 * vsmc_rng_u01_sorted / _stratified / _systematic (vsmc.h:76-83).  The
 * sorted form's running log sum is the reference's left-to-right sum
 * bit for bit; log/exp come from CUDA's libm. */
int vsmc_cuda_u01_sorted(size_t n, const double *u01, double *u01seq,
    void *stream);
int vsmc_cuda_u01_stratified(size_t n, const double *u01, double *u01seq,
    void *stream);
int vsmc_cuda_u01_systematic(size_t n, double u01, double *u01seq,
    void *stream);

/* --------------------------------------------------------------- sums */

/* Left-to-right double sum s_i = (...((0 + x_0) + x_1) ... + x_i) of n
 * non-negative finite values, bit-identical to a sequential loop (the order
 * std::accumulate and the reference's resampling CDF use,
 * resample/transform.hpp:61-69, core/weight.hpp:228).  prefix may be NULL
 * (only *total_dev is written); total_dev (device, 1 double) may be NULL.
 * Returns VSMC_CUDA_ERR_NONFINITE for a negative or non-finite input;
 * synchronizes the stream to report it. */
int vsmc_cuda_sequential_sum(size_t n, const double *x, double *prefix,
    double *total_dev, void *stream);

/* ---------------------------------------------------------- resampling */

typedef enum {
    VSMC_CUDA_MULTINOMIAL = 0,
    VSMC_CUDA_STRATIFIED = 1,
    VSMC_CUDA_SYSTEMATIC = 2,
    VSMC_CUDA_RESIDUAL = 3,
    VSMC_CUDA_RESIDUAL_STRATIFIED = 4,
    VSMC_CUDA_RESIDUAL_SYSTEMATIC = 5
} vsmc_cuda_resample_scheme; /* = vsmc::ResampleScheme (internal/defines.hpp:57-64) */

/* Replication counts from m normalized weights and n uniforms, identical to
 * the reference's two-pointer loop (resample/transform.hpp:43-71) for the
 * same inputs, including unsorted uniforms (counted up to the first
 * uniform above each cumulative weight).
 * Replaces vsmc_resample_trans_u01_rep (vsmc.h:286, lib/src/vsmc_resample.cpp:48-53). */
int vsmc_cuda_resample_trans_u01_rep(size_t m, size_t n, const double *weight,
    const double *u01, int *replication, void *stream);
/* Parent index per uniform (resample/transform.hpp:75-96).
 * Replaces vsmc_resample_trans_u01_index (vsmc.h:288). */
int vsmc_cuda_resample_trans_u01_index(size_t m, size_t n,
    const double *weight, const double *u01, int *index, void *stream);
/* Replication counts -> parent indices with the reference's slot layout:
 * for m == n a parent keeps its own slot and empty slots are filled, in
 * order, by surplus copies of parents taken in order
 * (resample/transform.hpp:100-134).
 * Replaces vsmc_resample_trans_rep_index (vsmc.h:290). */
int vsmc_cuda_resample_trans_rep_index(size_t m, size_t n,
    const int *replication, int *index, void *stream);
/* Parent indices -> replication counts (resample/transform.hpp:138-150).
 * Replaces vsmc_resample_trans_index_rep (vsmc.h:292). */
int vsmc_cuda_resample_trans_index_rep(size_t m, size_t n, const int *index,
    int *replication, void *stream);
/* Residual split (resample/transform.hpp:155-168): resid = frac(n * w)
 * normalized by its left-to-right sum, integ = integer parts; *r_host gets
 * n - sum(integ).  Synchronizes the stream.
 * Replaces vsmc_resample_trans_residual (vsmc.h:294). */
int vsmc_cuda_resample_trans_residual(size_t m, size_t n,
    const double *weight, double *resid, int *integ, size_t *r_host,
    void *stream);

/* Resampling schemes with an engine: counts identical to the reference
 * functors for the same weights and engine state, and the engine advanced by
 * exactly the words the reference consumes.  Multinomial / Residual build
 * their sorted uniforms with CUDA's log/exp, so a uniform can differ from the
 * reference's in the last bit; every other scheme is bit-exact end to end.
 * `rng` (host) is advanced; the call synchronizes the stream.  Philox4x32
 * engines only.  Replaces vsmc_resample_<scheme> and vsmc_resample
 * (vsmc.h:277-310, lib/src/vsmc_resample.cpp:84-116) and
 * Resample<Scheme>::operator() (resample/multinomial.hpp:46-52,
 * stratified.hpp:46-52, systematic.hpp:46-52, residual.hpp:46-57,
 * residual_stratified.hpp:46-57, residual_systematic.hpp:46-57). */
int vsmc_cuda_resample(size_t m, size_t n, vsmc_cuda_rng *rng,
    const double *weight, int *replication, int scheme, void *stream);
int vsmc_cuda_resample_multinomial(size_t m, size_t n, vsmc_cuda_rng *rng,
    const double *weight, int *replication, void *stream);
int vsmc_cuda_resample_stratified(size_t m, size_t n, vsmc_cuda_rng *rng,
    const double *weight, int *replication, void *stream);
int vsmc_cuda_resample_systematic(size_t m, size_t n, vsmc_cuda_rng *rng,
    const double *weight, int *replication, void *stream);
int vsmc_cuda_resample_residual(size_t m, size_t n, vsmc_cuda_rng *rng,
    const double *weight, int *replication, void *stream);
int vsmc_cuda_resample_residual_stratified(size_t m, size_t n,
    vsmc_cuda_rng *rng, const double *weight, int *replication, void *stream);
int vsmc_cuda_resample_residual_systematic(size_t m, size_t n,
    vsmc_cuda_rng *rng, const double *weight, int *replication, void *stream);

/* Resampling on an integer CDF, as the precision-32 filter does it: q holds
 * n non-negative 64-bit weights whose total stays below 2^63; uniform j
 * (stratified: its own word; systematic: one shared word a of the engine)
 * is u_j = (j + a 2^-32) / n and counts toward the first i with
 * u_j <= (q_0 + ... + q_i) / total, compared exactly in integers.  The last
 * slot takes the rest, as in resample/transform.hpp:70.  replication (n) and
 * index (n, the reference slot layout of resample/transform.hpp:116-133) are
 * device outputs (either may be NULL); the engine consumes the words the
 * reference's U01SequenceStratified / U01SequenceSystematic would
 * (rng/u01_sequence.hpp:177-259).  Synchronizes the stream.  No reference
 * counterpart for the integer CDF itself (the reference sums doubles).
 * A total of 0 or of 2^63 and more returns VSMC_CUDA_ERR_NONFINITE. */
int vsmc_cuda_resample_fixed(size_t n, const uint64_t *q, int scheme,
    vsmc_cuda_rng *rng, int *replication, int *index, void *stream);

/* vsmc_cuda_resample_fixed without any allocation, for callers that must not
 * allocate device memory while they run (inside an allocator or memory-pool
 * callback, or in a loop that reserved all device memory beforehand).  Same
 * arguments, results and engine advance as vsmc_cuda_resample_fixed; its
 * scratch is one fixed array of about 3 MiB in the library's device image.
 *   - n must be at most VSMC_CUDA_RESAMPLE_FIXED_NOALLOC_MAX_N, otherwise
 *     VSMC_CUDA_ERR_SIZE is returned before any device work;
 *   - the first call on each device (that device current) looks up the
 *     array's address and may load the library's device code: make it
 *     before any stream capture;
 *   - all callers on a device share the array, so calls whose work overlaps
 *     in time race and give wrong results.  Serialize the calls on the host:
 *     one call at a time per device (each call synchronizes its stream
 *     before returning, so one host thread calling in turn is safe; several
 *     host threads need a lock of their own, even on one stream, since each
 *     call queues several launches that could interleave);
 *   - the array's address is looked up once per device for the life of the
 *     process: a device reset (cudaDeviceReset) between calls is not
 *     supported;
 *   - synchronizes the stream.
 * No reference counterpart (the reference allocates nothing on a device). */
#define VSMC_CUDA_RESAMPLE_FIXED_NOALLOC_MAX_N (1u << 18)
int vsmc_cuda_resample_fixed_noalloc(size_t n, const uint64_t *q, int scheme,
    vsmc_cuda_rng *rng, int *replication, int *index, void *stream);

/* In-place particle copy state[d][dst] = state[d][index[dst]] for a SoA
 * state of `dim` rows of n values; safe in place for indices produced by
 * vsmc_cuda_resample_trans_rep_index (every parent keeps its slot).
 * Replaces StateMatrix<ColMajor,Dim,T>::copy (core/state_matrix.hpp:357-364)
 * and StateOMP::copy (smp/backend_omp.hpp:53-59). */
int vsmc_cuda_state_copy_f32(size_t n, size_t dim, const int *index,
    float *state, void *stream);
int vsmc_cuda_state_copy_f64(size_t n, size_t dim, const int *index,
    double *state, void *stream);

/* ------------------------------------------------------------- weights */

/* The Weight class on device (core/weight.hpp:67-230).  W holds normalized
 * weights (n doubles); *ess_dev (device, 1 double) receives 1 / sum W^2.
 * Sums run left to right in the reference's order, so set() is bit-exact;
 * set_log / add_log use CUDA's exp / log.
 *   set:       Weight::set (weight.hpp:115-120)     W = w / sum(w)
 *   set_log:   Weight::set_log (weight.hpp:145-149) W = exp(lw - max) normalized
 *   add_log:   Weight::add_log (weight.hpp:168-173) W = W * exp(l) normalized
 *   set_equal: Weight::set_equal (weight.hpp:99-103) */
int vsmc_cuda_weight_set(size_t n, const double *w, double *W,
    double *ess_dev, void *stream);
int vsmc_cuda_weight_set_log(size_t n, const double *lw, double *W,
    double *ess_dev, void *stream);
int vsmc_cuda_weight_add_log(size_t n, const double *l, double *W,
    double *ess_dev, void *stream);
int vsmc_cuda_weight_set_equal(size_t n, double *W, double *ess_dev,
    void *stream);

/* Weighted mean of each SoA row: out_dev[d] = sum_i W_i * state[d][i] for
 * d < dim (the Monitor::eval dgemv, core/monitor.hpp:252-267). */
int vsmc_cuda_monitor_mean_f64(size_t n, size_t dim, const double *state,
    const double *W, double *out_dev, void *stream);
int vsmc_cuda_monitor_mean_f32(size_t n, size_t dim, const float *state,
    const double *W, double *out_dev, void *stream);

/* ------------------------------------------------------ particle filter */

/* Constant-velocity tracking model with Student-t position observations:
 * state (x, y, vx, vy); x_t = F x_{t-1} + G a_t, a ~ N(0, sigma_a^2 I2);
 * prior x, y ~ N(0, sd_pos0^2), vx, vy ~ N(0, sd_vel0^2); observation
 * (x, y) + obs_scale * t_nu per coordinate.  The user move of
 * example/pf/include/pf.hpp:154-170 in this model's form. */
typedef struct {
    double dt, sigma_a, obs_scale, nu, sd_pos0, sd_vel0;
} vsmc_cuda_cv_model;

typedef struct vsmc_cuda_pf vsmc_cuda_pf; /* opaque */

/* A bootstrap filter over n particles.
 *   precision 64: FP64 state; weights kept as the reference's Weight class
 *     (normalized doubles, left-to-right sums) and resampled by the exact
 *     scheme path above -- the reference's arithmetic step for step.
 *   precision 32: FP32 SoA state and log-weights in one fused move /
 *     likelihood / reduction kernel; FP64 block-level log-sum-exp; an exact
 *     64-bit fixed-point CDF for resampling.
 * `stream` NULL gives the filter a private non-blocking stream (the legacy
 * stream cannot be captured in a CUDA graph); vsmc_cuda_pf_stream returns
 * the stream in use.
 * Particle streams: Philox4x32 key {step, seed}, counter {0, particle, 0, 0};
 * resampling engine key {0, seed} from counter {0, 0, 1, 0}.
 * Replaces Sampler<T>(N, scheme, threshold) (core/sampler.hpp:107-114) with
 * a CUDA state / move / weight / monitor (smp/backend_omp.hpp:45-133 are the
 * CPU siblings). */
int vsmc_cuda_pf_create(vsmc_cuda_pf **pf, size_t n, int precision,
    int scheme, double threshold, uint32_t seed,
    const vsmc_cuda_cv_model *model, size_t max_steps, void *stream);
int vsmc_cuda_pf_destroy(vsmc_cuda_pf *pf);
/* Sampler::initialize (core/sampler.hpp:443-455) with observation obs_dev[0..1]
 * (device, 2 doubles). */
int vsmc_cuda_pf_initialize(vsmc_cuda_pf *pf, const double *obs_dev);
/* Sampler::iterate() (core/sampler.hpp:464-476) with observation obs_dev[0..1]. */
int vsmc_cuda_pf_iterate(vsmc_cuda_pf *pf, const double *obs_dev);
/* initialize + (T-1) iterates over obs_dev[2t..2t+1] (device), recording
 * per step: mean (2 doubles), ESS, resampled flag and cumulative log
 * evidence into the device histories. */
int vsmc_cuda_pf_run_device(vsmc_cuda_pf *pf, size_t T, const double *obs_dev);
/* Whole run through host buffers (the end-to-end entry point): copies the
 * T x 2 observations in, runs, copies the histories out, synchronizes.
 * Any output pointer may be NULL. */
int vsmc_cuda_pf_run(vsmc_cuda_pf *pf, size_t T, const double *obs_host,
    double *mean_host, double *ess_host, int *resampled_host,
    double *logz_host);
/* Copy the first T recorded history entries to host (synchronizes). */
int vsmc_cuda_pf_history(vsmc_cuda_pf *pf, size_t T, double *mean_host,
    double *ess_host, int *resampled_host, double *logz_host);
/* Device views: SoA state (4 rows x, y, vx, vy, each of stride
 * ((n + 255) / 256) * 256 elements, float or double by precision), and the
 * weight array (precision 64: normalized W doubles; precision 32: float
 * log-weights; after a resampling step every weight is equal and the stored
 * log-weights are stale until the next step).  Precision 32 keeps the state
 * in two buffers that alternate every step (a step reads one and writes the
 * other, gathering resampled particles on the way), so the state pointer is
 * valid until the next step; the call applies a pending resampling gather
 * first (and may synchronize the stream to do so). */
int vsmc_cuda_pf_state(vsmc_cuda_pf *pf, void **state_dev, void **weight_dev);
int vsmc_cuda_pf_stream(vsmc_cuda_pf *pf, void **stream);
/* Enable (1) / disable (0) capturing each filter step in a CUDA graph and
 * replaying it (precision 32 only; default on). */
int vsmc_cuda_pf_use_graph(vsmc_cuda_pf *pf, int on);
/* Profiling hook (precision 32, after initialize): launch only the fused
 * move / likelihood / weight-reduction kernel of one step on the filter's
 * stream, without the resampling kernels.  Steps past max_steps reuse the
 * last observation and record no history.  No reference counterpart: it
 * times the dominant kernel of MoveOMP::operator() + Weight::add_log
 * (smp/backend_omp.hpp:93-105, core/weight.hpp:168-173). */
int vsmc_cuda_pf_launch_step_kernel(vsmc_cuda_pf *pf);

/* ------------------------------------------- filters of user models */

/* A precision-32 filter whose move and log-likelihood come from the caller's
 * device model (vsmc_cuda_filter.cuh): dim state components (1..8, SoA rows
 * of ((n + 255) / 256) * 256 floats), the weighted mean of the first
 * monitor_dim (0..4, <= dim) recorded every step, scheme stratified or
 * systematic on the exact integer CDF.  threshold >= 0: the step kernel
 * flags a resample when ESS < threshold * n and vsmc_cuda_pf_step_commit
 * runs it; threshold < 0: the host decides (vsmc_cuda_pf_resample_now), as
 * Particle::resample does under Sampler<T> (core/particle.hpp:170-197).
 * Replaces Sampler<T>(N, scheme, threshold) (core/sampler.hpp:107-114)
 * with a state matrix StateMatrix<ColMajor, dim, float>
 * (core/state_matrix.hpp:320-364) and a user move
 * (smp/backend_base.hpp:243-363). */
int vsmc_cuda_pf_create_model(vsmc_cuda_pf **pf, size_t n, size_t dim,
    size_t monitor_dim, int scheme, double threshold, uint32_t seed,
    size_t max_steps, void *stream);

/* Buffers of a precision-32 filter's next step, for a step kernel of the
 * caller's model (vsmc_cuda::pf_step_launch in vsmc_cuda_filter.cuh). */
typedef struct {
    const float *state_in;   /* dim rows of `stride` floats: before the step */
    float *state_out;        /* dim rows: after the step */
    float *log_weight;       /* n FP32 log-weights (updated in place) */
    const int32_t *index;    /* slot encoding of the last resample */
    const uint32_t *sources; /* parents of the empty slots */
    void *partials;          /* max_grid per-block records */
    void *scalars;           /* the filter's device scalars */
    double *hist_mean;       /* max_steps x monitor_dim */
    double *hist_ess, *hist_logz;
    int *hist_resampled;
    size_t n, stride, dim, monitor_dim, max_steps, max_grid;
    size_t step;             /* index of the step (0 = initialize) */
    uint32_t seed;
    double threshold;        /* the device's resampling threshold (< 0: never) */
    void *stream;            /* the filter's stream */
    int record_previous_mean; /* nonzero: the step records the previous
                                 step's monitor from the particles it reads
                                 (and not its own), as the filter's own
                                 runs do; 0: its own (after a resample the
                                 resampling passes replace it) */
} vsmc_cuda_pf_step_desc;

/* The first call after creation or vsmc_cuda_pf_reset (step 0) also resets
 * the filter's device scalars on its stream. */
int vsmc_cuda_pf_step_desc_get(vsmc_cuda_pf *pf, vsmc_cuda_pf_step_desc *d);
/* Back to step 0 (Sampler::initialize, core/sampler.hpp:443-455) for a
 * filter of vsmc_cuda_pf_create_model. */
int vsmc_cuda_pf_reset(vsmc_cuda_pf *pf);
/* After the step kernel was launched on the descriptor's stream: the
 * resampling passes (threshold >= 0; they return at once unless the step
 * flagged a resample), then the buffers swap and the step index advances. */
int vsmc_cuda_pf_step_commit(vsmc_cuda_pf *pf);
/* The host-side part of vsmc_cuda_pf_step_commit (the buffers swap, the
 * step index advances) without its launches: for a caller that replays a
 * step it captured in a CUDA graph from one step_desc_get ->
 * pf_step_launch -> step_commit sequence on the filter's stream (the graph
 * holds the step kernel and the resampling passes; a graph per buffer
 * parity, since the descriptor's buffers alternate).  No reference
 * counterpart. */
int vsmc_cuda_pf_step_advance(vsmc_cuda_pf *pf);
/* Resample the current particles now (precision 32): the host decided
 * ESS < threshold * N.  Particle::resample -> StateCUDA::copy(N, nullptr)
 * (core/particle.hpp:186-192); the weights become equal, and the monitor
 * mean becomes that of the resampled particles. */
int vsmc_cuda_pf_resample_now(vsmc_cuda_pf *pf);
/* Weight::set_equal (core/weight.hpp:99-103) on a precision-32 filter. */
int vsmc_cuda_pf_set_equal(vsmc_cuda_pf *pf);
/* Weight::set_log (add = 0) / Weight::add_log (add = 1)
 * (core/weight.hpp:145-149, 168-173) on a precision-32 filter from n device
 * doubles; ESS, the monitor sums' weights and (add) the log-evidence follow. */
int vsmc_cuda_pf_weight_log(vsmc_cuda_pf *pf, const double *lw_dev, int add);

/* Host view of the filter scalars after the work queued so far
 * (synchronizes the filter's stream). */
typedef struct {
    double ess;           /* ESS of the current weights */
    double log_evidence;  /* cumulative log-evidence */
    double max_log_weight;
    double sum_weight;    /* sum exp(lw - max_log_weight) */
    double mean[4];       /* monitor: weighted mean of the first components */
    size_t step;          /* steps taken */
    int resampled;        /* the current weights are equal after a resample */
    int monitor_dim;
} vsmc_cuda_pf_status;

int vsmc_cuda_pf_get_status(vsmc_cuda_pf *pf, vsmc_cuda_pf_status *out);
/* vsmc_cuda_pf_get_status in two halves.  status_enqueue queues the copy of
 * the device scalars into the filter's pinned host copy on its stream (no
 * wait; it may be captured into a graph with the step).  status_read waits
 * for the stream and reads that copy, with no copy of its own: it returns
 * what the last queued copy saw.  No reference counterpart. */
int vsmc_cuda_pf_status_enqueue(vsmc_cuda_pf *pf);
int vsmc_cuda_pf_status_read(vsmc_cuda_pf *pf, vsmc_cuda_pf_status *out);

/* ------------------------------------- bearings-only model, proposal */

/* Bearings-only tracking: state (x, y, vx, vy); constant velocity with
 * continuous white-noise acceleration of spectral density q per axis
 * (Q = q [[dt^3/3, dt^2/2], [dt^2/2, dt]]); bearing observation
 * atan2(y, x) + N(0, sigma_z^2) from a sensor at the origin; prior
 * N((x0, y0, vx0, vy0), diag(sd_pos0^2, sd_pos0^2, sd_vel0^2, sd_vel0^2)).
 * No reference counterpart (the reference's pf example is the position
 * model above). */
typedef struct {
    double dt, q, sigma_z, x0, y0, vx0, vy0, sd_pos0, sd_vel0;
} vsmc_cuda_bearings_model;

/* Simulate T steps from CounterEngine(seed) (Philox4x32): prior and
 * transition noise from fresh NormalDistribution<double> pairs (x axis, then
 * y axis), bearing noise from one NormalDistribution<double>(0, sigma_z)
 * kept for the run.  truth: T x 4 (may be NULL), obs: T (device). */
int vsmc_cuda_bearings_simulate(uint32_t seed, size_t T,
    const vsmc_cuda_bearings_model *model, double *truth, double *obs,
    void *stream);

/* The proposal network: inputs from the previous state and the bearing z,
 * in the bearing frame (along = (cos z, sin z), across = (-sin z, cos z)):
 * with the predicted position p = (x + dt vx, y + dt vy) and r = |p|,
 * p_along / (10 + r); e / sqrt(1 + (e / 8)^2) / 8 with e = p_across /
 * (sigma_z r); the velocity's along and across parts over (1 + |v|); sin z;
 * cos z.  Two hidden layers of 64 (GELU, tanh form); outputs (m, l): the
 * mean and diagonal log-variance of the whitened transition noise in the
 * bearing frame, nu' = (along, along, across, across) of the position and
 * velocity noise pairs (x = F x' + L nu, L = chol(Q), nu the pairs rotated
 * back).  Parameters: FP32, *nparams floats (W1[64][6], b1[64],
 * W2[64][64], b2[64], W3[8][64], b3[8]); the packed copy (BF16 operand
 * fragments + FP32 biases, *npacked 32-bit words) is what the kernels read. */
int vsmc_cuda_mlp_sizes(size_t *nparams, size_t *npacked);
int vsmc_cuda_mlp_init(uint32_t seed, float *params, void *stream);
int vsmc_cuda_mlp_pack(const float *params, uint32_t *packed, void *stream);
/* out[B][8] = network(feat[B][6]) (BF16 operands, FP32 accumulation):
 * mma.sync fragments per warp (16 rows at a time, activations kept in
 * registers). */
int vsmc_cuda_mlp_forward(const uint32_t *packed, size_t B, const float *feat,
    float *out, void *stream);
/* The same network on the Blackwell tensor core (tcgen05.mma, accumulators
 * in tensor memory), 128 rows per tile and one thread per row.  Results
 * agree with vsmc_cuda_mlp_forward up to FP32 summation order (and the BF16
 * rounding of an activation that lands on a rounding boundary).  A block
 * whose tensor-core wait runs out writes NaN for its rows. */
int vsmc_cuda_mlp_forward_tc(const uint32_t *packed, size_t B,
    const float *feat, float *out, void *stream);
/* Mean loss 0.5 sum_d [(nu_d - m_d)^2 exp(-l_d) + l_d] over B rows
 * (loss_dev: 1 double, may be NULL) and its gradient with respect to the
 * parameters (grad_dev: nparams floats); the sum over rows is in a fixed
 * order.  The weight gradients are contractions over the rows on the
 * Blackwell tensor core (tcgen05.mma into tensor memory, FP32 deltas split
 * into BF16 hi + lo parts); a block whose tensor-core wait runs out makes
 * the result NaN. */
int vsmc_cuda_mlp_loss_grad(const uint32_t *packed, size_t B,
    const float *feat, const float *nu, double *loss_dev, float *grad_dev,
    void *stream);
/* Train params in place with Adam (lr): ntraj trajectories simulated from
 * the model (seed) for T steps give ntraj * (T - 1) stored (x_{t-1}, z_t,
 * nu_t) samples (inputs and noise in the bearing frame of z_t); then `steps` Adam steps on minibatches of `batch` samples
 * drawn uniformly with replacement.  loss_host (may be NULL) receives the
 * mean loss of each minibatch (`steps` values).  Synchronizes. */
int vsmc_cuda_mlp_train(const vsmc_cuda_bearings_model *model, uint32_t seed,
    size_t ntraj, size_t T, size_t batch, size_t steps, double lr,
    float *params, double *loss_host, void *stream);
/* Training rows from the particle clouds of a bootstrap filter, one block
 * per track: ntracks tracks simulated from the model, each filtered by P
 * particles (a multiple of 32, at most 1024) for T steps (2 <= T <= 1024),
 * resampled every step.  At step t >= 1 each particle x' of the cloud
 * approximating p(x_{t-1} | z_{0:t-1}) gives a row: its inputs for z_t
 * (feat, 6 floats) and a noise chosen among K draws of N(0, I) with
 * probability proportional to g(z_t | F x' + L nu) (nu, 4 floats, bearing
 * frame) -- a sampling-importance-resampling draw toward the locally
 * optimal proposal the loss targets.  ntracks * P * (T - 1) rows (device).
 * No reference counterpart. */
int vsmc_cuda_mlp_cloud_rows(const vsmc_cuda_bearings_model *model,
    uint32_t seed, size_t ntracks, size_t P, size_t T, size_t K, float *feat,
    float *nu, void *stream);
/* vsmc_cuda_mlp_train with nx extra rows (device xfeat[nx][6], xnu[nx][4],
 * for instance from vsmc_cuda_mlp_cloud_rows): minibatch rows are drawn
 * uniformly over the simulated samples and the extra rows together.
 * Synchronizes.  No reference counterpart. */
int vsmc_cuda_mlp_train_rows(const vsmc_cuda_bearings_model *model,
    uint32_t seed, size_t ntraj, size_t T, const float *xfeat,
    const float *xnu, size_t nx, size_t batch, size_t steps, double lr,
    float *params, double *loss_host, void *stream);
/* One FP32 move + weight increment on caller-owned SoA state [4][n]: t == 0
 * draws the prior; t > 0 draws nu ~ N(0, I) (packed == NULL, bootstrap) or
 * nu' ~ N(m, diag(exp(l))) from the network in the bearing frame of z,
 * rotated to nu (packed != NULL).  lw_inc gets log g(z | x)
 * (+ log N(nu'; 0, I) - log N(nu'; m, exp(l)) for the learned proposal).  Particle streams: Philox4x32 key {t, seed}, counter
 * {0, i, 0, 0}, pre-incremented, two Box-Muller pairs. */
int vsmc_cuda_bearings_move_f32(size_t n, size_t t, uint32_t seed,
    const vsmc_cuda_bearings_model *model, double z, const uint32_t *packed,
    float *state, float *lw_inc, void *stream);

/* ----------------------------------------------------- batched filters */

typedef struct vsmc_cuda_batch vsmc_cuda_batch; /* opaque */

/* nfilters independent precision-32 bootstrap filters run together.  Filter
 * f has n[f] >= 2 particles, horizon T[f] >= 1, model models[f] and seed
 * seeds[f] (host arrays).  Per step, one persistent kernel moves, weights and
 * reduces the particles of every filter still running, and one kernel
 * resamples (one block per filter) those whose ESS fell below
 * threshold * n[f]; a whole run is one CUDA graph.  Filter f draws the
 * streams and makes the counts of a single vsmc_cuda_pf with seed seeds[f]
 * (the order of its FP64 sums differs).  Observations and histories are the
 * filters' blocks concatenated in the caller's order: filter f's T[f] steps
 * start at entry T[0] + ... + T[f-1] (2 doubles per entry for observations
 * and means).  scheme: stratified or systematic.  No reference counterpart:
 * the reference runs one Sampler<T> per filter (core/sampler.hpp:107-114). */
int vsmc_cuda_batch_create(vsmc_cuda_batch **batch, size_t nfilters,
    const uint32_t *n, const uint32_t *T, const vsmc_cuda_cv_model *models,
    const uint32_t *seeds, int scheme, double threshold, void *stream);
/* Bearings-only filters (vsmc_cuda_bearings_model each): the bootstrap
 * (packed == NULL) or the learned proposal (packed: the packed proposal
 * network, device, kept by pointer for the batch's lifetime).  Observations
 * are one bearing per step (filter f's block starts at entry
 * T[0] + ... + T[f-1]).  The learned kind has a fixed kernel shape (32
 * particles per warp; set_shape and autotune refuse it). */
int vsmc_cuda_batch_create_bearings(vsmc_cuda_batch **batch, size_t nfilters,
    const uint32_t *n, const uint32_t *T,
    const vsmc_cuda_bearings_model *models, const uint32_t *seeds,
    const uint32_t *packed, int scheme, double threshold, void *stream);
int vsmc_cuda_batch_destroy(vsmc_cuda_batch *batch);
int vsmc_cuda_batch_stream(vsmc_cuda_batch *batch, void **stream);
/* Each filter's truth (4 per step, may be NULL) and observations simulated
 * from its own model and seed, as vsmc_cuda_cv_simulate /
 * vsmc_cuda_bearings_simulate do for one filter (device outputs,
 * concatenated layout).  Synchronizes. */
int vsmc_cuda_batch_simulate(vsmc_cuda_batch *batch, double *truth_dev,
    double *obs_dev);
/* Run every filter to its horizon over device observations (asynchronous). */
int vsmc_cuda_batch_run_device(vsmc_cuda_batch *batch, const double *obs_dev);
/* Host observations in, histories out (the end-to-end entry; synchronizes). */
int vsmc_cuda_batch_run(vsmc_cuda_batch *batch, const double *obs_host,
    double *mean_host, double *ess_host, int *resampled_host,
    double *logz_host);
/* Copy the histories of the last run to host (synchronizes; NULL skips). */
int vsmc_cuda_batch_history(vsmc_cuda_batch *batch, double *mean_host,
    double *ess_host, int *resampled_host, double *logz_host);
/* Step-kernel shape: particles per thread (1, 2, 4) x threads (128, 256). */
int vsmc_cuda_batch_set_shape(vsmc_cuda_batch *batch, int ppt, int block);
int vsmc_cuda_batch_get_shape(vsmc_cuda_batch *batch, int *ppt, int *block);
/* Time the first `steps` steps of the batch over obs_dev for each shape and
 * keep the fastest; ms_host (6 floats, may be NULL) receives the times in
 * the order (1,128) (2,128) (4,128) (1,256) (2,256) (4,256).  Then tunes the
 * scan schedule for that shape (vsmc_cuda_batch_autotune_schedule).
 * Synchronizes. */
int vsmc_cuda_batch_autotune(vsmc_cuda_batch *batch, const double *obs_dev,
    int steps, float *ms_host);
/* Scan schedule of the batched resampling: a filter's particles are
 * resampled in chunks of min_chunk (4096, 8192, 16384 or 32768), doubled
 * until the filter has at most 32 chunks; each chunk is one entry of the
 * step's resampling list.  Results do not depend on it (the counts are
 * exact integers).  autotune_schedule times the first `steps` steps for each
 * of the four and keeps the fastest; ms_host (4 floats, may be NULL) gets
 * the times.  No reference counterpart. */
int vsmc_cuda_batch_set_schedule(vsmc_cuda_batch *batch, uint32_t min_chunk);
int vsmc_cuda_batch_get_schedule(vsmc_cuda_batch *batch, uint32_t *min_chunk);
int vsmc_cuda_batch_autotune_schedule(vsmc_cuda_batch *batch,
    const double *obs_dev, int steps, float *ms_host);

/* --------------------------------------------- genealogy and summary */

/* Lineage over a history of resampling index rows (device, row-major
 * [iters][N]: row k = each particle's parent among the particles before
 * iteration k, the identity for an iteration without resampling).
 * trace: out[id] = the ancestor at iteration `iter` of particle id of the
 * last iteration -- ResampleIndex::index(id, iter) (resample/index.hpp:
 * 117-129) for every id.  matrix: every line, layout 0 = [N][iters]
 * (index_matrix<RowMajor>), 1 = [iters][N] (index_matrix<ColMajor>)
 * (resample/index.hpp:131-201).  An index outside [0, N) gives
 * VSMC_CUDA_ERR_ARG.  Synchronize. */
int vsmc_cuda_resample_index_trace(size_t N, size_t iters, const int *rows,
    size_t iter, int *out, void *stream);
int vsmc_cuda_resample_index_matrix(size_t N, size_t iters, const int *rows,
    int layout, int *out, void *stream);
/* Sampler::print (core/sampler.hpp:646-689) for a sampler with naccept
 * moves / MCMC steps and one monitor of nmon variables named mon_name.0,
 * mon_name.1, ...: header "Size Resampled Accept.0 ... ESS <monitor>" and
 * one row per iteration, every field followed by sep, doubles as the
 * ostream default (6 significant digits).  Host arrays: resampled, ess (T),
 * mon (T x nmon), accept (T x naccept; NULL = one column of N).  buf (cap
 * bytes) gets the text, NUL-terminated; *len its length; VSMC_CUDA_ERR_SIZE
 * if it does not fit (cap 0: length only). */
int vsmc_cuda_sampler_print(size_t T, size_t N, const int *resampled,
    const double *ess, size_t nmon, const char *mon_name, const double *mon,
    size_t naccept, const size_t *accept, char sep, char *buf, size_t cap,
    size_t *len);
/* Precision-32 filters: record each step's resampling index row (the
 * parents after resampling, or the identity) into a max_steps x n device
 * array; rows_dev points at it (valid while the filter lives). */
int vsmc_cuda_pf_record_genealogy(vsmc_cuda_pf *pf, int on);
int vsmc_cuda_pf_genealogy(vsmc_cuda_pf *pf, const int **rows_dev);
/* Resample-move (precision 32, before initialize): after every step t >= 1
 * that resampled, `sweeps` random-walk Metropolis steps on each particle's
 * acceleration innovation a (the RandomWalk / NormalMVProposal update of
 * rng/random_walk.hpp:95-114, proposal a' = a + scale * N(0, I2), target
 * N(a; 0, sigma_a^2 I2) g(y_t | x_t), x_t = F x_{t-1} + G a), the mcmc
 * queue of Sampler::iterate (core/sampler.hpp:409-438, 746-754).  Steps
 * that did not resample (weights not equal) are left unmoved.  sweeps 0
 * turns it off.  accepts: the accepted steps per step (host, T). */
int vsmc_cuda_pf_set_mcmc(vsmc_cuda_pf *pf, size_t sweeps, double scale);
int vsmc_cuda_pf_mcmc_accepts(vsmc_cuda_pf *pf, size_t T, uint32_t *host);
/* Kernel-level resample-move step: `sweeps` such moves at step t on
 * caller-owned SoA state [4][n] after step t's move (particle i's
 * innovation is that of parent[i], or of i when parent is NULL);
 * accepted (device, 1 uint32) is incremented by the accepted steps. */
int vsmc_cuda_cv_mcmc_f32(size_t n, size_t t, size_t sweeps, uint32_t seed,
    const vsmc_cuda_cv_model *model, const double obs[2], double scale,
    const int *parent, float *state, uint32_t *accepted, void *stream);
/* The filter's first T steps as Sampler::print text (monitor "pos", the
 * weighted position mean; Accept.0 = n for the move, Accept.1 = the
 * MCMC accepts when resample-move is on). */
int vsmc_cuda_pf_print(vsmc_cuda_pf *pf, size_t T, char sep, char *buf,
    size_t cap, size_t *len);

/* One move + log-likelihood step on caller-owned SoA state (kernel-level
 * parity entry point): t == 0 draws the prior, t > 0 propagates.  ll
 * receives the per-particle log-likelihood of obs (host, 2 doubles). */
int vsmc_cuda_cv_move_f64(size_t n, size_t t, uint32_t seed,
    const vsmc_cuda_cv_model *model, const double obs[2], double *state,
    double *ll, void *stream);
int vsmc_cuda_cv_move_f32(size_t n, size_t t, uint32_t seed,
    const vsmc_cuda_cv_model *model, const double obs[2], float *state,
    float *ll, void *stream);

/* Simulate T steps of the model from the Philox4x32 engine seeded with seed
 * (truth: T x 4, obs: T x 2, device), prior pairs and acceleration pairs from
 * fresh NormalDistribution<double> objects, observation noise from one
 * StudentTDistribution<double>(nu) kept for the whole run. */
int vsmc_cuda_cv_simulate(uint32_t seed, size_t T,
    const vsmc_cuda_cv_model *model, double *truth, double *obs,
    void *stream);

#ifdef __cplusplus
}
#endif

#endif /* VSMC_CUDA_H */
