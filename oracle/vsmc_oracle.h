/* vsmc_oracle.h - CPU restatement of the vSMC particle-filter path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle and the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * arm may load it; the product library never does.
 *
 * Every function follows a reference file:line (paths inside the vSMC tree),
 * cited at its definition in vsmc_oracle.c.  It is pinned against the
 * reference itself through the fixtures in tests/golden/, which
 * tests/golden/make_golden.py generates from the reference compiled by
 * `make -C oracle ref`. */
#ifndef VSMC_ORACLE_H
#define VSMC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ engines */

typedef struct {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    uint32_t index; /* 4 = buffer exhausted */
} vo_philox;

typedef struct {
    uint64_t key[4];
    uint64_t ctr[4];
    uint64_t buf[4];
    uint32_t index;
} vo_threefry;

/* raw generator: one block from an explicit counter (no pre-increment) */
void vo_philox4x32_block(
    const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void vo_threefry4x64_block(
    const uint64_t ctr[4], const uint64_t key[4], uint64_t out[4]);

/* engine placed by key(k) then ctr(c), exactly as CounterEngine::key/ctr */
void vo_philox_init(vo_philox *e, const uint32_t key[2], const uint32_t ctr[4]);
uint32_t vo_philox_next(vo_philox *e);
void vo_philox_rand(vo_philox *e, size_t n, uint32_t *r);
void vo_threefry_init(
    vo_threefry *e, const uint64_t key[4], const uint64_t ctr[4]);
uint64_t vo_threefry_next(vo_threefry *e);
void vo_threefry_rand(vo_threefry *e, size_t n, uint64_t *r);

/* word streams, matching the harness entry points used by the fixtures */
void vo_philox4x32_words(const uint32_t key[2], const uint32_t ctr[4],
    size_t n, uint32_t *out, int bulk);
void vo_threefry4x64_words(const uint64_t key[4], const uint64_t ctr[4],
    size_t n, uint64_t *out, int bulk);

/* ---------------------------------------------------------------- u01 */
/* lr: 0 = [0,1], 1 = [0,1), 2 = (0,1], 3 = (0,1) */
double vo_u01_u32_f64(int lr, uint32_t u);
float vo_u01_u32_f32(int lr, uint32_t u);
double vo_u01_u64_f64(int lr, uint64_t u);
float vo_u01_u64_f32(int lr, uint64_t u);
void vo_u01_u32_f64_n(int lr, size_t n, const uint32_t *u, double *r);
void vo_u01_u32_f32_n(int lr, size_t n, const uint32_t *u, float *r);
void vo_u01_u64_f64_n(int lr, size_t n, const uint64_t *u, double *r);

/* ------------------------------------------------------ distributions */
/* eng: 0 = Philox4x32 (low 32 bits of key[0..1], ctr[0..3]), 1 = Threefry4x64 */
void vo_u01_dist_f64(int eng, const uint64_t key[4], const uint64_t ctr[4],
    size_t n, double *r, int batch);
void vo_u01_dist_f32(int eng, const uint64_t key[4], const uint64_t ctr[4],
    size_t n, float *r, int batch);
void vo_normal_f64(int eng, const uint64_t key[4], const uint64_t ctr[4],
    size_t n, double mean, double sd, double *r, int batch);
void vo_normal_f32(int eng, const uint64_t key[4], const uint64_t ctr[4],
    size_t n, float mean, float sd, float *r, int batch);
/* scalar StudentTDistribution semantics only */
void vo_student_t_f64(int eng, const uint64_t key[4], const uint64_t ctr[4],
    size_t n, double df, double *r);
/* student_t_distribution (batch form; vsmc_rng_student_t) after `skip`
 * scalar words; the engine state afterwards in ctr_out / index_out */
void vo_student_t_batch_f64(int eng, const uint64_t key[4],
    const uint64_t ctr[4], size_t skip, size_t n, double df, double *r,
    uint64_t ctr_out[4], uint32_t *index_out);

/* ------------------------------------------------------- u01 sequences */
void vo_u01_sequence(int kind, size_t N, const uint32_t key[2],
    const uint32_t ctr[4], double *out, uint32_t next_words[4]);
void vo_u01_sorted(size_t N, const double *u01, double *u01seq);
void vo_u01_stratified(size_t N, const double *u01, double *u01seq);
void vo_u01_systematic(size_t N, double u01, double *u01seq);

/* ---------------------------------------------------------- resampling */
/* scheme numbering = vsmc::ResampleScheme (internal/defines.hpp:57-64):
 * Multinomial 0, Stratified 1, Systematic 2, Residual 3,
 * ResidualStratified 4, ResidualSystematic 5 */
void vo_resample_trans_u01_rep(size_t M, size_t N, const double *w,
    const double *u01, int *rep);
void vo_resample_trans_u01_index(size_t M, size_t N, const double *w,
    const double *u01, int *idx);
void vo_resample_trans_rep_index(size_t M, size_t N, const int *rep, int *idx);
void vo_resample_trans_index_rep(size_t M, size_t N, const int *idx, int *rep);
size_t vo_resample_trans_residual(
    size_t M, size_t N, const double *w, double *resid, int *integ);
void vo_resample(int scheme, size_t M, size_t N, vo_philox *eng,
    const double *w, int *rep);
void vo_resample_words(int scheme, size_t M, size_t N, const uint32_t key[2],
    const uint32_t ctr[4], const double *w, int *rep, uint32_t next_words[4]);
void vo_state_copy_f32(size_t N, const int *idx, float *state);
void vo_state_copy_f64(size_t N, const int *idx, double *state);

/* ------------------------------------------------------------- weights */
double vo_weight_set_log(size_t N, const double *lw, double *W);
double vo_weight_add_log(size_t N, const double *W0, const double *l, double *W);
double vo_weight_set(size_t N, const double *w, double *W);

/* ------------------------------------------------------ particle filter */
typedef struct {
    double dt, sigma_a, obs_scale, nu, sd_pos0, sd_vel0;
} vo_model;

void vo_pf_simulate(uint32_t seed, size_t T, const vo_model *m, double *truth,
    double *obs);
/* precision 64 or 32; threads <= 0 means all OpenMP threads.  Uses the
 * (key = {step, seed}, counter = {0, particle, 0, 0}) particle streams and a
 * resampling engine keyed {0, seed} starting at counter {0, 0, 1, 0}. */
/* vo_pf_run with the resampling replayed from a record: at step t with
 * resampled[t] set, particle i takes particle parents[t * N + i]'s state */
int vo_pf_run_replay(int precision, size_t N, size_t T, uint32_t seed,
    const vo_model *m, const double *obs, const int *resampled,
    const int *parents, double *mean_out, double *ess_out, double *logz_out);
int vo_pf_run(int precision, size_t N, size_t T, uint32_t seed, int scheme,
    double threshold, const vo_model *m, const double *obs, int threads,
    double *mean_out, double *ess_out, int *resampled_out, double *logz_out);

/* Move + log-likelihood for one step on given inputs (kernel-level parity):
 * state is SoA [4][N]; ll_out receives the log-likelihoods. */
void vo_pf_move_f64(size_t N, size_t t, uint32_t seed, const vo_model *m,
    const double obs[2], double *state, double *ll_out);
void vo_pf_move_f32(size_t N, size_t t, uint32_t seed, const vo_model *m,
    const double obs[2], float *state, float *ll_out);
void vo_pf_init_f64(size_t N, uint32_t seed, const vo_model *m,
    const double obs[2], double *state, double *ll_out);
void vo_pf_init_f32(size_t N, uint32_t seed, const vo_model *m,
    const double obs[2], float *state, float *ll_out);
double vo_student_t_norm_const(double nu, double s);

/* ---------------------------- bearings-only model, learned proposal */
/* project-written (no reference counterpart); see vsmc_oracle.c */
typedef struct {
    double dt, q, sigma_z, x0, y0, vx0, vy0, sd_pos0, sd_vel0;
} vo_bmodel;

void vo_bearings_simulate(
    uint32_t seed, size_t T, const vo_bmodel *m, double *truth, double *obs);
/* FP32 move + weight increment (params NULL: bootstrap) on SoA [4][N] */
void vo_bearings_move_f32(size_t N, size_t t, uint32_t seed,
    const vo_bmodel *m, double z, const float *params, float *state,
    float *lw_inc);
/* proposal network: forward (out[B][8]) and mean loss + gradient (FP64,
 * BF16 operand rounding as on the device) */
void vo_mlp_forward(const float *params, size_t B, const float *feat,
    float *out);
void vo_mlp_loss_grad(const float *params, size_t B, const float *feat,
    const float *nu, double *loss, double *grad);
/* 1 (default): device rounding (BF16 operands, FP32 values); 0: exact */
void vo_mlp_set_rounding(int on);
/* bearings filter: precision 64 (bootstrap, FP64 state) or 32 (FP32 state,
 * bootstrap or learned proposal with params) */
int vo_bearings_pf_run(int precision, size_t N, size_t T, uint32_t seed,
    int scheme, double threshold, const vo_bmodel *m, const double *obs,
    const float *params, int threads, double *mean_out, double *ess_out,
    int *resampled_out, double *logz_out);

/* resample-move: `sweeps` random-walk Metropolis steps on each particle's
 * acceleration innovation (parent: NULL = identity); *accepted += accepts */
void vo_cv_mcmc_f32(size_t N, size_t t, size_t sweeps, uint32_t seed,
    const vo_model *m, const double obs[2], double scale, const int *parent,
    float *state, uint32_t *accepted, float *margin);

/* ResampleIndex::index for every id at `iter`, and index_matrix (layout 0
 * row-major [N][iters], 1 column-major [iters][N]); rows: [iters][N] */
void vo_resample_index_trace(
    size_t N, size_t iters, const int *rows, size_t iter, int *out);
void vo_resample_index_matrix(
    size_t N, size_t iters, const int *rows, int layout, int *out);

/* test helper: k scalar words, then one bulk / u01 / normal batch operation */
void vo_engine_run(int kind, const uint64_t key[4], const uint64_t ctr[4],
    size_t k, int op, size_t n, double mean, double sd, void *out,
    uint64_t ctr_out[4], uint32_t *index_out);

#ifdef __cplusplus
}
#endif

#endif
