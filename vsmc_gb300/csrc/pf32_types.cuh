// Data layout of the FP32 filter step (device structs shared by the driver).
#pragma once

#include "common.cuh"
#include "pf_model.cuh"

namespace vsmc_cuda
{

constexpr int kPfBlock = 256;
constexpr int kPfTile = kPfBlock * 4; // particles per block iteration

// FP64 per-block record of the fused step
struct MovePartial {
    double sx, sy, sw; // previous-step monitor sums
    double m, s, s2;   // new log-weights: block max, sum exp, sum exp^2
};

// Device-resident filter scalars (one per filter)
struct PfScalars {
    double M;    // max of the stored log-weights after the last weighting
    double S;    // sum exp(lw - M)
    double logz; // cumulative log-evidence
    double ess;
    uint64_t Q;          // fixed-point CDF total of the pending resample
    uint32_t step;       // next step index t
    int32_t resampled;   // last step resampled: weights equal, lw stale
    int32_t gather;      // state must be read through idx (after a resample)
    uint32_t done;       // completion counter of the fused step
    uint32_t err;        // DEV_ERR_* bits
    uint32_t nempty;     // empty slots of the pending resample
    uint32_t rindex;     // resampling engine: next word index in gen(rctr)
    uint32_t rkey[2];
    uint32_t rctr[4];
    float Mf; // M as a float (the batched filters' kernels read it per tile)
};

// The state lives in two SoA buffers; a step reads one (A) and writes the
// other (B).  After a resample, A is read through the parent index idx.
struct Pf32Args {
    const float *ax, *ay, *avx, *avy; // state in
    float *bx, *by, *bvx, *bvy;       // state out
    float *lw;                        // log-weights (in place)
    const int32_t *idx;               // parent of each slot after a resample
    const uint32_t *srcs;             // sources of the empty slots, by rank
    uint32_t n;
    uint32_t seed;
    uint32_t max_steps; // history / observation capacity
    double threshold;
    CvConst<float> c;
    const double *obs; // T x 2 observations (device)
    MovePartial *part;
    PfScalars *sc;
    double *h_mean, *h_ess, *h_logz;
    int *h_res;
};

struct Rs32Args {
    const float *lw;
    const uint64_t *q; // integer weights given directly (lw unused), or null
    uint32_t n;
    uint32_t shift;  // fixed-point K
    uint32_t chunk;  // particles per block (multiple of kPfTile)
    int scheme;      // VSMC_CUDA_STRATIFIED or VSMC_CUDA_SYSTEMATIC
    uint64_t *qpart; // per-block sum of q
    uint32_t *epart; // per-block empty count
    uint32_t *cpart; // per-block copy count (sum of rep)
    uint32_t *mpart; // per-block max of marks
    int32_t *rep;
    int32_t *idx;      // per slot: itself (>= 0) or -(empty rank + 1)
    uint32_t *marks;   // N entries, zero between resamples
    uint32_t *srcs;    // N entries: source of the k-th empty slot
    PfScalars *sc;
};

} // namespace vsmc_cuda
