/* vsmc_oracle.c - CPU restatement of the vSMC particle-filter path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity oracle and the timed CPU baseline.
 * The product library never links or loads this file.
 *
 * Paths in citations are inside the vSMC source tree.  Build flags keep
 * a*b+c as two roundings (-ffp-contract=off), matching the x86 reference
 * build, on every host. */
#include "vsmc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define VO_PI 3.14159265358979323846
#define VO_PI_2 6.283185307179586476925286766559005768394
#define VO_PI_2F 6.283185307179586476925286766559005768394f

/* =====================================================================
 * Philox4x32-10  (rng/philox.hpp:76-101 constants, 212-232 round,
 * 162-188 key bump before rounds 2..10, 263-294 generator)
 * ===================================================================== */
void vo_philox4x32_block(
    const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t s0 = ctr[0], s1 = ctr[1], s2 = ctr[2], s3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 1; r <= 10; ++r) {
        if (r > 1) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t pa = (uint64_t)0xCD9E8D57u * s2;
        const uint64_t pb = (uint64_t)0xD2511F53u * s0;
        const uint32_t hi0 = (uint32_t)(pa >> 32) ^ k0;
        const uint32_t lo1 = (uint32_t)pa;
        const uint32_t hi2 = (uint32_t)(pb >> 32) ^ k1;
        const uint32_t lo3 = (uint32_t)pb;
        s0 = hi0 ^ s1;
        s1 = lo1;
        s2 = hi2 ^ s3;
        s3 = lo3;
    }
    out[0] = s0;
    out[1] = s1;
    out[2] = s2;
    out[3] = s3;
}

/* =====================================================================
 * Threefry4x64-20  (rng/threefry.hpp:71-82 parity constant, 130-146
 * rotations, 219-242 lane pairing, 279-298 key insertion every 4 rounds)
 * ===================================================================== */
static inline uint64_t vo_rotl64(uint64_t x, int r)
{
    return (x << r) | (x >> (64 - r));
}

void vo_threefry4x64_block(
    const uint64_t ctr[4], const uint64_t key[4], uint64_t out[4])
{
    static const int R[8][2] = {{14, 16}, {52, 57}, {23, 40}, {5, 37},
        {25, 33}, {46, 12}, {58, 22}, {32, 32}};
    uint64_t par[5];
    par[4] = 0x1BD11BDAA9FC1A22ull;
    for (int i = 0; i != 4; ++i) {
        par[i] = key[i];
        par[4] ^= key[i];
    }
    uint64_t s[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    for (int i = 0; i != 4; ++i)
        s[i] += par[i];
    for (int n = 1; n <= 20; ++n) {
        const int r = (n - 1) % 8;
        if (n % 2) {
            s[0] += s[1];
            s[1] = vo_rotl64(s[1], R[r][0]) ^ s[0];
            s[2] += s[3];
            s[3] = vo_rotl64(s[3], R[r][1]) ^ s[2];
        } else {
            s[0] += s[3];
            s[3] = vo_rotl64(s[3], R[r][0]) ^ s[0];
            s[2] += s[1];
            s[1] = vo_rotl64(s[1], R[r][1]) ^ s[2];
        }
        if (n % 4 == 0) {
            const int inc = n / 4;
            for (int i = 0; i != 4; ++i)
                s[i] += par[(inc + i) % 5];
            s[3] += (uint64_t)inc;
        }
    }
    for (int i = 0; i != 4; ++i)
        out[i] = s[i];
}

/* =====================================================================
 * CounterEngine  (rng/counter.hpp:43-93 increment, 230-262 bulk counter
 * blocks, 288-496 engine)
 * ===================================================================== */
#define VO_DEFINE_INCREMENT(T, name)                                          \
    static inline void name##_inc(T *c)                                       \
    {                                                                         \
        for (int i = 0; i != 4; ++i)                                          \
            if (++c[i] != 0)                                                  \
                return;                                                       \
    }                                                                         \
    /* increment(ctr, nskip) (counter.hpp:78-89): note the carry into limb 1  \
     * also fires when front + nskip == max exactly. */                      \
    static inline void name##_inc_skip(T *c, T nskip, T maxv)                 \
    {                                                                         \
        if (c[0] < maxv - nskip) {                                            \
            c[0] += nskip;                                                    \
        } else {                                                              \
            c[0] += nskip;                                                    \
            for (int i = 1; i != 4; ++i)                                      \
                if (++c[i] != 0)                                              \
                    break;                                                    \
        }                                                                     \
    }                                                                         \
    /* increment(ctr, n, ctr_block) (counter.hpp:230-262) */                 \
    static void name##_inc_blocks(T *ctr, size_t n, T *blocks, T maxv)        \
    {                                                                         \
        if (n == 0)                                                           \
            return;                                                           \
        name##_inc(ctr);                                                      \
        const uint64_t m = (uint64_t)maxv;                                    \
        const uint64_t l = (uint64_t)ctr[0];                                  \
        const uint64_t k = (uint64_t)n;                                       \
        if (k < m && l < m - k) {                                             \
            for (size_t i = 0; i != n; ++i) {                                 \
                memcpy(blocks + 4 * i, ctr, 4 * sizeof(T));                   \
                blocks[4 * i] += (T)i;                                        \
            }                                                                 \
        } else if (k < m) {                                                   \
            for (size_t i = 0; i != n; ++i) {                                 \
                memcpy(blocks + 4 * i, ctr, 4 * sizeof(T));                   \
                name##_inc_skip(blocks + 4 * i, (T)i, maxv);                  \
            }                                                                 \
        } else {                                                              \
            for (size_t i = 0; i != n; ++i) {                                 \
                memcpy(blocks + 4 * i, ctr, 4 * sizeof(T));                   \
                name##_inc(ctr);                                              \
            }                                                                 \
        }                                                                     \
        memcpy(ctr, blocks + 4 * (n - 1), 4 * sizeof(T));                     \
    }

VO_DEFINE_INCREMENT(uint32_t, vo_c32)
VO_DEFINE_INCREMENT(uint64_t, vo_c64)

void vo_philox_init(vo_philox *e, const uint32_t key[2], const uint32_t ctr[4])
{
    e->key[0] = key[0];
    e->key[1] = key[1];
    memcpy(e->ctr, ctr, sizeof(e->ctr));
    memset(e->buf, 0, sizeof(e->buf));
    e->index = 4;
}

uint32_t vo_philox_next(vo_philox *e)
{
    if (e->index == 4) {
        vo_c32_inc(e->ctr);
        vo_philox4x32_block(e->ctr, e->key, e->buf);
        e->index = 0;
    }
    return e->buf[e->index++];
}

/* CounterEngine::operator()(n, r) (counter.hpp:357-390): drain the buffer,
 * then generator calls of 256 blocks, one call for the remaining whole
 * blocks, then scalar draws for the last < 4 words. */
void vo_philox_rand(vo_philox *e, size_t n, uint32_t *r)
{
    const size_t remain = 4 - e->index;
    if (n < remain) {
        memcpy(r, e->buf + e->index, n * sizeof(uint32_t));
        e->index += (uint32_t)n;
        return;
    }
    memcpy(r, e->buf + e->index, remain * sizeof(uint32_t));
    r += remain;
    n -= remain;
    e->index = 4;
    const size_t k = 256;
    const size_t m = (n / 4) / k;
    const size_t l = (n / 4) % k;
    uint32_t *blocks = (uint32_t *)malloc(sizeof(uint32_t) * 4 * k);
    for (size_t c = 0; c != m + 1; ++c) {
        const size_t nb = c < m ? k : l;
        vo_c32_inc_blocks(e->ctr, nb, blocks, 0xFFFFFFFFu);
        for (size_t i = 0; i != nb; ++i)
            vo_philox4x32_block(blocks + 4 * i, e->key, r + 4 * i);
        r += 4 * nb;
        n -= 4 * nb;
    }
    free(blocks);
    for (size_t i = 0; i != n; ++i)
        r[i] = vo_philox_next(e);
}

void vo_threefry_init(
    vo_threefry *e, const uint64_t key[4], const uint64_t ctr[4])
{
    memcpy(e->key, key, sizeof(e->key));
    memcpy(e->ctr, ctr, sizeof(e->ctr));
    memset(e->buf, 0, sizeof(e->buf));
    e->index = 4;
}

uint64_t vo_threefry_next(vo_threefry *e)
{
    if (e->index == 4) {
        vo_c64_inc(e->ctr);
        vo_threefry4x64_block(e->ctr, e->key, e->buf);
        e->index = 0;
    }
    return e->buf[e->index++];
}

void vo_threefry_rand(vo_threefry *e, size_t n, uint64_t *r)
{
    const size_t remain = 4 - e->index;
    if (n < remain) {
        memcpy(r, e->buf + e->index, n * sizeof(uint64_t));
        e->index += (uint32_t)n;
        return;
    }
    memcpy(r, e->buf + e->index, remain * sizeof(uint64_t));
    r += remain;
    n -= remain;
    e->index = 4;
    const size_t k = 256;
    const size_t m = (n / 4) / k;
    const size_t l = (n / 4) % k;
    uint64_t *blocks = (uint64_t *)malloc(sizeof(uint64_t) * 4 * k);
    for (size_t c = 0; c != m + 1; ++c) {
        const size_t nb = c < m ? k : l;
        vo_c64_inc_blocks(e->ctr, nb, blocks, 0xFFFFFFFFFFFFFFFFull);
        for (size_t i = 0; i != nb; ++i)
            vo_threefry4x64_block(blocks + 4 * i, e->key, r + 4 * i);
        r += 4 * nb;
        n -= 4 * nb;
    }
    free(blocks);
    for (size_t i = 0; i != n; ++i)
        r[i] = vo_threefry_next(e);
}

void vo_philox4x32_words(const uint32_t key[2], const uint32_t ctr[4],
    size_t n, uint32_t *out, int bulk)
{
    vo_philox e;
    vo_philox_init(&e, key, ctr);
    if (bulk) {
        vo_philox_rand(&e, n, out);
    } else {
        for (size_t i = 0; i != n; ++i)
            out[i] = vo_philox_next(&e);
    }
}

void vo_threefry4x64_words(const uint64_t key[4], const uint64_t ctr[4],
    size_t n, uint64_t *out, int bulk)
{
    vo_threefry e;
    vo_threefry_init(&e, key, ctr);
    if (bulk) {
        vo_threefry_rand(&e, n, out);
    } else {
        for (size_t i = 0; i != n; ++i)
            out[i] = vo_threefry_next(&e);
    }
}

/* =====================================================================
 * u01 conversions  (rng/u01.hpp:77-172).  W = integer bits, M = real
 * mantissa bits; all scale factors are exact powers of two.
 * ===================================================================== */
#define VO_DEFINE_U01(UT, RT, W, M, name)                                     \
    RT name(int lr, UT u)                                                     \
    {                                                                         \
        if (lr == 0) { /* [0,1]: U01LRImpl<Closed,Closed> */                 \
            const int P = (W) - 1 < (M) ? (W) - 1 : (M);                      \
            const int V = P + 1;                                              \
            const int L = V < (W) ? 1 : 0;                                    \
            const int R = V < (W) ? (W) - 1 - V : 0;                          \
            const UT t = (UT)((UT)(u << L) >> (R + L));                       \
            RT v;                                                             \
            if (V < (W))                                                      \
                v = (RT)(UT)((t & 1) + t);                                    \
            else                                                              \
                v = (RT)(t & 1) + (RT)t;                                      \
            return v * (RT)ldexp(1.0, -(P + 1));                              \
        }                                                                     \
        if (lr == 1) { /* [0,1): Closed,Open */                              \
            const int P = (W) < (M) ? (W) : (M);                              \
            const int R = (W) - P;                                            \
            return (RT)(u >> R) * (RT)ldexp(1.0, -P);                         \
        }                                                                     \
        if (lr == 2) { /* (0,1]: Open,Closed */                              \
            const int P = (W) < (M) ? (W) : (M);                              \
            const int R = (W) - P;                                            \
            return (RT)(u >> R) * (RT)ldexp(1.0, -P) + (RT)ldexp(1.0, -P);    \
        }                                                                     \
        { /* (0,1): Open,Open */                                             \
            const int P = (W) + 1 < (M) ? (W) + 1 : (M);                      \
            const int R = (W) + 1 - P;                                        \
            return (RT)(u >> R) * (RT)ldexp(1.0, -(P - 1)) +                  \
                (RT)ldexp(1.0, -P);                                           \
        }                                                                     \
    }

VO_DEFINE_U01(uint32_t, double, 32, 53, vo_u01_u32_f64)
VO_DEFINE_U01(uint32_t, float, 32, 24, vo_u01_u32_f32)
VO_DEFINE_U01(uint64_t, double, 64, 53, vo_u01_u64_f64)
VO_DEFINE_U01(uint64_t, float, 64, 24, vo_u01_u64_f32)

void vo_u01_u32_f64_n(int lr, size_t n, const uint32_t *u, double *r)
{
    for (size_t i = 0; i != n; ++i)
        r[i] = vo_u01_u32_f64(lr, u[i]);
}

void vo_u01_u32_f32_n(int lr, size_t n, const uint32_t *u, float *r)
{
    for (size_t i = 0; i != n; ++i)
        r[i] = vo_u01_u32_f32(lr, u[i]);
}

void vo_u01_u64_f64_n(int lr, size_t n, const uint64_t *u, double *r)
{
    for (size_t i = 0; i != n; ++i)
        r[i] = vo_u01_u64_f64(lr, u[i]);
}

/* =====================================================================
 * Engine-generic draws.  U01Distribution picks a 32-bit integer for a
 * 32-bit engine and a 64-bit one otherwise (rng/u01_distribution.hpp:45-47,
 * 67-72); batch draws take words through the bulk path in 1024-word calls
 * (rng/u01_distribution.hpp:215-233).
 * ===================================================================== */
typedef struct {
    int kind; /* 0 Philox4x32, 1 Threefry4x64 */
    vo_philox p;
    vo_threefry t;
} vo_eng;

static void vo_eng_init(vo_eng *e, int kind, const uint64_t key[4],
    const uint64_t ctr[4])
{
    e->kind = kind;
    if (kind == 0) {
        uint32_t k[2] = {(uint32_t)key[0], (uint32_t)key[1]};
        uint32_t c[4] = {(uint32_t)ctr[0], (uint32_t)ctr[1],
            (uint32_t)ctr[2], (uint32_t)ctr[3]};
        vo_philox_init(&e->p, k, c);
    } else {
        vo_threefry_init(&e->t, key, ctr);
    }
}

static double vo_eng_u01d(vo_eng *e)
{
    if (e->kind == 0)
        return vo_u01_u32_f64(1, vo_philox_next(&e->p));
    return vo_u01_u64_f64(1, vo_threefry_next(&e->t));
}

static float vo_eng_u01f(vo_eng *e)
{
    if (e->kind == 0)
        return vo_u01_u32_f32(1, vo_philox_next(&e->p));
    return vo_u01_u64_f32(1, vo_threefry_next(&e->t));
}

/* one bulk call of n <= 1024 words turned into [0,1) reals */
static void vo_eng_u01d_bulk(vo_eng *e, size_t n, double *r)
{
    if (e->kind == 0) {
        uint32_t s[1024];
        vo_philox_rand(&e->p, n, s);
        for (size_t i = 0; i != n; ++i)
            r[i] = vo_u01_u32_f64(1, s[i]);
    } else {
        uint64_t s[1024];
        vo_threefry_rand(&e->t, n, s);
        for (size_t i = 0; i != n; ++i)
            r[i] = vo_u01_u64_f64(1, s[i]);
    }
}

static void vo_eng_u01f_bulk(vo_eng *e, size_t n, float *r)
{
    if (e->kind == 0) {
        uint32_t s[1024];
        vo_philox_rand(&e->p, n, s);
        for (size_t i = 0; i != n; ++i)
            r[i] = vo_u01_u32_f32(1, s[i]);
    } else {
        uint64_t s[1024];
        vo_threefry_rand(&e->t, n, s);
        for (size_t i = 0; i != n; ++i)
            r[i] = vo_u01_u64_f32(1, s[i]);
    }
}

/* u01_distribution (rng/u01_distribution.hpp:215-233) */
static void vo_u01_distribution_d(vo_eng *e, size_t n, double *r)
{
    const size_t k = 1024, m = n / k, l = n % k;
    for (size_t i = 0; i != m; ++i, r += k)
        vo_eng_u01d_bulk(e, k, r);
    vo_eng_u01d_bulk(e, l, r);
}

static void vo_u01_distribution_f(vo_eng *e, size_t n, float *r)
{
    const size_t k = 1024, m = n / k, l = n % k;
    for (size_t i = 0; i != m; ++i, r += k)
        vo_eng_u01f_bulk(e, k, r);
    vo_eng_u01f_bulk(e, l, r);
}

void vo_u01_dist_f64(int eng, const uint64_t key[4], const uint64_t ctr[4],
    size_t n, double *r, int batch)
{
    vo_eng e;
    vo_eng_init(&e, eng, key, ctr);
    if (batch) {
        vo_u01_distribution_d(&e, n, r);
    } else {
        for (size_t i = 0; i != n; ++i)
            r[i] = vo_eng_u01d(&e);
    }
}

void vo_u01_dist_f32(int eng, const uint64_t key[4], const uint64_t ctr[4],
    size_t n, float *r, int batch)
{
    vo_eng e;
    vo_eng_init(&e, eng, key, ctr);
    if (batch) {
        vo_u01_distribution_f(&e, n, r);
    } else {
        for (size_t i = 0; i != n; ++i)
            r[i] = vo_eng_u01f(&e);
    }
}

/* =====================================================================
 * Normal  (rng/normal_distribution.hpp:199-216 scalar with cached sine
 * value; 222-267 batch: per 1024-chunk the first half are radii, the second
 * half angles, out[0..nu) = sine branch, out[nu..2nu) = cosine branch, and
 * an odd total draws two extra scalar uniforms for the last element)
 * ===================================================================== */
typedef struct {
    double mean, sd, v;
    int saved;
} vo_normal_d;

static double vo_normal_d_draw(vo_normal_d *nd, vo_eng *e)
{
    double z;
    if (nd->saved) {
        z = nd->v;
        nd->saved = 0;
    } else {
        const double u1 = sqrt(-2 * log(vo_eng_u01d(e)));
        const double u2 = VO_PI_2 * vo_eng_u01d(e);
        z = u1 * cos(u2);
        nd->v = u1 * sin(u2);
        nd->saved = 1;
    }
    return nd->mean + nd->sd * z;
}

typedef struct {
    float mean, sd, v;
    int saved;
} vo_normal_f;

static float vo_normal_f_draw(vo_normal_f *nd, vo_eng *e)
{
    float z;
    if (nd->saved) {
        z = nd->v;
        nd->saved = 0;
    } else {
        const float u1 = sqrtf(-2 * logf(vo_eng_u01f(e)));
        const float u2 = VO_PI_2F * vo_eng_u01f(e);
        z = u1 * cosf(u2);
        nd->v = u1 * sinf(u2);
        nd->saved = 1;
    }
    return nd->mean + nd->sd * z;
}

static void vo_normal_impl_d(
    vo_eng *e, size_t n, double *r, double mean, double sd)
{
    double s[512];
    const size_t nu = n / 2;
    double *u1 = r, *u2 = r + nu;
    vo_u01_distribution_d(e, n, r);
    for (size_t i = 0; i != nu; ++i)
        s[i] = log(u1[i]);
    for (size_t i = 0; i != nu; ++i)
        s[i] = -2.0 * s[i];
    for (size_t i = 0; i != nu; ++i)
        s[i] = sqrt(s[i]);
    for (size_t i = 0; i != nu; ++i)
        u2[i] = VO_PI_2 * u2[i];
    for (size_t i = 0; i != nu; ++i) {
        const double a = u2[i];
        u1[i] = sin(a);
        u2[i] = cos(a);
    }
    for (size_t i = 0; i != nu; ++i)
        s[i] = sd * s[i];
    for (size_t i = 0; i != nu; ++i)
        u1[i] = s[i] * u1[i] + mean;
    for (size_t i = 0; i != nu; ++i)
        u2[i] = s[i] * u2[i] + mean;
}

static void vo_normal_impl_f(vo_eng *e, size_t n, float *r, float mean, float sd)
{
    float s[512];
    const size_t nu = n / 2;
    float *u1 = r, *u2 = r + nu;
    vo_u01_distribution_f(e, n, r);
    for (size_t i = 0; i != nu; ++i)
        s[i] = logf(u1[i]);
    for (size_t i = 0; i != nu; ++i)
        s[i] = -2.0f * s[i];
    for (size_t i = 0; i != nu; ++i)
        s[i] = sqrtf(s[i]);
    for (size_t i = 0; i != nu; ++i)
        u2[i] = VO_PI_2F * u2[i];
    for (size_t i = 0; i != nu; ++i) {
        const float a = u2[i];
        u1[i] = sinf(a);
        u2[i] = cosf(a);
    }
    for (size_t i = 0; i != nu; ++i)
        s[i] = sd * s[i];
    for (size_t i = 0; i != nu; ++i)
        u1[i] = s[i] * u1[i] + mean;
    for (size_t i = 0; i != nu; ++i)
        u2[i] = s[i] * u2[i] + mean;
}

void vo_normal_f64(int eng, const uint64_t key[4], const uint64_t ctr[4],
    size_t n, double mean, double sd, double *r, int batch)
{
    vo_eng e;
    vo_eng_init(&e, eng, key, ctr);
    /* NormalDistribution::operator()(rng, n, r) uses scalar draws below 100
     * (normal_distribution.hpp:122-131); callers here choose explicitly. */
    if (!batch) {
        vo_normal_d nd = {mean, sd, 0, 0};
        for (size_t i = 0; i != n; ++i)
            r[i] = vo_normal_d_draw(&nd, &e);
        return;
    }
    const size_t k = 1024, m = n / k, l = n % k;
    for (size_t i = 0; i != m; ++i, r += k)
        vo_normal_impl_d(&e, k, r, mean, sd);
    vo_normal_impl_d(&e, l, r, mean, sd);
    if (n % 2 != 0) {
        const double u = vo_eng_u01d(&e);
        const double v = vo_eng_u01d(&e);
        r[l - 1] = mean + sd * sqrt(-2 * log(u)) * cos(VO_PI_2 * v);
    }
}

void vo_normal_f32(int eng, const uint64_t key[4], const uint64_t ctr[4],
    size_t n, float mean, float sd, float *r, int batch)
{
    vo_eng e;
    vo_eng_init(&e, eng, key, ctr);
    if (!batch) {
        vo_normal_f nd = {mean, sd, 0, 0};
        for (size_t i = 0; i != n; ++i)
            r[i] = vo_normal_f_draw(&nd, &e);
        return;
    }
    const size_t k = 1024, m = n / k, l = n % k;
    for (size_t i = 0; i != m; ++i, r += k)
        vo_normal_impl_f(&e, k, r, mean, sd);
    vo_normal_impl_f(&e, l, r, mean, sd);
    if (n % 2 != 0) {
        const float u = vo_eng_u01f(&e);
        const float v = vo_eng_u01f(&e);
        r[l - 1] = mean + sd * sqrtf(-2 * logf(u)) * cosf(VO_PI_2F * v);
    }
}

/* =====================================================================
 * Gamma / chi-squared / Student-t, scalar forms
 * (rng/gamma_distribution.hpp:57-91 constants, 132-216 generators;
 * rng/chi_squared_distribution.hpp:64-78 = Gamma(n/2, 2);
 * rng/student_t_distribution.hpp:78-91: normal first, then chi-squared)
 * ===================================================================== */
enum { VO_GAMMA_T, VO_GAMMA_W, VO_GAMMA_N, VO_GAMMA_E };

typedef struct {
    double alpha, beta, d, c;
    int alg;
} vo_gamma;

static void vo_gamma_init(vo_gamma *g, double alpha, double beta)
{
    g->alpha = alpha;
    g->beta = beta;
    if (alpha < 0.6)
        g->alg = VO_GAMMA_T;
    else if (alpha < 1)
        g->alg = VO_GAMMA_W;
    else if (alpha > 1)
        g->alg = VO_GAMMA_N;
    else
        g->alg = VO_GAMMA_E;
    g->d = g->c = 0;
    switch (g->alg) {
        case VO_GAMMA_T:
            g->d = 1 - alpha;
            g->c = 1 / alpha;
            break;
        case VO_GAMMA_W:
            g->d = pow(alpha, alpha / (1 - alpha)) * (1 - alpha);
            g->c = 1 / alpha;
            break;
        case VO_GAMMA_N:
            g->d = alpha - 1.0 / 3;
            g->c = 1 / (3 * sqrt(g->d));
            break;
        default: break;
    }
}

static double vo_gamma_draw(const vo_gamma *g, vo_eng *e)
{
    double r = 0;
    switch (g->alg) {
        case VO_GAMMA_T:
            for (;;) {
                double u = vo_eng_u01d(e);
                double ee = -log(vo_eng_u01d(e));
                if (u > g->d) {
                    u = -log(g->c * (1 - u));
                    ee += u;
                    u = g->d + g->alpha * u;
                }
                const double x = exp(g->c * log(u));
                if (fabs(x) < ee) {
                    r = x;
                    break;
                }
            }
            break;
        case VO_GAMMA_W: {
            double u, ee, x;
            do {
                u = -log(vo_eng_u01d(e));
                ee = -log(vo_eng_u01d(e));
                x = exp(g->c * log(u));
            } while (u + ee < g->d + x);
            r = x;
            break;
        }
        case VO_GAMMA_N: {
            vo_normal_d rnorm = {0, 1, 0, 0};
            for (;;) {
                const double u = vo_eng_u01d(e);
                double w, v;
                do {
                    w = vo_normal_d_draw(&rnorm, e);
                    v = 1 + g->c * w;
                } while (v <= 0);
                v = v * v * v;
                double ee = 1 - 0.0331 * (w * w) * (w * w);
                if (u < ee) {
                    r = g->d * v;
                    break;
                }
                ee = w * w / 2 + g->d * (1 - v + log(v));
                if (log(u) < ee) {
                    r = g->d * v;
                    break;
                }
            }
            break;
        }
        default: r = -log(vo_eng_u01d(e)); break;
    }
    return g->beta * r;
}

void vo_student_t_f64(int eng, const uint64_t key[4], const uint64_t ctr[4],
    size_t n, double df, double *r)
{
    vo_eng e;
    vo_eng_init(&e, eng, key, ctr);
    vo_normal_d nd = {0, 1, 0, 0};
    vo_gamma g;
    vo_gamma_init(&g, df / 2, 2);
    for (size_t i = 0; i != n; ++i) {
        const double z = vo_normal_d_draw(&nd, &e);
        const double u = df / vo_gamma_draw(&g, &e);
        r[i] = z * sqrt(u);
    }
}

/* =====================================================================
 * Student-t, batch form  (rng/student_t_distribution.hpp:97-128, which the
 * C ABI's vsmc_rng_student_t calls, lib/src/vsmc_rng.cpp:41-64, 207): per
 * chunk of at most 1024 variates, chi-squared = Gamma(df/2, 2) by the batch
 * gamma (rng/gamma_distribution.hpp:230-410: one vectorised attempt of the
 * chunk, the accepted values packed in order, then scalar draws for the
 * rest), r = sqrt(r * (1/df)), a batch of normals z, r = z / r.
 * ===================================================================== */

/* one vectorised gamma attempt over n <= 1024 values; returns how many were
 * accepted (rng/gamma_distribution.hpp:230-355) */
static size_t vo_gamma_batch_once(
    const vo_gamma *g, vo_eng *e, size_t n, double *r)
{
    static double s[5 * 1024];
    const double d = g->d, c = g->c, beta = g->beta;
    size_t m = 0;
    if (g->alg == VO_GAMMA_T) {
        double *u = s, *ee = s + n, *x = s + 2 * n;
        vo_u01_distribution_d(e, 2 * n, s);
        for (size_t i = 0; i != n; ++i)
            ee[i] = log(ee[i]);
        for (size_t i = 0; i != n; ++i)
            ee[i] = -1.0 * ee[i];
        for (size_t i = 0; i != n; ++i) {
            if (u[i] > d) {
                u[i] = -log(c * (1 - u[i]));
                ee[i] += u[i];
                u[i] = d + g->alpha * u[i];
            }
        }
        for (size_t i = 0; i != n; ++i)
            x[i] = log(u[i]);
        for (size_t i = 0; i != n; ++i)
            x[i] = c * x[i];
        for (size_t i = 0; i != n; ++i)
            x[i] = exp(x[i]);
        for (size_t i = 0; i != n; ++i)
            u[i] = fabs(x[i]);
        for (size_t i = 0; i != n; ++i)
            x[i] = beta * x[i];
        for (size_t i = 0; i != n; ++i)
            if (u[i] < ee[i])
                r[m++] = x[i];
    } else if (g->alg == VO_GAMMA_W) {
        double *u = s, *ee = s + n, *x = s + 2 * n;
        vo_u01_distribution_d(e, 2 * n, s);
        for (size_t i = 0; i != 2 * n; ++i)
            s[i] = log(s[i]);
        for (size_t i = 0; i != 2 * n; ++i)
            s[i] = -1.0 * s[i];
        for (size_t i = 0; i != n; ++i)
            x[i] = log(s[i]);
        for (size_t i = 0; i != n; ++i)
            x[i] = c * x[i];
        for (size_t i = 0; i != n; ++i)
            x[i] = exp(x[i]);
        for (size_t i = 0; i != n; ++i)
            u[i] = u[i] + ee[i];
        for (size_t i = 0; i != n; ++i)
            ee[i] = d + x[i];
        for (size_t i = 0; i != n; ++i)
            x[i] = beta * x[i];
        for (size_t i = 0; i != n; ++i)
            if (u[i] > ee[i])
                r[m++] = x[i];
    } else if (g->alg == VO_GAMMA_N) {
        double *u = s, *ee = s + n, *v = s + 2 * n, *w = s + 3 * n,
               *x = s + 4 * n;
        vo_u01_distribution_d(e, n, u);
        vo_normal_impl_d(e, n, w, 0, 1);
        if (n % 2 != 0) { /* normal_distribution's odd tail */
            const double a = vo_eng_u01d(e);
            const double b = vo_eng_u01d(e);
            w[n - 1] = 0 + 1 * sqrt(-2 * log(a)) * cos(VO_PI_2 * b);
        }
        for (size_t i = 0; i != n; ++i)
            v[i] = c * w[i] + 1;
        vo_normal_d rnorm = {0, 1, 0, 0};
        for (size_t i = 0; i != n; ++i) {
            if (v[i] <= 0) {
                do {
                    w[i] = vo_normal_d_draw(&rnorm, e);
                    v[i] = 1 + c * w[i];
                } while (v[i] <= 0);
            }
        }
        for (size_t i = 0; i != n; ++i)
            ee[i] = v[i] * v[i];
        for (size_t i = 0; i != n; ++i)
            v[i] = v[i] * ee[i];
        for (size_t i = 0; i != n; ++i)
            ee[i] = w[i] * w[i];
        for (size_t i = 0; i != n; ++i)
            ee[i] = ee[i] * ee[i];
        for (size_t i = 0; i != n; ++i)
            ee[i] = -0.0331 * ee[i] + 1;
        const double db = d * beta;
        for (size_t i = 0; i != n; ++i)
            x[i] = db * v[i];
        for (size_t i = 0; i != n; ++i) {
            if (u[i] < ee[i]) {
                r[m++] = x[i];
            } else {
                ee[i] = w[i] * w[i] / 2 + d * (1 - v[i] + log(v[i]));
                if (log(u[i]) < ee[i])
                    r[m++] = x[i];
            }
        }
    } else {
        vo_u01_distribution_d(e, n, r);
        for (size_t i = 0; i != n; ++i)
            r[i] = log(r[i]);
        for (size_t i = 0; i != n; ++i)
            r[i] = -beta * r[i];
        m = n;
    }
    return m;
}

/* The engine placed at (key, ctr) with an exhausted buffer, `skip` words
 * drawn through the scalar path, then student_t_distribution(rng, n, r, df).
 * The engine's counter and buffer index afterwards go to ctr_out /
 * index_out (either may be NULL). */
void vo_student_t_batch_f64(int eng, const uint64_t key[4],
    const uint64_t ctr[4], size_t skip, size_t n, double df, double *r,
    uint64_t ctr_out[4], uint32_t *index_out)
{
    vo_eng e;
    vo_eng_init(&e, eng, key, ctr);
    for (size_t i = 0; i != skip; ++i)
        (void)vo_eng_u01d(&e);
    vo_gamma g;
    vo_gamma_init(&g, df / 2, 2);
    double z[1024];
    for (size_t base = 0; base < n; base += 1024) {
        const size_t k = n - base < 1024 ? n - base : 1024;
        double *rr = r + base;
        const size_t m = vo_gamma_batch_once(&g, &e, k, rr);
        for (size_t i = m; i < k; ++i)
            rr[i] = vo_gamma_draw(&g, &e);
        const double inv = 1 / df;
        for (size_t i = 0; i != k; ++i)
            rr[i] = inv * rr[i];
        for (size_t i = 0; i != k; ++i)
            rr[i] = sqrt(rr[i]);
        vo_normal_impl_d(&e, k, z, 0, 1);
        if (k % 2 != 0) {
            const double a = vo_eng_u01d(&e);
            const double b = vo_eng_u01d(&e);
            z[k - 1] = 0 + 1 * sqrt(-2 * log(a)) * cos(VO_PI_2 * b);
        }
        for (size_t i = 0; i != k; ++i)
            rr[i] = z[i] / rr[i];
    }
    if (ctr_out) {
        for (int i = 0; i < 4; ++i)
            ctr_out[i] = eng == 0 ? e.p.ctr[i] : e.t.ctr[i];
    }
    if (index_out)
        *index_out = eng == 0 ? e.p.index : e.t.index;
}

/* =====================================================================
 * u01 sequences  (rng/u01_sequence.hpp:53-89 array forms; 131-259 lazy
 * classes: only indices that are read consume engine words)
 * ===================================================================== */
void vo_u01_sorted(size_t N, const double *u01, double *u01seq)
{
    for (size_t i = 0; i != N; ++i)
        u01seq[i] = log(u01[i]);
    double lmax = 0;
    for (size_t i = 0; i != N; ++i) {
        lmax += u01seq[i] / (double)(N - i);
        u01seq[i] = 1 - exp(lmax);
    }
}

void vo_u01_stratified(size_t N, const double *u01, double *u01seq)
{
    const double delta = 1 / (double)N;
    for (size_t i = 0; i != N; ++i)
        u01seq[i] = u01[i] * delta + (double)i * delta;
}

void vo_u01_systematic(size_t N, double u01, double *u01seq)
{
    if (N == 0)
        return;
    const double delta = 1.0 / (double)N;
    u01seq[0] = u01 * delta;
    for (size_t i = 1; i != N; ++i)
        u01seq[i] = u01seq[i - 1] + delta;
}

typedef struct {
    int kind; /* 0 sorted, 1 stratified, 2 systematic, 3 array */
    size_t N, n;
    double u, lmax, delta, u0;
    vo_philox *rng;
    const double *arr;
} vo_seq;

static void vo_seq_init(vo_seq *s, int kind, size_t N, vo_philox *rng)
{
    s->kind = kind;
    s->N = N;
    s->n = N;
    s->u = 0;
    s->lmax = 0;
    s->u0 = 0;
    s->rng = rng;
    s->arr = NULL;
    s->delta = 1 / (double)N;
    if (kind == 2)
        s->u0 = vo_u01_u32_f64(1, vo_philox_next(rng)) * s->delta;
}

static double vo_seq_get(vo_seq *s, size_t n)
{
    if (s->kind == 3)
        return s->arr[n];
    if (n == s->n)
        return s->u;
    s->n = n;
    if (s->kind == 0) {
        s->lmax += log(vo_u01_u32_f64(1, vo_philox_next(s->rng))) /
            (double)(s->N - n);
        s->u = 1 - exp(s->lmax);
    } else if (s->kind == 1) {
        s->u = vo_u01_u32_f64(1, vo_philox_next(s->rng)) * s->delta +
            (double)n * s->delta;
    } else {
        s->u = s->u0 + (double)n * s->delta;
    }
    return s->u;
}

void vo_u01_sequence(int kind, size_t N, const uint32_t key[2],
    const uint32_t ctr[4], double *out, uint32_t next_words[4])
{
    vo_philox e;
    vo_philox_init(&e, key, ctr);
    vo_seq s;
    vo_seq_init(&s, kind, N, &e);
    for (size_t i = 0; i != N; ++i)
        out[i] = vo_seq_get(&s, i);
    for (int i = 0; i != 4; ++i)
        next_words[i] = vo_philox_next(&e);
}

/* =====================================================================
 * Resampling transforms  (resample/transform.hpp:43-71 u01 -> rep,
 * 75-96 u01 -> index, 100-134 rep -> index, 138-150 index -> rep,
 * 155-168 residual)
 * ===================================================================== */
static void vo_trans_u01_rep_seq(
    size_t M, size_t N, const double *w, vo_seq *u01seq, int *rep)
{
    if (M == 0)
        return;
    if (M == 1) {
        *rep = (int)N;
        return;
    }
    memset(rep, 0, sizeof(int) * M);
    if (N == 0)
        return;
    double accw = 0;
    size_t j = 0;
    for (size_t i = 0; i != M - 1; ++i) {
        accw += w[i];
        while (j != N && vo_seq_get(u01seq, j) <= accw) {
            ++rep[i];
            ++j;
        }
    }
    rep[M - 1] = (int)(N - j);
}

void vo_resample_trans_u01_rep(
    size_t M, size_t N, const double *w, const double *u01, int *rep)
{
    vo_seq s;
    memset(&s, 0, sizeof(s));
    s.kind = 3;
    s.arr = u01;
    vo_trans_u01_rep_seq(M, N, w, &s, rep);
}

void vo_resample_trans_u01_index(
    size_t M, size_t N, const double *w, const double *u01, int *idx)
{
    if (M == 0 || N == 0)
        return;
    memset(idx, 0, sizeof(int) * N);
    if (M == 1)
        return;
    double accw = 0;
    size_t j = 0;
    for (size_t i = 0; i != M - 1; ++i) {
        accw += w[i];
        while (j != N && u01[j] <= accw)
            idx[j++] = (int)i;
    }
    while (j != N)
        idx[j++] = (int)(M - 1);
}

void vo_resample_trans_rep_index(size_t M, size_t N, const int *rep, int *idx)
{
    if (M == 0 || N == 0)
        return;
    if (M != N) {
        size_t dst = 0;
        for (size_t src = 0; src != M; ++src)
            for (int r = 0; r != rep[src]; ++r)
                idx[dst++] = (int)src;
        return;
    }
    int time = 0;
    size_t src = 0;
    for (size_t dst = 0; dst != N; ++dst) {
        if (rep[dst] != 0) {
            idx[dst] = (int)dst;
        } else {
            if (rep[src] < time + 2) {
                time = 0;
                do
                    ++src;
                while (rep[src] < 2);
            }
            idx[dst] = (int)src;
            ++time;
        }
    }
}

void vo_resample_trans_index_rep(size_t M, size_t N, const int *idx, int *rep)
{
    if (M == 0 || N == 0)
        return;
    memset(rep, 0, sizeof(int) * M);
    for (size_t i = 0; i != N; ++i)
        ++rep[idx[i]];
}

size_t vo_resample_trans_residual(
    size_t M, size_t N, const double *w, double *resid, int *integ)
{
    double integral = 0;
    const double coeff = (double)N;
    for (size_t i = 0; i != M; ++i) {
        resid[i] = modf(coeff * w[i], &integral);
        integ[i] = (int)integral;
    }
    double acc = 0;
    for (size_t i = 0; i != M; ++i)
        acc += resid[i];
    const double inv = 1 / acc;
    for (size_t i = 0; i != M; ++i)
        resid[i] = inv * resid[i];
    int R = 0;
    for (size_t i = 0; i != M; ++i)
        R += integ[i];
    return N - (size_t)R;
}

/* scheme functors (resample/multinomial.hpp:46-52, stratified.hpp:46-52,
 * systematic.hpp:46-52, residual*.hpp:46-57) */
void vo_resample(int scheme, size_t M, size_t N, vo_philox *eng,
    const double *w, int *rep)
{
    if (scheme <= 2) { /* Multinomial, Stratified, Systematic */
        const int kind = scheme;
        vo_seq s;
        vo_seq_init(&s, kind, N, eng);
        vo_trans_u01_rep_seq(M, N, w, &s, rep);
        return;
    }
    int *integ = (int *)malloc(sizeof(int) * (M ? M : 1));
    double *resid = (double *)malloc(sizeof(double) * (M ? M : 1));
    const size_t R = vo_resample_trans_residual(M, N, w, resid, integ);
    const int kind = scheme - 3; /* Residual, ResidualStratified, ResidualSystematic */
    vo_seq s;
    vo_seq_init(&s, kind, R, eng);
    vo_trans_u01_rep_seq(M, R, resid, &s, rep);
    for (size_t i = 0; i != M; ++i)
        rep[i] = rep[i] + integ[i];
    free(integ);
    free(resid);
}

void vo_resample_words(int scheme, size_t M, size_t N, const uint32_t key[2],
    const uint32_t ctr[4], const double *w, int *rep, uint32_t next_words[4])
{
    vo_philox e;
    vo_philox_init(&e, key, ctr);
    vo_resample(scheme, M, N, &e, w, rep);
    for (int i = 0; i != 4; ++i)
        next_words[i] = vo_philox_next(&e);
}

/* StateMatrix<ColMajor,Dim,T>::copy (core/state_matrix.hpp:357-364) */
void vo_state_copy_f32(size_t N, const int *idx, float *state)
{
    for (size_t d = 0; d != 4; ++d)
        for (size_t dst = 0; dst != N; ++dst)
            state[d * N + dst] = state[d * N + (size_t)idx[dst]];
}

void vo_state_copy_f64(size_t N, const int *idx, double *state)
{
    for (size_t d = 0; d != 4; ++d)
        for (size_t dst = 0; dst != N; ++dst)
            state[d * N + dst] = state[d * N + (size_t)idx[dst]];
}

/* =====================================================================
 * Weight  (core/weight.hpp:41-63 helpers, 99-103 set_equal, 145-149
 * set_log, 168-173 add_log, 202-230 normalize: exp and a running sum in
 * 1024-element chunks, scale by 1/sum, ESS = 1/dot(W, W))
 * ===================================================================== */
static double vo_weight_normalize(size_t N, double *w, int use_log)
{
    double accw = 0;
    for (size_t i = 0; i != N; ++i) {
        if (use_log)
            w[i] = exp(w[i]);
        accw = accw + w[i];
    }
    const double inv = 1 / accw;
    for (size_t i = 0; i != N; ++i)
        w[i] = inv * w[i];
    double dot = 0;
    for (size_t i = 0; i != N; ++i)
        dot += w[i] * w[i];
    return 1 / dot;
}

static double vo_weight_post_set_log(size_t N, double *w)
{
    double wmax = w[0];
    for (size_t i = 1; i < N; ++i)
        if (wmax < w[i])
            wmax = w[i];
    for (size_t i = 0; i != N; ++i)
        w[i] -= wmax;
    return vo_weight_normalize(N, w, 1);
}

static double vo_weight_set_equal(size_t N, double *W)
{
    const double v = 1.0 / (double)N;
    for (size_t i = 0; i != N; ++i)
        W[i] = v;
    return vo_weight_normalize(N, W, 0);
}

double vo_weight_set_log(size_t N, const double *lw, double *W)
{
    memcpy(W, lw, sizeof(double) * N);
    return vo_weight_post_set_log(N, W);
}

double vo_weight_add_log(size_t N, const double *W0, const double *l, double *W)
{
    memcpy(W, W0, sizeof(double) * N);
    vo_weight_normalize(N, W, 0); /* Weight::set(W0) */
    for (size_t i = 0; i != N; ++i)
        W[i] = log(W[i]);
    for (size_t i = 0; i != N; ++i)
        W[i] = W[i] + l[i];
    return vo_weight_post_set_log(N, W);
}

double vo_weight_set(size_t N, const double *w, double *W)
{
    memcpy(W, w, sizeof(double) * N);
    return vo_weight_normalize(N, W, 0);
}

/* =====================================================================
 * Particle filter: constant-velocity model, Student-t position
 * observations, in the example/pf/include/pf.hpp:70-193 form, driven in
 * the Sampler order (core/sampler.hpp:443-476, 735-785): weight, record
 * ESS, resample if ESS < threshold * N (core/particle.hpp:170-197), then the
 * weighted position mean (core/monitor.hpp:242-268, MonitorMCMC stage).
 * The log-evidence increment log sum_i W_{t-1,i} exp(l_{t,i}) follows
 * user_guide/tex/smc.tex:176-182.
 * ===================================================================== */
double vo_student_t_norm_const(double nu, double s)
{
    return lgamma(0.5 * (nu + 1)) - lgamma(0.5 * nu) - 0.5 * log(nu * VO_PI) -
        log(s);
}

static inline void vo_particle_engine(
    vo_philox *e, size_t t, uint32_t seed, size_t id)
{
    const uint32_t key[2] = {(uint32_t)t, seed};
    const uint32_t ctr[4] = {0, (uint32_t)id, 0, 0};
    vo_philox_init(e, key, ctr);
}

static inline void vo_pair_d(vo_philox *p, double sd, double *z1, double *z2)
{
    vo_eng e;
    e.kind = 0;
    e.p = *p;
    vo_normal_d nd = {0, sd, 0, 0};
    *z1 = vo_normal_d_draw(&nd, &e);
    *z2 = vo_normal_d_draw(&nd, &e);
    *p = e.p;
}

/* FP32 pair: Box-Muller with the (0,1] u01_oc radius uniform */
static inline void vo_pair_f(vo_philox *p, float sd, float *z1, float *z2)
{
    const uint32_t w0 = vo_philox_next(p);
    const uint32_t w1 = vo_philox_next(p);
    const float u1 = vo_u01_u32_f32(2, w0);
    const float u2 = vo_u01_u32_f32(1, w1);
    const float r = sqrtf(-2 * logf(u1));
    const float th = VO_PI_2F * u2;
    *z1 = sd * (r * cosf(th));
    *z2 = sd * (r * sinf(th));
}

#define VO_DEFINE_PF_KERNELS(T, SFX, PAIR, LOG1P, CAST)                       \
    static inline T vo_ll_##SFX(const vo_model *m, const double obs[2], T x,  \
        T y)                                                                  \
    {                                                                         \
        const T c2 = (T)(2 * vo_student_t_norm_const(m->nu, m->obs_scale));   \
        const T inv_s = (T)(1 / m->obs_scale);                                \
        const T inv_nu = (T)(1 / m->nu);                                      \
        const T half_nu1 = (T)(0.5 * (m->nu + 1));                            \
        const T zx = ((T)obs[0] - x) * inv_s;                                 \
        const T zy = ((T)obs[1] - y) * inv_s;                                 \
        const T qx = zx * zx * inv_nu;                                        \
        const T qy = zy * zy * inv_nu;                                        \
        return c2 - half_nu1 * (LOG1P(qx) + LOG1P(qy));                       \
    }                                                                         \
    void vo_pf_init_##SFX(size_t N, uint32_t seed, const vo_model *m,         \
        const double obs[2], T *state, T *ll_out)                             \
    {                                                                         \
        _Pragma("omp parallel for schedule(static)")                          \
        for (size_t i = 0; i < N; ++i) {                                      \
            vo_philox e;                                                      \
            vo_particle_engine(&e, 0, seed, i);                               \
            T x, y, vx, vy;                                                   \
            PAIR(&e, (T)m->sd_pos0, &x, &y);                                  \
            PAIR(&e, (T)m->sd_vel0, &vx, &vy);                                \
            state[0 * N + i] = x;                                             \
            state[1 * N + i] = y;                                             \
            state[2 * N + i] = vx;                                            \
            state[3 * N + i] = vy;                                            \
            ll_out[i] = vo_ll_##SFX(m, obs, x, y);                            \
        }                                                                     \
    }                                                                         \
    void vo_pf_move_##SFX(size_t N, size_t t, uint32_t seed,                  \
        const vo_model *m, const double obs[2], T *state, T *ll_out)          \
    {                                                                         \
        const T dt = (T)m->dt;                                                \
        const T h = (T)(0.5 * m->dt * m->dt);                                 \
        _Pragma("omp parallel for schedule(static)")                          \
        for (size_t i = 0; i < N; ++i) {                                      \
            vo_philox e;                                                      \
            vo_particle_engine(&e, t, seed, i);                               \
            T ax, ay;                                                         \
            PAIR(&e, (T)m->sigma_a, &ax, &ay);                                \
            const T x = state[0 * N + i], y = state[1 * N + i];               \
            const T vx = state[2 * N + i], vy = state[3 * N + i];             \
            const T nx = x + dt * vx + h * ax;                                \
            const T ny = y + dt * vy + h * ay;                                \
            state[0 * N + i] = nx;                                            \
            state[1 * N + i] = ny;                                            \
            state[2 * N + i] = vx + dt * ax;                                  \
            state[3 * N + i] = vy + dt * ay;                                  \
            ll_out[i] = vo_ll_##SFX(m, obs, nx, ny);                          \
        }                                                                     \
    }

VO_DEFINE_PF_KERNELS(double, f64, vo_pair_d, log1p, double)
VO_DEFINE_PF_KERNELS(float, f32, vo_pair_f, log1pf, float)

void vo_pf_simulate(
    uint32_t seed, size_t T, const vo_model *m, double *truth, double *obs)
{
    /* CounterEngine(seed): key {seed, 0}, counter 0 */
    vo_eng e;
    e.kind = 0;
    const uint32_t key[2] = {seed, 0};
    const uint32_t ctr[4] = {0, 0, 0, 0};
    vo_philox_init(&e.p, key, ctr);
    vo_normal_d st_normal = {0, 1, 0, 0};
    vo_gamma st_gamma;
    vo_gamma_init(&st_gamma, m->nu / 2, 2);
    double x, y, vx, vy;
    vo_pair_d(&e.p, m->sd_pos0, &x, &y);
    vo_pair_d(&e.p, m->sd_vel0, &vx, &vy);
    const double h = 0.5 * m->dt * m->dt;
    for (size_t t = 0; t != T; ++t) {
        if (t > 0) {
            double ax, ay;
            vo_pair_d(&e.p, m->sigma_a, &ax, &ay);
            x = x + m->dt * vx + h * ax;
            y = y + m->dt * vy + h * ay;
            vx = vx + m->dt * ax;
            vy = vy + m->dt * ay;
        }
        truth[4 * t + 0] = x;
        truth[4 * t + 1] = y;
        truth[4 * t + 2] = vx;
        truth[4 * t + 3] = vy;
        double ex, ey;
        {
            const double z = vo_normal_d_draw(&st_normal, &e);
            ex = z * sqrt(m->nu / vo_gamma_draw(&st_gamma, &e));
        }
        {
            const double z = vo_normal_d_draw(&st_normal, &e);
            ey = z * sqrt(m->nu / vo_gamma_draw(&st_gamma, &e));
        }
        obs[2 * t + 0] = x + m->obs_scale * ex;
        obs[2 * t + 1] = y + m->obs_scale * ey;
    }
}

/* Particle::resample + Sampler::do_resample; returns 1 if resampled */
static int vo_pf_resample(int scheme, double threshold, size_t N,
    vo_philox *reng, double *W, double *ess, int *rep, int *idx,
    void *state, int precision)
{
    const int resampled = *ess < threshold * (double)N;
    if (resampled) {
        vo_resample(scheme, N, N, reng, W, rep);
        vo_resample_trans_rep_index(N, N, rep, idx);
        if (precision == 32) {
            float *s = (float *)state;
            _Pragma("omp parallel for schedule(static)")
            for (size_t i = 0; i < N; ++i)
                for (size_t d = 0; d != 4; ++d)
                    s[d * N + i] = s[d * N + (size_t)idx[i]];
        } else {
            double *s = (double *)state;
            _Pragma("omp parallel for schedule(static)")
            for (size_t i = 0; i < N; ++i)
                for (size_t d = 0; d != 4; ++d)
                    s[d * N + i] = s[d * N + (size_t)idx[i]];
        }
        *ess = vo_weight_set_equal(N, W);
    }
    return resampled;
}

static void vo_pf_mean(size_t N, const void *state, int precision,
    const double *W, double out[2])
{
    for (size_t d = 0; d != 2; ++d) {
        double s = 0;
        if (precision == 32) {
            const float *st = (const float *)state + d * N;
            for (size_t i = 0; i != N; ++i)
                s += (double)st[i] * W[i];
        } else {
            const double *st = (const double *)state + d * N;
            for (size_t i = 0; i != N; ++i)
                s += st[i] * W[i];
        }
        out[d] = s;
    }
}

/* The filter of vo_pf_run with its resampling replayed from a record
 * instead of drawn (core/sampler.hpp:772-778 with the op's indices given):
 * at step t with resampled[t] set, particle i takes the state of particle
 * parents[t * N + i] and the weights become equal (core/particle.hpp:
 * 186-193).  With a device run's recorded decisions and genealogy rows this
 * isolates the move, weight, evidence and monitor arithmetic from the
 * resampler, step by step. */
int vo_pf_run_replay(int precision, size_t N, size_t T, uint32_t seed,
    const vo_model *m, const double *obs, const int *resampled,
    const int *parents, double *mean_out, double *ess_out, double *logz_out)
{
    const size_t esz = precision == 32 ? sizeof(float) : sizeof(double);
    void *state = malloc(esz * 4 * N);
    void *tmp = malloc(esz * 4 * N);
    double *W = (double *)malloc(sizeof(double) * N);
    double *ll = (double *)malloc(sizeof(double) * N);
    float *llf = (float *)malloc(sizeof(float) * N);
    double ess = vo_weight_set_equal(N, W);
    double logz = 0;
    for (size_t t = 0; t != T; ++t) {
        if (precision == 32) {
            if (t == 0)
                vo_pf_init_f32(N, seed, m, obs, (float *)state, llf);
            else
                vo_pf_move_f32(N, t, seed, m, obs + 2 * t, (float *)state, llf);
            for (size_t i = 0; i != N; ++i)
                ll[i] = (double)llf[i];
        } else {
            if (t == 0)
                vo_pf_init_f64(N, seed, m, obs, (double *)state, ll);
            else
                vo_pf_move_f64(N, t, seed, m, obs + 2 * t, (double *)state, ll);
        }
        double mx = -INFINITY;
        for (size_t i = 0; i != N; ++i)
            if (mx < ll[i])
                mx = ll[i];
        double s = 0;
        if (t == 0) {
            for (size_t i = 0; i != N; ++i)
                s += exp(ll[i] - mx);
            logz += mx + log(s / (double)N);
            ess = vo_weight_set_log(N, ll, W);
        } else {
            for (size_t i = 0; i != N; ++i)
                s += W[i] * exp(ll[i] - mx);
            logz += mx + log(s);
            for (size_t i = 0; i != N; ++i)
                W[i] = log(W[i]) + ll[i];
            ess = vo_weight_post_set_log(N, W);
        }
        logz_out[t] = logz;
        ess_out[t] = ess;
        if (resampled[t]) {
            const int *par = parents + t * N;
            memcpy(tmp, state, esz * 4 * N);
            for (size_t i = 0; i != N; ++i) {
                const size_t p = (size_t)par[i];
                for (size_t d = 0; d != 4; ++d) {
                    if (precision == 32)
                        ((float *)state)[d * N + i] =
                            ((const float *)tmp)[d * N + p];
                    else
                        ((double *)state)[d * N + i] =
                            ((const double *)tmp)[d * N + p];
                }
            }
            vo_weight_set_equal(N, W);
        }
        vo_pf_mean(N, state, precision, W, mean_out + 2 * t);
    }
    free(state);
    free(tmp);
    free(W);
    free(ll);
    free(llf);
    return 0;
}

int vo_pf_run(int precision, size_t N, size_t T, uint32_t seed, int scheme,
    double threshold, const vo_model *m, const double *obs, int threads,
    double *mean_out, double *ess_out, int *resampled_out, double *logz_out)
{
#ifdef _OPENMP
    int saved_threads = omp_get_max_threads();
    if (threads > 0)
        omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    const size_t esz = precision == 32 ? sizeof(float) : sizeof(double);
    void *state = malloc(esz * 4 * N);
    double *W = (double *)malloc(sizeof(double) * N);
    double *ll = (double *)malloc(sizeof(double) * N);
    float *llf = (float *)malloc(sizeof(float) * N);
    int *rep = (int *)malloc(sizeof(int) * N);
    int *idx = (int *)malloc(sizeof(int) * N);
    vo_philox reng;
    const uint32_t rkey[2] = {0, seed};
    const uint32_t rctr[4] = {0, 0, 1, 0};
    vo_philox_init(&reng, rkey, rctr);
    double ess = vo_weight_set_equal(N, W);
    double logz = 0;
    for (size_t t = 0; t != T; ++t) {
        if (precision == 32) {
            if (t == 0)
                vo_pf_init_f32(N, seed, m, obs, (float *)state, llf);
            else
                vo_pf_move_f32(N, t, seed, m, obs + 2 * t, (float *)state, llf);
            for (size_t i = 0; i != N; ++i)
                ll[i] = (double)llf[i];
        } else {
            if (t == 0)
                vo_pf_init_f64(N, seed, m, obs, (double *)state, ll);
            else
                vo_pf_move_f64(N, t, seed, m, obs + 2 * t, (double *)state, ll);
        }
        double mx = -INFINITY;
        for (size_t i = 0; i != N; ++i)
            if (mx < ll[i])
                mx = ll[i];
        double s = 0;
        if (t == 0) {
            for (size_t i = 0; i != N; ++i)
                s += exp(ll[i] - mx);
            logz += mx + log(s / (double)N);
            double *tmp = (double *)malloc(sizeof(double) * N);
            ess = vo_weight_set_log(N, ll, tmp);
            memcpy(W, tmp, sizeof(double) * N);
            free(tmp);
        } else {
            for (size_t i = 0; i != N; ++i)
                s += W[i] * exp(ll[i] - mx);
            logz += mx + log(s);
            for (size_t i = 0; i != N; ++i)
                W[i] = log(W[i]);
            for (size_t i = 0; i != N; ++i)
                W[i] = W[i] + ll[i];
            ess = vo_weight_post_set_log(N, W);
        }
        logz_out[t] = logz;
        ess_out[t] = ess;
        resampled_out[t] = vo_pf_resample(
            scheme, threshold, N, &reng, W, &ess, rep, idx, state, precision);
        vo_pf_mean(N, state, precision, W, mean_out + 2 * t);
    }
    free(state);
    free(W);
    free(ll);
    free(llf);
    free(rep);
    free(idx);
#ifdef _OPENMP
    omp_set_num_threads(saved_threads);
#endif
    return 0;
}

/* =====================================================================
 * Test helper: place an engine at (key, ctr), take k scalar words, then run
 * one operation -- op 0: n words through the bulk path; 1 / 2:
 * u01_distribution in f64 / f32; 3 / 4: normal_distribution in f64 / f32
 * (mean, sd).  The engine state afterwards goes to ctr_out / index_out.
 * Words and u01 values of a 32-bit engine are written as uint32 / real.
 * ===================================================================== */
void vo_engine_run(int kind, const uint64_t key[4], const uint64_t ctr[4],
    size_t k, int op, size_t n, double mean, double sd, void *out,
    uint64_t ctr_out[4], uint32_t *index_out)
{
    vo_eng e;
    vo_eng_init(&e, kind, key, ctr);
    for (size_t i = 0; i != k; ++i) {
        if (kind == 0)
            (void)vo_philox_next(&e.p);
        else
            (void)vo_threefry_next(&e.t);
    }
    if (op == 0) {
        if (kind == 0)
            vo_philox_rand(&e.p, n, (uint32_t *)out);
        else
            vo_threefry_rand(&e.t, n, (uint64_t *)out);
    } else if (op == 1) {
        vo_u01_distribution_d(&e, n, (double *)out);
    } else if (op == 2) {
        vo_u01_distribution_f(&e, n, (float *)out);
    } else if (op == 3 || op == 4) {
        const size_t kk = 1024, m = n / kk, l = n % kk;
        if (op == 3) {
            double *r = (double *)out;
            for (size_t i = 0; i != m; ++i, r += kk)
                vo_normal_impl_d(&e, kk, r, mean, sd);
            vo_normal_impl_d(&e, l, r, mean, sd);
            if (n % 2 != 0) {
                const double u = vo_eng_u01d(&e), v = vo_eng_u01d(&e);
                r[l - 1] = mean + sd * sqrt(-2 * log(u)) * cos(VO_PI_2 * v);
            }
        } else {
            float *r = (float *)out;
            const float fm = (float)mean, fs = (float)sd;
            for (size_t i = 0; i != m; ++i, r += kk)
                vo_normal_impl_f(&e, kk, r, fm, fs);
            vo_normal_impl_f(&e, l, r, fm, fs);
            if (n % 2 != 0) {
                const float u = vo_eng_u01f(&e), v = vo_eng_u01f(&e);
                r[l - 1] = fm + fs * sqrtf(-2 * logf(u)) * cosf(VO_PI_2F * v);
            }
        }
    }
    if (kind == 0) {
        for (int i = 0; i != 4; ++i)
            ctr_out[i] = e.p.ctr[i];
        *index_out = e.p.index;
    } else {
        for (int i = 0; i != 4; ++i)
            ctr_out[i] = e.t.ctr[i];
        *index_out = e.t.index;
    }
}

/* =====================================================================
 * Bearings-only tracking and the learned proposal.  Project-written test
 * infrastructure with no reference counterpart: the simulator (FP64, the
 * reference's CounterEngine / NormalDistribution draws), the FP32 particle
 * move and weight increment (bootstrap or learned proposal), the proposal
 * network's forward pass and loss gradient in FP64 with the device's BF16
 * operand rounding reproduced, and bearings filters for reference runs.
 *
 * Model: per axis [p; v]_t = [p + dt v; v]_{t-1} + L nu, L = chol(Q),
 * Q = q [[dt^3/3, dt^2/2], [dt^2/2, dt]]; bearing atan2(y, x) + N(0, sz^2).
 * Proposals draw the whitened noise nu (bootstrap N(0, I); learned
 * N(m, diag exp(l)) from the network) and weight by
 * log g(z | x) + log N(nu; 0, I) - log N(nu; m, diag exp(l)).
 * ===================================================================== */
static void vo_bchol(const vo_bmodel *m, double *l11, double *l21, double *l22)
{
    const double q11 = m->q * m->dt * m->dt * m->dt / 3;
    const double q12 = m->q * m->dt * m->dt / 2;
    const double q22 = m->q * m->dt;
    *l11 = sqrt(q11);
    *l21 = q12 / *l11;
    *l22 = sqrt(q22 - *l21 * *l21);
}

void vo_bearings_simulate(
    uint32_t seed, size_t T, const vo_bmodel *m, double *truth, double *obs)
{
    vo_eng e;
    e.kind = 0;
    const uint32_t key[2] = {seed, 0};
    const uint32_t ctr[4] = {0, 0, 0, 0};
    vo_philox_init(&e.p, key, ctr);
    vo_normal_d zn = {0, m->sigma_z, 0, 0};
    double l11, l21, l22;
    vo_bchol(m, &l11, &l21, &l22);
    double x, y, vx, vy, a, b, c, d;
    vo_pair_d(&e.p, m->sd_pos0, &a, &b);
    x = m->x0 + a;
    y = m->y0 + b;
    vo_pair_d(&e.p, m->sd_vel0, &a, &b);
    vx = m->vx0 + a;
    vy = m->vy0 + b;
    for (size_t t = 0; t != T; ++t) {
        if (t > 0) {
            vo_pair_d(&e.p, 1.0, &a, &b);
            vo_pair_d(&e.p, 1.0, &c, &d);
            x = (x + m->dt * vx) + l11 * a;
            vx = vx + (l21 * a + l22 * b);
            y = (y + m->dt * vy) + l11 * c;
            vy = vy + (l21 * c + l22 * d);
        }
        if (truth) {
            truth[4 * t + 0] = x;
            truth[4 * t + 1] = y;
            truth[4 * t + 2] = vx;
            truth[4 * t + 3] = vy;
        }
        obs[t] = atan2(y, x) + vo_normal_d_draw(&zn, &e);
    }
}

/* 1: round the network's tensor-core operands to BF16 and its FP32 values
 * to float as the device does; 0: exact FP64 (for finite-difference checks
 * of the gradient) */
static int vo_mlp_device_rounding = 1;

void vo_mlp_set_rounding(int on)
{
    vo_mlp_device_rounding = on;
}

/* float rounding of a device FP32 value (identity in exact mode) */
static double vo_rf(double x)
{
    return vo_mlp_device_rounding ? (double)(float)x : x;
}

/* BF16 round to nearest even (finite inputs; identity in exact mode) */
static double vo_bf16d(double x);

static float vo_bf16(float x)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    memcpy(&x, &u, 4);
    return x;
}

static double vo_gelu(double x, double *grad)
{
    const double k0 = -1.5957691216057308, k1 = -0.0713548162726009;
    const double e = exp(x * (k1 * x * x + k0));
    const double s = 1 / (1 + e);
    if (grad)
        *grad = s - x * s * (1 - s) * (3 * k1 * x * x + k0);
    return x * s;
}

/* GELU of a pre-activation as the filter kernels evaluate it (mlp.cuh,
 * gelu2_bf16): the FP32 pre-activation rounded to BF16, then
 * 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))) with every product and
 * fused multiply-add rounded to BF16.  The device takes tanh from the
 * hardware approximation; here it is tanhf rounded to BF16, so the two
 * can differ by a BF16 unit in the last place. */
static double vo_gelu_bf16(double pre)
{
    const float c0 = vo_bf16(0.7978845608028654f);
    const float c1 = vo_bf16(0.0356774081363001f);
    const float x = vo_bf16((float)pre);
    const float x2 = vo_bf16(x * x);
    const float t = vo_bf16(fmaf(x2, c1, c0));
    const float u = vo_bf16(x * t);
    const float th = vo_bf16(tanhf(u));
    const float h = vo_bf16(x * 0.5f);
    return vo_bf16(fmaf(h, th, h));
}

#define VO_IN 6
#define VO_HID 64
#define VO_OUT 8
#define VO_W1 0
#define VO_B1 (VO_W1 + VO_HID * VO_IN)
#define VO_W2 (VO_B1 + VO_HID)
#define VO_B2 (VO_W2 + VO_HID * VO_HID)
#define VO_W3 (VO_B2 + VO_HID)
#define VO_B3 (VO_W3 + VO_OUT * VO_HID)
#define VO_NP (VO_B3 + VO_OUT)

static double vo_bf16d(double x)
{
    return vo_mlp_device_rounding ? (double)vo_bf16((float)x) : x;
}

typedef struct {
    double a0[VO_IN];          /* bf16 inputs */
    double pre1[VO_HID];       /* hidden pre-activations */
    double a1[VO_HID];         /* bf16 gelu(pre1) */
    double pre2[VO_HID];
    double a2[VO_HID];
    double out[VO_OUT];
} vo_mlp_row;

static float p_w3(const float *p, int d, int j)
{
    return p[VO_W3 + d * VO_HID + j];
}

/* one row of the forward pass: BF16 weights and activations, FP64 sums;
 * filter = 1: the hidden activations as the filter kernels form them
 * (vo_gelu_bf16, device rounding mode only), else GELU in FP64 rounded to
 * BF16 as the training and parity kernels form them */
static void vo_mlp_row_forward(
    const float *p, const float *f, vo_mlp_row *r, int filter)
{
    const int fast = filter && vo_mlp_device_rounding;
    for (int k = 0; k < VO_IN; ++k)
        r->a0[k] = vo_bf16d(f[k]);
    for (int j = 0; j < VO_HID; ++j) {
        double s = 0;
        for (int k = 0; k < VO_IN; ++k)
            s += vo_bf16d(p[VO_W1 + j * VO_IN + k]) * r->a0[k];
        r->pre1[j] = s + p[VO_B1 + j];
        r->a1[j] = fast ? vo_gelu_bf16(r->pre1[j])
                        : vo_bf16d(vo_gelu(r->pre1[j], NULL));
    }
    for (int j = 0; j < VO_HID; ++j) {
        double s = 0;
        for (int k = 0; k < VO_HID; ++k)
            s += vo_bf16d(p[VO_W2 + j * VO_HID + k]) * r->a1[k];
        r->pre2[j] = s + p[VO_B2 + j];
        r->a2[j] = fast ? vo_gelu_bf16(r->pre2[j])
                        : vo_bf16d(vo_gelu(r->pre2[j], NULL));
    }
    for (int d = 0; d < VO_OUT; ++d) {
        double s = 0;
        for (int k = 0; k < VO_HID; ++k)
            s += vo_bf16d(p[VO_W3 + d * VO_HID + k]) * r->a2[k];
        r->out[d] = s + p[VO_B3 + d];
    }
}

void vo_mlp_forward(const float *params, size_t B, const float *feat,
    float *out)
{
    _Pragma("omp parallel for schedule(static)")
    for (size_t i = 0; i < B; ++i) {
        vo_mlp_row r;
        vo_mlp_row_forward(params, feat + 6 * i, &r, 0);
        for (int d = 0; d < VO_OUT; ++d)
            out[8 * i + d] = (float)r.out[d];
    }
}

/* mean loss 0.5 sum_d [(nu_d - m_d)^2 exp(-l_d) + l_d] and its gradient;
 * the backward data path rounds its operands to BF16 as the device does */
void vo_mlp_loss_grad(const float *params, size_t B, const float *feat,
    const float *nu, double *loss, double *grad)
{
    for (int i = 0; i < VO_NP; ++i)
        grad[i] = 0;
    double L = 0;
    const double inv_b = 1.0 / (double)B;
    for (size_t i = 0; i < B; ++i) {
        vo_mlp_row r;
        vo_mlp_row_forward(params, feat + 6 * i, &r, 0);
        double dout[VO_OUT];
        for (int d = 0; d < 4; ++d) {
            const double res = nu[4 * i + d] - r.out[d];
            const double el = exp(-r.out[4 + d]);
            L += 0.5 * (res * res * el + r.out[4 + d]);
            dout[d] = vo_rf(-res * el * inv_b);
            dout[4 + d] = vo_rf(0.5 * (1 - res * res * el) * inv_b);
        }
        double dp2[VO_HID], dp1[VO_HID];
        for (int j = 0; j < VO_HID; ++j) {
            double s = 0;
            for (int d = 0; d < VO_OUT; ++d)
                s += vo_bf16d(p_w3(params, d, j)) * vo_bf16d(dout[d]);
            double gg;
            vo_gelu(r.pre2[j], &gg);
            dp2[j] = vo_rf(s * gg);
        }
        for (int k = 0; k < VO_HID; ++k) {
            double s = 0;
            for (int j = 0; j < VO_HID; ++j)
                s += vo_bf16d(params[VO_W2 + j * VO_HID + k]) *
                    vo_bf16d(dp2[j]);
            double gg;
            vo_gelu(r.pre1[k], &gg);
            dp1[k] = vo_rf(s * gg);
        }
        for (int d = 0; d < VO_OUT; ++d) {
            grad[VO_B3 + d] += dout[d];
            for (int k = 0; k < VO_HID; ++k)
                grad[VO_W3 + d * VO_HID + k] += dout[d] * r.a2[k];
        }
        for (int j = 0; j < VO_HID; ++j) {
            grad[VO_B2 + j] += dp2[j];
            for (int k = 0; k < VO_HID; ++k)
                grad[VO_W2 + j * VO_HID + k] += dp2[j] * r.a1[k];
            grad[VO_B1 + j] += dp1[j];
            for (int k = 0; k < VO_IN; ++k)
                grad[VO_W1 + j * VO_IN + k] += dp1[j] * r.a0[k];
        }
    }
    *loss = L * inv_b;
}

static inline double vo_bwrap(double d)
{
    return d - VO_PI_2 * nearbyint(d / VO_PI_2);
}

void vo_bearings_move_f32(size_t N, size_t t, uint32_t seed,
    const vo_bmodel *m, double z, const float *params, float *state,
    float *lw_inc)
{
    double l11d, l21d, l22d;
    vo_bchol(m, &l11d, &l21d, &l22d);
    const float l11 = (float)l11d, l21 = (float)l21d, l22 = (float)l22d;
    const float dt = (float)m->dt;
    const float inv_sz = (float)(1 / m->sigma_z);
    const float ll_c = (float)(-log(m->sigma_z * sqrt(2 * VO_PI)));
    const float zf = (float)z;
    const float sz = sinf(zf), cz = cosf(zf);
    _Pragma("omp parallel for schedule(static)")
    for (size_t i = 0; i < N; ++i) {
        vo_philox e;
        vo_particle_engine(&e, t, seed, i);
        float ev[4];
        vo_pair_f(&e, 1.0f, &ev[0], &ev[1]);
        vo_pair_f(&e, 1.0f, &ev[2], &ev[3]);
        float x = state[i], y = state[N + i];
        float vx = state[2 * N + i], vy = state[3 * N + i];
        float lq = 0;
        if (t == 0) {
            x = (float)m->x0 + (float)m->sd_pos0 * ev[0];
            y = (float)m->y0 + (float)m->sd_pos0 * ev[1];
            vx = (float)m->vx0 + (float)m->sd_vel0 * ev[2];
            vy = (float)m->vy0 + (float)m->sd_vel0 * ev[3];
        } else {
            float nu[4] = {ev[0], ev[1], ev[2], ev[3]};
            if (params) {
                /* inputs in the bearing frame of z: the predicted position
                 * along it on a saturating range scale, across it in
                 * units of sigma_z r (softly held below 8, scaled by 1/8),
                 * the velocity's along / across parts on a bounded scale,
                 * sin z and cos z */
                const float px = x + dt * vx, py = y + dt * vy;
                const float rng = sqrtf(px * px + py * py);
                const float pa = cz * px + sz * py;
                const float pb = cz * py - sz * px;
                const float e = pb * inv_sz / (rng > 1e-6f ? rng : 1e-6f);
                const float eb = e / sqrtf(1.0f + 0.015625f * e * e);
                const float iv = 1.0f / (1.0f + sqrtf(vx * vx + vy * vy));
                const float f[6] = {pa / (10.0f + rng), 0.125f * eb,
                    (cz * vx + sz * vy) * iv, (cz * vy - sz * vx) * iv, sz,
                    cz};
                vo_mlp_row r;
                vo_mlp_row_forward(params, f, &r, 1);
                /* the draw nu' = (a1, a2, b1, b2) in the bearing frame,
                 * then rotated pairwise to the axes */
                float fr[4];
                for (int d = 0; d < 4; ++d) {
                    float l = (float)r.out[4 + d];
                    l = l < -12.0f ? -12.0f : (l > 4.0f ? 4.0f : l);
                    fr[d] = (float)r.out[d] + expf(0.5f * l) * ev[d];
                    lq += 0.5f * (ev[d] * ev[d] - fr[d] * fr[d]) + 0.5f * l;
                }
                nu[0] = cz * fr[0] - sz * fr[2];
                nu[2] = sz * fr[0] + cz * fr[2];
                nu[1] = cz * fr[1] - sz * fr[3];
                nu[3] = sz * fr[1] + cz * fr[3];
            }
            const float dx = l11 * nu[0], dvx = l21 * nu[0] + l22 * nu[1];
            const float dy = l11 * nu[2], dvy = l21 * nu[2] + l22 * nu[3];
            x = (x + dt * vx) + dx;
            y = (y + dt * vy) + dy;
            vx = vx + dvx;
            vy = vy + dvy;
        }
        state[i] = x;
        state[N + i] = y;
        state[2 * N + i] = vx;
        state[3 * N + i] = vy;
        float d = zf - atan2f(y, x);
        d -= (float)VO_PI_2 * nearbyintf(d / (float)VO_PI_2);
        const float s = d * inv_sz;
        lw_inc[i] = ll_c - 0.5f * s * s + lq;
    }
}

static void vo_bearings_move_f64(size_t N, size_t t, uint32_t seed,
    const vo_bmodel *m, double z, double *state, double *ll)
{
    double l11, l21, l22;
    vo_bchol(m, &l11, &l21, &l22);
    const double ll_c = -log(m->sigma_z * sqrt(2 * VO_PI));
    _Pragma("omp parallel for schedule(static)")
    for (size_t i = 0; i < N; ++i) {
        vo_philox e;
        vo_particle_engine(&e, t, seed, i);
        double a, b, c, d;
        double x = state[i], y = state[N + i];
        double vx = state[2 * N + i], vy = state[3 * N + i];
        if (t == 0) {
            vo_pair_d(&e, m->sd_pos0, &a, &b);
            vo_pair_d(&e, m->sd_vel0, &c, &d);
            x = m->x0 + a;
            y = m->y0 + b;
            vx = m->vx0 + c;
            vy = m->vy0 + d;
        } else {
            vo_pair_d(&e, 1.0, &a, &b);
            vo_pair_d(&e, 1.0, &c, &d);
            x = (x + m->dt * vx) + l11 * a;
            vx = vx + (l21 * a + l22 * b);
            y = (y + m->dt * vy) + l11 * c;
            vy = vy + (l21 * c + l22 * d);
        }
        state[i] = x;
        state[N + i] = y;
        state[2 * N + i] = vx;
        state[3 * N + i] = vy;
        const double s = vo_bwrap(z - atan2(y, x)) / m->sigma_z;
        ll[i] = ll_c - 0.5 * s * s;
    }
}

int vo_bearings_pf_run(int precision, size_t N, size_t T, uint32_t seed,
    int scheme, double threshold, const vo_bmodel *m, const double *obs,
    const float *params, int threads, double *mean_out, double *ess_out,
    int *resampled_out, double *logz_out)
{
#ifdef _OPENMP
    int saved_threads = omp_get_max_threads();
    if (threads > 0)
        omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    const size_t esz = precision == 32 ? sizeof(float) : sizeof(double);
    void *state = calloc(4 * N, esz);
    double *W = (double *)malloc(sizeof(double) * N);
    double *ll = (double *)malloc(sizeof(double) * N);
    float *llf = (float *)malloc(sizeof(float) * N);
    int *rep = (int *)malloc(sizeof(int) * N);
    int *idx = (int *)malloc(sizeof(int) * N);
    vo_philox reng;
    const uint32_t rkey[2] = {0, seed};
    const uint32_t rctr[4] = {0, 0, 1, 0};
    vo_philox_init(&reng, rkey, rctr);
    double ess = vo_weight_set_equal(N, W);
    double logz = 0;
    for (size_t t = 0; t != T; ++t) {
        if (precision == 32) {
            vo_bearings_move_f32(
                N, t, seed, m, obs[t], params, (float *)state, llf);
            for (size_t i = 0; i != N; ++i)
                ll[i] = (double)llf[i];
        } else {
            vo_bearings_move_f64(N, t, seed, m, obs[t], (double *)state, ll);
        }
        double mx = -INFINITY;
        for (size_t i = 0; i != N; ++i)
            if (mx < ll[i])
                mx = ll[i];
        double s = 0;
        for (size_t i = 0; i != N; ++i)
            s += W[i] * exp(ll[i] - mx);
        logz += mx + log(s);
        for (size_t i = 0; i != N; ++i)
            W[i] = log(W[i]) + ll[i];
        ess = vo_weight_post_set_log(N, W);
        logz_out[t] = logz;
        ess_out[t] = ess;
        resampled_out[t] = vo_pf_resample(
            scheme, threshold, N, &reng, W, &ess, rep, idx, state, precision);
        vo_pf_mean(N, state, precision, W, mean_out + 2 * t);
    }
    free(state);
    free(W);
    free(ll);
    free(llf);
    free(rep);
    free(idx);
#ifdef _OPENMP
    omp_set_num_threads(saved_threads);
#endif
    return 0;
}

/* =====================================================================
 * ResampleIndex (resample/index.hpp:46-206): rows[k] holds each particle's
 * parent before iteration k.  index(id, iter) follows rows back from the
 * last iteration (index.hpp:117-129); index_matrix gives every line,
 * row-major [N][iters] or column-major [iters][N] (index.hpp:131-201).
 * ===================================================================== */
void vo_resample_index_trace(
    size_t N, size_t iters, const int *rows, size_t iter, int *out)
{
    for (size_t id = 0; id != N; ++id) {
        size_t cur = iters - 1;
        int idx = rows[cur * N + id];
        while (cur != iter) {
            --cur;
            idx = rows[cur * N + (size_t)idx];
        }
        out[id] = idx;
    }
}

void vo_resample_index_matrix(
    size_t N, size_t iters, const int *rows, int layout, int *out)
{
    if (N * iters == 0)
        return;
    if (layout == 0) { /* row major: out[i * iters + k] */
        for (size_t i = 0; i != N; ++i)
            out[i * iters + iters - 1] = rows[(iters - 1) * N + i];
        for (size_t k = iters - 1; k != 0; --k)
            for (size_t i = 0; i != N; ++i)
                out[i * iters + k - 1] =
                    rows[(k - 1) * N + (size_t)out[i * iters + k]];
    } else { /* column major: out[k * N + i] */
        for (size_t i = 0; i != N; ++i)
            out[(iters - 1) * N + i] = rows[(iters - 1) * N + i];
        for (size_t k = iters - 1; k != 0; --k)
            for (size_t i = 0; i != N; ++i)
                out[(k - 1) * N + i] =
                    rows[(k - 1) * N + (size_t)out[k * N + i]];
    }
}

/* =====================================================================
 * Resample-move step: random-walk Metropolis on a particle's acceleration
 * innovation a (RandomWalk with an unbounded Normal proposal,
 * rng/random_walk.hpp:95-114), target N(a; 0, sigma_a^2 I) g(y | x),
 * x = F x' + G a, so a' = a + s e moves the state by G (a' - a).  Proposal
 * and uniform: Philox4x32 block of counter {2 + k, i, 0, 0}, key {t, seed}
 * (words 0, 1 -> Box-Muller pair, word 2 -> u in [0, 1)); particle i's
 * current innovation is the pair its parent j drew at step t.
 * ===================================================================== */
void vo_cv_mcmc_f32(size_t N, size_t t, size_t sweeps, uint32_t seed,
    const vo_model *m, const double obs[2], double scale, const int *parent,
    float *state, uint32_t *accepted, float *margin)
{
    const float dt = (float)m->dt, h = (float)(0.5 * m->dt * m->dt);
    const float sa = (float)m->sigma_a;
    const float inv_var = 1.0f / (sa * sa), s_rw = (float)scale;
    uint32_t acc = 0;
    for (size_t i = 0; i < N; ++i) {
        const size_t j = parent ? (size_t)parent[i] : i;
        vo_philox e;
        vo_particle_engine(&e, t, seed, j);
        float ax, ay;
        vo_pair_f(&e, sa, &ax, &ay);
        float x = state[i], y = state[N + i];
        float vx = state[2 * N + i], vy = state[3 * N + i];
        float lt = -0.5f * inv_var * (ax * ax + ay * ay) +
            vo_ll_f32(m, obs, x, y);
        float closest = INFINITY; /* min |log u - (lt2 - lt)| over sweeps */
        for (size_t k = 0; k < sweeps; ++k) {
            const uint32_t ctr[4] = {(uint32_t)(2 + k), (uint32_t)i, 0, 0};
            const uint32_t key[2] = {(uint32_t)t, seed};
            uint32_t w[4];
            vo_philox4x32_block(ctr, key, w);
            const float u1 = vo_u01_u32_f32(2, w[0]);
            const float u2 = vo_u01_u32_f32(1, w[1]);
            const float r = sqrtf(-2 * logf(u1));
            const float th = VO_PI_2F * u2;
            const float e1 = r * cosf(th), e2 = r * sinf(th);
            const float bx = ax + s_rw * e1, by = ay + s_rw * e2;
            const float dx = bx - ax, dy = by - ay;
            const float nx = x + h * dx, ny = y + h * dy;
            const float nvx = vx + dt * dx, nvy = vy + dt * dy;
            const float lt2 = -0.5f * inv_var * (bx * bx + by * by) +
                vo_ll_f32(m, obs, nx, ny);
            const float lu = logf(vo_u01_u32_f32(1, w[2]));
            if (fabsf(lu - (lt2 - lt)) < closest)
                closest = fabsf(lu - (lt2 - lt));
            if (lu < lt2 - lt) {
                x = nx;
                y = ny;
                vx = nvx;
                vy = nvy;
                ax = bx;
                ay = by;
                lt = lt2;
                ++acc;
            }
        }
        state[i] = x;
        state[N + i] = y;
        state[2 * N + i] = vx;
        state[3 * N + i] = vy;
        if (margin)
            margin[i] = closest;
    }
    *accepted += acc;
}
