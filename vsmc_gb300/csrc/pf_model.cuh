// Constant-velocity tracking model with Student-t position observations:
// the per-particle move and log-likelihood of the filter step, in the form
// of the reference's pf example (example/pf/include/pf.hpp:81-93 likelihood,
// 117-131 init, 154-170 move) with the benchmark model's constants.
#pragma once

#include "common.cuh"

#include <cmath>

namespace vsmc_cuda
{

template <typename T>
struct CvConst {
    T dt, h, sigma_a, sd_pos0, sd_vel0;
    T c2, inv_s, inv_nu, half_nu1;
};

// Student-t log density normalizing constant for one coordinate:
// lgamma((nu+1)/2) - lgamma(nu/2) - log(nu pi)/2 - log(s).
inline double student_t_norm_const(double nu, double s)
{
    return std::lgamma(0.5 * (nu + 1)) - std::lgamma(0.5 * nu) -
        0.5 * std::log(nu * 3.14159265358979323846) - std::log(s);
}

template <typename T>
inline CvConst<T> make_cv_const(const vsmc_cuda_cv_model &m)
{
    CvConst<T> c;
    c.dt = static_cast<T>(m.dt);
    c.h = static_cast<T>(0.5 * m.dt * m.dt);
    c.sigma_a = static_cast<T>(m.sigma_a);
    c.sd_pos0 = static_cast<T>(m.sd_pos0);
    c.sd_vel0 = static_cast<T>(m.sd_vel0);
    c.c2 = static_cast<T>(2 * student_t_norm_const(m.nu, m.obs_scale));
    c.inv_s = static_cast<T>(1 / m.obs_scale);
    c.inv_nu = static_cast<T>(1 / m.nu);
    c.half_nu1 = static_cast<T>(0.5 * (m.nu + 1));
    return c;
}

inline bool valid_cv_model(const vsmc_cuda_cv_model *m)
{
    return m != nullptr && m->dt > 0 && m->sigma_a >= 0 && m->obs_scale > 0 &&
        m->nu > 0 && m->sd_pos0 >= 0 && m->sd_vel0 >= 0 &&
        std::isfinite(m->dt) && std::isfinite(m->sigma_a) &&
        std::isfinite(m->obs_scale) && std::isfinite(m->nu) &&
        std::isfinite(m->sd_pos0) && std::isfinite(m->sd_vel0);
}

// Particle streams: Philox4x32 key {step, seed}, counter {0, particle, 0, 0};
// the first (pre-incremented) block is gen({1, particle, 0, 0}).
__device__ __forceinline__ u32x4 particle_block(
    uint32_t t, uint32_t seed, uint32_t i)
{
    return philox4x32_10(1u, i, 0u, 0u, t, seed);
}

// FP64 standard-normal pair: NormalDistribution<double> (cosine value
// first, sine value cached), [0,1) uniforms from 32-bit words.
__device__ __forceinline__ void normal_pair_d(uint32_t w0, uint32_t w1,
    double &z1, double &z2)
{
    const double u1 = sqrt(__dmul_rn(-2.0, log(u01_co_d(w0))));
    const double u2 = __dmul_rn(kPi2, u01_co_d(w1));
    double sv, cv;
    sincos(u2, &sv, &cv);
    z1 = __dmul_rn(u1, cv);
    z2 = __dmul_rn(u1, sv);
}

// FP32: log1p(qx) + log1p(qy) as one log1p((1 + qx)(1 + qy) - 1)
// FP32: log(1 + a) of a = qx + qy + qx qy >= 0 by the hardware log2.  Its
// absolute error (~2^-21, plus the rounding of 1 + a for small a) stays
// below ~3e-6 in the log-likelihood.
__device__ __forceinline__ float cv_loglik(
    const CvConst<float> &c, float ox, float oy, float x, float y)
{
    const float zx = (ox - x) * c.inv_s;
    const float zy = (oy - y) * c.inv_s;
    const float qx = zx * zx * c.inv_nu;
    const float qy = zy * zy * c.inv_nu;
    return c.c2 - c.half_nu1 * __logf(1.0f + fmaf(qx, qy, qx + qy));
}

__device__ __forceinline__ double cv_loglik(
    const CvConst<double> &c, double ox, double oy, double x, double y)
{
    const double zx = __dmul_rn(__dadd_rn(ox, -x), c.inv_s);
    const double zy = __dmul_rn(__dadd_rn(oy, -y), c.inv_s);
    const double qx = __dmul_rn(__dmul_rn(zx, zx), c.inv_nu);
    const double qy = __dmul_rn(__dmul_rn(zy, zy), c.inv_nu);
    return __dadd_rn(
        c.c2, -__dmul_rn(c.half_nu1, __dadd_rn(log1p(qx), log1p(qy))));
}

// move: x += dt vx + h ax, y += dt vy + h ay, v += dt a
__device__ __forceinline__ void cv_move(const CvConst<float> &c, float ax,
    float ay, float &x, float &y, float &vx, float &vy)
{
    x = x + c.dt * vx + c.h * ax;
    y = y + c.dt * vy + c.h * ay;
    vx = vx + c.dt * ax;
    vy = vy + c.dt * ay;
}

__device__ __forceinline__ void cv_move(const CvConst<double> &c, double ax,
    double ay, double &x, double &y, double &vx, double &vy)
{
    x = __dadd_rn(__dadd_rn(x, __dmul_rn(c.dt, vx)), __dmul_rn(c.h, ax));
    y = __dadd_rn(__dadd_rn(y, __dmul_rn(c.dt, vy)), __dmul_rn(c.h, ay));
    vx = __dadd_rn(vx, __dmul_rn(c.dt, ax));
    vy = __dadd_rn(vy, __dmul_rn(c.dt, ay));
}

// The acceleration innovation (2D) of particle j at step t >= 1: the pair
// cv_move drew for it.
__device__ __forceinline__ void cv_innovation(const CvConst<float> &c,
    uint32_t t, uint32_t seed, uint32_t j, float &ax, float &ay)
{
    const u32x4 w = particle_block(t, seed, j);
    float z1, z2;
    normal_pair_f(w.x, w.y, z1, z2);
    ax = c.sigma_a * z1;
    ay = c.sigma_a * z2;
}

// One random-walk Metropolis step on a particle's acceleration innovation
// a, the RandomWalk / NormalMVProposal update of rng/random_walk.hpp:95-114
// with an unbounded Normal proposal (log q ratio 0): the state is
// x_t = F x_{t-1} + G a, so a' = a + s e moves it by G (a' - a); the target
// is N(a; 0, sigma_a^2 I) g(y | x_t) and the step accepts when
// log u < lt' - lt with u in [0, 1).  Words: Philox4x32 key {t, seed},
// counter {2 + k, i, 0, 0} (k the sweep, i the particle's slot): the first
// two give the proposal pair, the third u.  lt holds the log target of the
// current (x, a); returns 1 on acceptance.
__device__ __forceinline__ int cv_mcmc_step(const CvConst<float> &c,
    float ox, float oy, float s_rw, float inv_var, uint32_t t, uint32_t seed,
    uint32_t i, uint32_t k, float &x, float &y, float &vx, float &vy,
    float &ax, float &ay, float &lt)
{
    const u32x4 w = philox4x32_10(2u + k, i, 0u, 0u, t, seed);
    float e1, e2;
    normal_pair_f(w.x, w.y, e1, e2);
    const float bx = ax + s_rw * e1, by = ay + s_rw * e2;
    const float dx = bx - ax, dy = by - ay;
    const float nx = x + c.h * dx, ny = y + c.h * dy;
    const float nvx = vx + c.dt * dx, nvy = vy + c.dt * dy;
    const float lt2 =
        -0.5f * inv_var * (bx * bx + by * by) + cv_loglik(c, ox, oy, nx, ny);
    if (logf(u01_co_f(w.z)) < lt2 - lt) {
        x = nx;
        y = ny;
        vx = nvx;
        vy = nvy;
        ax = bx;
        ay = by;
        lt = lt2;
        return 1;
    }
    return 0;
}

} // namespace vsmc_cuda
