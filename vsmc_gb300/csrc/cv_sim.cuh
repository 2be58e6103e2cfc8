// Sequential simulation of the constant-velocity / Student-t model on one
// thread: a Philox4x32 engine seeded with `seed` (CounterEngine(seed)), fresh
// NormalDistribution<double> pairs for the prior and the accelerations
// (rng/normal_distribution.hpp:199-216), one StudentTDistribution<double>(nu)
// for the observation noise (rng/student_t_distribution.hpp:78-91) kept for
// the whole run.  truth: T x 4, obs: T x 2 (either may be null).
#pragma once

#include "common.cuh"
#include "rng_device.cuh"

namespace vsmc_cuda
{

__device__ inline void cv_simulate_seq(uint32_t seed, uint32_t T, double dt,
    double sigma_a, double obs_scale, double nu, double sd_pos0,
    double sd_vel0, double *truth, double *obs)
{
    PhiloxScalar eng(PhiloxScalar::key_t{seed, 0u}, 0);
    StudentTScalar st(nu);
    auto pair = [&](double sd, double &a, double &b) {
        NormalScalar<double> nd(0, sd);
        a = nd(eng);
        b = nd(eng);
    };
    double x, y, vx, vy;
    pair(sd_pos0, x, y);
    pair(sd_vel0, vx, vy);
    const double h = 0.5 * dt * dt;
    for (uint32_t t = 0; t < T; ++t) {
        if (t > 0) {
            double ax, ay;
            pair(sigma_a, ax, ay);
            x = __dadd_rn(__dadd_rn(x, __dmul_rn(dt, vx)), __dmul_rn(h, ax));
            y = __dadd_rn(__dadd_rn(y, __dmul_rn(dt, vy)), __dmul_rn(h, ay));
            vx = __dadd_rn(vx, __dmul_rn(dt, ax));
            vy = __dadd_rn(vy, __dmul_rn(dt, ay));
        }
        if (truth) {
            truth[4 * t + 0] = x;
            truth[4 * t + 1] = y;
            truth[4 * t + 2] = vx;
            truth[4 * t + 3] = vy;
        }
        const double ex = st(eng);
        const double ey = st(eng);
        if (obs) {
            obs[2 * t + 0] = __dadd_rn(x, __dmul_rn(obs_scale, ex));
            obs[2 * t + 1] = __dadd_rn(y, __dmul_rn(obs_scale, ey));
        }
    }
}

} // namespace vsmc_cuda
