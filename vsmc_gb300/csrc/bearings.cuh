// Bearings-only tracking model and its proposal-corrected weights.
//
// State (x, y, vx, vy).  Transition: constant velocity with continuous
// white-noise acceleration of spectral density q, per axis
//   [p; v]_t = [p + dt v; v]_{t-1} + L nu,  nu ~ N(0, I2),
//   Q = q [[dt^3/3, dt^2/2], [dt^2/2, dt]],  L = chol(Q).
// Observation: bearing z = atan2(y, x) + N(0, sigma_z^2) from a sensor at the
// origin.  Prior: N((x0, y0, vx0, vy0), diag(sd_pos0^2, sd_pos0^2, sd_vel0^2,
// sd_vel0^2)).
//
// Proposals work in the transition's whitened coordinates nu = (nu_x1,
// nu_x2, nu_y1, nu_y2): the bootstrap draws nu ~ N(0, I); the learned
// proposal draws nu' ~ N(m, diag(exp(l))) in the bearing frame of z (see
// frame_to_axes) with (m, l) from the network, rotates it to nu, and the
// state follows as x = F x' + L nu.  The weight increment is
//   log g(z | x) + log N(nu'; 0, I) - log N(nu'; m, diag(exp(l)))
// (the Jacobian of nu' -> x is the same in both densities and cancels).
//
// No reference counterpart: the reference's pf example is the Student-t
// position model (example/pf/include/pf.hpp); this model and the learned
// proposal are the project's own.
#pragma once

#include "common.cuh"
#include "pf_model.cuh"
#include "rng_device.cuh"

#include <cmath>

namespace vsmc_cuda
{

struct BearingsConst {
    float dt, l11, l21, l22; // transition Cholesky factor per axis
    float inv_sz, ll_c;      // 1 / sigma_z, -log(sigma_z sqrt(2 pi))
    float x0, y0, vx0, vy0, sd_pos0, sd_vel0;
    float lmin, lmax; // log-variance clamp of the learned proposal
    float pad[2];
};

inline bool valid_bearings_model(const vsmc_cuda_bearings_model *m)
{
    return m != nullptr && m->dt > 0 && m->q > 0 && m->sigma_z > 0 &&
        m->sd_pos0 >= 0 && m->sd_vel0 >= 0 && std::isfinite(m->dt) &&
        std::isfinite(m->q) && std::isfinite(m->sigma_z) &&
        std::isfinite(m->x0) && std::isfinite(m->y0) &&
        std::isfinite(m->vx0) && std::isfinite(m->vy0) &&
        std::isfinite(m->sd_pos0) && std::isfinite(m->sd_vel0);
}

// per-axis Cholesky factor of Q (FP64)
inline void bearings_chol(
    const vsmc_cuda_bearings_model &m, double &l11, double &l21, double &l22)
{
    const double q11 = m.q * m.dt * m.dt * m.dt / 3;
    const double q12 = m.q * m.dt * m.dt / 2;
    const double q22 = m.q * m.dt;
    l11 = std::sqrt(q11);
    l21 = q12 / l11;
    l22 = std::sqrt(q22 - l21 * l21);
}

inline BearingsConst make_bearings_const(const vsmc_cuda_bearings_model &m)
{
    double l11, l21, l22;
    bearings_chol(m, l11, l21, l22);
    BearingsConst c;
    c.dt = static_cast<float>(m.dt);
    c.l11 = static_cast<float>(l11);
    c.l21 = static_cast<float>(l21);
    c.l22 = static_cast<float>(l22);
    c.inv_sz = static_cast<float>(1 / m.sigma_z);
    c.ll_c = static_cast<float>(
        -std::log(m.sigma_z * std::sqrt(2 * 3.14159265358979323846)));
    c.x0 = static_cast<float>(m.x0);
    c.y0 = static_cast<float>(m.y0);
    c.vx0 = static_cast<float>(m.vx0);
    c.vy0 = static_cast<float>(m.vy0);
    c.sd_pos0 = static_cast<float>(m.sd_pos0);
    c.sd_vel0 = static_cast<float>(m.sd_vel0);
    c.lmin = -12.0f;
    c.lmax = 4.0f;
    c.pad[0] = c.pad[1] = 0;
    return c;
}

// the four standard normals of particle i at step t (two Box-Muller pairs)
__device__ __forceinline__ void bearings_normals(
    uint32_t t, uint32_t seed, uint32_t i, float (&e)[4])
{
    const u32x4 w = particle_block(t, seed, i);
    normal_pair_f(w.x, w.y, e[0], e[1]);
    normal_pair_f(w.z, w.w, e[2], e[3]);
}

__device__ __forceinline__ void bearings_prior(const BearingsConst &c,
    const float (&e)[4], float &x, float &y, float &vx, float &vy)
{
    x = c.x0 + c.sd_pos0 * e[0];
    y = c.y0 + c.sd_pos0 * e[1];
    vx = c.vx0 + c.sd_vel0 * e[2];
    vy = c.vy0 + c.sd_vel0 * e[3];
}

// x = F x' + L nu
__device__ __forceinline__ void bearings_step(const BearingsConst &c,
    const float (&nu)[4], float &x, float &y, float &vx, float &vy)
{
    const float dx = c.l11 * nu[0];
    const float dvx = c.l21 * nu[0] + c.l22 * nu[1];
    const float dy = c.l11 * nu[2];
    const float dvy = c.l21 * nu[2] + c.l22 * nu[3];
    x = (x + c.dt * vx) + dx;
    y = (y + c.dt * vy) + dy;
    vx = vx + dvx;
    vy = vy + dvy;
}

// log g(z | x, y): Gaussian on the bearing error wrapped to [-pi, pi]
__device__ __forceinline__ float bearings_loglik(
    const BearingsConst &c, float z, float x, float y)
{
    float d = z - atan2f(y, x);
    d -= 6.283185307179586f * rintf(d * 0.15915494309189535f);
    const float s = d * c.inv_sz;
    return c.ll_c - 0.5f * s * s;
}

// The bearing frame of an observation z: along = (cos z, sin z), across =
// (-sin z, cos z).  The whitened transition noise nu = (x1, x2, y1, y2)
// (position and velocity parts per axis) rotates pairwise into
// nu' = (a1, a2, b1, b2), the along and across parts of the position pair
// (x1, y1) and of the velocity pair (x2, y2).  The rotation is orthogonal,
// so N(nu; 0, I) = N(nu'; 0, I) with Jacobian 1; the factor L is the same on
// both axes, so the position noise across the bearing is l11 b1 alone.  The
// proposal's mean and diagonal log-variance live in this frame.
__device__ __forceinline__ void frame_to_axes(
    float sz, float cz, const float (&v)[4], float (&nu)[4])
{
    nu[0] = cz * v[0] - sz * v[2];
    nu[2] = sz * v[0] + cz * v[2];
    nu[1] = cz * v[1] - sz * v[3];
    nu[3] = sz * v[1] + cz * v[3];
}

__device__ __forceinline__ void axes_to_frame(
    float sz, float cz, const float (&nu)[4], float (&v)[4])
{
    v[0] = cz * nu[0] + sz * nu[2];
    v[2] = cz * nu[2] - sz * nu[0];
    v[1] = cz * nu[1] + sz * nu[3];
    v[3] = cz * nu[3] - sz * nu[1];
}

// The network inputs of a particle at its previous state and the bearing z,
// in the bearing frame.  With the predicted position p = (x + dt vx,
// y + dt vy) and r = |p|: p along the bearing on a saturating range scale,
// p_a / (10 + r); p across it in units of the bearing's resolution,
// e = p_b / (sigma_z r), held below 8 by e / sqrt(1 + (e / 8)^2) and scaled
// by 1/8; the velocity's along and across parts as v / (1 + |v|); and
// (sin z, cos z).  Every input is bounded whatever the state.  The inputs
// are rounded to BF16 for the network, so the quotients use the fast
// division and reciprocal square root.
__device__ __forceinline__ void bearings_features(const BearingsConst &c,
    float x, float y, float vx, float vy, float sz, float cz, float (&f)[6])
{
    const float px = x + c.dt * vx, py = y + c.dt * vy;
    const float r = sqrtf(px * px + py * py);
    const float pa = cz * px + sz * py;
    const float pb = cz * py - sz * px;
    const float e = __fdividef(pb * c.inv_sz, fmaxf(r, 1e-6f));
    const float eb = e * rsqrtf(1.0f + 0.015625f * e * e);
    const float iv = __fdividef(1.0f, 1.0f + sqrtf(vx * vx + vy * vy));
    f[0] = __fdividef(pa, 10.0f + r);
    f[1] = 0.125f * eb;
    f[2] = (cz * vx + sz * vy) * iv;
    f[3] = (cz * vy - sz * vx) * iv;
    f[4] = sz;
    f[5] = cz;
}

// Sequential FP64 simulation on one thread: CounterEngine(seed), fresh
// NormalDistribution<double> pairs for the prior and the transition noise
// (x axis pair, then y axis pair), one NormalDistribution<double>(0, sigma_z)
// for the bearing noise kept for the whole run (the draw conventions of
// rng/normal_distribution.hpp:199-216).  truth: T x 4 (may be null), obs: T.
__device__ inline void bearings_simulate_seq(uint32_t seed, uint32_t T,
    const vsmc_cuda_bearings_model &m, double *truth, double *obs)
{
    const double q11 = m.q * m.dt * m.dt * m.dt / 3;
    const double q12 = m.q * m.dt * m.dt / 2;
    const double q22 = m.q * m.dt;
    const double l11 = sqrt(q11);
    const double l21 = q12 / l11;
    const double l22 = sqrt(q22 - l21 * l21);
    PhiloxScalar eng(PhiloxScalar::key_t{seed, 0u}, 0);
    NormalScalar<double> zn(0, m.sigma_z);
    auto pair = [&](double sd, double &a, double &b) {
        NormalScalar<double> nd(0, sd);
        a = nd(eng);
        b = nd(eng);
    };
    double x, y, vx, vy, a, b;
    pair(m.sd_pos0, a, b);
    x = __dadd_rn(m.x0, a);
    y = __dadd_rn(m.y0, b);
    pair(m.sd_vel0, a, b);
    vx = __dadd_rn(m.vx0, a);
    vy = __dadd_rn(m.vy0, b);
    for (uint32_t t = 0; t < T; ++t) {
        if (t > 0) {
            double c, d;
            pair(1.0, a, b);
            pair(1.0, c, d);
            x = __dadd_rn(__dadd_rn(x, __dmul_rn(m.dt, vx)), __dmul_rn(l11, a));
            vx = __dadd_rn(vx, __dadd_rn(__dmul_rn(l21, a), __dmul_rn(l22, b)));
            y = __dadd_rn(__dadd_rn(y, __dmul_rn(m.dt, vy)), __dmul_rn(l11, c));
            vy = __dadd_rn(vy, __dadd_rn(__dmul_rn(l21, c), __dmul_rn(l22, d)));
        }
        if (truth) {
            truth[4 * t + 0] = x;
            truth[4 * t + 1] = y;
            truth[4 * t + 2] = vx;
            truth[4 * t + 3] = vy;
        }
        obs[t] = __dadd_rn(atan2(y, x), zn(eng));
    }
}

} // namespace vsmc_cuda
