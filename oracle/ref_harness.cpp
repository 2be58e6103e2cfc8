// Reference harness: test infrastructure, not product code.
//
// Compiled (by oracle/Makefile) against the reference's own headers, together
// with the reference's own C-ABI sources lib/src/vsmc_{rng,resample,memory}.cpp,
// into oracle/_ref/libvsmcref.so.  It exposes, with plain C signatures, the
// pieces of the reference the C-ABI library does not export:
//   * CounterEngine<Philox4x32 / Threefry4x64> word streams placed at an
//     explicit (key, ctr)                          rng/counter.hpp:288-496
//   * u01 conversions                              rng/u01.hpp:126-172
//   * Normal / Student-t scalar and batch draws    rng/normal_distribution.hpp,
//                                                  rng/student_t_distribution.hpp
//   * U01Sequence* lazy sequences                  rng/u01_sequence.hpp:131-259
//   * resampling functors with an explicit engine  resample/*.hpp
//   * Weight::set / set_log / add_log              core/weight.hpp:145-230
//   * a full Sampler<T> particle-filter run        core/sampler.hpp, smp/backend_omp.hpp
//     in the constant-velocity / Student-t form of example/pf/include/pf.hpp,
//     with the log-evidence increment the user guide defines
//     (user_guide/tex/smc.tex:176-182) computed from weight().data() before
//     add_log.
// The golden fixtures under tests/golden/ are produced from this library by
// tests/golden/make_golden.py.

#include <vsmc/core/sampler.hpp>
#include <vsmc/core/state_matrix.hpp>
#include <vsmc/rng/rng.hpp>
#include <vsmc/rng/normal_distribution.hpp>
#include <vsmc/rng/student_t_distribution.hpp>
#include <vsmc/rng/u01_sequence.hpp>
#include <vsmc/resample/index.hpp>
#include <vsmc/resample/resample.hpp>
#include <vsmc/smp/backend_omp.hpp>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

namespace
{

using Eng32 = vsmc::Philox4x32;
using Eng64 = vsmc::Threefry4x64;

Eng32 make_philox(const uint32_t *key, const uint32_t *ctr)
{
    Eng32 eng;
    Eng32::key_type k;
    k[0] = key[0];
    k[1] = key[1];
    eng.key(k);
    Eng32::ctr_type c;
    for (int i = 0; i != 4; ++i)
        c[i] = ctr[i];
    eng.ctr(c);
    return eng;
}

Eng64 make_threefry(const uint64_t *key, const uint64_t *ctr)
{
    Eng64 eng;
    Eng64::key_type k;
    for (int i = 0; i != 4; ++i)
        k[i] = key[i];
    eng.key(k);
    Eng64::ctr_type c;
    for (int i = 0; i != 4; ++i)
        c[i] = ctr[i];
    eng.ctr(c);
    return eng;
}

template <typename Left, typename Right, typename U, typename R>
void u01_conv(std::size_t n, const U *u, R *r)
{
    for (std::size_t i = 0; i != n; ++i)
        r[i] = vsmc::u01_lr<U, R, Left, Right>(u[i]);
}

template <typename U, typename R>
void u01_dispatch(int lr, std::size_t n, const U *u, R *r)
{
    switch (lr) {
        case 0: u01_conv<vsmc::Closed, vsmc::Closed>(n, u, r); break;
        case 1: u01_conv<vsmc::Closed, vsmc::Open>(n, u, r); break;
        case 2: u01_conv<vsmc::Open, vsmc::Closed>(n, u, r); break;
        default: u01_conv<vsmc::Open, vsmc::Open>(n, u, r); break;
    }
}

template <typename Eng, typename R>
void u01_draw(Eng &eng, std::size_t n, R *r, int batch)
{
    if (batch) {
        vsmc::u01_distribution(eng, n, r);
    } else {
        vsmc::U01Distribution<R> u01;
        for (std::size_t i = 0; i != n; ++i)
            r[i] = u01(eng);
    }
}

template <typename Eng, typename R>
void normal_draw(Eng &eng, std::size_t n, R mean, R sd, R *r, int batch)
{
    if (batch) {
        vsmc::normal_distribution(eng, n, r, mean, sd);
    } else {
        vsmc::NormalDistribution<R> nd(mean, sd);
        for (std::size_t i = 0; i != n; ++i)
            r[i] = nd(eng);
    }
}

template <typename Eng, typename R>
void student_t_draw(Eng &eng, std::size_t n, R df, R *r, int batch)
{
    if (batch) {
        vsmc::student_t_distribution(eng, n, r, df);
    } else {
        vsmc::StudentTDistribution<R> st(df);
        for (std::size_t i = 0; i != n; ++i)
            r[i] = st(eng);
    }
}

// ---------------------------------------------------------------------------
// Constant-velocity tracking model with Student-t position observations.
// Written against the pf_state / pf_move pattern of example/pf/include/pf.hpp,
// with the model constants of the benchmark workload.
// ---------------------------------------------------------------------------

struct ModelParam {
    double dt, sigma_a, obs_scale, nu, sd_pos0, sd_vel0;
};

inline double student_t_norm_const(double nu, double s)
{
    return std::lgamma(0.5 * (nu + 1)) - std::lgamma(0.5 * nu) -
        0.5 * std::log(nu * vsmc::const_pi<double>()) - std::log(s);
}

template <typename T>
using PFBase = vsmc::StateOMP<vsmc::StateMatrix<vsmc::ColMajor, 4, T>>;

template <typename T>
class PFState : public PFBase<T>
{
    public:
    using size_type = typename PFBase<T>::size_type;

    explicit PFState(size_type N) : PFBase<T>(N), obs_(nullptr) {}

    void setup(const double *obs, const ModelParam &p, uint32_t seed,
        int native_rng)
    {
        obs_ = obs;
        p_ = p;
        seed_ = seed;
        native_ = native_rng;
        c2_ = static_cast<T>(2 * student_t_norm_const(p.nu, p.obs_scale));
        inv_s_ = static_cast<T>(1 / p.obs_scale);
        inv_nu_ = static_cast<T>(1 / p.nu);
        half_nu1_ = static_cast<T>(0.5 * (p.nu + 1));
    }

    T log_likelihood(std::size_t t, size_type id) const
    {
        const T ox = static_cast<T>(obs_[2 * t + 0]);
        const T oy = static_cast<T>(obs_[2 * t + 1]);
        const T zx = (ox - this->state(id, 0)) * inv_s_;
        const T zy = (oy - this->state(id, 1)) * inv_s_;
        const T qx = zx * zx * inv_nu_;
        const T qy = zy * zy * inv_nu_;
        return c2_ - half_nu1_ * (std::log1p(qx) + std::log1p(qy));
    }

    const ModelParam &param() const { return p_; }
    uint32_t seed() const { return seed_; }
    int native() const { return native_; }

    private:
    const double *obs_;
    ModelParam p_;
    uint32_t seed_;
    int native_;
    T c2_, inv_s_, inv_nu_, half_nu1_;
};

// The per-particle stream: Philox4x32 with key = {step, seed} and counter
// {0, particle, 0, 0}; the engine pre-increments, so the first block is
// generated from counter {1, particle, 0, 0}.
inline Eng32 particle_engine(std::size_t t, uint32_t seed, std::size_t id)
{
    uint32_t key[2] = {static_cast<uint32_t>(t), seed};
    uint32_t ctr[4] = {0, static_cast<uint32_t>(id), 0, 0};
    return make_philox(key, ctr);
}

// One standard-normal pair.  FP64: the reference NormalDistribution<double>
// (u01_co radius).  FP32: Box-Muller with the (0,1] u01_oc radius uniform so
// log(0) cannot occur at 24-bit resolution.
template <typename RNG>
inline void normal_pair(RNG &eng, double sd, double &z1, double &z2)
{
    vsmc::NormalDistribution<double> nd(0, sd);
    z1 = nd(eng);
    z2 = nd(eng);
}

template <typename RNG>
inline void normal_pair(RNG &eng, float sd, float &z1, float &z2)
{
    const uint32_t w0 = static_cast<uint32_t>(eng());
    const uint32_t w1 = static_cast<uint32_t>(eng());
    const float u1 = vsmc::u01_oc<uint32_t, float>(w0);
    const float u2 = vsmc::u01_co<uint32_t, float>(w1);
    const float r = std::sqrt(-2 * std::log(u1));
    const float th = vsmc::const_pi_2<float>() * u2;
    z1 = sd * (r * std::cos(th));
    z2 = sd * (r * std::sin(th));
}

template <typename T>
class PFInit : public vsmc::InitializeOMP<PFState<T>, PFInit<T>>
{
    public:
    std::size_t eval_sp(vsmc::SingleParticle<PFState<T>> sp)
    {
        const PFState<T> &s = sp.particle().value();
        const ModelParam &p = s.param();
        T x, y, vx, vy;
        if (s.native()) {
            normal_pair(sp.rng(), static_cast<T>(p.sd_pos0), x, y);
            normal_pair(sp.rng(), static_cast<T>(p.sd_vel0), vx, vy);
        } else {
            Eng32 eng = particle_engine(0, s.seed(), sp.id());
            normal_pair(eng, static_cast<T>(p.sd_pos0), x, y);
            normal_pair(eng, static_cast<T>(p.sd_vel0), vx, vy);
        }
        sp.state(0) = x;
        sp.state(1) = y;
        sp.state(2) = vx;
        sp.state(3) = vy;
        ll_[sp.id()] = static_cast<double>(s.log_likelihood(0, sp.id()));
        return 1;
    }

    void eval_pre(vsmc::Particle<PFState<T>> &particle)
    {
        ll_.resize(particle.size());
    }

    void eval_post(vsmc::Particle<PFState<T>> &particle)
    {
        // Evidence increment with W_{-1} = 1/N (core/sampler.hpp:732).
        const std::size_t N = particle.size();
        double m = -std::numeric_limits<double>::infinity();
        for (std::size_t i = 0; i != N; ++i)
            m = std::max(m, ll_[i]);
        double s = 0;
        for (std::size_t i = 0; i != N; ++i)
            s += std::exp(ll_[i] - m);
        logz_inc = m + std::log(s / static_cast<double>(N));
        particle.weight().set_log(ll_.data());
    }

    double logz_inc = 0;

    private:
    std::vector<double> ll_;
};

template <typename T>
class PFMove : public vsmc::MoveOMP<PFState<T>, PFMove<T>>
{
    public:
    std::size_t eval_sp(std::size_t t, vsmc::SingleParticle<PFState<T>> sp)
    {
        const PFState<T> &s = sp.particle().value();
        const ModelParam &p = s.param();
        const T dt = static_cast<T>(p.dt);
        const T h = static_cast<T>(0.5 * p.dt * p.dt);
        T ax, ay;
        if (s.native()) {
            normal_pair(sp.rng(), static_cast<T>(p.sigma_a), ax, ay);
        } else {
            Eng32 eng = particle_engine(t, s.seed(), sp.id());
            normal_pair(eng, static_cast<T>(p.sigma_a), ax, ay);
        }
        const T x = sp.state(0), y = sp.state(1);
        const T vx = sp.state(2), vy = sp.state(3);
        sp.state(0) = x + dt * vx + h * ax;
        sp.state(1) = y + dt * vy + h * ay;
        sp.state(2) = vx + dt * ax;
        sp.state(3) = vy + dt * ay;
        ll_[sp.id()] = static_cast<double>(s.log_likelihood(t, sp.id()));
        return 1;
    }

    void eval_pre(std::size_t, vsmc::Particle<PFState<T>> &particle)
    {
        ll_.resize(particle.size());
    }

    void eval_post(std::size_t, vsmc::Particle<PFState<T>> &particle)
    {
        const std::size_t N = particle.size();
        const double *W = particle.weight().data();
        double m = -std::numeric_limits<double>::infinity();
        for (std::size_t i = 0; i != N; ++i)
            m = std::max(m, ll_[i]);
        double s = 0;
        for (std::size_t i = 0; i != N; ++i)
            s += W[i] * std::exp(ll_[i] - m);
        logz_inc = m + std::log(s);
        particle.weight().add_log(ll_.data());
    }

    double logz_inc = 0;

    private:
    std::vector<double> ll_;
};

template <typename T>
class PFMean : public vsmc::MonitorEvalOMP<PFState<T>, PFMean<T>>
{
    public:
    void eval_sp(std::size_t, std::size_t,
        vsmc::SingleParticle<PFState<T>> sp, double *res)
    {
        res[0] = static_cast<double>(sp.state(0));
        res[1] = static_cast<double>(sp.state(1));
    }
};

template <typename T>
int pf_run(std::size_t N, std::size_t T_, uint32_t seed, int scheme,
    double threshold, int native_rng, const ModelParam &p, const double *obs,
    double *mean_out, double *ess_out, int *resampled_out, double *logz_out,
    std::string *tsv = nullptr)
{
    if (native_rng)
        vsmc::Seed::instance().set(seed);
    vsmc::Sampler<PFState<T>> sampler(
        N, static_cast<vsmc::ResampleScheme>(scheme), threshold);
    sampler.particle().value().setup(obs, p, seed, native_rng);
    if (!native_rng) {
        // Resampling engine: key {0, seed}, counter {0, 0, 1, 0}.
        Eng32::key_type k = {{0, seed}};
        sampler.particle().rng().key(k);
        Eng32::ctr_type c = {{0, 0, 1, 0}};
        sampler.particle().rng().ctr(c);
    }
    PFInit<T> init;
    PFMove<T> move;
    sampler.init(std::ref(init));
    sampler.move(std::ref(move), false);
    sampler.monitor("pos", 2, PFMean<T>());

    double logz = 0;
    sampler.initialize();
    logz += init.logz_inc;
    logz_out[0] = logz;
    for (std::size_t t = 1; t < T_; ++t) {
        sampler.iterate();
        logz += move.logz_inc;
        logz_out[t] = logz;
    }
    const auto &mon = sampler.monitor("pos");
    for (std::size_t t = 0; t < T_; ++t) {
        mean_out[2 * t + 0] = mon.record(0, t);
        mean_out[2 * t + 1] = mon.record(1, t);
        ess_out[t] = sampler.ess_history(t);
        resampled_out[t] = sampler.resampled_history(t) ? 1 : 0;
    }
    if (tsv) {
        std::ostringstream os;
        sampler.print(os);
        *tsv = os.str();
    }
    return 0;
}

} // namespace

extern "C" {

// ----------------------------------------------------------------- engines

void ref_philox4x32_words(const uint32_t *key, const uint32_t *ctr,
    std::size_t n, uint32_t *out, int bulk)
{
    Eng32 eng = make_philox(key, ctr);
    if (bulk) {
        vsmc::rng_rand(eng, n, out);
    } else {
        for (std::size_t i = 0; i != n; ++i)
            out[i] = eng();
    }
}

void ref_threefry4x64_words(const uint64_t *key, const uint64_t *ctr,
    std::size_t n, uint64_t *out, int bulk)
{
    Eng64 eng = make_threefry(key, ctr);
    if (bulk) {
        vsmc::rng_rand(eng, n, out);
    } else {
        for (std::size_t i = 0; i != n; ++i)
            out[i] = eng();
    }
}

// ------------------------------------------------------------------- u01

void ref_u01_u32_f64(int lr, std::size_t n, const uint32_t *u, double *r)
{
    u01_dispatch(lr, n, u, r);
}

void ref_u01_u32_f32(int lr, std::size_t n, const uint32_t *u, float *r)
{
    u01_dispatch(lr, n, u, r);
}

void ref_u01_u64_f64(int lr, std::size_t n, const uint64_t *u, double *r)
{
    u01_dispatch(lr, n, u, r);
}

// ---------------------------------------------------- distributions
// eng: 0 = Philox4x32 (key/ctr read as 2/4 uint32 from the low words of the
// uint64 arrays), 1 = Threefry4x64.

#define REF_WITH_ENGINE(call)                                                 \
    if (eng == 0) {                                                           \
        uint32_t k32[2] = {static_cast<uint32_t>(key[0]),                     \
            static_cast<uint32_t>(key[1])};                                   \
        uint32_t c32[4] = {static_cast<uint32_t>(ctr[0]),                     \
            static_cast<uint32_t>(ctr[1]), static_cast<uint32_t>(ctr[2]),     \
            static_cast<uint32_t>(ctr[3])};                                   \
        Eng32 e = make_philox(k32, c32);                                      \
        call;                                                                 \
    } else {                                                                  \
        Eng64 e = make_threefry(key, ctr);                                    \
        call;                                                                 \
    }

void ref_u01_dist_f64(int eng, const uint64_t *key, const uint64_t *ctr,
    std::size_t n, double *r, int batch)
{
    REF_WITH_ENGINE(u01_draw(e, n, r, batch))
}

void ref_u01_dist_f32(int eng, const uint64_t *key, const uint64_t *ctr,
    std::size_t n, float *r, int batch)
{
    REF_WITH_ENGINE(u01_draw(e, n, r, batch))
}

void ref_normal_f64(int eng, const uint64_t *key, const uint64_t *ctr,
    std::size_t n, double mean, double sd, double *r, int batch)
{
    REF_WITH_ENGINE(normal_draw(e, n, mean, sd, r, batch))
}

void ref_normal_f32(int eng, const uint64_t *key, const uint64_t *ctr,
    std::size_t n, float mean, float sd, float *r, int batch)
{
    REF_WITH_ENGINE(normal_draw(e, n, mean, sd, r, batch))
}

void ref_student_t_f64(int eng, const uint64_t *key, const uint64_t *ctr,
    std::size_t n, double df, double *r, int batch)
{
    REF_WITH_ENGINE(student_t_draw(e, n, df, r, batch))
}

// ----------------------------------------------------------- u01 sequences
// kind: 0 sorted, 1 stratified, 2 systematic.  Accesses indices 0..N-1 in
// order (all N values are generated) and then returns the next 4 words of
// the engine in next_words.
void ref_u01_sequence(int kind, std::size_t N, const uint32_t *key,
    const uint32_t *ctr, double *out, uint32_t *next_words)
{
    Eng32 eng = make_philox(key, ctr);
    if (kind == 0) {
        vsmc::U01SequenceSorted<Eng32, double> seq(N, eng);
        for (std::size_t i = 0; i != N; ++i)
            out[i] = seq[i];
    } else if (kind == 1) {
        vsmc::U01SequenceStratified<Eng32, double> seq(N, eng);
        for (std::size_t i = 0; i != N; ++i)
            out[i] = seq[i];
    } else {
        vsmc::U01SequenceSystematic<Eng32, double> seq(N, eng);
        for (std::size_t i = 0; i != N; ++i)
            out[i] = seq[i];
    }
    for (int i = 0; i != 4; ++i)
        next_words[i] = eng();
}

// ------------------------------------------------------------- resampling
// scheme: vsmc::ResampleScheme (Multinomial 0, Stratified 1, Systematic 2,
// Residual 3, ResidualStratified 4, ResidualSystematic 5).  The engine is
// placed at (key, ctr); next_words gets the 4 words it produces afterwards,
// which pins how many words the scheme consumed.
void ref_resample(int scheme, std::size_t M, std::size_t N,
    const uint32_t *key, const uint32_t *ctr, const double *w, int *rep,
    uint32_t *next_words)
{
    Eng32 eng = make_philox(key, ctr);
    switch (scheme) {
        case vsmc::Multinomial:
            vsmc::ResampleMultinomial()(M, N, eng, w, rep);
            break;
        case vsmc::Residual: vsmc::ResampleResidual()(M, N, eng, w, rep); break;
        case vsmc::Stratified:
            vsmc::ResampleStratified()(M, N, eng, w, rep);
            break;
        case vsmc::Systematic:
            vsmc::ResampleSystematic()(M, N, eng, w, rep);
            break;
        case vsmc::ResidualStratified:
            vsmc::ResampleResidualStratified()(M, N, eng, w, rep);
            break;
        case vsmc::ResidualSystematic:
            vsmc::ResampleResidualSystematic()(M, N, eng, w, rep);
            break;
    }
    for (int i = 0; i != 4; ++i)
        next_words[i] = eng();
}

void ref_state_copy_f32(std::size_t N, const int *idx, float *state)
{
    vsmc::StateMatrix<vsmc::ColMajor, 4, float> s(N);
    std::memcpy(s.data(), state, sizeof(float) * 4 * N);
    s.copy(N, idx);
    std::memcpy(state, s.data(), sizeof(float) * 4 * N);
}

void ref_state_copy_f64(std::size_t N, const int *idx, double *state)
{
    vsmc::StateMatrix<vsmc::ColMajor, 4, double> s(N);
    std::memcpy(s.data(), state, sizeof(double) * 4 * N);
    s.copy(N, idx);
    std::memcpy(state, s.data(), sizeof(double) * 4 * N);
}

// ----------------------------------------------------------------- weights

double ref_weight_set_log(std::size_t N, const double *lw, double *W)
{
    vsmc::Weight wt(N);
    wt.set_log(lw);
    std::memcpy(W, wt.data(), sizeof(double) * N);
    return wt.ess();
}

double ref_weight_add_log(
    std::size_t N, const double *W0, const double *l, double *W)
{
    vsmc::Weight wt(N);
    wt.set(W0);
    wt.add_log(l);
    std::memcpy(W, wt.data(), sizeof(double) * N);
    return wt.ess();
}

double ref_weight_set(std::size_t N, const double *w, double *W)
{
    vsmc::Weight wt(N);
    wt.set(w);
    std::memcpy(W, wt.data(), sizeof(double) * N);
    return wt.ess();
}

// ---------------------------------------------------------- particle filter
// precision: 64 or 32 (state type).  native_rng: 0 = the (key = step,
// counter = particle) assignment, 1 = the reference's own per-particle
// engines (RNGSetVector seeded by Seed::instance().set(seed)).
int ref_pf_run(int precision, std::size_t N, std::size_t T, uint32_t seed,
    int scheme, double threshold, int native_rng, double dt, double sigma_a,
    double obs_scale, double nu, double sd_pos0, double sd_vel0,
    const double *obs, double *mean_out, double *ess_out, int *resampled_out,
    double *logz_out)
{
    ModelParam p = {dt, sigma_a, obs_scale, nu, sd_pos0, sd_vel0};
    if (precision == 32)
        return pf_run<float>(N, T, seed, scheme, threshold, native_rng, p,
            obs, mean_out, ess_out, resampled_out, logz_out);
    return pf_run<double>(N, T, seed, scheme, threshold, native_rng, p, obs,
        mean_out, ess_out, resampled_out, logz_out);
}

// Sampler::print (core/sampler.hpp:646-689) of an FP64 run of the filter
// above; buf receives the text (truncated to cap - 1 bytes, NUL-terminated);
// returns its full length.
std::size_t ref_pf_print(std::size_t N, std::size_t T, uint32_t seed,
    int scheme, double threshold, double dt, double sigma_a, double obs_scale,
    double nu, double sd_pos0, double sd_vel0, const double *obs,
    double *mean_out, double *ess_out, int *resampled_out, double *logz_out,
    char *buf, std::size_t cap)
{
    ModelParam p = {dt, sigma_a, obs_scale, nu, sd_pos0, sd_vel0};
    std::string tsv;
    pf_run<double>(N, T, seed, scheme, threshold, 0, p, obs, mean_out,
        ess_out, resampled_out, logz_out, &tsv);
    if (cap > 0) {
        const std::size_t k = tsv.size() < cap - 1 ? tsv.size() : cap - 1;
        std::memcpy(buf, tsv.data(), k);
        buf[k] = 0;
    }
    return tsv.size();
}

// ResampleIndex<int> fed `iters` index rows of N (row-major [iter][N]);
// out: index_matrix<RowMajor> (layout 0) or <ColMajor> (layout 1)
// (resample/index.hpp:127-201); trace: index(id, iter) for every id and iter
// ([iter][N]).
void ref_resample_index(std::size_t N, std::size_t iters, const int *rows,
    int layout, int *out, int *trace)
{
    vsmc::ResampleIndex<int> ri(N);
    ri.reset(); // the constructor leaves the iteration count unset
    for (std::size_t i = 0; i != iters; ++i)
        ri.push_back(rows + i * N);
    vsmc::Vector<int> m = layout == 0
        ? ri.index_matrix<vsmc::RowMajor>()
        : ri.index_matrix<vsmc::ColMajor>();
    std::memcpy(out, m.data(), sizeof(int) * N * iters);
    for (std::size_t it = 0; it != iters; ++it)
        for (std::size_t id = 0; id != N; ++id)
            trace[it * N + id] = ri.index(id, it);
}

// Observation simulation: Philox4x32 engine seeded with `seed` (key {seed,0},
// counter 0).  Prior pairs and acceleration pairs each come from a fresh
// NormalDistribution<double>; the Student-t noise comes from one
// StudentTDistribution<double>(nu) object kept for the whole run.
void ref_pf_simulate(uint32_t seed, std::size_t T, double dt, double sigma_a,
    double obs_scale, double nu, double sd_pos0, double sd_vel0,
    double *truth, double *obs)
{
    Eng32 eng(seed);
    vsmc::StudentTDistribution<double> st(nu);
    double x, y, vx, vy;
    normal_pair(eng, sd_pos0, x, y);
    normal_pair(eng, sd_vel0, vx, vy);
    const double h = 0.5 * dt * dt;
    for (std::size_t t = 0; t != T; ++t) {
        if (t > 0) {
            double ax, ay;
            normal_pair(eng, sigma_a, ax, ay);
            x = x + dt * vx + h * ax;
            y = y + dt * vy + h * ay;
            vx = vx + dt * ax;
            vy = vy + dt * ay;
        }
        truth[4 * t + 0] = x;
        truth[4 * t + 1] = y;
        truth[4 * t + 2] = vx;
        truth[4 * t + 3] = vy;
        const double ex = st(eng);
        const double ey = st(eng);
        obs[2 * t + 0] = x + obs_scale * ex;
        obs[2 * t + 1] = y + obs_scale * ey;
    }
}

} // extern "C"
