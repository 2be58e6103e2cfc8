// The pf example's filter run by vSMC's own Sampler<T> on the fused FP32
// CUDA backend (include/vsmc_cuda_sampler.cuh), with the constant-velocity
// model written here as a user device functor.  Built with nvcc against the
// reference's headers by tests/test_sampler_cuda_gpu.py and by bench.py's
// sampler workload.
//
//   sampler_cuda N T seed scheme threshold device_threshold obs.bin out.bin
//                [runs]
//
// obs.bin: T x 2 doubles.  out.bin: the Sampler's own histories of the last
// run -- monitor "pos" (T x 2), ESS (T), resampled (T, as doubles), then the
// weight's cumulative log-evidence after each step (T).  device_threshold 1
// gives the state the Sampler's threshold (the device resamples right after
// the step); 0 leaves the decision to Particle::resample alone.  runs > 1:
// repeated initialize + iterate(T - 1), each timed on the host clock (the
// Sampler's API waits for each step); prints one line
//   {"runs": R, "ms": [...]}
#include <vsmc_cuda_sampler.cuh>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace
{

struct PfModel {
    static constexpr int dim = 4;
    static constexpr int monitor_dim = 2;
    struct step_type {
        float ox, oy;
    };

    float dt, h, sigma_a, sd_pos0, sd_vel0;
    float lconst2, inv_s, inv_nu, half_nu1;
    const double *obs;
    uint32_t T;

    __device__ step_type step(uint32_t t) const
    {
        const uint32_t k = t < T ? t : T - 1;
        return {static_cast<float>(obs[2 * k]),
            static_cast<float>(obs[2 * k + 1])};
    }

    __device__ void init(
        const step_type &, vsmc_cuda::ParticleRng &rng, float (&x)[4]) const
    {
        float a, b, c, d;
        rng.normal_pair(a, b);
        rng.normal_pair(c, d);
        x[0] = sd_pos0 * a;
        x[1] = sd_pos0 * b;
        x[2] = sd_vel0 * c;
        x[3] = sd_vel0 * d;
    }

    __device__ void move(
        const step_type &, vsmc_cuda::ParticleRng &rng, float (&x)[4]) const
    {
        float e1, e2;
        rng.normal_pair(e1, e2);
        const float ax = sigma_a * e1, ay = sigma_a * e2;
        x[0] = x[0] + dt * x[2] + h * ax;
        x[1] = x[1] + dt * x[3] + h * ay;
        x[2] = x[2] + dt * ax;
        x[3] = x[3] + dt * ay;
    }

    __device__ float log_likelihood(
        const step_type &s, const float (&x)[4]) const
    {
        const float zx = (s.ox - x[0]) * inv_s;
        const float zy = (s.oy - x[1]) * inv_s;
        const float qx = zx * zx * inv_nu;
        const float qy = zy * zy * inv_nu;
        return lconst2 - half_nu1 * __logf(1.0f + fmaf(qx, qy, qx + qy));
    }
};

PfModel make_model(const double *obs_dev, uint32_t T)
{
    // dt 0.1, acceleration sd 1, Student-t(10) with scale 0.5, prior sds 2, 1
    const double dt = 0.1, sa = 1.0, s = 0.5, nu = 10.0;
    const double lc = std::lgamma(0.5 * (nu + 1)) - std::lgamma(0.5 * nu) -
        0.5 * std::log(nu * 3.14159265358979323846) - std::log(s);
    PfModel m;
    m.dt = static_cast<float>(dt);
    m.h = static_cast<float>(0.5 * dt * dt);
    m.sigma_a = static_cast<float>(sa);
    m.sd_pos0 = 2.0f;
    m.sd_vel0 = 1.0f;
    m.lconst2 = static_cast<float>(2 * lc);
    m.inv_s = static_cast<float>(1 / s);
    m.inv_nu = static_cast<float>(1 / nu);
    m.half_nu1 = static_cast<float>(0.5 * (nu + 1));
    m.obs = obs_dev;
    m.T = T;
    return m;
}

} // namespace

int main(int argc, char **argv)
{
    if (argc < 9) {
        std::fprintf(stderr, "usage: %s N T seed scheme threshold "
                             "device_threshold obs.bin out.bin [runs] "
                             "[graph]\n",
            argv[0]);
        return 2;
    }
    const std::size_t N = std::stoul(argv[1]);
    const std::size_t T = std::stoul(argv[2]);
    const auto seed = static_cast<std::uint32_t>(std::stoul(argv[3]));
    const int scheme = std::stoi(argv[4]);
    const double threshold = std::stod(argv[5]);
    const bool dev_thr = std::stoi(argv[6]) != 0;
    const int runs = argc > 9 ? std::stoi(argv[9]) : 1;
    const bool graph = argc > 10 ? std::stoi(argv[10]) != 0 : true;

    std::vector<double> obs(2 * T);
    {
        std::FILE *f = std::fopen(argv[7], "rb");
        if (f == nullptr || std::fread(obs.data(), sizeof(double), 2 * T, f) !=
                2 * T) {
            std::fprintf(stderr, "cannot read %s\n", argv[7]);
            return 2;
        }
        std::fclose(f);
    }
    double *obs_dev = nullptr;
    vsmc::cuda::check_cuda(cudaMalloc(&obs_dev, sizeof(double) * 2 * T),
        "cudaMalloc");
    vsmc::cuda::check_cuda(cudaMemcpy(obs_dev, obs.data(),
                               sizeof(double) * 2 * T, cudaMemcpyHostToDevice),
        "cudaMemcpy");
    const PfModel model = make_model(obs_dev, static_cast<uint32_t>(T));

    using State = vsmc::cuda::StateCUDA<4, float>;
    const auto sch = static_cast<vsmc::ResampleScheme>(scheme);
    vsmc::Sampler<State> sampler(N, sch, threshold);
    sampler.particle().value().resample_scheme(sch, seed);
    if (dev_thr)
        sampler.particle().value().resample_threshold(threshold);
    sampler.particle().value().use_graph(graph);
    sampler.init(vsmc::cuda::InitializeCUDA<PfModel>(model));
    sampler.move(vsmc::cuda::MoveCUDA<PfModel>(model), false);
    sampler.monitor("pos", 2, vsmc::cuda::MonitorMeanCUDA<4, float>(), true);

    std::vector<double> logz(T);
    std::vector<double> ms;
    for (int r = 0; r < runs; ++r) {
        const auto t0 = std::chrono::steady_clock::now();
        sampler.initialize();
        logz[0] = sampler.particle().weight().log_evidence();
        for (std::size_t t = 1; t < T; ++t) {
            sampler.iterate();
            logz[t] = sampler.particle().weight().log_evidence();
        }
        const auto t1 = std::chrono::steady_clock::now();
        ms.push_back(
            std::chrono::duration<double, std::milli>(t1 - t0).count());
    }

    std::vector<double> out;
    const auto &mon = sampler.monitor("pos");
    for (std::size_t t = 0; t < T; ++t) {
        out.push_back(mon.record(0, t));
        out.push_back(mon.record(1, t));
    }
    for (std::size_t t = 0; t < T; ++t)
        out.push_back(sampler.ess_history(t));
    for (std::size_t t = 0; t < T; ++t)
        out.push_back(sampler.resampled_history(t) ? 1.0 : 0.0);
    for (std::size_t t = 0; t < T; ++t)
        out.push_back(logz[t]);
    std::FILE *f = std::fopen(argv[8], "wb");
    if (f == nullptr ||
        std::fwrite(out.data(), sizeof(double), out.size(), f) != out.size()) {
        std::fprintf(stderr, "cannot write %s\n", argv[8]);
        return 2;
    }
    std::fclose(f);
    std::printf("{\"runs\": %d, \"ms\": [", runs);
    for (std::size_t k = 0; k < ms.size(); ++k)
        std::printf("%s%.4f", k ? ", " : "", ms[k]);
    std::printf("]}\n");
    cudaFree(obs_dev);
    return 0;
}
