// The pf example run through vSMC's own Sampler<T> with the CUDA backend
// classes of include/vsmc_cuda_backend.hpp.  Built by
// tests/test_backend_cpu.py wherever the reference headers exist; run it on a
// GPU host to print the filtering means and the ESS history.
#include <vsmc_cuda_backend.hpp>

#include <cstdio>
#include <vector>

int main(int argc, char **argv)
{
    const std::size_t N = argc > 1 ? std::stoul(argv[1]) : 16384;
    const std::size_t T = 100;
    vsmc_cuda_cv_model model = {0.1, 1.0, 0.5, 10.0, 2.0, 1.0};
    std::vector<double> obs(2 * T);
    {
        double *d_truth = nullptr, *d_obs = nullptr;
        cudaMalloc(&d_truth, sizeof(double) * 4 * T);
        cudaMalloc(&d_obs, sizeof(double) * 2 * T);
        vsmc::cuda::check(
            vsmc_cuda_cv_simulate(0, T, &model, d_truth, d_obs, nullptr),
            "simulate");
        cudaMemcpy(obs.data(), d_obs, sizeof(double) * 2 * T,
            cudaMemcpyDeviceToHost);
        cudaFree(d_truth);
        cudaFree(d_obs);
    }
    using State = vsmc::cuda::StateCUDA<4, double>;
    vsmc::Sampler<State> sampler(N, vsmc::Stratified, 0.5);
    sampler.particle().value().resample_scheme(vsmc::Stratified, 5);
    sampler.init(vsmc::cuda::InitializeCV<4, double>(model, 5, obs));
    sampler.move(vsmc::cuda::MoveCV<4, double>(model, 5, obs), false);
    sampler.monitor("pos", 2, vsmc::cuda::MonitorMeanCUDA<4, double>(), true);
    sampler.initialize();
    sampler.iterate(T - 1);
    const auto &mon = sampler.monitor("pos");
    for (std::size_t t = 0; t < T; ++t)
        std::printf("%zu %.12g %.12g %.12g %d\n", t, mon.record(0, t),
            mon.record(1, t), sampler.ess_history(t),
            sampler.resampled_history(t) ? 1 : 0);
    return 0;
}
