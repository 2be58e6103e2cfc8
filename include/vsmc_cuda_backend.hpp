// vsmc_cuda_backend.hpp - CUDA backend classes for vSMC's Sampler<T>.
//
// The CUDA sibling of the reference's smp/backend_{seq,omp,tbb}.hpp for the
// particle-filter path, built on the C ABI of libvsmc_cuda (vsmc_cuda.h).
// This header holds the FP64 classes, which keep the reference's arithmetic
// step for step (normalized double weights, the exact resampling schemes):
//
//   StateCUDA<Dim, double> particle state on the device (SoA, StateMatrix
//                         <ColMajor, Dim, T> layout, core/state_matrix.hpp:
//                         320-364); resampling runs in copy(N, nullptr)
//   WeightCUDA            the Weight class (core/weight.hpp:67-230) on the
//                         device, chosen through the weight_type trait
//                         (core/weight.hpp:321); resample_data() is nullptr,
//                         so Particle::resample hands resampling to the state
//                         (core/particle.hpp:175-192)
//   InitializeCV / MoveCV the constant-velocity / Student-t model's init and
//                         move (the pf example's pf_init / pf_move,
//                         example/pf/include/pf.hpp:111-178) as Sampler
//                         init_type / move_type functors
//   MonitorMeanCUDA       Monitor eval functor (record_only) computing the
//                         weighted mean on the device (core/monitor.hpp:
//                         242-268)
//
// StateCUDA<Dim, float> -- the fused FP32 filter with a user device model
// (InitializeCUDA<Model> / MoveCUDA<Model>) -- is in vsmc_cuda_sampler.cuh,
// which needs nvcc.
//
// Usage (the pf example with the FP64 CUDA backend):
//
//   using State = vsmc::cuda::StateCUDA<4, double>;
//   vsmc::Sampler<State> sampler(N, vsmc::Stratified, 0.5);
//   sampler.particle().value().resample_scheme(vsmc::Stratified, seed);
//   sampler.init(vsmc::cuda::InitializeCV<4, double>(model, seed, obs));
//   sampler.move(vsmc::cuda::MoveCV<4, double>(model, seed, obs), false);
//   sampler.monitor("pos", 2, vsmc::cuda::MonitorMeanCUDA<4, double>(), true);
//   sampler.initialize();
//   sampler.iterate(T - 1);
//
// Requires the reference's headers (vsmc/core/sampler.hpp), the CUDA runtime
// headers and linking with libvsmc_cuda.so and cudart.  Errors from the C ABI
// throw vsmc::cuda::Error.
#ifndef VSMC_CUDA_BACKEND_HPP
#define VSMC_CUDA_BACKEND_HPP

#include <vsmc/core/sampler.hpp>

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "vsmc_cuda.h"

namespace vsmc
{

namespace cuda
{

class Error : public std::runtime_error
{
    public:
    Error(int status, const char *where)
        : std::runtime_error(std::string(where) + ": " +
              vsmc_cuda_status_string(status)),
          status_(status)
    {
    }

    int status() const { return status_; }

    private:
    int status_;
};

inline void check(int status, const char *where)
{
    if (status != VSMC_CUDA_OK)
        throw Error(status, where);
}

inline void check_cuda(cudaError_t e, const char *where)
{
    if (e != cudaSuccess)
        throw Error(VSMC_CUDA_ERR_CUDA, where);
}

// Owning device array.
template <typename T>
class DeviceArray
{
    public:
    DeviceArray() = default;
    explicit DeviceArray(std::size_t n) { resize(n); }
    DeviceArray(const DeviceArray &other) { *this = other; }
    DeviceArray &operator=(const DeviceArray &other)
    {
        if (this != &other) {
            resize(other.n_);
            if (n_)
                check_cuda(cudaMemcpy(p_, other.p_, sizeof(T) * n_,
                               cudaMemcpyDeviceToDevice),
                    "DeviceArray copy");
        }
        return *this;
    }
    ~DeviceArray() { release(); }

    void resize(std::size_t n)
    {
        if (n == n_)
            return;
        release();
        if (n)
            check_cuda(cudaMalloc(&p_, sizeof(T) * n), "cudaMalloc");
        n_ = n;
    }

    T *get() { return p_; }
    const T *get() const { return p_; }
    std::size_t size() const { return n_; }

    void upload(const T *host, std::size_t n)
    {
        check_cuda(cudaMemcpy(p_, host, sizeof(T) * n, cudaMemcpyHostToDevice),
            "upload");
    }

    void download(T *host, std::size_t n) const
    {
        check_cuda(cudaMemcpy(host, p_, sizeof(T) * n, cudaMemcpyDeviceToHost),
            "download");
    }

    private:
    void release()
    {
        if (p_)
            cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
    }

    T *p_ = nullptr;
    std::size_t n_ = 0;
};

// Device-resident Weight (core/weight.hpp:67-230) with the reference's
// arithmetic: normalized doubles, left-to-right sums, ESS = 1 / sum W^2.
class WeightCUDA
{
    public:
    using size_type = std::size_t;

    explicit WeightCUDA(size_type N) : W_(N), ess_dev_(1), host_(N) {}

    size_type size() const { return W_.size(); }
    size_type resample_size() const { return size(); }

    double ess() const
    {
        double e = 0;
        ess_dev_.download(&e, 1);
        return e;
    }

    // host copy of the normalized weights (downloaded on request)
    const double *data() const
    {
        W_.download(host_.data(), size());
        return host_.data();
    }

    // nullptr: Particle::resample calls value().copy(N, nullptr), which
    // resamples on the device (core/particle.hpp:175-192)
    const double *resample_data() const { return nullptr; }

    template <typename OutputIter>
    void read_weight(OutputIter first) const
    {
        const double *w = data();
        for (size_type i = 0; i != size(); ++i, ++first)
            *first = w[i];
    }

    void set_equal()
    {
        check(vsmc_cuda_weight_set_equal(size(), W_.get(), ess_dev_.get(),
                  nullptr),
            "WeightCUDA::set_equal");
    }

    template <typename InputIter>
    void set(InputIter first)
    {
        upload_host(first);
        check(vsmc_cuda_weight_set(size(), W_.get(), W_.get(), ess_dev_.get(),
                  nullptr),
            "WeightCUDA::set");
    }

    template <typename InputIter>
    void set_log(InputIter first)
    {
        upload_host(first);
        set_log_device(W_.get());
    }

    template <typename InputIter>
    void add_log(InputIter first)
    {
        DeviceArray<double> l(size());
        std::vector<double> tmp(size());
        for (size_type i = 0; i != size(); ++i, ++first)
            tmp[i] = *first;
        l.upload(tmp.data(), size());
        add_log_device(l.get());
    }

    // device-pointer forms used by the CUDA init / move functors
    void set_log_device(const double *lw)
    {
        check(vsmc_cuda_weight_set_log(size(), lw, W_.get(), ess_dev_.get(),
                  nullptr),
            "WeightCUDA::set_log");
    }

    void add_log_device(const double *l)
    {
        check(vsmc_cuda_weight_add_log(size(), l, W_.get(), ess_dev_.get(),
                  nullptr),
            "WeightCUDA::add_log");
    }

    double *device_data() { return W_.get(); }
    const double *device_data() const { return W_.get(); }

    private:
    template <typename InputIter>
    void upload_host(InputIter first)
    {
        for (size_type i = 0; i != size(); ++i, ++first)
            host_[i] = *first;
        W_.upload(host_.data(), size());
    }

    DeviceArray<double> W_;
    DeviceArray<double> ess_dev_;
    mutable std::vector<double> host_;
};

// Particle state on the device: Dim rows of N values (StateMatrix<ColMajor,
// Dim, T> layout).  state(id, pos) reads a host copy downloaded on request.
// This is the FP64 state; StateCUDA<Dim, float> (vsmc_cuda_sampler.cuh) is
// the fused FP32 filter.
template <std::size_t Dim, typename T>
class StateCUDA
{
    static_assert(sizeof(T) == 8,
        "StateCUDA<Dim, double> here; StateCUDA<Dim, float> is the fused "
        "FP32 filter of vsmc_cuda_sampler.cuh (compile with nvcc)");

    public:
    using size_type = std::size_t;
    using state_type = T;
    using weight_type = WeightCUDA;

    explicit StateCUDA(size_type N)
        : N_(N), data_(Dim * N), rep_(N), idx_(N), host_(Dim * N)
    {
        resample_scheme(Stratified, 0);
    }

    size_type size() const { return N_; }
    static constexpr std::size_t dim() { return Dim; }

    T *device_data() { return data_.get(); }
    const T *device_data() const { return data_.get(); }

    // host copy (downloaded by read_host())
    const T &state(size_type id, std::size_t pos) const
    {
        return host_[pos * N_ + id];
    }

    void read_host() { data_.download(host_.data(), Dim * N_); }

    template <typename OutputIter>
    void read_state(std::size_t pos, OutputIter first)
    {
        read_host();
        for (size_type i = 0; i != N_; ++i, ++first)
            *first = host_[pos * N_ + i];
    }

    // The resampling scheme and engine of the device path (the reference's
    // Particle::rng_, core/particle.hpp:149, 187): Philox4x32 keyed
    // {0, seed} from counter {0, 0, 1, 0}.
    void resample_scheme(ResampleScheme scheme, std::uint32_t seed)
    {
        scheme_ = static_cast<int>(scheme);
        check(vsmc_cuda_rng_init(&rng_, VSMC_CUDA_PHILOX4X32, 0),
            "StateCUDA::resample_scheme");
        const std::uint64_t key[2] = {0, seed};
        check(vsmc_cuda_rng_set_key(&rng_, 2, key), "rng key");
        const std::uint64_t ctr[4] = {0, 0, 1, 0};
        check(vsmc_cuda_rng_set_ctr(&rng_, 4, ctr), "rng ctr");
    }

    void bind_weight(WeightCUDA *w) { weight_ = w; }

    // Particle::resample with host weights: copy through host indices
    template <typename IntType>
    void copy(size_type N, const IntType *index)
    {
        if (index == nullptr) {
            resample_device(N);
            return;
        }
        std::vector<int> idx(N);
        for (size_type i = 0; i != N; ++i)
            idx[i] = static_cast<int>(index[i]);
        idx_.upload(idx.data(), N);
        copy_device(N);
    }

    private:
    void resample_device(size_type N)
    {
        if (weight_ == nullptr)
            throw Error(VSMC_CUDA_ERR_ARG, "StateCUDA: no bound WeightCUDA");
        check(vsmc_cuda_resample(N, N, &rng_, weight_->device_data(),
                  rep_.get(), scheme_, nullptr),
            "vsmc_cuda_resample");
        check(vsmc_cuda_resample_trans_rep_index(
                  N, N, rep_.get(), idx_.get(), nullptr),
            "vsmc_cuda_resample_trans_rep_index");
        copy_device(N);
    }

    void copy_device(size_type N)
    {
        check(vsmc_cuda_state_copy_f64(N, Dim, idx_.get(),
                  reinterpret_cast<double *>(data_.get()), nullptr),
            "vsmc_cuda_state_copy");
    }

    size_type N_;
    DeviceArray<T> data_;
    DeviceArray<int> rep_;
    DeviceArray<int> idx_;
    std::vector<T> host_;
    WeightCUDA *weight_ = nullptr;
    vsmc_cuda_rng rng_;
    int scheme_ = static_cast<int>(Stratified);
};

// init_type functor: prior draws and weights from observation 0
// (pf_init, example/pf/include/pf.hpp:111-144).  obs: T x 2 host values.
template <std::size_t Dim, typename T>
class InitializeCV
{
    static_assert(Dim == 4, "the constant-velocity model has 4 components");
    static_assert(sizeof(T) == 8,
        "FP64 only; the FP32 filter takes InitializeCUDA<Model> / "
        "MoveCUDA<Model> (vsmc_cuda_sampler.cuh)");

    public:
    InitializeCV(const vsmc_cuda_cv_model &model, std::uint32_t seed,
        std::vector<double> obs)
        : model_(model), seed_(seed), obs_(std::move(obs))
    {
    }

    std::size_t operator()(Particle<StateCUDA<Dim, T>> &particle, void *)
    {
        auto &s = particle.value();
        s.bind_weight(&particle.weight());
        const std::size_t N = particle.size();
        ll_.resize(N);
        loglik(0, s, N);
        particle.weight().set_log_device(ll_.get());
        return N;
    }

    protected:
    void loglik(std::size_t t, StateCUDA<Dim, T> &s, std::size_t N)
    {
        check(vsmc_cuda_cv_move_f64(N, t, seed_, &model_, obs_.data() + 2 * t,
                  reinterpret_cast<double *>(s.device_data()), ll_.get(),
                  nullptr),
            "vsmc_cuda_cv_move_f64");
    }

    vsmc_cuda_cv_model model_;
    std::uint32_t seed_;
    std::vector<double> obs_;
    DeviceArray<double> ll_;
};

// move_type functor: propagate and weight by observation `iter`
// (pf_move, example/pf/include/pf.hpp:146-178); returns N (bootstrap).
template <std::size_t Dim, typename T>
class MoveCV : public InitializeCV<Dim, T>
{
    public:
    using InitializeCV<Dim, T>::InitializeCV;

    std::size_t operator()(std::size_t iter, Particle<StateCUDA<Dim, T>> &particle)
    {
        auto &s = particle.value();
        s.bind_weight(&particle.weight());
        const std::size_t N = particle.size();
        this->ll_.resize(N);
        this->loglik(iter, s, N);
        particle.weight().add_log_device(this->ll_.get());
        return N;
    }
};

// Monitor eval functor (record_only): r[d] = sum_i W_i state(i, d), d < dim
template <std::size_t Dim, typename T>
class MonitorMeanCUDA
{
    public:
    void operator()(std::size_t, std::size_t dim,
        Particle<StateCUDA<Dim, T>> &particle, double *r)
    {
        const std::size_t N = particle.size();
        out_.resize(dim);
        check(vsmc_cuda_monitor_mean_f64(N, dim,
                  reinterpret_cast<const double *>(
                      particle.value().device_data()),
                  particle.weight().device_data(), out_.get(), nullptr),
            "vsmc_cuda_monitor_mean");
        out_.download(r, dim);
    }

    private:
    DeviceArray<double> out_;
};

} // namespace vsmc::cuda

} // namespace vsmc

#endif // VSMC_CUDA_BACKEND_HPP
