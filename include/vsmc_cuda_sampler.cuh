// vsmc_cuda_sampler.cuh - the fused FP32 particle filter of libvsmc_cuda as
// vSMC Sampler<T> classes, with the user's model as a device functor.
// Compile with nvcc (sm_103a); needs the reference's headers, the CUDA
// runtime and libvsmc_cuda.so.
//
// The reference's backends plug a state type, a weight type and move
// functors into Sampler<T> (smp/backend_omp.hpp:45-133, the CRTP bases of
// smp/backend_base.hpp:92-363).  The classes here plug in the same way:
//
//   StateCUDA<Dim, float>   the particle state and its filter on the device:
//                           two SoA buffers (StateMatrix<ColMajor, Dim, float>
//                           rows), FP32 log-weights, the resampling passes.
//                           copy(N, nullptr) resamples on the device
//                           (core/particle.hpp:186-192).
//   WeightCUDAF32           its weight_type (core/weight.hpp:321): ess(),
//                           set_equal(), set_log(), add_log(), data() on the
//                           device log-weights; resample_data() is nullptr.
//   InitializeCUDA<Model>   init_type / move_type functors (core/sampler.hpp:
//   MoveCUDA<Model>         64-65): one fused kernel per step moves every
//                           particle with the user's device model, weights it
//                           and reduces ESS, log-evidence and the monitor.
//   MonitorMeanCUDA<Dim, float>  Monitor eval (record_only): the weighted
//                           mean of the model's first monitor_dim components,
//                           reduced inside the step (core/monitor.hpp:242-268).
//
// Model: see vsmc_cuda_filter.cuh.  Usage:
//
//   using State = vsmc::cuda::StateCUDA<4, float>;
//   vsmc::Sampler<State> sampler(N, vsmc::Systematic, 0.5);
//   sampler.particle().value().resample_scheme(vsmc::Systematic, seed);
//   sampler.particle().value().resample_threshold(0.5);  // optional, below
//   sampler.init(vsmc::cuda::InitializeCUDA<MyModel>(model));
//   sampler.move(vsmc::cuda::MoveCUDA<MyModel>(model), false);
//   sampler.monitor("pos", 2, vsmc::cuda::MonitorMeanCUDA<4, float>(), true);
//   sampler.initialize();
//   sampler.iterate(T - 1);
//
// Sampler<T> decides resampling on the host from weight().ess(), which
// waits for the step.  With resample_threshold(t) set to the Sampler's own
// threshold, the device takes the same decision right after the step and
// runs the resampling passes before the host asks, so one host wait per step
// covers the step, the resample and the monitor.  Without it, the passes run
// when Particle::resample calls copy(N, nullptr).  A device decision the
// host did not take (the two thresholds differ) throws at the next step.
//
// Each step queues the copy of the filter's scalars (ESS, log-evidence,
// monitor, decision) behind its kernels, and the host's first read after it
// waits for that copy alone.  From the third step on, a step (the fused
// kernel, with a device threshold the three resampling passes, and the
// scalars' copy) is replayed as a CUDA graph: one
// graph per buffer parity, captured the first time that parity comes up
// and captured again when the model's bytes change.  use_graph(false) on
// the state launches every step on its own.
#ifndef VSMC_CUDA_SAMPLER_CUH
#define VSMC_CUDA_SAMPLER_CUH

#include "vsmc_cuda_backend.hpp"
#include "vsmc_cuda_filter.cuh"

#include <vsmc/rng/engine.hpp>
#include <vsmc/rng/rng_set.hpp>

#include <cmath>
#include <cstring>
#include <memory>

namespace vsmc
{

namespace cuda
{

// A precision-32 filter of vsmc_cuda_pf_create_model, shared by a
// StateCUDA<Dim, float> and its weight.
class FilterCore
{
    public:
    FilterCore(std::size_t N, std::size_t dim) : N_(N), dim_(dim) {}
    FilterCore(const FilterCore &) = delete;
    FilterCore &operator=(const FilterCore &) = delete;
    ~FilterCore()
    {
        drop_graphs();
        if (pf_ != nullptr)
            vsmc_cuda_pf_destroy(pf_);
    }

    std::size_t size() const { return N_; }

    // settings of the next open()
    void configure(int scheme, std::uint32_t seed)
    {
        scheme_ = scheme;
        seed_ = seed;
        drop();
    }
    void threshold(double t)
    {
        threshold_ = t;
        drop();
    }
    void history(std::size_t T)
    {
        history_ = T > 0 ? T : 1;
        drop();
    }
    void use_graph(bool on)
    {
        use_graph_ = on;
        drop_graphs();
    }

    // a filter at step 0 for a model with monitor_dim monitored components
    void open(std::size_t monitor_dim)
    {
        if (pf_ != nullptr && monitor_dim != monitor_dim_)
            drop();
        if (pf_ == nullptr) {
            check(vsmc_cuda_pf_create_model(&pf_, N_, dim_, monitor_dim,
                      scheme_, threshold_, seed_, history_, nullptr),
                "vsmc_cuda_pf_create_model");
            monitor_dim_ = monitor_dim;
        } else {
            check(vsmc_cuda_pf_reset(pf_), "vsmc_cuda_pf_reset");
        }
        ++version_;
        equal_ = false;
        pending_ = false;
    }

    bool is_open() const { return pf_ != nullptr; }

    // one fused step of the model: kernel, then the device's resampling
    // passes (with a device threshold) and the buffer swap
    template <typename Model>
    void step(const Model &model)
    {
        require_open();
        if (pending_)
            throw Error(VSMC_CUDA_ERR_ARG,
                "StateCUDA: the device resampled where Particle::resample "
                "did not (resample_threshold differs from the Sampler's)");
        vsmc_cuda_pf_step_desc d;
        check(vsmc_cuda_pf_step_desc_get(pf_, &d),
            "vsmc_cuda_pf_step_desc_get");
        if (use_graph_ && d.step >= 2) {
            replay(d, model);
        } else {
            check(::vsmc_cuda::pf_step_launch(d, model), "pf_step_launch");
            check(vsmc_cuda_pf_step_commit(pf_), "vsmc_cuda_pf_step_commit");
            check(vsmc_cuda_pf_status_enqueue(pf_),
                "vsmc_cuda_pf_status_enqueue");
        }
        ++version_;
        queued_version_ = version_;
        equal_ = false;
        fresh_ = true;
    }

    // Particle::resample decided to resample (the device may have already)
    void resample()
    {
        require_open();
        const vsmc_cuda_pf_status &st = status();
        if (fresh_ && threshold_ >= 0 && st.resampled) {
            pending_ = false; // the device's resample, now the host's too
        } else {
            check(vsmc_cuda_pf_resample_now(pf_), "vsmc_cuda_pf_resample_now");
            ++version_;
        }
        equal_ = true;
        fresh_ = false;
    }

    void set_equal()
    {
        if (pf_ == nullptr || equal_)
            return;
        check(vsmc_cuda_pf_set_equal(pf_), "vsmc_cuda_pf_set_equal");
        ++version_;
        equal_ = true;
        fresh_ = false;
    }

    // set_log (add false) / add_log (add true) from n device doubles
    void weight_log(const double *lw_dev, bool add)
    {
        require_open();
        check(vsmc_cuda_pf_weight_log(pf_, lw_dev, add ? 1 : 0),
            "vsmc_cuda_pf_weight_log");
        ++version_;
        equal_ = false;
        fresh_ = false;
    }

    // the device scalars after the queued work (waits once per change)
    const vsmc_cuda_pf_status &status()
    {
        require_open();
        if (status_version_ != version_) {
            // the step queued the copy of the scalars after its work
            if (queued_version_ == version_)
                check(vsmc_cuda_pf_status_read(pf_, &status_),
                    "vsmc_cuda_pf_status_read");
            else
                check(vsmc_cuda_pf_get_status(pf_, &status_),
                    "vsmc_cuda_pf_get_status");
            status_version_ = version_;
            if (fresh_ && threshold_ >= 0 && status_.resampled)
                pending_ = true; // until Particle::resample agrees
        }
        return status_;
    }

    vsmc_cuda_pf *handle() { return pf_; }
    std::size_t dim() const { return dim_; }
    std::size_t monitor_dim() const { return monitor_dim_; }

    private:
    void require_open() const
    {
        if (pf_ == nullptr)
            throw Error(VSMC_CUDA_ERR_ARG,
                "StateCUDA: no filter (run InitializeCUDA first)");
    }

    void drop()
    {
        drop_graphs();
        if (pf_ != nullptr)
            vsmc_cuda_pf_destroy(pf_);
        pf_ = nullptr;
        ++version_;
    }

    template <typename Model>
    static const void *model_tag()
    {
        static const char tag = 0;
        return &tag;
    }

    void drop_graphs()
    {
        for (int k = 0; k != 2; ++k) {
            if (graph_[k] != nullptr)
                cudaGraphExecDestroy(graph_[k]);
            graph_[k] = nullptr;
            graph_in_[k] = nullptr;
        }
        graph_tag_ = nullptr;
        graph_model_.clear();
    }

    // the step of d as a graph launch; the host's half of step_commit
    // follows a replay, and runs inside the capture the first time
    template <typename Model>
    void replay(const vsmc_cuda_pf_step_desc &d, const Model &model)
    {
        const unsigned char *mb = reinterpret_cast<const unsigned char *>(&model);
        if (graph_tag_ != model_tag<Model>() ||
            graph_model_.size() != sizeof(Model) ||
            std::memcmp(graph_model_.data(), mb, sizeof(Model)) != 0) {
            drop_graphs();
            graph_tag_ = model_tag<Model>();
            graph_model_.assign(mb, mb + sizeof(Model));
        }
        cudaStream_t st = static_cast<cudaStream_t>(d.stream);
        for (int k = 0; k != 2; ++k) {
            if (graph_[k] != nullptr && graph_in_[k] == d.state_in) {
                check_cuda(cudaGraphLaunch(graph_[k], st), "cudaGraphLaunch");
                check(vsmc_cuda_pf_step_advance(pf_),
                    "vsmc_cuda_pf_step_advance");
                return;
            }
        }
        const int k = graph_[0] == nullptr ? 0 : 1;
        if (graph_[k] != nullptr)
            throw Error(VSMC_CUDA_ERR_ARG,
                "StateCUDA: a third state buffer for the step graphs");
        check_cuda(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal),
            "cudaStreamBeginCapture");
        int rc = ::vsmc_cuda::pf_step_launch(d, model);
        if (rc == VSMC_CUDA_OK)
            rc = vsmc_cuda_pf_step_commit(pf_);
        if (rc == VSMC_CUDA_OK)
            rc = vsmc_cuda_pf_status_enqueue(pf_);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(st, &g);
        if (rc != VSMC_CUDA_OK || e != cudaSuccess) {
            if (g != nullptr)
                cudaGraphDestroy(g);
            check(rc, "captured step");
            check_cuda(e, "cudaStreamEndCapture");
        }
        cudaGraphExec_t x = nullptr;
        const cudaError_t ei = cudaGraphInstantiate(&x, g, 0);
        cudaGraphDestroy(g);
        check_cuda(ei, "cudaGraphInstantiate");
        graph_[k] = x;
        graph_in_[k] = d.state_in;
        check_cuda(cudaGraphLaunch(x, st), "cudaGraphLaunch");
    }

    std::size_t N_, dim_;
    std::size_t monitor_dim_ = 0;
    int scheme_ = VSMC_CUDA_STRATIFIED;
    std::uint32_t seed_ = 0;
    double threshold_ = -1; // host decides
    std::size_t history_ = 1;
    vsmc_cuda_pf *pf_ = nullptr;
    vsmc_cuda_pf_status status_ = {};
    unsigned long long version_ = 1, status_version_ = 0;
    unsigned long long queued_version_ = 0; // a step queued its status copy
    bool equal_ = false;   // the host made the weights equal
    bool fresh_ = false;   // nothing changed the weights since the last step
    bool pending_ = false; // a device resample the host has not taken yet
    bool use_graph_ = true;
    cudaGraphExec_t graph_[2] = {nullptr, nullptr}; // by input buffer
    const float *graph_in_[2] = {nullptr, nullptr};
    const void *graph_tag_ = nullptr;               // the captured model
    std::vector<unsigned char> graph_model_;
};

// weight_type of StateCUDA<Dim, float>: the Weight interface
// (core/weight.hpp:67-230) over the filter's FP32 log-weights.
class WeightCUDAF32
{
    public:
    using size_type = std::size_t;

    explicit WeightCUDAF32(size_type N) : N_(N) {}

    void bind(const std::shared_ptr<FilterCore> &core) { core_ = core; }

    size_type size() const { return N_; }
    size_type resample_size() const { return N_; }

    double ess() const
    {
        if (!bound())
            return static_cast<double>(N_);
        return core_->status().ess;
    }

    // cumulative log-evidence of the run (no reference counterpart; the
    // user guide's estimator, user_guide/tex/smc.tex:176-182)
    double log_evidence() const
    {
        return bound() ? core_->status().log_evidence : 0.0;
    }

    // host copy of the normalized weights (downloaded on request)
    const double *data() const
    {
        host_.assign(N_, 1.0 / static_cast<double>(N_));
        if (!bound())
            return host_.data();
        const vsmc_cuda_pf_status st = core_->status();
        if (st.resampled)
            return host_.data();
        void *lw = nullptr;
        check(vsmc_cuda_pf_state(core_->handle(), nullptr, &lw),
            "vsmc_cuda_pf_state");
        std::vector<float> h(N_);
        check_cuda(cudaMemcpy(h.data(), lw, sizeof(float) * N_,
                       cudaMemcpyDeviceToHost),
            "WeightCUDAF32::data");
        double s = 0;
        for (size_type i = 0; i != N_; ++i) {
            host_[i] = std::exp(static_cast<double>(h[i]) - st.max_log_weight);
            s += host_[i];
        }
        for (size_type i = 0; i != N_; ++i)
            host_[i] /= s;
        return host_.data();
    }

    // nullptr: Particle::resample calls value().copy(N, nullptr)
    const double *resample_data() const { return nullptr; }

    template <typename OutputIter>
    void read_weight(OutputIter first) const
    {
        const double *w = data();
        for (size_type i = 0; i != N_; ++i, ++first)
            *first = w[i];
    }

    void set_equal()
    {
        if (bound())
            core_->set_equal();
    }

    template <typename InputIter>
    void set(InputIter first)
    {
        std::vector<double> l(N_);
        for (size_type i = 0; i != N_; ++i, ++first)
            l[i] = std::log(static_cast<double>(*first));
        upload_log(l, false);
    }

    template <typename InputIter>
    void set_log(InputIter first)
    {
        std::vector<double> l(N_);
        for (size_type i = 0; i != N_; ++i, ++first)
            l[i] = static_cast<double>(*first);
        upload_log(l, false);
    }

    template <typename InputIter>
    void add_log(InputIter first)
    {
        std::vector<double> l(N_);
        for (size_type i = 0; i != N_; ++i, ++first)
            l[i] = static_cast<double>(*first);
        upload_log(l, true);
    }

    private:
    bool bound() const { return core_ && core_->is_open(); }

    void upload_log(const std::vector<double> &l, bool add)
    {
        if (!bound())
            throw Error(VSMC_CUDA_ERR_ARG,
                "WeightCUDAF32: no filter (run InitializeCUDA first)");
        dev_.resize(N_);
        dev_.upload(l.data(), N_);
        core_->weight_log(dev_.get(), add);
    }

    size_type N_;
    std::shared_ptr<FilterCore> core_;
    DeviceArray<double> dev_;
    mutable std::vector<double> host_;
};

// FP32 state: the fused filter.  Dim state components as SoA rows.
template <std::size_t Dim>
class StateCUDA<Dim, float>
{
    public:
    using size_type = std::size_t;
    using state_type = float;
    using weight_type = WeightCUDAF32;
    // the device draws from counter-based streams: one host engine only
    // (the resampling engine lives on the device)
    using rng_set_type = ::vsmc::RNGSetScalar<::vsmc::RNG>;

    explicit StateCUDA(size_type N)
        : N_(N), core_(std::make_shared<FilterCore>(N, Dim))
    {
    }

    size_type size() const { return N_; }
    static constexpr std::size_t dim() { return Dim; }

    // Stratified or Systematic on the exact integer CDF; the engine is the
    // device's Philox4x32 keyed {0, seed} from counter {0, 0, 1, 0}.
    void resample_scheme(ResampleScheme scheme, std::uint32_t seed)
    {
        if (scheme != Stratified && scheme != Systematic)
            throw Error(VSMC_CUDA_ERR_ARG,
                "StateCUDA<Dim, float>: Stratified or Systematic");
        core_->configure(static_cast<int>(scheme), seed);
    }

    // the Sampler's resampling threshold, for the device to resample right
    // after each step (negative: wait for Particle::resample)
    void resample_threshold(double t) { core_->threshold(t); }

    // steps of device history kept (ESS, log-evidence, monitor)
    void reserve_history(std::size_t T) { core_->history(T); }

    // replay steps as CUDA graphs (default) or launch each on its own
    void use_graph(bool on) { core_->use_graph(on); }

    FilterCore &core() { return *core_; }
    const std::shared_ptr<FilterCore> &core_ptr() { return core_; }

    // the particles as host values (downloaded by read_host())
    const float &state(size_type id, std::size_t pos) const
    {
        return host_[pos * stride_ + id];
    }

    void read_host()
    {
        void *s = nullptr;
        check(vsmc_cuda_pf_state(core_->handle(), &s, nullptr),
            "vsmc_cuda_pf_state");
        stride_ = (N_ + 255) / 256 * 256;
        host_.resize(Dim * stride_);
        check_cuda(cudaMemcpy(host_.data(), s, sizeof(float) * Dim * stride_,
                       cudaMemcpyDeviceToHost),
            "StateCUDA::read_host");
    }

    template <typename OutputIter>
    void read_state(std::size_t pos, OutputIter first)
    {
        read_host();
        for (size_type i = 0; i != N_; ++i, ++first)
            *first = host_[pos * stride_ + i];
    }

    // Particle::resample: nullptr resamples on the device; host indices
    // (host-resident weights) are copied in place through the device
    template <typename IntType>
    void copy(size_type N, const IntType *index)
    {
        if (index == nullptr) {
            core_->resample();
            return;
        }
        std::vector<int> idx(N);
        for (size_type i = 0; i != N; ++i)
            idx[i] = static_cast<int>(index[i]);
        DeviceArray<int> d(N);
        d.upload(idx.data(), N);
        void *s = nullptr;
        check(vsmc_cuda_pf_state(core_->handle(), &s, nullptr),
            "vsmc_cuda_pf_state");
        const std::size_t stride = (N_ + 255) / 256 * 256;
        for (std::size_t k = 0; k != Dim; ++k)
            check(vsmc_cuda_state_copy_f32(N, 1, d.get(),
                      static_cast<float *>(s) + k * stride, nullptr),
                "vsmc_cuda_state_copy_f32");
    }

    private:
    size_type N_;
    std::shared_ptr<FilterCore> core_;
    std::vector<float> host_;
    std::size_t stride_ = 0;
};

// init_type functor: the fused step at t = 0 (the model's init draws the
// particles; their weights come from the first observation)
template <typename Model>
class InitializeCUDA
{
    public:
    using state_type = StateCUDA<static_cast<std::size_t>(Model::dim), float>;

    explicit InitializeCUDA(const Model &model) : model_(model) {}

    std::size_t operator()(Particle<state_type> &particle, void *)
    {
        auto &s = particle.value();
        s.core().open(static_cast<std::size_t>(Model::monitor_dim));
        particle.weight().bind(s.core_ptr());
        s.core().step(model_);
        return particle.size();
    }

    Model &model() { return model_; }

    private:
    Model model_;
};

// move_type functor: one fused step of the model; returns N (every
// particle moves, as the reference's bootstrap move reports)
template <typename Model>
class MoveCUDA
{
    public:
    using state_type = StateCUDA<static_cast<std::size_t>(Model::dim), float>;

    explicit MoveCUDA(const Model &model) : model_(model) {}

    std::size_t operator()(std::size_t, Particle<state_type> &particle)
    {
        particle.value().core().step(model_);
        return particle.size();
    }

    Model &model() { return model_; }

    private:
    Model model_;
};

// Monitor eval functor (record_only): r[d] = sum_i W_i x_{d,i} for the first
// dim <= monitor_dim components, from the step's own reduction (after a
// resample: the mean of the resampled particles)
template <std::size_t Dim>
class MonitorMeanCUDA<Dim, float>
{
    public:
    void operator()(std::size_t, std::size_t dim,
        Particle<StateCUDA<Dim, float>> &particle, double *r)
    {
        FilterCore &core = particle.value().core();
        if (dim > core.monitor_dim())
            throw Error(VSMC_CUDA_ERR_ARG,
                "MonitorMeanCUDA: more components than the model monitors");
        const vsmc_cuda_pf_status &st = core.status();
        for (std::size_t d = 0; d != dim; ++d)
            r[d] = st.mean[d];
    }
};

} // namespace vsmc::cuda

} // namespace vsmc

#endif // VSMC_CUDA_SAMPLER_CUH
