// Host runtime of the GB300 KNP backend: owns device memory, builds the device network at init,
// records the step as CUDA graphs of per-phase kernels (or, for small networks, launches the fused
// step kernel), stages external messages and drains spike recordings.
//
// The step order is the single-threaded backend's (knp/backends/cpu/cpu-single-threaded-backend/
// impl/backend.cpp:89-141): all populations (consume this step's ring slot, emit spikes), then all
// projections (scatter this step's spikes into future ring slots), then additive-STDP updates
// (after the scatter, as modify_weights follows impact construction in delta_impl.h:63-111), then the
// end-of-step kernel (per-phase path). Internal SpikeMessages / SynapticImpactMessages never leave
// the device.
#pragma once

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <thread>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/knp_gb300.h"
#include "kernels.h"

namespace knp_gb300
{

class Error : public std::runtime_error
{
public:
    Error(int code, const std::string &msg) : std::runtime_error(msg), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

struct Uid
{
    knp_uid v{};
    Uid() = default;
    explicit Uid(const knp_uid &u) : v(u) {}
    bool operator<(const Uid &o) const { return std::memcmp(v.bytes, o.v.bytes, 16) < 0; }
    bool operator==(const Uid &o) const { return std::memcmp(v.bytes, o.v.bytes, 16) == 0; }
    bool is_null() const
    {
        for (auto b : v.bytes)
            if (b) return false;
        return true;
    }
};

// Owner of device allocations made for one backend.
class DeviceArena
{
public:
    ~DeviceArena();
    void *alloc(size_t bytes, bool zero = true);
    template <class T>
    T *make(size_t n, bool zero = true)
    {
        return static_cast<T *>(alloc(n * sizeof(T), zero));
    }
    void release(void *p);
    void adopt(void *p, size_t bytes)  // take ownership of a cudaMalloc'd buffer
    {
        ptrs_.push_back(p);
        bytes_ += bytes;
    }
    size_t bytes() const { return bytes_; }

private:
    std::vector<void *> ptrs_;
    size_t bytes_ = 0;
};

// Words of a recorded bitmap per block of the parallel expansion.
constexpr size_t kExpandBlockWords = 4096;

struct RecordedStep
{
    std::vector<uint32_t> bits;  // bit i of word i / 32: neuron i fired
    uint32_t count = 0;
    std::vector<uint32_t> block_prefix;  // spikes before each block of kExpandBlockWords words
};

// Host worker threads for large bitmap expansions: run(n, fn) calls fn(0 .. n - 1) on the workers
// and the calling thread and returns once all calls are done. One run at a time (the backend is not
// reentrant).
class ExpandPool
{
public:
    explicit ExpandPool(unsigned workers);
    ~ExpandPool();
    void run(unsigned n_tasks, const std::function<void(unsigned)> &fn);
    unsigned workers() const { return static_cast<unsigned>(threads_.size()); }

private:
    void work();
    void drain_tasks();
    std::vector<std::thread> threads_;
    std::mutex m_;
    std::condition_variable go_, done_;
    const std::function<void(unsigned)> *fn_ = nullptr;
    unsigned n_tasks_ = 0;
    std::atomic<unsigned> next_{0};
    unsigned busy_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
};

struct ProjectionSlot;

struct PopulationSlot
{
    Uid uid;
    int kind = KNP_NEURON_BLIFAT;
    uint32_t n = 0, n_pad = 0;
    std::vector<knp_blifat_neuron> init_blifat;
    std::vector<knp_resource_stdp_state> init_res;
    std::vector<knp_lif_neuron> init_lif;
    std::vector<knp_altai_neuron> init_altai;
    int acc_request = KNP_GB300_ACC_AUTO;
    bool record = false;
    std::set<Uid> impact_senders;
    // device
    BlifatDev bdev{};
    LifDev ldev{};
    AltaiDev adev{};
    bool is_altai() const { return kind == KNP_NEURON_ALTAI_LIF || kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF; }
    // this step's spike list of the population, whatever its kind
    uint32_t *spike_list() const { return kind == KNP_NEURON_LIF ? ldev.spikes : is_altai() ? adev.spikes : bdev.spikes; }
    const RingView &input_ring() const { return kind == KNP_NEURON_LIF ? ldev.ring : is_altai() ? adev.ring : bdev.ring; }
    RingView ring{};
    uint32_t counter_index = 0;
    // spike recording: ring of rec_slots per-step bitmaps on the device (see BlifatDev)
    uint32_t *rec_bits = nullptr;
    uint32_t rec_words = 0, rec_slots = 0;
    bool has_external_impacts = false;
    // recorded spikes drained to the host: per step, the spike bitmap and its count
    std::map<uint64_t, RecordedStep> recorded;
    uint64_t record_from = 0;
    // SynapticResourceSTDPDeltaSynapse projections into this population (load order) and their
    // concatenated synapse arrays; the training runs for resource-STDP BLIFAT populations.
    std::vector<ProjectionSlot *> res_projs;
    ResSynDev res_syn{};
    uint32_t *res_locked = nullptr;  // device copy of the projections' lock flags
    std::vector<uint32_t> res_locked_host;
    uint32_t work_counter_index = 0;
};

struct ProjectionSlot
{
    Uid uid;
    int kind = KNP_SYNAPSE_DELTA;
    Uid pre_uid, post_uid;
    uint64_t n_syn = 0;
    // host copy until init
    std::vector<uint32_t> pre, post, delay;
    std::vector<float> weight, tau_plus, tau_minus;
    std::vector<uint8_t> type;
    bool generated = false;
    struct
    {
        int kind;  // GenKind
        uint32_t n_pre, n_post;
        uint32_t in_degree;  // largest number of synapses into one postsynaptic neuron (a bound)
        int32_t k_lo, k_hi;
        uint32_t d_lo, d_hi;
        uint64_t seed, stream;
        unsigned long long prob_threshold;  // FixedProbability: 53-bit draw below it keeps a pair
    } gen{};
    std::map<Uid, int> stdp_pops;
    std::set<Uid> spike_senders;
    uint32_t max_delay = 1;
    bool dyadic = true;  // every weight is k/256 with bounded column sums
    // device
    uint32_t n_rows = 0;
    long long *row_ptr = nullptr;
    int32_t *col = nullptr;
    float *w = nullptr;
    uint8_t *delay_d = nullptr;
    uint8_t *type_d = nullptr;
    uint32_t *perm = nullptr;  // CSR position -> loaded synapse index (null for generated projections)
    double pull_fraction = 0.1;  // pull a step when its spikes reach this share of presynaptic neurons (<0: never)
    bool pull = false;           // the gather layout was built
    ProjectionDev dev{};
    StdpDev stdp{};
    std::vector<std::pair<SpikeSource, int>> stdp_sources;  // (source, both lists)
    // resource-STDP synapses: rule state in load order (host copy until init, and for projections
    // with no target population on this backend), lock flag, slice of the target's arrays
    std::vector<knp_resource_synapse> rule;
    bool locked = true;
    PopulationSlot *res_pop = nullptr;
    uint64_t res_offset = 0;
};

struct Channel
{
    Uid uid;
    ChannelDev host{};
    ChannelDev *dev = nullptr;  // device descriptor read by kernels
    // device data
    long long *offsets = nullptr;
    uint32_t *idx = nullptr;
    uint64_t cap_idx = 0, cap_steps = 0;
    bool scheduled = false;        // a device schedule is loaded
    bool owns_generated = false;   // idx allocated by the device generator (cudaFree on replace)
    std::vector<uint32_t> pending;  // host-sent spikes for the next step
    bool has_pending = false;
};

struct PendingImpacts
{
    Uid receiver;
    bool forcing;
    std::vector<uint32_t> post;
    std::vector<float> value;
    std::vector<uint8_t> type;
};

class Backend
{
public:
    explicit Backend(int device);
    ~Backend();

    void load_blifat(const Uid &uid, int kind, uint32_t n, const knp_blifat_neuron *neurons,
                     const knp_resource_stdp_state *ext);
    void load_projection(const Uid &uid, int kind, const Uid &pre_uid, const Uid &post_uid, uint64_t n_syn,
                         const uint32_t *pre, const uint32_t *post, const float *w, const uint32_t *delay,
                         const uint8_t *type, const float *tau_plus, const float *tau_minus);
    void load_resource_projection(const Uid &uid, const Uid &pre_uid, const Uid &post_uid, uint64_t n_syn,
                                  const uint32_t *pre, const uint32_t *post, const float *w, const uint32_t *delay,
                                  const uint8_t *type, const knp_resource_synapse *rule, bool locked);
    void read_resource_synapses(const Uid &proj, knp_resource_synapse *out);
    void generate_projection(const Uid &uid, const Uid &pre_uid, const Uid &post_uid, int kind, uint32_t n_pre,
                             uint32_t n_post, uint64_t count, double probability, int32_t k_lo, int32_t k_hi,
                             uint32_t d_lo, uint32_t d_hi, uint64_t seed, uint64_t stream);
    void set_stdp_population(const Uid &proj, const Uid &pop, int processing);
    void subscribe(const Uid &receiver, const Uid &sender);
    void set_accumulator(const Uid &pop, int mode);
    void set_pull_threshold(const Uid &proj, double fraction);
    void set_step_mode(int mode);
    bool fused() const { return fused_; }
    int step_kernel() const { return fused_ ? KNP_GB300_STEP_FUSED : (grid_ ? KNP_GB300_STEP_GRID : KNP_GB300_STEP_PHASES); }
    void record_spikes(const Uid &pop, bool enable);
    void init();

    void send_spikes(const Uid &sender, uint64_t send_time, uint32_t n, const uint32_t *idx);
    void load_schedule(const Uid &sender, uint64_t first_step, uint64_t n_steps, const int64_t *offsets,
                       const uint32_t *idx);
    void generate_bernoulli(const Uid &sender, uint32_t n_sources, double p, uint64_t first_step, uint64_t n_steps,
                            uint64_t seed, uint64_t stream);
    void send_impacts(const Uid &sender, const Uid &receiver, bool forcing, uint32_t n, const uint32_t *post,
                      const float *value, const uint8_t *type);

    void step(uint64_t n);
    float step_timed(uint64_t n);
    void profile_phases(uint64_t n, float *ms);
    void profile_grid_phases(uint64_t n, double *us);
    uint64_t current_step() const { return step_; }
    void read_spikes(const Uid &pop, uint64_t step, uint32_t cap, uint32_t *out, uint32_t *n);
    void discard_spikes(uint64_t before);
    void read_blifat(const Uid &pop, knp_blifat_neuron *out, knp_resource_stdp_state *ext);
    void load_lif(const Uid &uid, uint32_t n, const knp_lif_neuron *neurons);
    void load_altai(const Uid &uid, int kind, uint32_t n, const knp_altai_neuron *neurons,
                    const knp_resource_stdp_state *ext);
    void read_altai(const Uid &pop, knp_altai_neuron *out, knp_resource_stdp_state *ext);
    void read_lif(const Uid &pop, knp_lif_neuron *out);
    void read_weights(const Uid &proj, float *out);
    uint64_t projection_size(const Uid &proj) const;
    void counters(uint64_t *events, uint64_t *spikes, uint64_t *updates);
    void synchronize();
    void set_learning(bool on);
    cudaStream_t stream() const { return stream_; }

private:
    PopulationSlot *find_pop(const Uid &u);
    ProjectionSlot *find_proj(const Uid &u);
    const ProjectionSlot *find_proj(const Uid &u) const;
    Channel *find_channel(const Uid &u);
    Channel &channel(const Uid &u);
    void require_not_init(const char *what) const;
    void require_init(const char *what) const;

    void build_population(PopulationSlot &p);
    void build_projection(ProjectionSlot &p);
    GenSpec gen_spec(const ProjectionSlot &p, const unsigned long long *cand) const;
    void build_stdp(ProjectionSlot &p);
    void build_pull(ProjectionSlot &p);
    void build_resource_synapses(PopulationSlot &q);
    void upload_locks();
    int gather_grid(const ProjectionSlot &p) const;
    void wire();
    void enqueue_step();
    void launch_population(const PopulationSlot &q);
    bool small_net_eligible(std::string &why) const;
    bool grid_net_eligible(std::string &why);
    void build_small_net();
    void setup_ring_window();
    void capture_graphs();
    void stage_host_inputs();
    void drain_recordings() { drain_recordings(step_); }
    void drain_recordings(uint64_t upto);
    void check_device_error();
    void alloc_recording(PopulationSlot &p);
    uint64_t steps_before_drain() const;

    int device_ = 0;
    int sm_count_ = 0;
    cudaStream_t stream_ = nullptr;
    DeviceArena arena_;
    bool initialized_ = false;
    bool learning_ = true;
    uint64_t step_ = 0;  // host mirror of Control::step
    std::vector<std::unique_ptr<PopulationSlot>> pops_;
    std::vector<std::unique_ptr<ProjectionSlot>> projs_;
    std::vector<std::unique_ptr<Channel>> channels_;
    std::vector<std::pair<Uid, Uid>> subs_;
    std::vector<PendingImpacts> pending_impacts_;
    Control *ctl_ = nullptr;
    uint32_t *counters_ = nullptr;  // per-step counters
    uint32_t n_counters_ = 0, n_spike_counters_ = 0;
    uint64_t drained_to_ = 0;  // recorded steps before this one have been copied to the host
    // pinned host buffer that recorded bitmaps are drained through
    uint32_t *rec_host_ = nullptr;
    size_t rec_host_words_ = 0;
    uint64_t neurons_total_ = 0;
    uint64_t updates_before_init_ = 0;
    cudaGraphExec_t graph1_ = nullptr, graphK_ = nullptr;
    static constexpr uint64_t kGraphSteps = 16;
    // Fused step kernel for small networks (small_net.cu: one CTA cluster runs whole steps), chosen at init.
    int step_mode_ = 0;  // knp_gb300_step_mode
    bool fused_ = false;
    SmallNet small_{};
    int small_cluster_ = 1;  // CTAs of the fused kernel's cluster
    uint32_t *counters_alt_ = nullptr;  // the fused kernel's second set of per-step counters
    std::vector<std::pair<const uint32_t *, uint32_t *>> spikes_alt_;  // spike list -> its second copy
    static constexpr uint64_t kSmallMaxNeurons = 16384;
    static constexpr uint64_t kSmallMaxSynapses = 1ull << 22;
    static constexpr uint64_t kSmallMaxStepsPerLaunch = 1ull << 16;
    // Persistent grid step kernel (grid_net.cu: one cooperative launch of one CTA per SM runs whole
    // steps), chosen at init for networks the fused kernel does not take.
    bool grid_ = false;
    GridNet grid_net_{};
    std::vector<uint32_t> small_pull_;  // indices (into the fused descriptor sets' projections) with a gather layout
    int grid_ctas_ = 0;
    size_t grid_smem_ = 0;
    // L2 access policy of the grid kernel's launches: the largest FP32 input ring kept persisting.
    cudaAccessPolicyWindow ring_window_{};
    bool persisting_l2_ = false;
    size_t persisting_before_ = 0;  // the context's set-aside before this backend changed it (restored at destroy)
    // pinned staging for host-sent messages
    void *pinned_ = nullptr;
    size_t pinned_bytes_ = 0;
    cudaEvent_t pinned_free_ = nullptr;
    bool any_recording_ = false;
    // Completion events of recent steps (while spikes are recorded), so that a step's bitmaps can be
    // copied to the host on copy_stream_ while later steps still run on stream_.
    static constexpr uint64_t kStepEvents = 16;
    cudaEvent_t step_ev_[kStepEvents] = {};
    uint64_t step_ev_of_[kStepEvents] = {};  // the step each event was last recorded after, plus one
    cudaStream_t copy_stream_ = nullptr;
    std::unique_ptr<ExpandPool> expand_pool_;  // created on the first large spike read
    Control *ctl_host_ = nullptr;  // pinned copy of the control block read after a drain
    void record_step_event(uint64_t last_step);
};

}  // namespace knp_gb300
