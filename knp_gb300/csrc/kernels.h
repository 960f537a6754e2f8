// Device data layout of the GB300 KNP backend and the host-side launchers of its kernels.
//
// Layout in HBM (one backend):
//   population  SoA arrays of n_pad = round_up(n, 4) entries (float4-aligned), one per live state
//               field; parameters either broadcast (uniform across the population) or SoA arrays.
//   input ring  [slots][n_pad] accumulators of postsynaptic input, slot = step mod slots, with
//               slots = the largest delay into the population. FP32 (exact for dyadic weights) or
//               two-word fixed point (order-independent, exact for every FP32 weight that is a
//               multiple of 2^-48 while the sum stays below 2^54): a high word in units of 2^-8 and
//               a low word in units of 2^-48 per neuron. Optional rings for conductance / dopamine
//               input and a forcing bitmap for resource-STDP neurons.
//   projection  presynaptic-major CSR: row_ptr int64[n_pre + 1], col int32[S], weight fp32[S],
//               delay u8[S], optional per-synapse output type u8[S]; STDP projections add a
//               postsynaptic-major index (col_ptr, CSR positions) and per-column spike histories.
//   spikes      per population a spike list (u32[n]) + count, written by the population kernel
//               with warp-ballot compaction, consumed by projection kernels in the same step.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>
#include <utility>

namespace knp_gb300
{

constexpr int kFxLoBits = 40;  // fixed-point input: value = hi * 2^-8 + lo * 2^-48
constexpr int kMaxSources = 8;

// Device-resident step control block (one per backend).
struct Control
{
    unsigned long long step;          // step being executed
    unsigned long long events_total;  // synaptic events (impacts created) since init
    unsigned long long spikes_total;  // spikes since init
    unsigned int error;               // sticky error bits a kernel can report through; checked by the host
    unsigned int pad;
};

// Bits of Control::error.
constexpr unsigned int kErrGridBarrier = 1u << 0;  // a grid barrier of the persistent grid kernel gave up
constexpr unsigned int kErrBlockingEvents = 1u << 1;  // more BLOCKING impacts on an AltAI population in a step than kept

struct RingView
{
    uint32_t n;      // neurons
    uint32_t pitch;  // elements per slot row (multiple of 4)
    uint32_t slots;  // ring length
    int fixed;       // 0: v32, 1: v64 + v64lo
    float *v32;
    long long *v64;    // fixed point, sums of high words (units of 2^-8)
    long long *v64lo;  // fixed point, sums of low words (units of 2^-48, each addend in [0, 2^40])
    float *g;          // conductance input, or null
    float *dopa;       // dopamine input, or null
    uint32_t *forced;  // forcing bitmap [slots][words], or null
    uint32_t words;
    // BLOCKING impacts (last writer in message order wins), or null: per (slot, neuron) the largest
    // key blocking_key() of the impacts arriving at that step; blk_w[order] is the weight array (CSR
    // order) of the projection with load order `order`, blk_ext[neuron] the value of this step's last
    // external BLOCKING impact (key kBlkExternal << kBlkOrderShift).
    unsigned long long *blk;
    const float *const *blk_w;
    long long *blk_ext;
    // Non-finite EXCITATORY / INHIBITORY_CURRENT impacts (trained resource-STDP weights can become NaN
    // or infinite), or null: one byte per (slot, neuron), packed four to a word, bit 0 NaN, bit 1 +inf,
    // bit 2 -inf; such impacts are not added to the fixed-point sum.
    uint32_t *nf;
    // BLOCKING impacts on an AltAI-LIF population, or null: every impact of a step kept as an event
    // (key blocking_key(), value, target) in its slot's list of bev_cap entries; the population's
    // blocking kernel applies them in key order (altai_impl.h:74-83 depends on their order).
    unsigned long long *bev_key;
    float *bev_val;
    uint32_t *bev_tgt;
    uint32_t *bev_count;  // [slots]
    uint32_t bev_cap;
};

// Key of a BLOCKING impact: the reference applies the impacts of a step in message order and the last
// one sets the blocking period (blifat_impl.h:86). Messages arrive in projection load order, then
// the external messages; within a projection's message, impacts of earlier source steps (larger
// delays) come first, then by ascending spike index and synapse order, which is the CSR position.
constexpr int kBlkOrderShift = 58;
constexpr int kBlkDelayShift = 50;
constexpr unsigned long long kBlkExternal = 63;  // external SynapticImpactMessages come last
constexpr unsigned long long kBlkPosMask = (1ull << kBlkDelayShift) - 1;
__host__ __device__ inline unsigned long long blocking_key(uint32_t order, uint32_t delay, long long csr_pos)
{
    return (static_cast<unsigned long long>(order + 1) << kBlkOrderShift) |
           (static_cast<unsigned long long>(255u - delay) << kBlkDelayShift) |
           (static_cast<unsigned long long>(csr_pos) & kBlkPosMask);
}

// Liveness flags of a BLIFAT population: a field that is not live keeps a value that follows from
// its initial value alone and is neither read nor written per step.
enum BlifatFlags : uint32_t
{
    kLiveVRead = 1u << 0,     // potential carries over between steps (potential_decay != 0 somewhere)
    kLiveThrDyn = 1u << 1,    // dynamic threshold
    kLiveTrace = 1u << 2,     // postsynaptic trace
    kLiveG = 1u << 3,         // inhibitory conductance
    kLiveBurst = 1u << 4,     // bursting phase
    kLiveBlock = 1u << 5,     // total blocking period
    kLiveRefract = 1u << 6,   // steps since last firing must be tracked per neuron
    kLiveDopa = 1u << 7,      // dopamine input
    kLiveVPre = 1u << 8,      // store pre-impact potential
    kResource = 1u << 9,      // synaptic-resource-STDP neuron bookkeeping
    kLiveRenorm = 1u << 10,   // free-resource renormalisation can fire
    kLiveAddThr = 1u << 11,   // additional threshold differs from 0 somewhere
    kResSyn = 1u << 12,       // resource-STDP neurons with SynapticResourceSTDPDeltaSynapse projections
};

// One parameter: a broadcast value, or a per-neuron array when `a` is not null.
struct ParamF
{
    const float *a;
    float u;
};
struct ParamU
{
    const uint32_t *a;
    uint32_t u;
};

struct ResourceDev
{
    // state
    int32_t *isi_status;
    unsigned long long *last_step, *last_spike_step, *first_isi_spike;
    float *stability, *free_resource;
    uint8_t *is_forced;  // is_being_forced_ of the last step
    // parameters
    ParamF add_thr_coef, resource_threshold, stability_change_param, stability_change_at_isi, d_h;
    ParamU isi_max, dopamine_time, drain;
};

// SynapticResourceSTDPDeltaSynapse synapses into one population: the synapses of all its
// resource-STDP projections, concatenated in projection load order, each projection's CSR range
// one slice (the projection's scatter reads its weights and writes last_spike there). Synapse
// state is the rule of stdp_synaptic_resource_rule.h:45-89.
constexpr int kResSlotShift = 56;  // col_pos entries: projection slot << 56 | position
struct ResSynDev
{
    float *w;                        // weight_
    float *resource;                 // synaptic_resource_
    const float *w_min, *w_max, *d_u;
    const uint32_t *period;          // dopamine_plasticity_period_
    unsigned long long *last_spike;  // last_spike_step_
    uint8_t *flags;                  // bit 0 had_hebbian_update_, bit 1 has_contributed_
    const uint8_t *delay;
    // By postsynaptic neuron, in get_all_connected_synapses order (projection load order, then
    // synapse index): entries col_pos[col_ptr[i] .. col_ptr[i + 1]).
    const long long *col_ptr;
    const unsigned long long *col_pos;
    const uint32_t *locked;          // [slot] 1: the projection's weights are locked (not trained)
    uint32_t *work;                  // non-spiking neurons with dopamine or renormalisation work this step
    uint32_t *work_count;            // this step (a per-step counter)
    double *add_thr;                 // additional_threshold_, FP64 as the reference keeps it
};

struct BlifatDev
{
    uint32_t n, n_pad;
    uint32_t flags;
    // state
    float *V, *V_pre, *thr_dyn, *trace, *g, *dopa, *add_thr;
    uint32_t *n_since, *burst_phase;
    long long *blocking;
    // parameters
    ParamF thr, thr_decay, thr_inc, trace_decay, trace_inc, g_decay, v_decay, reflexive, e_inh, v_reset, v_min;
    ParamU t_ref, burst_period;
    ResourceDev res;
    ResSynDev syn;  // kResSyn only
    // outputs
    uint32_t *spikes;
    uint32_t *spike_count;  // this step
    // Spike recording, or null: a ring of rec_slots per-step bitmaps of rec_words words each; step t
    // writes slot t % rec_slots completely (bit i of word i / 32 = neuron i fired).
    uint32_t *rec_bits;
    uint32_t rec_words, rec_slots;
    RingView ring;
};

struct LifDev
{
    uint32_t n, n_pad;
    float *V;
    uint32_t *refract;
    ParamF leak, thr, v_reset;
    ParamU refract_period;
    uint32_t *spikes;
    uint32_t *spike_count;
    uint32_t *rec_bits;  // spike recording ring, as for BlifatDev
    uint32_t rec_words, rec_slots;
    RingView ring;
};

// AltAI-LIF population (altai_lif.h:164-335, altai_impl.h:33-168): FP32 potential, integer
// thresholds, leak and reset, FP64 additional threshold (written by resource-STDP training), int64
// activity time. cfg bits per neuron: kAltaiDiff, kAltaiReset, kAltaiLeakRev, kAltaiSaturate,
// kAltaiNoSave.
enum AltaiCfg : uint32_t
{
    kAltaiDiff = 1u << 0,
    kAltaiReset = 1u << 1,
    kAltaiLeakRev = 1u << 2,
    kAltaiSaturate = 1u << 3,
    kAltaiNoSave = 1u << 4,
};
struct AltaiDev
{
    uint32_t n, n_pad;
    uint32_t flags;  // kResource, kResSyn, kLiveDopa
    float *V, *V_pre;
    long long *activity;
    ParamU cfg, thr, neg_thr, reset, leak;  // leak: the int16 value's int32 bits
    float *dopa;
    double *add_thr;
    ResourceDev res;
    ResSynDev syn;
    uint32_t *spikes;
    uint32_t *spike_count;
    uint32_t *rec_bits;  // spike recording ring, as for BlifatDev
    uint32_t rec_words, rec_slots;
    RingView ring;
};

// What the resource-STDP training kernel reads and writes of a population of either base type.
struct TrainView
{
    ResourceDev res;
    ResSynDev syn;
    const float *dopa;
    const uint32_t *spikes;
    const uint32_t *spike_count;
};

// External spike schedule of one sender channel (device-resident window).
struct ChannelDev
{
    unsigned long long first_step;
    unsigned long long n_steps;
    const long long *offsets;  // n_steps + 1
    const uint32_t *idx;
};

// A spike source of a projection: a population's spike list of this step, or a channel.
struct SpikeSource
{
    const uint32_t *idx;          // population spike list (null for a channel)
    const uint32_t *count;        // population spike count
    const ChannelDev *channel;    // channel descriptor (null for a population)
    uint32_t n;                   // population size (0 for a channel)
};

// Gather ("pull") form of a projection. A step whose spike count reaches `threshold` is not
// scattered: its spikes go to a bitmap slot instead, and the gather kernel adds, for every target,
// the weights of its synapses whose presynaptic neuron spiked d steps before the target step.
// Layout (sliced ELL): for each delay d and each window of kPullWindow consecutive targets, the
// targets are ordered by decreasing number of synapses with delay d (perm: sorted position -> target
// offset in the window) and cut into slices of kPullSlice. Slice q holds its 32 targets' synapses
// column-major: entry k of the slice's lane L (its L-th target) is at slice_ptr[q] + 32 k + L, and
// every lane's list is padded with zero entries (presynaptic 0, weight 0) to slice_len[q], the
// longest list of the slice. A lane therefore owns one target for a whole slice: no atomics, and
// each warp load reads 32 consecutive entries. Slices are indexed q = ((d - 1) * n_windows + window)
// * kPullSlicesPerWindow + slice-in-window.
constexpr int kPullWindow = 256;
constexpr int kPullSlice = 32;
constexpr int kPullSlicesPerWindow = kPullWindow / kPullSlice;

struct PullDev
{
    uint32_t *bitmap;       // [hist_slots][words] spikes of pulled steps
    uint32_t *pulled;       // [hist_slots] 1 if that step was pulled, 2 if every presynaptic neuron fired
    uint32_t hist_slots;    // max_delay + 1
    uint32_t words;         // ceil(n_rows / 32), rounded up to 4
    uint32_t threshold;     // minimum spike count for pulling a step
    uint32_t max_delay;
    uint32_t n_windows;     // ceil(n_post / kPullWindow)
    uint32_t n_post;
    const long long *slice_ptr;  // [max_delay * n_windows * kPullSlicesPerWindow + 1] first entry of each slice
    const uint32_t *slice_len;   // [max_delay * n_windows * kPullSlicesPerWindow] entries per lane
    const uint8_t *perm;         // [max_delay * n_windows * kPullWindow] target offset in its window
    const uint32_t *packed;      // presynaptic neuron of each entry (| weight index << 24 with wtab)
    const float *wtab;           // [256] weight dictionary (entry 0 is +0.0), used when the projection has at
                                 // most 256 distinct weights and fewer than 2^24 presynaptic neurons; else null
    uint32_t n_tab;              // dictionary entries in use
    uint32_t tab_rep;            // 1: the gather keeps 32 copies of the dictionary in shared memory (entry
                                 // i of lane l at 32 i + l: conflict-free lookups); 0: one copy
    const float *w;              // FP32 weights (negated for inhibitory current), or null
    const uint16_t *w16;         // FP16 bit patterns, used when every weight is exactly an FP16 value
    uint64_t padded_entries;     // entries of packed / w
};

// Device buffers of a gather layout (cudaMalloc'd; the caller takes ownership), with their sizes.
struct PullBuffers
{
    static constexpr int kCount = 7;
    void *ptr[kCount] = {};
    size_t bytes[kCount] = {};
};

struct ProjectionDev
{
    PullDev pull;  // pull.bitmap == nullptr: scatter only
    const long long *row_ptr;
    uint32_t n_rows;
    const int32_t *col;
    float *w;
    const uint8_t *delay;
    const uint8_t *type;  // per-synapse output type, or null (uniform_type)
    int uniform_type;
    int forcing;  // impacts of this projection carry is_forcing (plain delta projections)
    unsigned long long *last_spike;  // resource-STDP synapses: last_spike_step_ per CSR position, or null
    uint32_t order;  // load order among the backend's projections (message order of BLOCKING impacts)
    RingView ring;
    int n_src;
    SpikeSource src[kMaxSources];
};

// Additive-STDP state of one projection (per postsynaptic column).
struct StdpDev
{
    uint32_t n_cols;
    uint32_t period;  // list capacity and trigger count: smallest integer >= tau_plus + tau_minus
    uint32_t *pre_hist, *post_hist;  // [n_cols][period] step numbers
    uint32_t *pre_cnt, *post_cnt;    // [n_cols]
    uint32_t *touched;               // [n_cols] columns appended this step
    uint32_t *touched_count;         // this step
    unsigned long long *touched_stamp;  // [n_cols] step + 1 of the last append
    const long long *col_ptr;        // [n_cols + 1] into col_pos
    const uint64_t *col_pos;         // CSR positions of the column's synapses
    float *w;                        // CSR weights
    const float *table;              // stdp_w(d) for d in [0, table_len)
    uint32_t table_len;
};

// Per-step reset of this step's counters (launched at the end of every step for the next one).
struct StepEnd
{
    uint32_t *zero_u32;       // per-step counters to zero
    uint32_t n_zero_u32;
    uint32_t n_spike_counts;  // the first n_spike_counts counters are population spike counts
};

// A small network run by the fused step kernel (small_net.cu): device arrays of its populations,
// its projections (none with a gather layout) and its STDP rules, in step order.
enum SmallPopKind : int
{
    kSmallBlifat = 0,
    kSmallLif = 1,
};
struct SmallPop
{
    int kind;
    BlifatDev blifat;
    LifDev lif;
};
struct SmallStdp
{
    StdpDev d;
    uint32_t n_src;
    SpikeSource src[kMaxSources];
    int both[kMaxSources];  // the source fills both histories (STDPAndSpike)
};
// Two descriptor sets that differ only in their per-step counters (spike counts, STDP touched
// counts) and population spike lists: step t uses set t & 1, so step t - 1's STDP rules can read its
// spikes, and its counters can be zeroed, while step t runs; a step needs no end-of-step phase. Set 0
// uses the per-phase kernels' counters and lists; both sets' counters are zero between launches.
struct SmallNet
{
    const SmallPop *pops[2];
    const ProjectionDev *projs[2];
    const SmallStdp *stdp[2];
    uint32_t n_pops, n_projs, n_stdp;
    StepEnd end[2];
};

// A network run by the persistent grid step kernel (grid_net.cu): the fused kernel's descriptor
// sets, plus the projections with a gather layout (indices into net.projs) and the grid barrier's
// arrival counter (zeroed before every launch).
constexpr int kMaxGridPull = 8;
struct GridNet
{
    SmallNet net;
    unsigned long long *barrier;
    // Optional (nullptr: off): CTA 0 adds the global-timer nanoseconds of phase A, B and C of every
    // step it runs to phase_ns[0..2] (each phase up to the exit of the barrier that ends it).
    unsigned long long *phase_ns;
    uint32_t n_pull;
    uint32_t pull[kMaxGridPull];
};

// ---------------------------------------------------------------- launchers (stream-ordered)
void launch_blifat(const BlifatDev &p, Control *ctl, cudaStream_t s);
void launch_resource_train(const TrainView &p, int blocks, Control *ctl, cudaStream_t s);
void launch_altai(const AltaiDev &p, Control *ctl, cudaStream_t s);
void launch_altai_blocking(const AltaiDev &p, Control *ctl, cudaStream_t s);
void launch_lif(const LifDev &p, Control *ctl, cudaStream_t s);
void launch_projection(const ProjectionDev &p, Control *ctl, int grid, cudaStream_t s);
// Device rate (adds per second) of FP32 atomic adds at uniformly random positions of an n-float
// buffer, over about `adds` adds (three timed launches after one warm-up); 0, or -3 with *why.
int measure_add_rate(uint64_t n, uint64_t adds, double *rate, const char **why);
void launch_stdp_append(const StdpDev &d, SpikeSource src, int both_lists, Control *ctl, cudaStream_t s);
void launch_stdp_modify(const StdpDev &d, Control *ctl, cudaStream_t s);
void launch_step_end(const StepEnd &e, Control *ctl, cudaStream_t s);
// Runs n_steps whole steps of a small network in one launch of one cluster of `cluster` CTAs
// (advances Control::step). small_net_cluster() is the largest cluster size (8, 4, 2 or 1) the
// device can schedule for it.
int small_net_cluster();
cudaError_t launch_small_net(const SmallNet &net, Control *ctl, uint32_t n_steps, int cluster, cudaStream_t s);
// Runs n_steps whole steps of a network in one cooperative launch of `ctas` CTAs (advances
// Control::step). grid_net_ctas(smem) is the CTA count (one per SM) when the kernel fits with `smem`
// bytes of dynamic shared memory, else 0; grid_net_smem is the shared memory a gather projection
// needs in it. `window` (may be null): L2 access policy of the launch (persisting input ring).
int grid_net_ctas(size_t smem);
size_t grid_net_smem(const PullDev &p, int ctas);
cudaError_t launch_grid_net(const GridNet &g, Control *ctl, uint32_t n_steps, int ctas, size_t smem,
                            const cudaAccessPolicyWindow *window, cudaStream_t s);
void launch_gather(const ProjectionDev &p, Control *ctl, int grid, cudaStream_t s);
size_t gather_smem_bytes(const PullDev &p, int grid);
// Builds the gather layout of a projection from its CSR and fills `out`; the buffers go to `bufs`.
// Weights are stored losslessly in the smallest form that holds them: an 8-bit index into a
// 256-entry dictionary packed with the presynaptic neuron (at most 256 distinct weights), FP16 (every
// weight exactly an FP16 value), else FP32.
cudaError_t build_pull_layout(
    uint64_t n_syn, uint32_t n_rows, uint32_t n_post, const long long *row_ptr, const int32_t *col, const float *w,
    const uint8_t *delay, bool negate, PullDev &out, PullBuffers &bufs, cudaStream_t s);
// seq_base: the message-order index of the first impact among this step's external impacts on the
// population (AltAI-LIF BLOCKING events are ordered by it).
void launch_apply_impacts(
    const RingView &ring, const uint32_t *post, const float *value, const uint8_t *type, int forcing, uint32_t n,
    uint32_t seq_base, Control *ctl, cudaStream_t s);

// Network construction on the device.
cudaError_t build_csr(
    uint64_t n_syn, uint32_t n_rows, const uint32_t *d_row_key, uint32_t *d_perm_out, long long *d_row_ptr,
    void *d_temp, size_t temp_bytes, size_t *temp_needed, cudaStream_t s);
void launch_iota_u32(uint32_t *out, uint64_t n, cudaStream_t s);
void launch_gather_synapses(
    uint64_t n_syn, const uint32_t *perm, const uint32_t *post, const float *w, const uint32_t *delay,
    const uint8_t *type, int32_t *col_out, float *w_out, uint8_t *delay_out, uint8_t *type_out, cudaStream_t s);
// Device synapse generators: the index -> (presynaptic, postsynaptic) rules of the reference's
// synapse_generators.h (all_to_all, aligned, exclusive, one_to_one, FixedProbability,
// FixedNumberPost, FixedNumberPre), with counter-based draws instead of std::mt19937 so that a seed
// gives the same projection every time. Synapse i's weight is k/256 (k uniform in [k_lo, k_hi])
// and its delay uniform in [d_lo, d_hi], drawn from (key_w, i) and (key_d, i).
enum GenKind : int
{
    kGenAllToAll = 0,
    kGenAligned = 1,
    kGenExclusive = 2,
    kGenOneToOne = 3,
    kGenFixedProbability = 4,
    kGenFixedNumberPost = 5,
    kGenFixedNumberPre = 6,
};

struct GenSpec
{
    int kind;
    uint32_t n_pre, n_post;
    int32_t k_lo, k_hi;
    uint32_t d_lo, d_hi;
    unsigned long long key_pre, key_post, key_w, key_d;
    const unsigned long long *cand;  // FixedProbability: kept candidate pair indexes (pre + n_pre * post)
};

void launch_gen_keys(const GenSpec &g, uint64_t n_syn, uint32_t *pre_out, cudaStream_t s);
void launch_gen_gather(const GenSpec &g, uint64_t n_syn, const uint32_t *perm, int32_t *col_out, float *w_out,
                       uint8_t *delay_out, cudaStream_t s);
// Candidate pairs c in [0, n_cand) kept when the 53-bit draw (key, c) is below `threshold`: with
// out == nullptr only their number (*n_kept); else also written to out[] in ascending order.
cudaError_t gen_candidates(uint64_t n_cand, unsigned long long threshold, unsigned long long key,
                           unsigned long long *out, uint64_t *n_kept, cudaStream_t s);

cudaError_t gen_bernoulli_schedule(
    uint32_t n_sources, unsigned long long threshold, unsigned long long key, unsigned long long first_step,
    uint64_t n_steps, long long *d_offsets, uint32_t **d_idx, uint64_t *n_idx, cudaStream_t s);

// Counter-based generator shared with knp_gb300/network.py (SplitMix64 finaliser).
// ---------------------------------------------------------------- two-word fixed point
// An FP32 value w = s * m * 2^e (m < 2^24) is W = w * 2^48 = H * 2^40 + L with 0 <= L < 2^40: exact
// when w is a multiple of 2^-48 (every FP32 value of magnitude >= 2^-24 is), else rounded to the
// nearest multiple; |w| >= 2^54 saturates. Sums of H and of L over any order give the same exact
// total, which fx_normalize brings back to H * 2^40 + L form.
__host__ __device__ inline void fx_split(float w, long long &hi, long long &lo)
{
    uint32_t b;
    static_assert(sizeof(float) == sizeof(uint32_t), "32-bit float");
#ifdef __CUDA_ARCH__
    b = __float_as_uint(w);
#else
    __builtin_memcpy(&b, &w, 4);
#endif
    const int ex = static_cast<int>((b >> 23) & 0xFFu);
    unsigned long long m = b & 0x7FFFFFu;
    int e = -149;
    if (ex != 0)
    {
        m |= 0x800000u;
        e = ex - 150;
    }
    const unsigned long long mask = (1ull << kFxLoBits) - 1;
    const int s = e + 48;  // W = m * 2^s
    unsigned long long H = 0, L = 0;
    if (s >= 0)
    {
        if (s <= kFxLoBits)
        {
            const unsigned long long v = m << s;  // < 2^64
            H = v >> kFxLoBits;
            L = v & mask;
        }
        else if (s - kFxLoBits <= 38)
        {
            H = m << (s - kFxLoBits);
        }
        else
        {
            H = 1ull << 62;
        }
    }
    else if (s > -26)
    {
        // Below 2^-48: round m * 2^s to nearest, ties to even.
        const int r = -s;
        const unsigned long long q = m >> r, rem = m & ((1ull << r) - 1), half = 1ull << (r - 1);
        L = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
    }
    if (b >> 31)
    {
        if (L)
        {
            hi = -static_cast<long long>(H) - 1;
            lo = static_cast<long long>((1ull << kFxLoBits) - L);
        }
        else
        {
            hi = -static_cast<long long>(H);
            lo = 0;
        }
    }
    else
    {
        hi = static_cast<long long>(H);
        lo = static_cast<long long>(L);
    }
}

// Bring (hi, lo) with lo >= 0 back to 0 <= lo < 2^40.
__host__ __device__ inline void fx_normalize(long long &hi, long long &lo)
{
    hi += lo >> kFxLoBits;
    lo &= (1ll << kFxLoBits) - 1;
}

// The smallest two-word fixed-point value (hi * 2^-8 + lo * 2^-48, 0 <= lo < 2^40) that is >= x,
// for comparing an exact fixed-point sum V with an FP64 threshold: V >= x iff (V.hi, V.lo) >= (hi, lo)
// lexicographically. NaN and +inf give a value no sum reaches, -inf one every sum reaches;
// |x| >= 2^54 saturates as fx_split does.
__host__ __device__ inline void fx_ceil64(double x, long long &hi, long long &lo)
{
    unsigned long long b;
    static_assert(sizeof(double) == sizeof(unsigned long long), "64-bit double");
#ifdef __CUDA_ARCH__
    b = static_cast<unsigned long long>(__double_as_longlong(x));
#else
    __builtin_memcpy(&b, &x, 8);
#endif
    const bool neg = (b >> 63) != 0;
    const int ex = static_cast<int>((b >> 52) & 0x7FFu);
    unsigned long long m = b & ((1ull << 52) - 1);
    if (ex == 0x7FF)
    {
        if (neg && m == 0)
        {
            hi = -0x7FFFFFFFFFFFFFFFll - 1;
            lo = 0;
        }
        else
        {
            hi = 0x7FFFFFFFFFFFFFFFll;
            lo = 1ll << kFxLoBits;
        }
        return;
    }
    int e = -1074;
    if (ex != 0)
    {
        m |= 1ull << 52;
        e = ex - 1075;
    }
    const unsigned long long mask = (1ull << kFxLoBits) - 1;
    const int s = e + 48;  // |x| * 2^48 = m * 2^s
    // C = ceil(|x| * 2^48) for x > 0, floor(|x| * 2^48) for x < 0 (then negated), as H * 2^40 + L.
    unsigned long long H = 0, L = 0;
    if (s >= 0)
    {
        if (s <= 10)
        {
            const unsigned long long v = m << s;  // < 2^63
            H = v >> kFxLoBits;
            L = v & mask;
        }
        else if (s < kFxLoBits)
        {
            H = m >> (kFxLoBits - s);
            L = (m << s) & mask;  // the low 40 bits survive the shift's wrap
        }
        else if (s - kFxLoBits <= 9)
        {
            H = m << (s - kFxLoBits);  // < 2^62
        }
        else
        {
            H = 1ull << 62;
        }
    }
    else
    {
        const int r = -s;
        unsigned long long q = 0, rem = m;
        if (r < 64)
        {
            q = m >> r;
            rem = m & ((1ull << r) - 1);
        }
        if (!neg && rem) ++q;
        H = q >> kFxLoBits;
        L = q & mask;
    }
    if (neg)
    {
        if (L)
        {
            hi = -static_cast<long long>(H) - 1;
            lo = static_cast<long long>((1ull << kFxLoBits) - L);
        }
        else
        {
            hi = -static_cast<long long>(H);
            lo = 0;
        }
    }
    else
    {
        hi = static_cast<long long>(H);
        lo = static_cast<long long>(L);
    }
}

#ifdef __CUDACC__
// Correctly rounded FP32 value of hi * 2^-8 + lo * 2^-48 (0 <= lo < 2^40).
__device__ __forceinline__ float fx_to_float(long long hi, long long lo)
{
    const bool neg = hi < 0;
    unsigned long long H = static_cast<unsigned long long>(hi), L = static_cast<unsigned long long>(lo);
    if (neg)
    {
        if (L)
        {
            H = ~H;  // -hi - 1
            L = (1ull << kFxLoBits) - L;
        }
        else
        {
            H = 0ull - H;
        }
    }
    // Magnitude H * 2^40 + L as the 128-bit integer u1:u0.
    const unsigned long long u1 = H >> (64 - kFxLoBits), u0 = (H << kFxLoBits) | L;
    float f;
    if (u1 == 0)
    {
        f = __fmul_rn(__ull2float_rn(u0), 3.5527136788005009e-15f);  // 2^-48
    }
    else
    {
        const int lz = __clzll(static_cast<long long>(u1));
        const int sh = 64 - lz;  // bits of u0 below the 64-bit window
        const unsigned long long top = (u1 << lz) | (sh == 64 ? 0ull : (u0 >> sh));
        const unsigned long long sticky = (sh == 64 ? u0 : (u0 & ((1ull << sh) - 1))) != 0 ? 1ull : 0ull;
        f = __fmul_rn(__ull2float_rn(top | sticky), __int_as_float((127 + sh - 48) << 23));
    }
    return neg ? -f : f;
}

// Adds an FP32 impact to a two-word fixed-point accumulator.
__device__ __forceinline__ void fx_atomic_add(long long *hi, long long *lo, size_t o, float w)
{
    long long h, l;
    fx_split(w, h, l);
    if (h) atomicAdd(reinterpret_cast<unsigned long long *>(hi + o), static_cast<unsigned long long>(h));
    if (l) atomicAdd(reinterpret_cast<unsigned long long *>(lo + o), static_cast<unsigned long long>(l));
}
#endif

__host__ __device__ inline unsigned long long mix64(unsigned long long x)
{
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__host__ __device__ inline unsigned long long stream_key(unsigned long long seed, unsigned long long stream)
{
    return mix64(seed * 0x9E3779B97F4A7C15ull + stream);
}
__host__ __device__ inline unsigned long long rand64(unsigned long long key, unsigned long long ctr)
{
    return mix64(key ^ (ctr * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull));
}
__host__ __device__ inline long long uniform_int(unsigned long long key, unsigned long long ctr, long long lo, long long hi)
{
    const unsigned long long r = rand64(key, ctr) >> 32;
    const unsigned long long span = static_cast<unsigned long long>(hi - lo + 1);
    return static_cast<long long>((r * span) >> 32) + lo;
}

// Programmatic dependent launch of a step's kernels: each kernel is launched while its predecessor
// on the stream still runs, waits at its first instruction until the predecessor has completed and
// its memory is visible (so every kernel still sees the whole previous kernel's results), then lets
// its own successor start launching. Only the launch latency between kernels is overlapped.
#ifdef __CUDACC__
__device__ __forceinline__ void pdl_begin()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args &&...args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}
#endif

}  // namespace knp_gb300
