/*
 * knp_gb300 — C ABI of the GB300 (sm_103a) KNP backend: BLIFAT and synaptic-resource-STDP BLIFAT
 * populations, delta-synapse and additive-STDP delta-synapse projections.
 *
 * Every entry point replaces one operation of the KNP backend plugin interface
 * knp::core::Backend (knp/core-library/include/knp/core/backend.h) as the single-threaded CPU
 * backend implements it (knp/backends/cpu/cpu-single-threaded-backend/...). The reference interface is
 * C++ (std::shared_ptr<Backend>, variants of Population<Neuron>/Projection<Synapse>, messages on a
 * MessageBus); this ABI carries the same data as plain pointers and sizes:
 *   - populations as arrays of knp_blifat_neuron (+ knp_resource_stdp_state) structs,
 *   - projections as synapse arrays (pre index, post index, weight, delay, output type, STDP taus),
 *   - SpikeMessages as (sender UID, send time, index array),
 *   - SynapticImpactMessages to a population as (sender, receiver, is_forcing, impact arrays).
 * All buffers are caller-owned host memory unless a name says "device". Every call returns 0 on
 * success or a negative knp_gb300_status; knp_gb300_last_error() describes the last failure of the
 * calling thread. A backend handle is used by one thread at a time (as a reference backend is: one
 * step at a time, no reentrancy).
 */
#ifndef KNP_GB300_H
#define KNP_GB300_H

#include <stddef.h>
#include <stdint.h>

#include "knp_gb300_types.h"

#if defined(__GNUC__)
#define KNP_GB300_API __attribute__((visibility("default")))
#else
#define KNP_GB300_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct knp_gb300_backend knp_gb300_backend;

typedef enum knp_gb300_status
{
    KNP_GB300_OK = 0,
    KNP_GB300_E_INVALID = -1,      /* bad argument, unknown UID, unsupported type */
    KNP_GB300_E_STATE = -2,        /* call not allowed in the current state (e.g. load after init) */
    KNP_GB300_E_CUDA = -3,         /* CUDA runtime error */
    KNP_GB300_E_DEVICE_FLAG = -4,  /* a kernel reported an error through the device error word */
    KNP_GB300_E_NOMEM = -5         /* device allocation failed */
} knp_gb300_status;

/** Accumulator mode of a population's input ring. */
typedef enum knp_gb300_accumulator
{
    KNP_GB300_ACC_AUTO = 0,  /* FP32 when every incoming weight is a dyadic k/256 with bounded sums, else FIXED64 */
    KNP_GB300_ACC_FP32 = 1,  /* FP32 atomics: exact for dyadic weights, otherwise order-dependent rounding */
    KNP_GB300_ACC_FIXED64 = 2 /* int64 fixed point (2^-40): order-independent, exact for |w| >= 2^-17 */
} knp_gb300_accumulator;

/** How a step is executed (results are the same in every mode). */
typedef enum knp_gb300_step_mode
{
    KNP_GB300_STEP_AUTO = 0,   /* fused, else grid, when the network qualifies (see knp_gb300_set_step_mode), else phases */
    KNP_GB300_STEP_PHASES = 1, /* one kernel per phase (population, projection, STDP, end of step) in CUDA graphs */
    KNP_GB300_STEP_FUSED = 2,  /* one kernel (one CTA cluster) runs whole steps; init fails if the network does not qualify */
    KNP_GB300_STEP_GRID = 3    /* one persistent cooperative kernel (one CTA per SM) runs whole steps, gather
                                  form included; init fails if the network does not qualify */
} knp_gb300_step_mode;

/** Message text of the last failed call on this thread (never NULL). */
KNP_GB300_API const char *knp_gb300_last_error(void);

/** Library version string. */
KNP_GB300_API const char *knp_gb300_version(void);

/**
 * Create a backend on CUDA device `device`.
 * Replaces: SingleThreadedCPUBackend::create()
 *   (knp/backends/cpu/cpu-single-threaded-backend/impl/backend.cpp:48-52) reached through the exported
 *   alias create_knp_backend (:340) and BackendLoader::load (knp/base-framework/impl/backend_loader.cpp:57-68).
 */
KNP_GB300_API int knp_gb300_create(int device, knp_gb300_backend **out);

/** Destroy a backend and free its device memory. Replaces: Backend::~Backend (backend.h:70). */
KNP_GB300_API int knp_gb300_destroy(knp_gb300_backend *b);

/**
 * Load a BLIFAT (kind KNP_NEURON_BLIFAT) or resource-STDP BLIFAT (KNP_NEURON_RESOURCE_STDP_BLIFAT,
 * `ext` required) population of `n` neurons. Neuron order is the population's index order.
 * Replaces: load_populations / load_all_populations for Population<BLIFATNeuron> and
 *   Population<SynapticResourceSTDPBLIFATNeuron> (cpu-single-threaded-backend/include/knp/backends/
 *   cpu-single-threaded/backend.h:199; core backend.h:146; impl/backend.cpp:144-186).
 */
KNP_GB300_API int knp_gb300_load_blifat_population(
    knp_gb300_backend *b, knp_uid uid, int kind, uint32_t n, const knp_blifat_neuron *neurons,
    const knp_resource_stdp_state *ext);

/**
 * Load a LIF population (reference semantics of lif_impl.h:33-86: leak and impacts only outside the
 * refractory period, spike iff potential > threshold, reset to a value). Used by the batched form
 * and its FP32 comparison path. Replaces: load_populations for Population<LIFNeuron>
 * (cpu-single-threaded-backend/impl/backend.cpp:255-260).
 */
KNP_GB300_API int knp_gb300_load_lif_population(knp_gb300_backend *b, knp_uid uid, uint32_t n, const knp_lif_neuron *neurons);

/** Read back a LIF population's neurons. Replaces: get_network_data population range for LIF. */
KNP_GB300_API int knp_gb300_read_lif_population(knp_gb300_backend *b, knp_uid pop, knp_lif_neuron *out);

/**
 * Load an AltAI-LIF population: kind KNP_NEURON_ALTAI_LIF, or KNP_NEURON_RESOURCE_STDP_ALTAI_LIF with
 * `ext` (the resource-STDP extension, trained like the BLIFAT variant: altai/altai_stdp.h). Semantics
 * of altai/altai_impl.h:33-168: the potential is rounded (or reset when do_not_save) before the
 * impacts, leak with optional sign reversal, activity time counted towards INT64_MAX, threshold
 * crossing with difference or reset, negative threshold with saturation. Impacts of a step are summed
 * exactly and rounded once, which is the reference's impact-by-impact FP32 sum whenever its partial
 * sums are exact (integer or dyadic weights); BLOCKING impacts are applied in the reference's message
 * order (at most 2048 per population and step, else KNP_GB300_E_DEVICE_FLAG). INHIBITORY_CONDUCTANCE
 * impacts are refused, as the reference throws on them. Populations of these kinds run the per-phase
 * step. Replaces: load_populations for Population<AltAILIF> and
 * Population<SynapticResourceSTDPAltAILIFNeuron> (cpu-single-threaded-backend/impl/backend.cpp:144-186).
 */
KNP_GB300_API int knp_gb300_load_altai_population(
    knp_gb300_backend *b, knp_uid uid, int kind, uint32_t n, const knp_altai_neuron *neurons,
    const knp_resource_stdp_state *ext);

/** Read back an AltAI-LIF population's neurons (and their resource-STDP extension when `ext` is not
 * NULL). Replaces: get_network_data population range for the AltAI-LIF kinds. */
KNP_GB300_API int knp_gb300_read_altai_population(
    knp_gb300_backend *b, knp_uid pop, knp_altai_neuron *out, knp_resource_stdp_state *ext);

/**
 * Load a projection of `n_syn` synapses given in the reference's synapse order: synapse i is
 * (weight[i], delay[i], out_type[i]) from presynaptic neuron pre[i] to postsynaptic neuron post[i].
 * kind: KNP_SYNAPSE_DELTA or KNP_SYNAPSE_ADDITIVE_STDP_DELTA (tau_plus/tau_minus required, uniform
 * per projection). out_type may be NULL (all EXCITATORY). pre_uid may be the all-zero UID (the
 * projection then receives spikes only through knp_gb300_subscribe). KNP_OUT_BLOCKING synapses are
 * taken in delta projections (not in additive-STDP ones) of backends with at most 62 projections: of
 * the BLOCKING impacts a neuron receives in a step, the last one in the reference's message order
 * (projection load order; within a projection, larger delays first, then ascending spike index and
 * synapse order; external messages last) sets its total blocking period (blifat_impl.h:86).
 * Replaces: load_projections /
 * load_all_projections for Projection<DeltaSynapse> and Projection<AdditiveSTDPDeltaSynapse>
 * (backend.h:206; core backend.h:137; impl/backend.cpp:158-178).
 */
KNP_GB300_API int knp_gb300_load_projection(
    knp_gb300_backend *b, knp_uid uid, int kind, knp_uid pre_uid, knp_uid post_uid, uint64_t n_syn,
    const uint32_t *pre, const uint32_t *post, const float *weight, const uint32_t *delay,
    const uint8_t *out_type, const float *tau_plus, const float *tau_minus);

/**
 * Load a projection of `n_syn` SynapticResourceSTDPDeltaSynapse synapses (synaptic-resource STDP,
 * stdp_synaptic_resource_rule.h:45-89): synapse i is (weight[i], delay[i], out_type[i], rule[i]) from
 * pre[i] to post[i], as knp_gb300_load_projection; `locked` is the projection's is_locked()
 * (projection.h:384-396; a projection starts locked). The synapses deliver impacts like delta
 * synapses with is_forcing false (synaptic_resource_stdp.h:58-62), record the step of every
 * presynaptic spike (init_synapse, :36-41), and while unlocked are trained by their postsynaptic
 * resource-STDP BLIFAT population at the end of its step (blifat_stdp.h:35-172: Hebbian and
 * dopamine changes of the synaptic resource, free-resource renormalisation, weights recalculated
 * from the resource). out_type may not hold KNP_OUT_BLOCKING. A backend with such projections runs
 * the per-phase step (KNP_GB300_STEP_PHASES). Replaces: load_projections for
 * Projection<SynapticResourceSTDPDeltaSynapse> (cpu-single-threaded-backend/impl/backend.cpp:158-178).
 */
KNP_GB300_API int knp_gb300_load_resource_stdp_projection(
    knp_gb300_backend *b, knp_uid uid, knp_uid pre_uid, knp_uid post_uid, uint64_t n_syn, const uint32_t *pre,
    const uint32_t *post, const float *weight, const uint32_t *delay, const uint8_t *out_type,
    const knp_resource_synapse *rule, int locked);

/** Read back the rule state of a resource-STDP projection's synapses in the order they were loaded.
 * Replaces: get_network_data projection range for Projection<SynapticResourceSTDPDeltaSynapse>. */
KNP_GB300_API int knp_gb300_read_resource_synapses(knp_gb300_backend *b, knp_uid proj, knp_resource_synapse *out);

/**
 * Generate, on the device, a delta projection with fixed fan-in: synapse i has post = i % n_post,
 * pre = uniform [0, n_pre), weight = k/256 with k uniform in [k_lo, k_hi], delay uniform in
 * [d_lo, d_hi], drawn from the counter-based generator keyed by (seed, stream). Equivalent to
 * knp_gb300_load_projection with the arrays of knp_gb300/network.py:fixed_fan_in_pre, without
 * materialising them on the host. Replaces: Projection construction from the FixedNumberPre
 * generator (knp/base-framework/include/knp/framework/projection/synapse_generators.h:410-457).
 */
KNP_GB300_API int knp_gb300_generate_fixed_fan_in_projection(
    knp_gb300_backend *b, knp_uid uid, knp_uid pre_uid, knp_uid post_uid, uint32_t n_pre, uint32_t n_post,
    uint32_t fan_in, int32_t k_lo, int32_t k_hi, uint32_t d_lo, uint32_t d_hi, uint64_t seed, uint64_t stream);

/**
 * Generate, on the device, a delta projection by one of the reference's synapse generators
 * (knp_generator_kind: all_to_all, aligned (the larger size a multiple of the smaller), exclusive
 * (equal sizes), one_to_one (equal sizes), FixedProbability (at most 2^40 candidate pairs) with
 * `probability`, FixedNumberPost and FixedNumberPre with `count` synapses; `count` and
 * `probability` are ignored by the other kinds). Synapse i connects the pair the generator's index
 * rule gives (FixedProbability: the i-th kept all_to_all pair in index order, each pair kept when
 * its draw is below the probability); the random choices, weights (k/256, k uniform in
 * [k_lo, k_hi]) and delays (uniform in [d_lo, d_hi]) are counter-based draws keyed by (seed,
 * stream), so one seed gives one projection, where the reference draws from std::mt19937 seeded
 * by std::random_device. knp_gb300/network.py:generated_synapses gives the same synapses on the
 * host. Replaces: Projection construction from those generators
 * (knp/base-framework/include/knp/framework/projection/synapse_generators.h:58-457).
 */
KNP_GB300_API int knp_gb300_generate_projection(
    knp_gb300_backend *b, knp_uid uid, knp_uid pre_uid, knp_uid post_uid, int kind, uint32_t n_pre, uint32_t n_post,
    uint64_t count, double probability, int32_t k_lo, int32_t k_hi, uint32_t d_lo, uint32_t d_hi, uint64_t seed,
    uint64_t stream);

/**
 * Register `pop_uid` in an STDP projection's stdp_populations_ map with processing type
 * KNP_STDP_ONLY or KNP_STDP_AND_SPIKE. Replaces: writing
 * Projection<STDP<...>>::get_shared_parameters().stdp_populations_ (knp/core-library/include/knp/core/projection.h:133-164).
 */
KNP_GB300_API int knp_gb300_set_stdp_population(knp_gb300_backend *b, knp_uid proj_uid, knp_uid pop_uid, int processing);

/**
 * Subscribe `receiver` (a projection: to SpikeMessages; a population: to SynapticImpactMessages) to
 * messages of `sender` (a population of this backend or an external channel UID).
 * Replaces: Backend::subscribe<MessageType> (core backend.h:222-226).
 */
KNP_GB300_API int knp_gb300_subscribe(knp_gb300_backend *b, knp_uid receiver, knp_uid sender);

/** Force the accumulator mode of a population (before init). */
KNP_GB300_API int knp_gb300_set_accumulator(knp_gb300_backend *b, knp_uid pop_uid, int mode);

/**
 * Direction choice of a delta projection: a step in which at least `fraction` x (presynaptic
 * neurons) spike is delivered by the gather kernel (synapses sorted by delay and target, no global
 * atomics) instead of the scatter kernel; results are identical. Default 0.1; a negative fraction
 * keeps every step on the scatter path. The gather form is built at init for delta projections of
 * at least 2^20 synapses fed by one population into an FP32 input ring. No reference counterpart:
 * the reference's delivery loop (delta_impl.h:65-107) is a scatter only.
 */
KNP_GB300_API int knp_gb300_set_pull_threshold(knp_gb300_backend *b, knp_uid proj_uid, double fraction);

/**
 * Step execution mode (before init). The fused mode runs every phase of a step, and many steps per
 * launch, in one thread-block cluster (up to 8 CTAs) with cluster barriers between the phases; it
 * takes networks of at most 16384 neurons and 2^22 synapses whose projections have no gather form
 * and at most 8 STDP populations each. The grid mode runs every phase of a step, and many steps per
 * launch, in one cooperative launch of one 1024-thread CTA per SM with bounded grid barriers
 * between the phases (gather form included); it takes networks whose projections have at most 8 STDP
 * populations each, with at most 8 gather-form projections whose shared memory fits one CTA.
 * AUTO (the default) picks the fused mode for networks it takes, else the grid mode for networks it
 * takes, else the per-phase kernels. No reference counterpart: the reference's step driver is
 * SingleThreadedCPUBackend::_step (knp/backends/cpu/cpu-single-threaded-backend/impl/backend.cpp:89-141),
 * whose phase order every mode keeps.
 */
KNP_GB300_API int knp_gb300_set_step_mode(knp_gb300_backend *b, int mode);

/** 1 when init chose the fused step kernel, else 0 (after init). */
KNP_GB300_API int knp_gb300_step_fused(const knp_gb300_backend *b, int *fused);

/** The step mode init chose: KNP_GB300_STEP_PHASES, _FUSED or _GRID (after init). */
KNP_GB300_API int knp_gb300_step_kernel(const knp_gb300_backend *b, int *mode);

/**
 * Enable or disable per-step spike recording of a population (SpikeMessages that an output
 * channel or observer subscribed to this population would receive).
 * Replaces: an external endpoint subscribing to the population's SpikeMessages
 *   (knp/base-framework/impl/model_loader.cpp:100-120; knp/tests/backend/single_thread_cpu_test.cpp:76).
 */
KNP_GB300_API int knp_gb300_record_spikes(knp_gb300_backend *b, knp_uid pop_uid, int enable);

/**
 * Build device structures (CSR, rings, subscriptions) and capture the step graph.
 * Replaces: Backend::_init (core backend.h:314) = cpu::init (knp/backends/cpu/cpu-library/include/
 *   knp/backends/cpu-library/init.h:93-110) as called by SingleThreadedCPUBackend::_init (impl/backend.cpp:207-214).
 */
KNP_GB300_API int knp_gb300_init(knp_gb300_backend *b);

/**
 * Send an external SpikeMessage {sender, send_time, indexes[n]}; it is delivered at the next step to
 * every projection subscribed to `sender`. Replaces: MessageEndpoint::send_message of a SpikeMessage
 *   by an input channel (knp/base-framework/include/knp/framework/io/input_channel.h:99-120).
 */
KNP_GB300_API int knp_gb300_send_spikes(knp_gb300_backend *b, knp_uid sender, uint64_t send_time, uint32_t n, const uint32_t *idx);

/**
 * Upload a whole external spike schedule for `sender` to device memory: step t (t in
 * [first_step, first_step + n_steps)) sends idx[offsets[t - first_step] : offsets[t - first_step + 1]].
 * Replaces: an input channel's per-step SpikeMessages, staged on the device ahead of time.
 */
KNP_GB300_API int knp_gb300_load_spike_schedule(
    knp_gb300_backend *b, knp_uid sender, uint64_t first_step, uint64_t n_steps, const int64_t *offsets,
    const uint32_t *idx);

/**
 * Generate on the device a Bernoulli schedule for `sender`: source s spikes at step t iff the
 * counter-based generator (seed, stream, t * n_sources + s) is below probability p.
 */
KNP_GB300_API int knp_gb300_generate_bernoulli_schedule(
    knp_gb300_backend *b, knp_uid sender, uint32_t n_sources, double p, uint64_t first_step, uint64_t n_steps,
    uint64_t seed, uint64_t stream);

/**
 * Allocation-free variant of knp_gb300_generate_bernoulli_schedule, for callers that cannot
 * allocate GPU memory when they need a schedule (code running while another component owns the
 * device memory pool, allocators that forbid cudaMalloc/cudaFree in the calling phase or thread,
 * plugins that may only use buffers their host hands them). No reference counterpart.
 *
 * Writes the schedule of `n_sources` Bernoulli(p) sources for steps [first_step, first_step +
 * n_steps) into caller-owned DEVICE buffers: d_offsets[n_steps + 1] and d_idx[capacity]; step
 * first_step + t sends d_idx[d_offsets[t] : d_offsets[t + 1]] (ascending), the same spikes the
 * allocating generator produces for (seed, stream). *n_idx (host) receives the number of spikes.
 * It calls no cudaMalloc, cudaFree or allocating library routine: its scratch is one fixed device
 * array of 2^18 + 1 int64 counters (2 MiB) that every GPU it runs on keeps until process exit, so
 * n_steps * ceil(n_sources / 4096) must not exceed 262144 and n_steps 65535, and p must be finite
 * (else KNP_GB300_E_INVALID with *n_idx = 0). If capacity is too small it returns
 * KNP_GB300_E_INVALID with the needed count (non-zero) in *n_idx and writes nothing to d_idx.
 * Set-up: the CUDA runtime loads device code and __device__ arrays lazily, and that load allocates
 * device memory. The first call in a CUDA context (per device, with that device current; again after
 * cudaDeviceReset) therefore loads this entry point's kernels and its scratch array (2 MiB) and looks
 * up the array's address: make that first call (any valid call) during set-up, where allocation is
 * allowed and no stream capture is active. Later calls in the same context allocate nothing.
 * Every call shares the scratch and finds the previous call's contents (each call rewrites every
 * counter it reads); calls that overlap on the GPU race and must be serialised by the caller. The
 * call waits for its own stream (`stream`, a cudaStream_t; NULL: legacy default stream) once, to read
 * the spike count, and returns with the index writes queued on that stream.
 */
KNP_GB300_API int knp_gb300_generate_bernoulli_schedule_noalloc(
    uint32_t n_sources, double p, uint64_t first_step, uint64_t n_steps, uint64_t seed, uint64_t stream_id,
    int64_t *d_offsets, uint32_t *d_idx, uint64_t capacity, uint64_t *n_idx, void *stream);

/**
 * Send an external SynapticImpactMessage to population `receiver` (impacts post_idx[i], value[i],
 * out_type[i] (NULL = EXCITATORY)); applied at the next step, after impacts of the backend's own
 * projections (so a BLOCKING impact here overrides theirs, and within one step the last message's last
 * BLOCKING impact on a neuron counts). Replaces: MessageEndpoint::send_message of a SynapticImpactMessage
 *   (knp/tests/framework/lif_test.cpp:78-86).
 */
KNP_GB300_API int knp_gb300_send_impacts(
    knp_gb300_backend *b, knp_uid sender, knp_uid receiver, int is_forcing, uint32_t n, const uint32_t *post_idx,
    const float *value, const uint8_t *out_type);

/**
 * Advance `n_steps` steps. Replaces: `n_steps` calls of Backend::_step (core backend.h:321;
 *   cpu-single-threaded-backend/impl/backend.cpp:89-141), as driven by Backend::start (core impl/backend.cpp:116-141).
 */
KNP_GB300_API int knp_gb300_step(knp_gb300_backend *b, uint64_t n_steps);

/** Current step number. Replaces: Backend::get_step (core backend.h:290). */
KNP_GB300_API int knp_gb300_get_step(const knp_gb300_backend *b, uint64_t *step);

/**
 * Spike indexes (ascending) that population `pop` emitted at step `step`, which must be among the
 * steps run since recording was enabled and not yet discarded. Writes min(count, cap) indexes and
 * the full count to *n. Waits only for step `step` itself: later steps already queued keep running
 * on the device while the step's bitmap is copied and expanded (a caller can queue step k + 1 before
 * reading step k). Replaces: receiving the population's SpikeMessage of that step on a subscribed
 * endpoint (single_thread_cpu_test.cpp:85, tests_messaging_common.h:48-56).
 */
KNP_GB300_API int knp_gb300_read_spikes(
    knp_gb300_backend *b, knp_uid pop, uint64_t step, uint32_t cap, uint32_t *out, uint32_t *n);

/** Discard recorded spikes of steps before `step` (frees log space). */
KNP_GB300_API int knp_gb300_discard_spikes(knp_gb300_backend *b, uint64_t step);

/**
 * Read back a BLIFAT population's neurons (and, for resource-STDP BLIFAT, `ext`, may be NULL).
 * Replaces: get_network_data population range (core backend.h:420;
 *   cpu-single-threaded-backend/impl/get_network.cpp:80-93).
 */
KNP_GB300_API int knp_gb300_read_blifat_population(
    knp_gb300_backend *b, knp_uid pop, knp_blifat_neuron *out, knp_resource_stdp_state *ext);

/** Read back projection weights in the order the synapses were loaded. Replaces: get_network_data projection range. */
KNP_GB300_API int knp_gb300_read_weights(knp_gb300_backend *b, knp_uid proj, float *out);

/** Number of synapses of a loaded projection. */
KNP_GB300_API int knp_gb300_projection_size(const knp_gb300_backend *b, knp_uid proj, uint64_t *n);

/**
 * Unlock / lock the weights of every loaded projection. Replaces: start_learning / stop_learning
 * (cpu-single-threaded-backend/include/.../backend.h:315-332). As in the reference, only
 * resource-STDP training reads the lock (populations_old.h:57-83 keeps unlocked projections);
 * additive-STDP weight updates ignore it (knp/backends/cpu/cpu-library/include/knp/backends/
 * cpu-library/impl/projections/training/stdp/additive_stdp.h:173-196).
 */
KNP_GB300_API int knp_gb300_start_learning(knp_gb300_backend *b);
KNP_GB300_API int knp_gb300_stop_learning(knp_gb300_backend *b);

/**
 * Cumulative counters since init: synaptic events (impacts created), spikes emitted by all
 * populations, and neuron updates. Any pointer may be NULL.
 */
KNP_GB300_API int knp_gb300_counters(knp_gb300_backend *b, uint64_t *events, uint64_t *spikes, uint64_t *neuron_updates);

/**
 * Time `n_steps` steps with CUDA events on the backend's stream and return the elapsed
 * milliseconds (device time). The steps run exactly as knp_gb300_step runs them.
 */
KNP_GB300_API int knp_gb300_step_timed(knp_gb300_backend *b, uint64_t n_steps, float *ms);

/**
 * Run `n_steps` steps with the kernels launched one by one (no graph) and CUDA events between the
 * step phases; ms[0..3] receive the summed device time of the population kernels, the projection
 * kernels, the STDP kernels and the end-of-step kernel. Results equal knp_gb300_step's.
 */
KNP_GB300_API int knp_gb300_profile_phases(knp_gb300_backend *b, uint64_t n_steps, float *ms);

/**
 * Runs n_steps normal steps (knp_gb300_step; results equal its own) on a backend that steps with the
 * persistent grid kernel (KNP_GB300_E_STATE otherwise, or with host messages pending), timing each
 * step's phases on the device's global timer: us[0] populations (and the previous step's STDP
 * rules), us[1] projections (scatter, or spike bitmaps of gathered steps), us[2] gathers and
 * bitmap clearing; each summed over the steps, a phase ending when every CTA has finished it.
 * A measurement aid beside knp_gb300_step_timed (no reference counterpart).
 */
KNP_GB300_API int knp_gb300_profile_grid_phases(knp_gb300_backend *b, uint64_t n_steps, double *us);

/**
 * Measures, on the current device, the rate of FP32 atomic adds at uniformly random positions of an
 * n_floats buffer (0 < n_floats < 2^32) (about n_adds adds, three timed launches after one warm-up): the ceiling of the
 * scatter's ring adds when n_floats is the input rings' size. A measurement aid for the scatter's
 * roofline (no reference counterpart). Allocates and frees the buffer; synchronous.
 */
KNP_GB300_API int knp_gb300_measure_add_rate(uint64_t n_floats, uint64_t n_adds, double *adds_per_s);

/*
 * Differentiation form (no reference counterpart: KNP has no gradient-based training). LIF layer
 * recurrence over T steps for BN = batch x neurons independent neurons, device buffers laid out
 * [T][BN] (I, S, dS, dI) and [ceil(T/K)][BN] (ckpt):
 *   U_t = beta V_{t-1} + I_t,  S_t = H(U_t - theta) (strict '>'),  V_t = U_t - theta S_t,  V_{-1} = 0.
 * The forward stores the membrane state entering every K-th step (K <= 16); the backward recomputes
 * each K-step segment from its checkpoint and returns dI = dL/dI from dS = dL/dS using the
 * fast-sigmoid surrogate dS/dU = (k/2) / (1 + k|U - theta|)^2. relaxed != 0 replaces H by the
 * fast sigmoid (1 + kx/(1+k|x|))/2 in the forward, whose exact derivative the backward then is.
 * `stream` is a cudaStream_t (NULL: legacy default stream). Launches only; returns before completion.
 */
KNP_GB300_API int knp_gb300_lif_scan_forward(
    const float *I, float *S, float *ckpt, int T, int64_t BN, float beta, float theta, int K, int relaxed, float k,
    void *stream);
KNP_GB300_API int knp_gb300_lif_scan_backward(
    const float *I, const float *ckpt, const float *dS, float *dI, int T, int64_t BN, float beta, float theta, int K,
    int relaxed, float k, void *stream);

/**
 * Differentiation form: a BF16 GEMM operand (K contiguous) from X[R][C] (FP32, or BF16 when x_bf16
 * != 0; device memory) in one pass. Each output row holds one (mode 0) or two (modes 1, 2) halves of
 * width P, zero past the copied extent: mode 0 bf16(x); mode 1 bf16(x) twice; mode 2 hi = bf16(x)
 * and lo = bf16(x - hi) (round to nearest even). transpose == 0: out[R][H P], row r from X's row r
 * (P >= C, P even); transpose != 0: out[C][H P], row c from X's column c (P >= R). Launch only.
 */
KNP_GB300_API int knp_gb300_bf16_operand(const void *X, int x_bf16, int64_t R, int64_t C, int mode, int transpose,
                                         int64_t P, void *out, void *stream);

/*
 * Batched / precision form (no reference counterpart). D[M x N] (FP32, row-major) = A[M x K] *
 * B[N x K]^T with BF16 operands (row-major, K contiguous, device memory) on the tcgen05 tensor
 * cores, accumulator in tensor memory. *d_err (device) receives bit 0 if a completion wait timed
 * out. Launch only.
 */
KNP_GB300_API int knp_gb300_bf16_gemm_tn(
    const void *A, const void *B, float *D, int M, int N, int K, unsigned int *d_err, void *stream);

/*
 * Batched / precision form (no reference counterpart: the reference steps one network at a time).
 * `batch` independent samples of a feed-forward LIF network with n_layers all-to-all delay-1
 * layers (sizes[0] inputs -> sizes[1] -> ... -> sizes[n_layers], each <= 4096, fan-in <= 2048; reference LIF
 * semantics lif_impl.h:33-86 with per-layer leak / threshold / reset / refractory period, NULL =
 * reference defaults 1, 1, 0, 0) run in a persistent kernel of CTA pairs on the tcgen05 tensor cores:
 * every step each layer's input is the previous layer's 0/1 spike matrix (BF16, exact) times its BF16
 * weights (device, d_weights[l] = [sizes[l + 1]][sizes[l]] row-major) with FP32 accumulation in tensor
 * memory. Sample b runs steps[b] (host array) steps; its input i spikes at step t iff
 * rand64(stream_key(seed, 5), (t * batch + b) * sizes[0] + i) >> 11 < d_rates[b][i] * 2^53 (the
 * generator of knp_gb300/network.py; a rate below 0 or NaN never fires, 1 or above always). Outputs: d_counts[batch][sizes[n_layers]] (device, int32) output
 * spike counts; optional d_record (device, uint32) with every layer's spike bitmap of every step,
 * laid out [max(steps)][layer 0..n_layers][batch][ceil(sizes[l] / 32)]; *events (host) synaptic events
 * (spikes x fan-out of their layer); *ms (host) device time of the run. Synchronous.
 */
KNP_GB300_API int knp_gb300_batched_lif_run(
    int n_layers, const uint32_t *sizes, const void *const *d_weights, const float *leak, const float *threshold,
    const float *reset, const uint32_t *refract, uint32_t batch, const uint32_t *steps, const float *d_rates,
    uint64_t seed, int32_t *d_counts, uint32_t *d_record, uint64_t *events, float *ms, void *stream);

/*
 * Batched form, prepared once and run as one CUDA-graph launch (no reference counterpart). The
 * arguments are those of knp_gb300_batched_lif_run plus:
 *   sample_sizes  optional host array [(n_layers + 1) * batch], layer-major: sample b's size of layer
 *                 l (<= sizes[l]); inputs and neurons beyond it do not exist for that sample (never
 *                 spike, carry no events). NULL: every sample has the full sizes (uneven network
 *                 instances over shared weights, or inputs of uneven width).
 *   autotune      > 0: each operand ring depth that fits (2..4 chunks of 32 KB) with each layer
 *                 ring length (4, 8, 16 steps) is run twice at creation and the fastest pair kept;
 *                 < 0: depth -autotune (layer rings of 8); 0: the deepest that fits. Neither choice
 *                 changes any result.
 *   segment_steps non-zero: at most this many steps per persistent launch (0: as many as a 256 MB
 *                 buffer of pre-drawn input spike bitmaps holds); segments do not change any result.
 * The device buffers (weights, rates, counts, record) must stay valid for the plan's life; their
 * contents are read / written by every knp_gb300_batched_plan_run, so rates and weights may be
 * rewritten between runs. One run: memsets of the run's state, the input-threshold kernel and, per
 * segment of steps, the input-drawing kernel and the persistent kernel (cluster launch of CTA pairs),
 * launched as one graph on `stream`; synchronous. Runs of one plan must not overlap (they share the
 * plan's device state).
 */
typedef struct knp_gb300_batched_plan knp_gb300_batched_plan;

KNP_GB300_API int knp_gb300_batched_plan_create(
    int n_layers, const uint32_t *sizes, const void *const *d_weights, const float *leak, const float *threshold,
    const float *reset, const uint32_t *refract, uint32_t batch, const uint32_t *steps, const uint32_t *sample_sizes,
    const float *d_rates, uint64_t seed, int32_t *d_counts, uint32_t *d_record, int autotune, uint32_t segment_steps,
    void *stream, knp_gb300_batched_plan **plan);

/** Runs the prepared batch once: *events (host) synaptic events, *ms device time of the graph launch. */
KNP_GB300_API int knp_gb300_batched_plan_run(knp_gb300_batched_plan *plan, uint64_t *events, float *ms);

/**
 * The operand ring depth and the layer ring length (steps a layer may hold; it runs at most that
 * many minus 2 steps ahead of the next layer) in use, and, after autotuning, the time of each pair
 * tried: tune_ms[9], index 3 * r + (depth - 2) for layer rings of 4, 8, 16 steps (r = 0, 1, 2) and
 * depths 2, 3, 4; 0 = not tried.
 */
KNP_GB300_API int knp_gb300_batched_plan_info(const knp_gb300_batched_plan *plan, int *stages, int *ring_steps,
                                              float *tune_ms);

KNP_GB300_API void knp_gb300_batched_plan_destroy(knp_gb300_batched_plan *plan);

/** Block until all queued device work of the backend has finished. */
KNP_GB300_API int knp_gb300_synchronize(knp_gb300_backend *b);

/** CUDA stream the backend launches on (a cudaStream_t), for callers that order their own work after it. */
KNP_GB300_API int knp_gb300_stream(knp_gb300_backend *b, void **stream);

#ifdef __cplusplus
}
#endif

#endif /* KNP_GB300_H */
