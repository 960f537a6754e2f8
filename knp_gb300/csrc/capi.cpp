// extern "C" layer of include/knp_gb300.h over the host runtime: argument checks, exception to
// status-code translation, thread-local error text.
#include <cuda_runtime.h>

#include <string>

#include "../../include/knp_gb300.h"
#include "engine.h"

namespace knp_gb300
{
int lif_scan_forward(
    const float *I, float *S, float *ckpt, int T, long long BN, float beta, float theta, int K, int relaxed, float k,
    cudaStream_t s);
int lif_scan_backward(
    const float *I, const float *ckpt, const float *dS, float *dI, int T, long long BN, float beta, float theta, int K,
    int relaxed, float k, cudaStream_t s);
int bf16_operand(const void *X, int x_bf16, long long R, long long C, int mode, int transpose, long long P, void *out,
                 cudaStream_t s);
}  // namespace knp_gb300

namespace knp_gb300
{
int bernoulli_schedule_noalloc(
    uint32_t n_sources, double p, uint64_t first_step, uint64_t n_steps, uint64_t seed, uint64_t stream,
    long long *d_offsets, uint32_t *d_idx, uint64_t capacity, uint64_t *n_idx, cudaStream_t s, const char **why);
}  // namespace knp_gb300

namespace knp_gb300
{
int bf16_gemm_tn(const void *A, const void *B, float *D, int M, int N, int K, unsigned int *d_err, cudaStream_t s);
int batched_lif_run(
    int n_layers, const uint32_t *sizes, const void *const *weights, const float *leak, const float *threshold,
    const float *reset, const uint32_t *refract, uint32_t batch, const uint32_t *steps, const float *rates,
    unsigned long long key, int *counts, uint32_t *record, unsigned long long *events_out, float *ms,
    cudaStream_t s, const char **why);
struct BatchedPlan;
int batched_plan_create(
    int n_layers, const uint32_t *sizes, const void *const *weights, const float *leak, const float *threshold,
    const float *reset, const uint32_t *refract, uint32_t batch, const uint32_t *steps, const uint32_t *sample_sizes,
    const float *rates, unsigned long long key, int *counts, uint32_t *record, int autotune, uint32_t segment_steps,
    cudaStream_t s, BatchedPlan **out, const char **why);
int batched_plan_run(BatchedPlan *p, unsigned long long *events_out, float *ms, const char **why);
void batched_plan_info(const BatchedPlan *p, int *stages, int *ring_steps, float *tune_ms);
void batched_plan_destroy(BatchedPlan *p);
}  // namespace knp_gb300

struct knp_gb300_batched_plan
{
    knp_gb300::BatchedPlan *impl;
};

struct knp_gb300_backend
{
    knp_gb300::Backend impl;
    explicit knp_gb300_backend(int device) : impl(device) {}
};

namespace
{
thread_local std::string g_error;

template <class F>
int guarded(F &&f)
{
    try
    {
        f();
        g_error.clear();
        return KNP_GB300_OK;
    }
    catch (const knp_gb300::Error &e)
    {
        g_error = e.what();
        return e.code();
    }
    catch (const std::bad_alloc &)
    {
        g_error = "host allocation failed";
        return KNP_GB300_E_NOMEM;
    }
    catch (const std::exception &e)
    {
        g_error = e.what();
        return KNP_GB300_E_INVALID;
    }
}

int null_handle()
{
    g_error = "null backend handle";
    return KNP_GB300_E_INVALID;
}

knp_gb300::Uid U(const knp_uid &u) { return knp_gb300::Uid(u); }
}  // namespace

extern "C" {

const char *knp_gb300_last_error(void) { return g_error.c_str(); }

const char *knp_gb300_version(void) { return "knp_gb300 0.1.0 (sm_103a)"; }

int knp_gb300_create(int device, knp_gb300_backend **out)
{
    if (!out) return null_handle();
    *out = nullptr;
    return guarded([&] { *out = new knp_gb300_backend(device); });
}

int knp_gb300_destroy(knp_gb300_backend *b)
{
    if (!b) return null_handle();
    return guarded([&] { delete b; });
}

int knp_gb300_load_blifat_population(
    knp_gb300_backend *b, knp_uid uid, int kind, uint32_t n, const knp_blifat_neuron *neurons,
    const knp_resource_stdp_state *ext)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.load_blifat(U(uid), kind, n, neurons, ext); });
}

int knp_gb300_load_lif_population(knp_gb300_backend *b, knp_uid uid, uint32_t n, const knp_lif_neuron *neurons)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.load_lif(U(uid), n, neurons); });
}

int knp_gb300_read_lif_population(knp_gb300_backend *b, knp_uid pop, knp_lif_neuron *out)
{
    if (!b || !out) return null_handle();
    return guarded([&] { b->impl.read_lif(U(pop), out); });
}

int knp_gb300_load_altai_population(
    knp_gb300_backend *b, knp_uid uid, int kind, uint32_t n, const knp_altai_neuron *neurons,
    const knp_resource_stdp_state *ext)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.load_altai(U(uid), kind, n, neurons, ext); });
}

int knp_gb300_read_altai_population(knp_gb300_backend *b, knp_uid pop, knp_altai_neuron *out, knp_resource_stdp_state *ext)
{
    if (!b || !out) return null_handle();
    return guarded([&] { b->impl.read_altai(U(pop), out, ext); });
}

int knp_gb300_load_projection(
    knp_gb300_backend *b, knp_uid uid, int kind, knp_uid pre_uid, knp_uid post_uid, uint64_t n_syn, const uint32_t *pre,
    const uint32_t *post, const float *weight, const uint32_t *delay, const uint8_t *out_type, const float *tau_plus,
    const float *tau_minus)
{
    if (!b) return null_handle();
    return guarded(
        [&]
        {
            if (kind == KNP_SYNAPSE_RESOURCE_STDP_DELTA)
                throw knp_gb300::Error(KNP_GB300_E_INVALID,
                                       "resource-STDP projections are loaded with knp_gb300_load_resource_stdp_projection");
            b->impl.load_projection(U(uid), kind, U(pre_uid), U(post_uid), n_syn, pre, post, weight, delay, out_type,
                                    tau_plus, tau_minus);
        });
}

int knp_gb300_generate_fixed_fan_in_projection(
    knp_gb300_backend *b, knp_uid uid, knp_uid pre_uid, knp_uid post_uid, uint32_t n_pre, uint32_t n_post,
    uint32_t fan_in, int32_t k_lo, int32_t k_hi, uint32_t d_lo, uint32_t d_hi, uint64_t seed, uint64_t stream)
{
    if (!b) return null_handle();
    return guarded(
        [&]
        {
            b->impl.generate_projection(U(uid), U(pre_uid), U(post_uid), KNP_GEN_FIXED_NUMBER_PRE, n_pre, n_post,
                                        static_cast<uint64_t>(n_post) * fan_in, 0.0, k_lo, k_hi, d_lo, d_hi, seed,
                                        stream);
        });
}

int knp_gb300_generate_projection(
    knp_gb300_backend *b, knp_uid uid, knp_uid pre_uid, knp_uid post_uid, int kind, uint32_t n_pre, uint32_t n_post,
    uint64_t count, double probability, int32_t k_lo, int32_t k_hi, uint32_t d_lo, uint32_t d_hi, uint64_t seed,
    uint64_t stream)
{
    if (!b) return null_handle();
    return guarded(
        [&]
        {
            b->impl.generate_projection(U(uid), U(pre_uid), U(post_uid), kind, n_pre, n_post, count, probability, k_lo,
                                        k_hi, d_lo, d_hi, seed, stream);
        });
}

int knp_gb300_set_stdp_population(knp_gb300_backend *b, knp_uid proj_uid, knp_uid pop_uid, int processing)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.set_stdp_population(U(proj_uid), U(pop_uid), processing); });
}

int knp_gb300_subscribe(knp_gb300_backend *b, knp_uid receiver, knp_uid sender)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.subscribe(U(receiver), U(sender)); });
}

int knp_gb300_set_accumulator(knp_gb300_backend *b, knp_uid pop_uid, int mode)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.set_accumulator(U(pop_uid), mode); });
}

int knp_gb300_set_pull_threshold(knp_gb300_backend *b, knp_uid proj_uid, double fraction)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.set_pull_threshold(U(proj_uid), fraction); });
}

int knp_gb300_set_step_mode(knp_gb300_backend *b, int mode)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.set_step_mode(mode); });
}

int knp_gb300_step_fused(const knp_gb300_backend *b, int *fused)
{
    if (!b || !fused) return null_handle();
    *fused = b->impl.fused() ? 1 : 0;
    return KNP_GB300_OK;
}

int knp_gb300_step_kernel(const knp_gb300_backend *b, int *mode)
{
    if (!b || !mode) return null_handle();
    *mode = b->impl.step_kernel();
    return KNP_GB300_OK;
}

int knp_gb300_record_spikes(knp_gb300_backend *b, knp_uid pop_uid, int enable)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.record_spikes(U(pop_uid), enable != 0); });
}

int knp_gb300_init(knp_gb300_backend *b)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.init(); });
}

int knp_gb300_send_spikes(knp_gb300_backend *b, knp_uid sender, uint64_t send_time, uint32_t n, const uint32_t *idx)
{
    if (!b) return null_handle();
    if (n && !idx)
    {
        g_error = "null index array";
        return KNP_GB300_E_INVALID;
    }
    return guarded([&] { b->impl.send_spikes(U(sender), send_time, n, idx); });
}

int knp_gb300_load_spike_schedule(
    knp_gb300_backend *b, knp_uid sender, uint64_t first_step, uint64_t n_steps, const int64_t *offsets,
    const uint32_t *idx)
{
    if (!b) return null_handle();
    if (!offsets)
    {
        g_error = "null offsets";
        return KNP_GB300_E_INVALID;
    }
    return guarded([&] { b->impl.load_schedule(U(sender), first_step, n_steps, offsets, idx); });
}

int knp_gb300_generate_bernoulli_schedule(
    knp_gb300_backend *b, knp_uid sender, uint32_t n_sources, double p, uint64_t first_step, uint64_t n_steps,
    uint64_t seed, uint64_t stream)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.generate_bernoulli(U(sender), n_sources, p, first_step, n_steps, seed, stream); });
}

int knp_gb300_send_impacts(
    knp_gb300_backend *b, knp_uid sender, knp_uid receiver, int is_forcing, uint32_t n, const uint32_t *post_idx,
    const float *value, const uint8_t *out_type)
{
    if (!b) return null_handle();
    if (n && (!post_idx || !value))
    {
        g_error = "null impact array";
        return KNP_GB300_E_INVALID;
    }
    return guarded([&] { b->impl.send_impacts(U(sender), U(receiver), is_forcing != 0, n, post_idx, value, out_type); });
}

int knp_gb300_step(knp_gb300_backend *b, uint64_t n_steps)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.step(n_steps); });
}

int knp_gb300_get_step(const knp_gb300_backend *b, uint64_t *step)
{
    if (!b || !step) return null_handle();
    *step = b->impl.current_step();
    return KNP_GB300_OK;
}

int knp_gb300_read_spikes(knp_gb300_backend *b, knp_uid pop, uint64_t step, uint32_t cap, uint32_t *out, uint32_t *n)
{
    if (!b || !n) return null_handle();
    if (cap && !out)
    {
        g_error = "null output array";
        return KNP_GB300_E_INVALID;
    }
    return guarded([&] { b->impl.read_spikes(U(pop), step, cap, out, n); });
}

int knp_gb300_discard_spikes(knp_gb300_backend *b, uint64_t step)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.discard_spikes(step); });
}

int knp_gb300_read_blifat_population(
    knp_gb300_backend *b, knp_uid pop, knp_blifat_neuron *out, knp_resource_stdp_state *ext)
{
    if (!b || !out) return null_handle();
    return guarded([&] { b->impl.read_blifat(U(pop), out, ext); });
}

int knp_gb300_load_resource_stdp_projection(
    knp_gb300_backend *b, knp_uid uid, knp_uid pre_uid, knp_uid post_uid, uint64_t n_syn, const uint32_t *pre,
    const uint32_t *post, const float *weight, const uint32_t *delay, const uint8_t *out_type,
    const knp_resource_synapse *rule, int locked)
{
    if (!b) return null_handle();
    return guarded(
        [&]
        {
            b->impl.load_resource_projection(U(uid), U(pre_uid), U(post_uid), n_syn, pre, post, weight, delay, out_type,
                                             rule, locked != 0);
        });
}

int knp_gb300_read_resource_synapses(knp_gb300_backend *b, knp_uid proj, knp_resource_synapse *out)
{
    if (!b || !out) return null_handle();
    return guarded([&] { b->impl.read_resource_synapses(U(proj), out); });
}

int knp_gb300_read_weights(knp_gb300_backend *b, knp_uid proj, float *out)
{
    if (!b || !out) return null_handle();
    return guarded([&] { b->impl.read_weights(U(proj), out); });
}

int knp_gb300_projection_size(const knp_gb300_backend *b, knp_uid proj, uint64_t *n)
{
    if (!b || !n) return null_handle();
    return guarded([&] { *n = b->impl.projection_size(U(proj)); });
}

int knp_gb300_start_learning(knp_gb300_backend *b)
{
    if (!b) return null_handle();
    b->impl.set_learning(true);
    return KNP_GB300_OK;
}

int knp_gb300_stop_learning(knp_gb300_backend *b)
{
    if (!b) return null_handle();
    b->impl.set_learning(false);
    return KNP_GB300_OK;
}

int knp_gb300_counters(knp_gb300_backend *b, uint64_t *events, uint64_t *spikes, uint64_t *neuron_updates)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.counters(events, spikes, neuron_updates); });
}

int knp_gb300_step_timed(knp_gb300_backend *b, uint64_t n_steps, float *ms)
{
    if (!b || !ms) return null_handle();
    return guarded([&] { *ms = b->impl.step_timed(n_steps); });
}

int knp_gb300_profile_phases(knp_gb300_backend *b, uint64_t n_steps, float *ms)
{
    if (!b || !ms) return null_handle();
    return guarded([&] { b->impl.profile_phases(n_steps, ms); });
}

int knp_gb300_profile_grid_phases(knp_gb300_backend *b, uint64_t n_steps, double *us)
{
    if (!b || !us) return null_handle();
    return guarded([&] { b->impl.profile_grid_phases(n_steps, us); });
}

int knp_gb300_lif_scan_forward(
    const float *I, float *S, float *ckpt, int T, int64_t BN, float beta, float theta, int K, int relaxed, float k,
    void *stream)
{
    if (!I || !S || !ckpt)
    {
        g_error = "null buffer";
        return KNP_GB300_E_INVALID;
    }
    const int rc = knp_gb300::lif_scan_forward(I, S, ckpt, T, BN, beta, theta, K, relaxed, k,
                                               static_cast<cudaStream_t>(stream));
    if (rc) g_error = rc == -1 ? "bad sizes (T >= 1, BN >= 1, 1 <= K <= 16)" : "kernel launch failed";
    return rc;
}

int knp_gb300_lif_scan_backward(
    const float *I, const float *ckpt, const float *dS, float *dI, int T, int64_t BN, float beta, float theta, int K,
    int relaxed, float k, void *stream)
{
    if (!I || !ckpt || !dS || !dI)
    {
        g_error = "null buffer";
        return KNP_GB300_E_INVALID;
    }
    const int rc = knp_gb300::lif_scan_backward(I, ckpt, dS, dI, T, BN, beta, theta, K, relaxed, k,
                                                static_cast<cudaStream_t>(stream));
    if (rc) g_error = rc == -1 ? "bad sizes (T >= 1, BN >= 1, 1 <= K <= 16)" : "kernel launch failed";
    return rc;
}

int knp_gb300_bf16_operand(const void *X, int x_bf16, int64_t R, int64_t C, int mode, int transpose, int64_t P,
                           void *out, void *stream)
{
    const int rc = knp_gb300::bf16_operand(X, x_bf16, R, C, mode, transpose, P, out, static_cast<cudaStream_t>(stream));
    if (rc == 0) return KNP_GB300_OK;
    g_error = rc == -1 ? "bad operand arguments (sizes >= 1, mode 0..2, P >= the copied extent)" : "kernel launch failed";
    return rc == -1 ? KNP_GB300_E_INVALID : KNP_GB300_E_CUDA;
}

int knp_gb300_generate_bernoulli_schedule_noalloc(
    uint32_t n_sources, double p, uint64_t first_step, uint64_t n_steps, uint64_t seed, uint64_t stream_id,
    int64_t *d_offsets, uint32_t *d_idx, uint64_t capacity, uint64_t *n_idx, void *stream)
{
    const char *why = "";
    const int rc = knp_gb300::bernoulli_schedule_noalloc(
        n_sources, p, first_step, n_steps, seed, stream_id, reinterpret_cast<long long *>(d_offsets), d_idx, capacity,
        n_idx, static_cast<cudaStream_t>(stream), &why);
    if (rc == 0) return KNP_GB300_OK;
    g_error = why;
    return rc == -3 ? KNP_GB300_E_CUDA : KNP_GB300_E_INVALID;
}

int knp_gb300_measure_add_rate(uint64_t n_floats, uint64_t n_adds, double *adds_per_s)
{
    if (!adds_per_s || n_floats == 0 || n_floats > 0xFFFFFFFFull || n_adds == 0)
    {
        g_error = "n_floats (below 2^32) and n_adds must be positive, adds_per_s not null";
        return KNP_GB300_E_INVALID;
    }
    const char *why = "";
    if (knp_gb300::measure_add_rate(n_floats, n_adds, adds_per_s, &why) == 0) return KNP_GB300_OK;
    g_error = why;
    return KNP_GB300_E_CUDA;
}

int knp_gb300_bf16_gemm_tn(
    const void *A, const void *B, float *D, int M, int N, int K, unsigned int *d_err, void *stream)
{
    const int rc = knp_gb300::bf16_gemm_tn(A, B, D, M, N, K, d_err, static_cast<cudaStream_t>(stream));
    if (rc) g_error = rc == -1 ? "bad GEMM arguments" : "kernel launch failed";
    return rc == 0 ? KNP_GB300_OK : (rc == -1 ? KNP_GB300_E_INVALID : KNP_GB300_E_CUDA);
}

static int batched_status(int rc, const char *why)
{
    if (rc == 0) return KNP_GB300_OK;
    g_error = why;
    switch (rc)
    {
        case -1:
            return KNP_GB300_E_INVALID;
        case -4:
            return KNP_GB300_E_DEVICE_FLAG;
        case -5:
            return KNP_GB300_E_NOMEM;
        default:
            return KNP_GB300_E_CUDA;
    }
}

int knp_gb300_batched_lif_run(
    int n_layers, const uint32_t *sizes, const void *const *d_weights, const float *leak, const float *threshold,
    const float *reset, const uint32_t *refract, uint32_t batch, const uint32_t *steps, const float *d_rates,
    uint64_t seed, int32_t *d_counts, uint32_t *d_record, uint64_t *events, float *ms, void *stream)
{
    const char *why = "";
    unsigned long long ev = 0;
    const int rc = knp_gb300::batched_lif_run(
        n_layers, sizes, d_weights, leak, threshold, reset, refract, batch, steps, d_rates,
        knp_gb300::stream_key(seed, 5), d_counts, d_record, &ev, ms, static_cast<cudaStream_t>(stream), &why);
    if (events) *events = ev;
    return batched_status(rc, why);
}

int knp_gb300_batched_plan_create(
    int n_layers, const uint32_t *sizes, const void *const *d_weights, const float *leak, const float *threshold,
    const float *reset, const uint32_t *refract, uint32_t batch, const uint32_t *steps, const uint32_t *sample_sizes,
    const float *d_rates, uint64_t seed, int32_t *d_counts, uint32_t *d_record, int autotune, uint32_t segment_steps,
    void *stream, knp_gb300_batched_plan **plan)
{
    if (!plan)
    {
        g_error = "plan is null";
        return KNP_GB300_E_INVALID;
    }
    *plan = nullptr;
    const char *why = "";
    knp_gb300::BatchedPlan *p = nullptr;
    const int rc = knp_gb300::batched_plan_create(
        n_layers, sizes, d_weights, leak, threshold, reset, refract, batch, steps, sample_sizes, d_rates,
        knp_gb300::stream_key(seed, 5), d_counts, d_record, autotune, segment_steps, static_cast<cudaStream_t>(stream),
        &p, &why);
    if (rc == 0) *plan = new knp_gb300_batched_plan{p};
    return batched_status(rc, why);
}

int knp_gb300_batched_plan_run(knp_gb300_batched_plan *plan, uint64_t *events, float *ms)
{
    if (!plan || !plan->impl)
    {
        g_error = "plan is null";
        return KNP_GB300_E_INVALID;
    }
    const char *why = "";
    unsigned long long ev = 0;
    const int rc = knp_gb300::batched_plan_run(plan->impl, &ev, ms, &why);
    if (events) *events = ev;
    return batched_status(rc, why);
}

int knp_gb300_batched_plan_info(const knp_gb300_batched_plan *plan, int *stages, int *ring_steps, float *tune_ms)
{
    if (!plan || !plan->impl)
    {
        g_error = "plan is null";
        return KNP_GB300_E_INVALID;
    }
    knp_gb300::batched_plan_info(plan->impl, stages, ring_steps, tune_ms);
    return KNP_GB300_OK;
}

void knp_gb300_batched_plan_destroy(knp_gb300_batched_plan *plan)
{
    if (!plan) return;
    knp_gb300::batched_plan_destroy(plan->impl);
    delete plan;
}

int knp_gb300_synchronize(knp_gb300_backend *b)
{
    if (!b) return null_handle();
    return guarded([&] { b->impl.synchronize(); });
}

int knp_gb300_stream(knp_gb300_backend *b, void **stream)
{
    if (!b || !stream) return null_handle();
    *stream = static_cast<void *>(b->impl.stream());
    return KNP_GB300_OK;
}

}  // extern "C"
