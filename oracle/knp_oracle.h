/*
 * TEST INFRASTRUCTURE — CPU oracle of the KNP single-threaded backend step.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arms load this.
 * The GB300 product path never calls it.
 *
 * Two implementations export this same C API:
 *   - knp_oracle.cpp (libknp_oracle.so): a restatement of the reference algorithm written for
 *     this repository (FP64 neuron state, the reference's container structure);
 *   - ref_driver.cpp (_ref/libknp_ref.so): the reference's own per-neuron / per-synapse headers
 *     compiled against a small shim, driven by the same message-routing loop.
 * Tests compare the two on seeded networks, and both against the reference's golden vectors.
 */
#ifndef KNP_ORACLE_H
#define KNP_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/knp_gb300_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_net or_net;

/** Last error message of the calling thread ("" if none). */
const char *or_last_error(void);

or_net *or_create(void);
void or_destroy(or_net *net);

/** Add a BLIFAT (kind 0), resource-STDP BLIFAT (kind 1) population. `ext` is required for kind 1. */
int or_add_blifat_population(
    or_net *net, knp_uid uid, int kind, uint32_t n, const knp_blifat_neuron *neurons,
    const knp_resource_stdp_state *ext);

/** Add a LIF population (kind 2). */
int or_add_lif_population(or_net *net, knp_uid uid, uint32_t n, const knp_lif_neuron *neurons);
/* AltAI-LIF populations (kind KNP_NEURON_ALTAI_LIF, or KNP_NEURON_RESOURCE_STDP_ALTAI_LIF with ext). */
int or_add_altai_population(
    or_net *net, knp_uid uid, int kind, uint32_t n, const knp_altai_neuron *neurons, const knp_resource_stdp_state *ext);
int or_read_altai(const or_net *net, knp_uid pop, knp_altai_neuron *out, knp_resource_stdp_state *ext);

/**
 * Add a projection. kind: knp_synapse_kind. pre_uid may be all-zero (no presynaptic population).
 * tau_plus / tau_minus are read only for additive-STDP projections.
 */
int or_add_projection(
    or_net *net, knp_uid uid, int kind, knp_uid pre_uid, knp_uid post_uid, uint64_t n_syn,
    const uint32_t *pre_idx, const uint32_t *post_idx, const float *weight, const uint32_t *delay,
    const uint8_t *out_type, const float *tau_plus, const float *tau_minus);

/** Register `pop_uid` in an STDP projection's stdp_populations_ map. */
int or_set_stdp_population(or_net *net, knp_uid proj_uid, knp_uid pop_uid, int processing);
/* SynapticResourceSTDPDeltaSynapse projection: the rule state of every synapse and the projection's
 * lock flag (a projection starts locked; start_learning unlocks every projection). */
int or_add_resource_projection(
    or_net *net, knp_uid uid, knp_uid pre_uid, knp_uid post_uid, uint64_t n_syn, const uint32_t *pre_idx,
    const uint32_t *post_idx, const float *weight, const uint32_t *delay, const uint8_t *out_type,
    const knp_resource_synapse *rule, int locked);
/* start_learning (on = 1) / stop_learning (on = 0). */
int or_set_learning(or_net *net, int on);
int or_read_resource_synapses(const or_net *net, knp_uid proj, knp_resource_synapse *out);

/** Extra subscription of `receiver` (projection or population) to messages of `sender`. */
int or_subscribe(or_net *net, knp_uid receiver, knp_uid sender);

/** Build the reference's subscriptions (knp/backends/cpu/cpu-library/include/knp/backends/cpu-library/init.h:93-110). */
int or_init(or_net *net);
/* Timing support (restated oracle only): or_snapshot keeps a copy of the network as it is now, and
 * or_reset returns the network to that copy (step 0, no messages in flight). */
int or_snapshot(or_net *net);
int or_reset(or_net *net);

/** An external SpikeMessage {sender, send_time, indexes}, delivered at the next step. */
int or_send_spikes(or_net *net, knp_uid sender, uint64_t send_time, uint32_t n, const uint32_t *idx);

/** An external SynapticImpactMessage to a population, delivered at the next step. */
int or_send_impacts(
    or_net *net, knp_uid sender, knp_uid receiver_pop, int is_forcing, uint32_t n, const uint32_t *post_idx,
    const float *value, const uint8_t *out_type);

/** One backend step. */
int or_step(or_net *net);

/**
 * One step of the reference's multi-threaded CPU backend structure on `threads` workers (for timing
 * the reference's multi-threaded path; its semantics differ from the single-threaded oracle: only
 * the first spike message per projection per step, impacts = weight x spike count, no additive STDP).
 */
int or_step_mt(or_net *net, int threads);
uint64_t or_get_step(const or_net *net);

/** Spike indexes a population emitted in the last step (ascending), count in *n. */
int or_read_spikes(const or_net *net, knp_uid pop, uint32_t cap, uint32_t *out, uint32_t *n);

int or_read_blifat(const or_net *net, knp_uid pop, knp_blifat_neuron *out, knp_resource_stdp_state *ext);
int or_read_lif(const or_net *net, knp_uid pop, knp_lif_neuron *out);

/** Projection weights in the projection's synapse order. */
int or_read_weights(const or_net *net, knp_uid proj, float *out);

/** Synaptic events (impacts created) since creation. */
uint64_t or_event_count(const or_net *net);

#ifdef __cplusplus
}
#endif

#endif /* KNP_ORACLE_H */
