// Host runtime of the GB300 KNP backend (see engine.h).
#include "engine.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <limits>
#include <numeric>

namespace knp_gb300
{

#define KNP_CUDA(call)                                                                                          \
    do                                                                                                          \
    {                                                                                                           \
        cudaError_t e_ = (call);                                                                                \
        if (e_ != cudaSuccess)                                                                                  \
            throw Error(e_ == cudaErrorMemoryAllocation ? KNP_GB300_E_NOMEM : KNP_GB300_E_CUDA,                 \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                                    \
    } while (0)

namespace
{

uint32_t round_up(uint32_t x, uint32_t m) { return (x + m - 1) / m * m; }

float to_f(double x) { return static_cast<float>(x); }

bool is_dyadic(float w)
{
    const double k = static_cast<double>(w) * 256.0;
    return std::floor(k) == k && std::fabs(k) < 16777216.0;
}

// The reference's stdp_w for d >= 0 (additive_stdp.h:50-55 with a_plus = a_minus = 1), evaluated
// with the host libm exactly as the reference evaluates it; 0 beyond the returned length.
std::vector<float> stdp_table(float tau_plus, float tau_minus)
{
    std::vector<float> t;
    for (uint64_t d = 0;; ++d)
    {
        const float wd = static_cast<float>(d);
        const float v = wd > 0 ? 1.0F * std::exp(-wd / tau_plus) : 1.0F * std::exp(wd / tau_minus);
        if (v == 0.0F && d > 0) break;
        t.push_back(v);
        if (t.size() > (1u << 24)) break;
    }
    return t;
}

}  // namespace

// ------------------------------------------------------------------------------- DeviceArena

DeviceArena::~DeviceArena()
{
    for (void *p : ptrs_) cudaFree(p);
}

void *DeviceArena::alloc(size_t bytes, bool zero)
{
    if (bytes == 0) bytes = 16;
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess)
        throw Error(KNP_GB300_E_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed: " +
                                           cudaGetErrorString(e));
    if (zero) KNP_CUDA(cudaMemset(p, 0, bytes));
    ptrs_.push_back(p);
    bytes_ += bytes;
    return p;
}

void DeviceArena::release(void *p)
{
    auto it = std::find(ptrs_.begin(), ptrs_.end(), p);
    if (it != ptrs_.end())
    {
        cudaFree(p);
        ptrs_.erase(it);
    }
}

// ----------------------------------------------------------------------------------- Backend

Backend::Backend(int device) : device_(device)
{
    int n = 0;
    KNP_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) throw Error(KNP_GB300_E_INVALID, "no CUDA device " + std::to_string(device));
    KNP_CUDA(cudaSetDevice(device));
    KNP_CUDA(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device));
    KNP_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    KNP_CUDA(cudaEventCreateWithFlags(&pinned_free_, cudaEventDisableTiming));
    KNP_CUDA(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking));
    for (auto &e : step_ev_) KNP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    KNP_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&ctl_host_), sizeof(Control), cudaHostAllocDefault));
    ctl_ = arena_.make<Control>(1);
}

Backend::~Backend()
{
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    if (persisting_l2_)
    {
        // The ring's lines go back to normal eviction and the L2 set-aside to its previous size, so
        // that later work in this process gets the whole L2 again.
        cudaCtxResetPersistingL2Cache();
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, persisting_before_);
    }
    if (graph1_) cudaGraphExecDestroy(graph1_);
    if (graphK_) cudaGraphExecDestroy(graphK_);
    for (auto &c : channels_)
        if (c->owns_generated && c->idx) cudaFree(c->idx);
    if (pinned_) cudaFreeHost(pinned_);
    if (rec_host_) cudaFreeHost(rec_host_);
    if (pinned_free_) cudaEventDestroy(pinned_free_);
    if (copy_stream_) cudaStreamSynchronize(copy_stream_);
    for (auto &e : step_ev_)
        if (e) cudaEventDestroy(e);
    if (ctl_host_) cudaFreeHost(ctl_host_);
    if (copy_stream_) cudaStreamDestroy(copy_stream_);
    if (stream_) cudaStreamDestroy(stream_);
}

void Backend::require_not_init(const char *what) const
{
    if (initialized_) throw Error(KNP_GB300_E_STATE, std::string(what) + " is not allowed after init");
}

void Backend::require_init(const char *what) const
{
    if (!initialized_) throw Error(KNP_GB300_E_STATE, std::string(what) + " requires init");
}

PopulationSlot *Backend::find_pop(const Uid &u)
{
    for (auto &p : pops_)
        if (p->uid == u) return p.get();
    return nullptr;
}

ProjectionSlot *Backend::find_proj(const Uid &u)
{
    for (auto &p : projs_)
        if (p->uid == u) return p.get();
    return nullptr;
}

const ProjectionSlot *Backend::find_proj(const Uid &u) const
{
    for (auto &p : projs_)
        if (p->uid == u) return p.get();
    return nullptr;
}

Channel *Backend::find_channel(const Uid &u)
{
    for (auto &c : channels_)
        if (c->uid == u) return c.get();
    return nullptr;
}

Channel &Backend::channel(const Uid &u)
{
    if (Channel *c = find_channel(u)) return *c;
    auto c = std::make_unique<Channel>();
    c->uid = u;
    c->dev = arena_.make<ChannelDev>(1);
    channels_.push_back(std::move(c));
    return *channels_.back();
}

void Backend::load_blifat(
    const Uid &uid, int kind, uint32_t n, const knp_blifat_neuron *neurons, const knp_resource_stdp_state *ext)
{
    require_not_init("load_blifat_population");
    if (kind != KNP_NEURON_BLIFAT && kind != KNP_NEURON_RESOURCE_STDP_BLIFAT)
        throw Error(KNP_GB300_E_INVALID, "unsupported neuron kind " + std::to_string(kind));
    if (kind == KNP_NEURON_RESOURCE_STDP_BLIFAT && !ext)
        throw Error(KNP_GB300_E_INVALID, "a resource-STDP population needs its knp_resource_stdp_state array");
    if (!neurons && n) throw Error(KNP_GB300_E_INVALID, "null neuron array");
    if (find_pop(uid) || find_proj(uid)) throw Error(KNP_GB300_E_INVALID, "duplicate UID");
    auto p = std::make_unique<PopulationSlot>();
    p->uid = uid;
    p->kind = kind;
    p->n = n;
    p->n_pad = round_up(std::max<uint32_t>(n, 1), 4);
    p->init_blifat.assign(neurons, neurons + n);
    if (ext) p->init_res.assign(ext, ext + n);
    pops_.push_back(std::move(p));
}

void Backend::load_altai(
    const Uid &uid, int kind, uint32_t n, const knp_altai_neuron *neurons, const knp_resource_stdp_state *ext)
{
    require_not_init("load_altai_population");
    if (kind != KNP_NEURON_ALTAI_LIF && kind != KNP_NEURON_RESOURCE_STDP_ALTAI_LIF)
        throw Error(KNP_GB300_E_INVALID, "unsupported neuron kind " + std::to_string(kind));
    if (kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF && !ext)
        throw Error(KNP_GB300_E_INVALID, "a resource-STDP population needs its knp_resource_stdp_state array");
    if (!neurons && n) throw Error(KNP_GB300_E_INVALID, "null neuron array");
    if (find_pop(uid) || find_proj(uid)) throw Error(KNP_GB300_E_INVALID, "duplicate UID");
    auto p = std::make_unique<PopulationSlot>();
    p->uid = uid;
    p->kind = kind;
    p->n = n;
    p->n_pad = round_up(std::max<uint32_t>(n, 1), 4);
    p->init_altai.assign(neurons, neurons + n);
    if (kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF) p->init_res.assign(ext, ext + n);
    pops_.push_back(std::move(p));
}

void Backend::load_lif(const Uid &uid, uint32_t n, const knp_lif_neuron *neurons)
{
    require_not_init("load_lif_population");
    if (!neurons && n) throw Error(KNP_GB300_E_INVALID, "null neuron array");
    if (find_pop(uid) || find_proj(uid)) throw Error(KNP_GB300_E_INVALID, "duplicate UID");
    auto p = std::make_unique<PopulationSlot>();
    p->uid = uid;
    p->kind = KNP_NEURON_LIF;
    p->n = n;
    p->n_pad = round_up(std::max<uint32_t>(n, 1), 4);
    p->init_lif.assign(neurons, neurons + n);
    pops_.push_back(std::move(p));
}

void Backend::load_projection(
    const Uid &uid, int kind, const Uid &pre_uid, const Uid &post_uid, uint64_t n_syn, const uint32_t *pre,
    const uint32_t *post, const float *w, const uint32_t *delay, const uint8_t *type, const float *tau_plus,
    const float *tau_minus)
{
    require_not_init("load_projection");
    if (kind != KNP_SYNAPSE_DELTA && kind != KNP_SYNAPSE_ADDITIVE_STDP_DELTA && kind != KNP_SYNAPSE_RESOURCE_STDP_DELTA)
        throw Error(KNP_GB300_E_INVALID, "unsupported synapse kind " + std::to_string(kind));
    if (n_syn && (!pre || !post || !w || !delay)) throw Error(KNP_GB300_E_INVALID, "null synapse array");
    if (n_syn > 0xFFFFFFFFull) throw Error(KNP_GB300_E_INVALID, "more than 2^32-1 synapses in one projection");
    if (kind == KNP_SYNAPSE_ADDITIVE_STDP_DELTA && n_syn && (!tau_plus || !tau_minus))
        throw Error(KNP_GB300_E_INVALID, "an additive-STDP projection needs tau_plus and tau_minus");
    if (find_pop(uid) || find_proj(uid)) throw Error(KNP_GB300_E_INVALID, "duplicate UID");
    auto p = std::make_unique<ProjectionSlot>();
    p->uid = uid;
    p->kind = kind;
    p->pre_uid = pre_uid;
    p->post_uid = post_uid;
    p->n_syn = n_syn;
    p->pre.assign(pre, pre + n_syn);
    p->post.assign(post, post + n_syn);
    p->weight.assign(w, w + n_syn);
    p->delay.assign(delay, delay + n_syn);
    if (type)
    {
        p->type.assign(type, type + n_syn);
        for (uint8_t t : p->type)
        {
            // A BLOCKING impact carries the synapse's weight at the spike; an additive-STDP weight can
            // change before the impact arrives, so BLOCKING synapses are taken in delta projections.
            if (t == KNP_OUT_BLOCKING && kind != KNP_SYNAPSE_DELTA)
                throw Error(KNP_GB300_E_INVALID, "BLOCKING synapses are supported in delta projections only");
            if (t > KNP_OUT_BLOCKING) throw Error(KNP_GB300_E_INVALID, "unhandled synapse type");
        }
        if (std::all_of(p->type.begin(), p->type.end(), [&](uint8_t t) { return t == p->type[0]; }) && n_syn)
        {
            // Uniform type: keep only the value.
            const uint8_t t0 = p->type[0];
            p->type.assign(1, t0);
        }
    }
    for (uint64_t i = 0; i < n_syn; ++i)
        if (p->delay[i] > 255)
            throw Error(KNP_GB300_E_INVALID, "synapse delay above 255 steps is not supported");
    if (kind == KNP_SYNAPSE_ADDITIVE_STDP_DELTA && n_syn)
    {
        p->tau_plus.assign(tau_plus, tau_plus + n_syn);
        p->tau_minus.assign(tau_minus, tau_minus + n_syn);
        for (uint64_t i = 0; i < n_syn; ++i)
            if (p->tau_plus[i] != p->tau_plus[0] || p->tau_minus[i] != p->tau_minus[0])
                throw Error(KNP_GB300_E_INVALID, "STDP time constants must be uniform within a projection");
    }
    projs_.push_back(std::move(p));
}

void Backend::load_resource_projection(
    const Uid &uid, const Uid &pre_uid, const Uid &post_uid, uint64_t n_syn, const uint32_t *pre, const uint32_t *post,
    const float *w, const uint32_t *delay, const uint8_t *type, const knp_resource_synapse *rule, bool locked)
{
    if (n_syn && !rule) throw Error(KNP_GB300_E_INVALID, "resource-STDP synapses need their rule state");
    load_projection(uid, KNP_SYNAPSE_RESOURCE_STDP_DELTA, pre_uid, post_uid, n_syn, pre, post, w, delay, type, nullptr,
                    nullptr);
    ProjectionSlot *p = projs_.back().get();
    p->rule.assign(rule, rule + n_syn);
    p->locked = locked;
}

void Backend::set_learning(bool on)
{
    // start_learning / stop_learning unlock / lock every projection (cpu-single-threaded/backend.h:
    // 315-332); only resource-STDP training reads the lock.
    learning_ = on;
    for (auto &p : projs_) p->locked = !on;
    if (initialized_) upload_locks();
}

void Backend::upload_locks()
{
    for (auto &q : pops_)
    {
        if (!q->res_locked) continue;
        for (size_t k = 0; k < q->res_projs.size(); ++k) q->res_locked_host[k] = q->res_projs[k]->locked ? 1u : 0u;
        // Ordered with the steps on the stream; the host vector outlives the copy.
        KNP_CUDA(cudaMemcpyAsync(q->res_locked, q->res_locked_host.data(), q->res_locked_host.size() * 4,
                                 cudaMemcpyHostToDevice, stream_));
        KNP_CUDA(cudaStreamSynchronize(stream_));
    }
}

static_assert(int(kGenAllToAll) == int(KNP_GEN_ALL_TO_ALL) && int(kGenAligned) == int(KNP_GEN_ALIGNED) &&
                  int(kGenExclusive) == int(KNP_GEN_EXCLUSIVE) && int(kGenOneToOne) == int(KNP_GEN_ONE_TO_ONE) &&
                  int(kGenFixedProbability) == int(KNP_GEN_FIXED_PROBABILITY) &&
                  int(kGenFixedNumberPost) == int(KNP_GEN_FIXED_NUMBER_POST) &&
                  int(kGenFixedNumberPre) == int(KNP_GEN_FIXED_NUMBER_PRE),
              "generator kinds of the C ABI");

GenSpec Backend::gen_spec(const ProjectionSlot &p, const unsigned long long *cand) const
{
    GenSpec g{};
    g.kind = p.gen.kind;
    g.n_pre = p.gen.n_pre;
    g.n_post = p.gen.n_post;
    g.k_lo = p.gen.k_lo;
    g.k_hi = p.gen.k_hi;
    g.d_lo = p.gen.d_lo;
    g.d_hi = p.gen.d_hi;
    g.key_pre = stream_key(p.gen.seed, p.gen.stream + 1);
    g.key_w = stream_key(p.gen.seed, p.gen.stream + 2);
    g.key_d = stream_key(p.gen.seed, p.gen.stream + 3);
    g.key_post = stream_key(p.gen.seed, p.gen.stream + 4);
    g.cand = cand;
    return g;
}

void Backend::generate_projection(const Uid &uid, const Uid &pre_uid, const Uid &post_uid, int kind, uint32_t n_pre,
                                  uint32_t n_post, uint64_t count, double probability, int32_t k_lo, int32_t k_hi,
                                  uint32_t d_lo, uint32_t d_hi, uint64_t seed, uint64_t stream)
{
    require_not_init("generate_projection");
    if (k_lo > k_hi || d_lo > d_hi || d_hi > 255 || n_pre == 0 || n_post == 0)
        throw Error(KNP_GB300_E_INVALID, "bad generator ranges");
    if (find_pop(uid) || find_proj(uid)) throw Error(KNP_GB300_E_INVALID, "duplicate UID");
    uint64_t n_syn = 0, in_degree = 0;
    unsigned long long thr = 0;
    switch (kind)
    {
        case KNP_GEN_ALL_TO_ALL:
            n_syn = static_cast<uint64_t>(n_pre) * n_post;
            in_degree = n_pre;
            break;
        case KNP_GEN_ALIGNED:
            // The larger size a multiple of the smaller (else the reference's rule makes indexes past
            // the smaller population).
            if (std::max(n_pre, n_post) % std::min(n_pre, n_post) != 0)
                throw Error(KNP_GB300_E_INVALID, "aligned: the larger population size must be a multiple of the smaller");
            n_syn = std::max(n_pre, n_post);
            in_degree = n_pre >= n_post ? n_pre / n_post : 1;
            break;
        case KNP_GEN_EXCLUSIVE:
            if (n_pre != n_post || n_pre < 2)
                throw Error(KNP_GB300_E_INVALID, "exclusive: equal population sizes of at least 2");
            n_syn = static_cast<uint64_t>(n_pre) * (n_pre - 1);
            in_degree = n_pre - 1;
            break;
        case KNP_GEN_ONE_TO_ONE:
            if (n_pre != n_post) throw Error(KNP_GB300_E_INVALID, "one_to_one: equal population sizes");
            n_syn = n_pre;
            in_degree = 1;
            break;
        case KNP_GEN_FIXED_PROBABILITY:
        {
            if (!(probability >= 0.0 && probability <= 1.0))
                throw Error(KNP_GB300_E_INVALID, "connection probability outside [0, 1]");
            const uint64_t n_cand = static_cast<uint64_t>(n_pre) * n_post;
            if (n_cand > (1ull << 40)) throw Error(KNP_GB300_E_INVALID, "more than 2^40 candidate pairs");
            thr = static_cast<unsigned long long>(probability * 9007199254740992.0);
            KNP_CUDA(cudaSetDevice(device_));
            KNP_CUDA(gen_candidates(n_cand, thr, stream_key(seed, stream + 5), nullptr, &n_syn, stream_));
            in_degree = n_pre;
            break;
        }
        case KNP_GEN_FIXED_NUMBER_POST:
            n_syn = count;
            in_degree = count;
            break;
        case KNP_GEN_FIXED_NUMBER_PRE:
            n_syn = count;
            in_degree = (count + n_post - 1) / n_post;
            break;
        default:
            throw Error(KNP_GB300_E_INVALID, "unknown generator kind");
    }
    if (n_syn > 0xFFFFFFFFull) throw Error(KNP_GB300_E_INVALID, "more than 2^32-1 synapses in one projection");
    auto p = std::make_unique<ProjectionSlot>();
    p->uid = uid;
    p->kind = KNP_SYNAPSE_DELTA;
    p->pre_uid = pre_uid;
    p->post_uid = post_uid;
    p->n_syn = n_syn;
    p->generated = true;
    p->gen.kind = kind;
    p->gen.n_pre = n_pre;
    p->gen.n_post = n_post;
    p->gen.in_degree = static_cast<uint32_t>(std::min<uint64_t>(in_degree, 0xFFFFFFFFull));
    p->gen.k_lo = k_lo;
    p->gen.k_hi = k_hi;
    p->gen.d_lo = d_lo;
    p->gen.d_hi = d_hi;
    p->gen.seed = seed;
    p->gen.stream = stream;
    p->gen.prob_threshold = thr;
    projs_.push_back(std::move(p));
}

void Backend::set_stdp_population(const Uid &proj, const Uid &pop, int processing)
{
    require_not_init("set_stdp_population");
    ProjectionSlot *p = find_proj(proj);
    if (!p) throw Error(KNP_GB300_E_INVALID, "unknown projection");
    if (p->kind != KNP_SYNAPSE_ADDITIVE_STDP_DELTA) throw Error(KNP_GB300_E_INVALID, "not an STDP projection");
    if (processing != KNP_STDP_ONLY && processing != KNP_STDP_AND_SPIKE)
        throw Error(KNP_GB300_E_INVALID, "bad STDP processing type");
    p->stdp_pops[pop] = processing;
}

void Backend::subscribe(const Uid &receiver, const Uid &sender)
{
    require_not_init("subscribe");
    subs_.emplace_back(receiver, sender);
}

void Backend::set_accumulator(const Uid &pop, int mode)
{
    require_not_init("set_accumulator");
    PopulationSlot *p = find_pop(pop);
    if (!p) throw Error(KNP_GB300_E_INVALID, "unknown population");
    if (mode < KNP_GB300_ACC_AUTO || mode > KNP_GB300_ACC_FIXED64) throw Error(KNP_GB300_E_INVALID, "bad mode");
    p->acc_request = mode;
}

void Backend::record_spikes(const Uid &pop, bool enable)
{
    PopulationSlot *p = find_pop(pop);
    if (!p) throw Error(KNP_GB300_E_INVALID, "unknown population");
    if (initialized_)
    {
        drain_recordings();
        if (enable && !p->rec_bits)
        {
            alloc_recording(*p);
            p->bdev.rec_words = p->ldev.rec_words = p->adev.rec_words = p->rec_words;
            p->bdev.rec_slots = p->ldev.rec_slots = p->adev.rec_slots = p->rec_slots;
        }
        p->record = enable;
        p->record_from = step_;
        p->bdev.rec_bits = enable ? p->rec_bits : nullptr;
        p->ldev.rec_bits = enable ? p->rec_bits : nullptr;
        p->adev.rec_bits = enable ? p->rec_bits : nullptr;
        capture_graphs();
        return;
    }
    p->record = enable;
}

// ------------------------------------------------------------------------------------- init

void Backend::wire()
{
    // cpu::init (knp/backends/cpu/cpu-library/include/knp/backends/cpu-library/init.h:93-110).
    for (auto &p : projs_)
    {
        for (auto &[u, _] : p->stdp_pops)
            if (!u.is_null()) p->spike_senders.insert(u);
        if (!p->pre_uid.is_null()) p->spike_senders.insert(p->pre_uid);
        if (!p->post_uid.is_null())
            if (PopulationSlot *q = find_pop(p->post_uid)) q->impact_senders.insert(p->uid);
    }
    for (auto &[recv, send] : subs_)
    {
        if (ProjectionSlot *p = find_proj(recv))
            p->spike_senders.insert(send);
        else if (PopulationSlot *q = find_pop(recv))
            q->impact_senders.insert(send);
        else
            throw Error(KNP_GB300_E_INVALID, "subscription receiver is neither a population nor a projection");
    }
    for (auto &q : pops_)
        for (const Uid &s : q->impact_senders)
            if (!find_proj(s)) q->has_external_impacts = true;
}

void Backend::build_population(PopulationSlot &p)
{
    const uint32_t n = p.n, np = p.n_pad;
    // Incoming projections decide ring length, accumulator mode and the live input channels.
    uint32_t slots = 1;
    bool dyadic = true, stdp_in = false, g_in = false, d_in = false, forcing_exc = false, blk_in = false;
    for (auto &pr : projs_)
    {
        if (!(pr->post_uid == p.uid)) continue;
        slots = std::max(slots, pr->max_delay);
        dyadic = dyadic && pr->dyadic;
        stdp_in = stdp_in || pr->kind == KNP_SYNAPSE_ADDITIVE_STDP_DELTA || pr->kind == KNP_SYNAPSE_RESOURCE_STDP_DELTA;
        const bool has_type = !pr->type.empty();
        auto any_type = [&](uint8_t t)
        { return has_type ? std::find(pr->type.begin(), pr->type.end(), t) != pr->type.end() : t == 0; };
        g_in = g_in || any_type(KNP_OUT_INHIBITORY_CONDUCTANCE);
        d_in = d_in || any_type(KNP_OUT_DOPAMINE);
        blk_in = blk_in || any_type(KNP_OUT_BLOCKING);
        if (pr->kind == KNP_SYNAPSE_DELTA && any_type(KNP_OUT_EXCITATORY)) forcing_exc = true;
    }
    if (p.has_external_impacts) g_in = d_in = forcing_exc = true;
    bool fixed = false;
    if (p.kind != KNP_NEURON_LIF)
    {
        if (p.acc_request == KNP_GB300_ACC_FIXED64)
            fixed = true;
        else if (p.acc_request == KNP_GB300_ACC_AUTO)
            fixed = !dyadic || stdp_in;
    }

    RingView &rg = p.ring;
    rg.n = n;
    rg.pitch = np;
    rg.slots = slots;
    rg.fixed = fixed ? 1 : 0;
    const size_t cells = static_cast<size_t>(slots) * np;
    if (fixed)
    {
        rg.v64 = arena_.make<long long>(cells);
        rg.v64lo = arena_.make<long long>(cells);
    }
    else
        rg.v32 = arena_.make<float>(cells);
    const bool res = p.kind == KNP_NEURON_RESOURCE_STDP_BLIFAT || p.kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF;
    if (p.is_altai())
    {
        if (d_in) rg.dopa = arena_.make<float>(cells);
        if (blk_in || p.has_external_impacts)
        {
            // Every BLOCKING impact of a step, kept as an ordered event.
            rg.bev_cap = 2048;
            const size_t ev = static_cast<size_t>(slots) * rg.bev_cap;
            rg.bev_key = arena_.make<unsigned long long>(ev, false);
            rg.bev_val = arena_.make<float>(ev, false);
            rg.bev_tgt = arena_.make<uint32_t>(ev, false);
            rg.bev_count = arena_.make<uint32_t>(slots);
        }
        if (fixed) rg.nf = arena_.make<uint32_t>(cells / 4);
        if (res && forcing_exc)
        {
            rg.words = (np + 31) / 32;
            rg.forced = arena_.make<uint32_t>(static_cast<size_t>(slots) * rg.words);
        }
    }
    else if (p.kind != KNP_NEURON_LIF)
    {
        if (g_in) rg.g = arena_.make<float>(cells);
        if (d_in) rg.dopa = arena_.make<float>(cells);
        if (blk_in || p.has_external_impacts)
        {
            // BLOCKING keys per (slot, neuron); the weight table by projection load order is filled once
            // every projection's CSR exists (init).
            rg.blk = arena_.make<unsigned long long>(cells);
            rg.blk_w = arena_.make<const float *>(std::max<size_t>(projs_.size(), 1));
            if (p.has_external_impacts) rg.blk_ext = arena_.make<long long>(np);
        }
        if (fixed && res)
            for (auto &pr : projs_)
                if (pr->kind == KNP_SYNAPSE_RESOURCE_STDP_DELTA && pr->post_uid == p.uid && !rg.nf)
                    rg.nf = arena_.make<uint32_t>(cells / 4);
        if (res && forcing_exc)
        {
            rg.words = (np + 31) / 32;
            rg.forced = arena_.make<uint32_t>(static_cast<size_t>(slots) * rg.words);
        }
    }

    // Spike list, count, recording log.
    uint32_t *spikes = arena_.make<uint32_t>(np);
    uint32_t *count = counters_ + p.counter_index;
    if (p.record)
    {
        alloc_recording(p);
        p.record_from = 0;
    }

    if (p.is_altai())
    {
        AltaiDev &d = p.adev;
        const auto &nn = p.init_altai;
        d.n = n;
        d.n_pad = np;
        d.flags = (res ? kResource : 0u) | (rg.dopa ? kLiveDopa : 0u);
        auto upload = [&](auto get, auto *dst)
        {
            using V = std::remove_pointer_t<decltype(dst)>;
            std::vector<V> a(np, V{});
            for (uint32_t i = 0; i < n; ++i) a[i] = get(i);
            V *dp = arena_.make<V>(np);
            KNP_CUDA(cudaMemcpy(dp, a.data(), np * sizeof(V), cudaMemcpyHostToDevice));
            return dp;
        };
        auto param_u = [&](auto get) -> ParamU
        {
            ParamU r{nullptr, n ? static_cast<uint32_t>(get(0)) : 0u};
            bool uni = true;
            for (uint32_t i = 1; i < n && uni; ++i) uni = static_cast<uint32_t>(get(i)) == r.u;
            if (!uni) r.a = upload([&](uint32_t i) { return static_cast<uint32_t>(get(i)); }, static_cast<uint32_t *>(nullptr));
            return r;
        };
        d.V = upload([&](uint32_t i) { return nn[i].potential; }, static_cast<float *>(nullptr));
        d.V_pre = upload([&](uint32_t i) { return nn[i].pre_impact_potential; }, static_cast<float *>(nullptr));
        d.activity = upload([&](uint32_t i) { return static_cast<long long>(nn[i].activity_time); },
                            static_cast<long long *>(nullptr));
        d.add_thr = upload([&](uint32_t i) { return nn[i].additional_threshold; }, static_cast<double *>(nullptr));
        d.dopa = (rg.dopa || res)
                     ? upload([&](uint32_t i) { return static_cast<float>(nn[i].dopamine_value); }, static_cast<float *>(nullptr))
                     : nullptr;
        d.cfg = param_u(
            [&](uint32_t i)
            {
                const knp_altai_neuron &x = nn[i];
                return (x.is_diff ? kAltaiDiff : 0u) | (x.is_reset ? kAltaiReset : 0u) | (x.leak_rev ? kAltaiLeakRev : 0u) |
                       (x.saturate ? kAltaiSaturate : 0u) | (x.do_not_save ? kAltaiNoSave : 0u);
            });
        d.thr = param_u([&](uint32_t i) { return nn[i].activation_threshold; });
        d.neg_thr = param_u([&](uint32_t i) { return nn[i].negative_activation_threshold; });
        d.reset = param_u([&](uint32_t i) { return nn[i].potential_reset_value; });
        d.leak = param_u([&](uint32_t i) { return static_cast<uint32_t>(static_cast<int32_t>(nn[i].potential_leak)); });
        if (res)
        {
            ResourceDev &r = d.res;
            const auto &rr = p.init_res;
            using R = knp_resource_stdp_state;
            auto up64 = [&](auto get)
            { return upload([&](uint32_t i) { return static_cast<unsigned long long>(get(rr[i])); },
                            static_cast<unsigned long long *>(nullptr)); };
            auto rpf = [&](auto get) -> ParamF
            {
                ParamF x{nullptr, n ? get(rr[0]) : 0.f};
                bool uni = true;
                for (uint32_t i = 1; i < n && uni; ++i) uni = get(rr[i]) == x.u;
                if (!uni) x.a = upload([&](uint32_t i) { return get(rr[i]); }, static_cast<float *>(nullptr));
                return x;
            };
            auto rpu = [&](auto get) -> ParamU { return param_u([&](uint32_t i) { return get(rr[i]); }); };
            r.isi_status = reinterpret_cast<int32_t *>(
                upload([&](uint32_t i) { return static_cast<uint32_t>(rr[i].isi_status); }, static_cast<uint32_t *>(nullptr)));
            r.last_step = up64([](const R &x) { return x.last_step; });
            r.last_spike_step = up64([](const R &x) { return x.last_spike_step; });
            r.first_isi_spike = up64([](const R &x) { return x.first_isi_spike; });
            r.stability = upload([&](uint32_t i) { return rr[i].stability; }, static_cast<float *>(nullptr));
            r.free_resource = upload([&](uint32_t i) { return rr[i].free_synaptic_resource; }, static_cast<float *>(nullptr));
            r.is_forced = upload([&](uint32_t i) { return static_cast<uint8_t>(rr[i].is_being_forced ? 1 : 0); },
                                 static_cast<uint8_t *>(nullptr));
            r.add_thr_coef = rpf([](const R &x) { return x.synapse_sum_threshold_coefficient; });
            r.resource_threshold = rpf([](const R &x) { return x.synaptic_resource_threshold; });
            r.stability_change_param = rpf([](const R &x) { return x.stability_change_parameter; });
            r.stability_change_at_isi = rpf([](const R &x) { return x.stability_change_at_isi; });
            r.d_h = rpf([](const R &x) { return x.d_h; });
            r.isi_max = rpu([](const R &x) { return x.isi_max; });
            r.dopamine_time = rpu([](const R &x) { return x.dopamine_plasticity_time; });
            r.drain = rpu([](const R &x) { return x.resource_drain_coefficient; });
            // Training kernel's work list and FP64 additional threshold (shared with the neuron state);
            // the synapse arrays follow in build_resource_synapses.
            d.syn.add_thr = d.add_thr;
            d.syn.work = arena_.make<uint32_t>(np);
            d.syn.work_count = counters_ + p.work_counter_index;
        }
        d.spikes = spikes;
        d.spike_count = count;
        d.rec_bits = p.record ? p.rec_bits : nullptr;
        d.rec_words = p.rec_words;
        d.rec_slots = p.rec_slots;
        d.ring = rg;
        return;
    }

    if (p.kind == KNP_NEURON_LIF)
    {
        LifDev &d = p.ldev;
        d.n = n;
        d.n_pad = np;
        d.V = arena_.make<float>(np);
        d.refract = arena_.make<uint32_t>(np);
        std::vector<float> V(np, 0.f);
        std::vector<uint32_t> rc(np, 0);
        for (uint32_t i = 0; i < n; ++i)
        {
            V[i] = p.init_lif[i].potential;
            rc[i] = p.init_lif[i].refract_counter;
        }
        KNP_CUDA(cudaMemcpy(d.V, V.data(), np * 4, cudaMemcpyHostToDevice));
        KNP_CUDA(cudaMemcpy(d.refract, rc.data(), np * 4, cudaMemcpyHostToDevice));
        auto pf = [&](auto get) -> ParamF
        {
            ParamF r{nullptr, n ? get(p.init_lif[0]) : 0.f};
            bool uni = true;
            for (uint32_t i = 1; i < n && uni; ++i) uni = get(p.init_lif[i]) == r.u;
            if (!uni)
            {
                std::vector<float> a(np, 0.f);
                for (uint32_t i = 0; i < n; ++i) a[i] = get(p.init_lif[i]);
                float *dp = arena_.make<float>(np);
                KNP_CUDA(cudaMemcpy(dp, a.data(), np * 4, cudaMemcpyHostToDevice));
                r.a = dp;
            }
            return r;
        };
        d.leak = pf([](const knp_lif_neuron &x) { return x.leak_coefficient; });
        d.thr = pf([](const knp_lif_neuron &x) { return x.activation_threshold; });
        d.v_reset = pf([](const knp_lif_neuron &x) { return x.potential_reset_value; });
        {
            ParamU r{nullptr, n ? p.init_lif[0].refract_period : 0u};
            bool uni = true;
            for (uint32_t i = 1; i < n && uni; ++i) uni = p.init_lif[i].refract_period == r.u;
            if (!uni)
            {
                std::vector<uint32_t> a(np, 0);
                for (uint32_t i = 0; i < n; ++i) a[i] = p.init_lif[i].refract_period;
                uint32_t *dp = arena_.make<uint32_t>(np);
                KNP_CUDA(cudaMemcpy(dp, a.data(), np * 4, cudaMemcpyHostToDevice));
                r.a = dp;
            }
            d.refract_period = r;
        }
        d.spikes = spikes;
        d.spike_count = count;
        d.rec_bits = p.record ? p.rec_bits : nullptr;
        d.rec_words = p.rec_words;
        d.rec_slots = p.rec_slots;
        d.ring = rg;
        return;
    }

    const auto &nn = p.init_blifat;
    BlifatDev &d = p.bdev;
    d.n = n;
    d.n_pad = np;
    auto any = [&](auto pred)
    {
        for (uint32_t i = 0; i < n; ++i)
            if (pred(nn[i])) return true;
        return false;
    };
    uint32_t f = 0;
    if (any([](const knp_blifat_neuron &x) { return x.potential_decay != 0.0; })) f |= kLiveVRead;
    if (any([](const knp_blifat_neuron &x)
            { return x.dynamic_threshold != 0.0 || x.threshold_decay != 0.0 || x.threshold_increment != 0.0; }))
        f |= kLiveThrDyn;
    if (any([](const knp_blifat_neuron &x)
            {
                return x.postsynaptic_trace != 0.0 || x.postsynaptic_trace_decay != 0.0 ||
                       x.postsynaptic_trace_increment != 0.0;
            }))
        f |= kLiveTrace;
    if (g_in || any([](const knp_blifat_neuron &x)
                    { return x.inhibitory_conductance != 0.0 || x.inhibitory_conductance_decay != 0.0; }))
        f |= kLiveG;
    if (any([](const knp_blifat_neuron &x) { return x.bursting_period != 0 || x.bursting_phase != 0; })) f |= kLiveBurst;
    if (any([](const knp_blifat_neuron &x) { return x.total_blocking_period != std::numeric_limits<int64_t>::max(); }))
        f |= kLiveBlock;
    if (any([](const knp_blifat_neuron &x)
            {
                return x.absolute_refractory_period != 0 ||
                       x.n_time_steps_since_last_firing != std::numeric_limits<uint64_t>::max();
            }))
        f |= kLiveRefract;
    if (d_in) f |= kLiveDopa;
    if (rg.blk) f |= kLiveBlock;
    if (f & (kLiveBlock | kLiveVRead | kLiveBurst)) f |= kLiveVPre;
    bool res_syn = false;
    if (res)
        for (auto &pr : projs_)
            if (pr->kind == KNP_SYNAPSE_RESOURCE_STDP_DELTA && pr->post_uid == p.uid) res_syn = true;
    if (res)
    {
        f |= kResource | kLiveAddThr;
        if (res_syn) f |= kResSyn;
        for (uint32_t i = 0; i < n; ++i)
            if (!(std::fabs(p.init_res[i].free_synaptic_resource) < p.init_res[i].synaptic_resource_threshold))
                f |= kLiveRenorm;
    }
    if (any([](const knp_blifat_neuron &x) { return x.additional_threshold != 0.0; })) f |= kLiveAddThr;
    d.flags = f;

    auto upload_f = [&](auto get) -> float *
    {
        std::vector<float> a(np, 0.f);
        for (uint32_t i = 0; i < n; ++i) a[i] = get(i);
        float *dp = arena_.make<float>(np);
        KNP_CUDA(cudaMemcpy(dp, a.data(), np * sizeof(float), cudaMemcpyHostToDevice));
        return dp;
    };
    auto upload_u = [&](auto get) -> uint32_t *
    {
        std::vector<uint32_t> a(np, 0);
        for (uint32_t i = 0; i < n; ++i) a[i] = get(i);
        uint32_t *dp = arena_.make<uint32_t>(np);
        KNP_CUDA(cudaMemcpy(dp, a.data(), np * sizeof(uint32_t), cudaMemcpyHostToDevice));
        return dp;
    };
    auto param_f = [&](auto get) -> ParamF
    {
        ParamF r{nullptr, n ? to_f(get(nn[0])) : 0.f};
        bool uni = true;
        for (uint32_t i = 1; i < n && uni; ++i) uni = to_f(get(nn[i])) == r.u;
        if (!uni) r.a = upload_f([&](uint32_t i) { return to_f(get(nn[i])); });
        return r;
    };
    auto param_u = [&](auto get) -> ParamU
    {
        ParamU r{nullptr, n ? static_cast<uint32_t>(get(nn[0])) : 0u};
        bool uni = true;
        for (uint32_t i = 1; i < n && uni; ++i) uni = static_cast<uint32_t>(get(nn[i])) == r.u;
        if (!uni) r.a = upload_u([&](uint32_t i) { return static_cast<uint32_t>(get(nn[i])); });
        return r;
    };
    using N = knp_blifat_neuron;
    d.thr = param_f([](const N &x) { return x.activation_threshold; });
    d.thr_decay = param_f([](const N &x) { return x.threshold_decay; });
    d.thr_inc = param_f([](const N &x) { return x.threshold_increment; });
    d.trace_decay = param_f([](const N &x) { return x.postsynaptic_trace_decay; });
    d.trace_inc = param_f([](const N &x) { return x.postsynaptic_trace_increment; });
    d.g_decay = param_f([](const N &x) { return x.inhibitory_conductance_decay; });
    d.v_decay = param_f([](const N &x) { return x.potential_decay; });
    d.reflexive = param_f([](const N &x) { return x.reflexive_weight; });
    d.e_inh = param_f([](const N &x) { return x.reversal_inhibitory_potential; });
    d.v_reset = param_f([](const N &x) { return x.potential_reset_value; });
    d.v_min = param_f([](const N &x) { return x.min_potential; });
    d.t_ref = param_u([](const N &x) { return x.absolute_refractory_period; });
    d.burst_period = param_u([](const N &x) { return x.bursting_period; });

    d.V = upload_f([&](uint32_t i) { return to_f(nn[i].potential); });
    d.V_pre = (f & kLiveVPre) ? upload_f([&](uint32_t i) { return to_f(nn[i].pre_impact_potential); }) : nullptr;
    d.thr_dyn = (f & kLiveThrDyn) ? upload_f([&](uint32_t i) { return to_f(nn[i].dynamic_threshold); }) : nullptr;
    d.trace = (f & kLiveTrace) ? upload_f([&](uint32_t i) { return to_f(nn[i].postsynaptic_trace); }) : nullptr;
    d.g = (f & kLiveG) ? upload_f([&](uint32_t i) { return to_f(nn[i].inhibitory_conductance); }) : nullptr;
    d.dopa = ((f & kLiveDopa) || res) ? upload_f([&](uint32_t i) { return to_f(nn[i].dopamine_value); }) : nullptr;
    d.add_thr = (f & kLiveAddThr) ? upload_f([&](uint32_t i) { return to_f(nn[i].additional_threshold); }) : nullptr;
    d.n_since = upload_u(
        [&](uint32_t i) -> uint32_t
        {
            if (!(f & kLiveRefract)) return 0u;  // step of the last spike (lazy tracking)
            const uint64_t v = nn[i].n_time_steps_since_last_firing;
            if (v == std::numeric_limits<uint64_t>::max()) return 0xFFFFFFFFu;
            return v >= 0xFFFFFFFEull ? 0xFFFFFFFEu : static_cast<uint32_t>(v);
        });
    d.burst_phase = (f & kLiveBurst) ? upload_u([&](uint32_t i) { return nn[i].bursting_phase; }) : nullptr;
    if (f & kLiveBlock)
    {
        std::vector<long long> a(np, 0);
        for (uint32_t i = 0; i < n; ++i) a[i] = nn[i].total_blocking_period;
        d.blocking = arena_.make<long long>(np);
        KNP_CUDA(cudaMemcpy(d.blocking, a.data(), np * 8, cudaMemcpyHostToDevice));
    }
    if (res)
    {
        ResourceDev &r = d.res;
        const auto &rr = p.init_res;
        auto up64 = [&](auto get)
        {
            std::vector<unsigned long long> a(np, 0);
            for (uint32_t i = 0; i < n; ++i) a[i] = get(rr[i]);
            auto *dp = arena_.make<unsigned long long>(np);
            KNP_CUDA(cudaMemcpy(dp, a.data(), np * 8, cudaMemcpyHostToDevice));
            return dp;
        };
        using R = knp_resource_stdp_state;
        r.isi_status = reinterpret_cast<int32_t *>(upload_u([&](uint32_t i) { return static_cast<uint32_t>(rr[i].isi_status); }));
        r.last_step = up64([](const R &x) { return x.last_step; });
        r.last_spike_step = up64([](const R &x) { return x.last_spike_step; });
        r.first_isi_spike = up64([](const R &x) { return x.first_isi_spike; });
        r.stability = upload_f([&](uint32_t i) { return rr[i].stability; });
        r.free_resource = upload_f([&](uint32_t i) { return rr[i].free_synaptic_resource; });
        {
            std::vector<uint8_t> a(np, 0);
            for (uint32_t i = 0; i < n; ++i) a[i] = rr[i].is_being_forced ? 1 : 0;
            r.is_forced = arena_.make<uint8_t>(np);
            KNP_CUDA(cudaMemcpy(r.is_forced, a.data(), np, cudaMemcpyHostToDevice));
        }
        auto rpf = [&](auto get) -> ParamF
        {
            ParamF x{nullptr, n ? get(rr[0]) : 0.f};
            bool uni = true;
            for (uint32_t i = 1; i < n && uni; ++i) uni = get(rr[i]) == x.u;
            if (!uni) x.a = upload_f([&](uint32_t i) { return get(rr[i]); });
            return x;
        };
        r.add_thr_coef = rpf([](const R &x) { return x.synapse_sum_threshold_coefficient; });
        r.resource_threshold = rpf([](const R &x) { return x.synaptic_resource_threshold; });
        r.stability_change_param = rpf([](const R &x) { return x.stability_change_parameter; });
        r.stability_change_at_isi = rpf([](const R &x) { return x.stability_change_at_isi; });
        r.d_h = rpf([](const R &x) { return x.d_h; });
        auto rpu = [&](auto get) -> ParamU
        {
            ParamU x{nullptr, n ? get(rr[0]) : 0u};
            bool uni = true;
            for (uint32_t i = 1; i < n && uni; ++i) uni = get(rr[i]) == x.u;
            if (!uni) x.a = upload_u([&](uint32_t i) { return get(rr[i]); });
            return x;
        };
        r.isi_max = rpu([](const R &x) { return x.isi_max; });
        r.dopamine_time = rpu([](const R &x) { return x.dopamine_plasticity_time; });
        r.drain = rpu([](const R &x) { return x.resource_drain_coefficient; });
        if (f & kResSyn)
        {
            // FP64 additional threshold and the training kernel's work list; the synapse arrays
            // follow once every projection's CSR exists (build_resource_synapses).
            std::vector<double> a(np, 0.0);
            for (uint32_t i = 0; i < n; ++i) a[i] = nn[i].additional_threshold;
            d.syn.add_thr = arena_.make<double>(np);
            KNP_CUDA(cudaMemcpy(d.syn.add_thr, a.data(), np * 8, cudaMemcpyHostToDevice));
            d.syn.work = arena_.make<uint32_t>(np);
            d.syn.work_count = counters_ + p.work_counter_index;
        }
    }
    d.spikes = spikes;
    d.spike_count = count;
    d.rec_bits = p.record ? p.rec_bits : nullptr;
    d.rec_words = p.rec_words;
    d.rec_slots = p.rec_slots;
    d.ring = rg;
}

void Backend::build_projection(ProjectionSlot &p)
{
    PopulationSlot *post = find_pop(p.post_uid);
    const uint64_t S = p.n_syn;
    // Rows: presynaptic indexes 0..max(pre).
    uint32_t *d_key = nullptr;
    uint32_t *d_post = nullptr, *d_delay = nullptr;
    float *d_w = nullptr;
    uint8_t *d_type = nullptr;
    unsigned long long *cand = nullptr;  // FixedProbability: the kept pairs, until the gather
    if (p.generated)
    {
        p.n_rows = p.gen.n_pre;
        if (p.gen.kind == KNP_GEN_FIXED_PROBABILITY)
        {
            cand = arena_.make<unsigned long long>(std::max<uint64_t>(S, 1), false);
            uint64_t kept = 0;
            KNP_CUDA(gen_candidates(static_cast<uint64_t>(p.gen.n_pre) * p.gen.n_post, p.gen.prob_threshold,
                                    stream_key(p.gen.seed, p.gen.stream + 5), cand, &kept, stream_));
            if (kept != S) throw Error(KNP_GB300_E_CUDA, "generated pair count changed");
        }
        d_key = arena_.make<uint32_t>(S, false);
        launch_gen_keys(gen_spec(p, cand), S, d_key, stream_);
    }
    else
    {
        uint32_t max_pre = 0;
        for (uint32_t v : p.pre) max_pre = std::max(max_pre, v + 1);
        p.n_rows = max_pre;
        d_key = arena_.make<uint32_t>(S, false);
        d_post = arena_.make<uint32_t>(S, false);
        d_delay = arena_.make<uint32_t>(S, false);
        d_w = arena_.make<float>(S, false);
        KNP_CUDA(cudaMemcpyAsync(d_key, p.pre.data(), S * 4, cudaMemcpyHostToDevice, stream_));
        KNP_CUDA(cudaMemcpyAsync(d_post, p.post.data(), S * 4, cudaMemcpyHostToDevice, stream_));
        KNP_CUDA(cudaMemcpyAsync(d_delay, p.delay.data(), S * 4, cudaMemcpyHostToDevice, stream_));
        KNP_CUDA(cudaMemcpyAsync(d_w, p.weight.data(), S * 4, cudaMemcpyHostToDevice, stream_));
        if (p.type.size() > 1)
        {
            d_type = arena_.make<uint8_t>(S, false);
            KNP_CUDA(cudaMemcpyAsync(d_type, p.type.data(), S, cudaMemcpyHostToDevice, stream_));
        }
    }
    p.row_ptr = arena_.make<long long>(static_cast<size_t>(p.n_rows) + 1);
    uint32_t *perm = arena_.make<uint32_t>(S, false);
    size_t temp_need = 0;
    KNP_CUDA(build_csr(S, p.n_rows, d_key, perm, p.row_ptr, nullptr, 0, &temp_need, stream_));
    void *temp = arena_.alloc(temp_need, false);
    KNP_CUDA(build_csr(S, p.n_rows, d_key, perm, p.row_ptr, temp, temp_need, &temp_need, stream_));
    p.col = arena_.make<int32_t>(S, false);
    p.w = arena_.make<float>(S, false);
    p.delay_d = arena_.make<uint8_t>(S, false);
    if (p.generated)
    {
        launch_gen_gather(gen_spec(p, cand), S, perm, p.col, p.w, p.delay_d, stream_);
    }
    else
    {
        if (d_type) p.type_d = arena_.make<uint8_t>(S, false);
        launch_gather_synapses(S, perm, d_post, d_w, d_delay, d_type, p.col, p.w, p.delay_d, p.type_d, stream_);
    }
    KNP_CUDA(cudaGetLastError());
    KNP_CUDA(cudaStreamSynchronize(stream_));
    arena_.release(temp);
    arena_.release(d_key);
    if (cand) arena_.release(cand);
    if (d_post) arena_.release(d_post);
    if (d_delay) arena_.release(d_delay);
    if (d_w) arena_.release(d_w);
    if (d_type) arena_.release(d_type);
    if (p.generated)
        arena_.release(perm);  // weights of a generated projection are regenerated, not permuted
    else
        p.perm = perm;

    ProjectionDev &d = p.dev;
    d.row_ptr = p.row_ptr;
    d.n_rows = p.n_rows;
    d.col = p.col;
    d.w = p.w;
    d.delay = p.delay_d;
    d.type = p.type_d;
    d.uniform_type = p.type.size() == 1 ? p.type[0] : 0;
    d.forcing = p.kind == KNP_SYNAPSE_DELTA ? 1 : 0;  // is_forced(): stdp_dispatcher.h:54-58, additive_stdp.h:199-203
    for (size_t k = 0; k < projs_.size(); ++k)
        if (projs_[k].get() == &p) d.order = static_cast<uint32_t>(k);
    if (post) d.ring = post->ring;
    // Spike sources: every subscribed sender, except STDP-only populations whose messages the
    // projection empties before propagating them (additive_stdp.h:162-166).
    d.n_src = 0;
    for (const Uid &s : p.spike_senders)
    {
        auto it = p.stdp_pops.find(s);
        if (it != p.stdp_pops.end() && it->second == KNP_STDP_ONLY) continue;
        SpikeSource src{};
        if (PopulationSlot *q = find_pop(s))
        {
            src.idx = q->spike_list();
            src.count = counters_ + q->counter_index;
            src.n = q->n;
        }
        else
        {
            src.channel = channel(s).dev;
        }
        if (d.n_src >= kMaxSources) throw Error(KNP_GB300_E_INVALID, "too many spike sources for one projection");
        d.src[d.n_src++] = src;
    }
    if (!post) d.n_src = 0;  // no target population on this backend: impacts go nowhere
}

void Backend::build_stdp(ProjectionSlot &p)
{
    if (p.kind != KNP_SYNAPSE_ADDITIVE_STDP_DELTA || p.n_syn == 0) return;
    const float tp = p.tau_plus[0], tm = p.tau_minus[0];
    const float period_f = tp + tm;
    uint32_t period = 0;
    while (static_cast<float>(period) < period_f) ++period;  // smallest n with n >= tau+ + tau- (float compare)
    if (period == 0) period = 0;
    uint32_t n_cols = 0;
    for (uint32_t v : p.post) n_cols = std::max(n_cols, v + 1);
    StdpDev &s = p.stdp;
    s.n_cols = n_cols;
    s.period = period;
    s.pre_hist = arena_.make<uint32_t>(static_cast<size_t>(n_cols) * std::max<uint32_t>(period, 1));
    s.post_hist = arena_.make<uint32_t>(static_cast<size_t>(n_cols) * std::max<uint32_t>(period, 1));
    s.pre_cnt = arena_.make<uint32_t>(n_cols);
    s.post_cnt = arena_.make<uint32_t>(n_cols);
    s.touched = arena_.make<uint32_t>(n_cols);
    s.touched_stamp = arena_.make<unsigned long long>(n_cols);
    s.w = p.w;
    // Column index: CSR positions grouped by postsynaptic neuron (stable).
    std::vector<uint32_t> perm(p.n_syn);
    KNP_CUDA(cudaMemcpy(perm.data(), p.perm, p.n_syn * 4, cudaMemcpyDeviceToHost));
    std::vector<long long> col_ptr(static_cast<size_t>(n_cols) + 1, 0);
    for (uint64_t e = 0; e < p.n_syn; ++e) ++col_ptr[p.post[perm[e]] + 1];
    for (uint32_t c = 0; c < n_cols; ++c) col_ptr[c + 1] += col_ptr[c];
    std::vector<uint64_t> col_pos(p.n_syn);
    std::vector<long long> fill(col_ptr.begin(), col_ptr.end() - 1);
    for (uint64_t e = 0; e < p.n_syn; ++e) col_pos[fill[p.post[perm[e]]]++] = e;
    auto *cp = arena_.make<long long>(col_ptr.size());
    auto *cpos = arena_.make<uint64_t>(col_pos.size());
    KNP_CUDA(cudaMemcpy(cp, col_ptr.data(), col_ptr.size() * 8, cudaMemcpyHostToDevice));
    KNP_CUDA(cudaMemcpy(cpos, col_pos.data(), col_pos.size() * 8, cudaMemcpyHostToDevice));
    s.col_ptr = cp;
    s.col_pos = cpos;
    std::vector<float> table = stdp_table(tp, tm);
    auto *tb = arena_.make<float>(table.size());
    KNP_CUDA(cudaMemcpy(tb, table.data(), table.size() * 4, cudaMemcpyHostToDevice));
    s.table = tb;
    s.table_len = static_cast<uint32_t>(table.size());
    // Append sources: STDP populations in population load order (the order their SpikeMessages
    // arrive in one step).
    for (auto &q : pops_)
    {
        auto it = p.stdp_pops.find(q->uid);
        if (it == p.stdp_pops.end()) continue;
        SpikeSource src{};
        src.idx = q->spike_list();
        src.count = counters_ + q->counter_index;
        p.stdp_sources.emplace_back(src, it->second == KNP_STDP_AND_SPIKE ? 1 : 0);
    }
}

// The resource-STDP projections into population q, concatenated in load order: each projection's
// CSR weights, delays and last-spike steps become a slice of the population's arrays (its scatter
// reads and writes them there), its rule state is uploaded in CSR order, and the column index lists
// every neuron's synapses in get_all_connected_synapses order (training/stdp.h:55-72: projection
// order, then the synapse index within the projection).
void Backend::build_resource_synapses(PopulationSlot &q)
{
    for (auto &p : projs_)
        if (p->kind == KNP_SYNAPSE_RESOURCE_STDP_DELTA && p->post_uid == q.uid) q.res_projs.push_back(p.get());
    if (q.res_projs.empty())
    {
        if (q.kind != KNP_NEURON_RESOURCE_STDP_ALTAI_LIF) return;
        // A resource-STDP AltAI-LIF population always runs the training kernel: no synapses.
        ResSynDev y = q.adev.syn;
        y.col_ptr = arena_.make<long long>(static_cast<size_t>(q.n) + 1);
        q.adev.syn = y;
        return;
    }
    if (q.res_projs.size() > 255)
        throw Error(KNP_GB300_E_INVALID, "more than 255 resource-STDP projections into one population");
    uint64_t total = 0;
    for (ProjectionSlot *p : q.res_projs) total += p->n_syn;
    const size_t T = std::max<uint64_t>(total, 1);
    ResSynDev &y = q.res_syn;
    y.w = arena_.make<float>(T, false);
    y.resource = arena_.make<float>(T, false);
    float *w_min = arena_.make<float>(T, false), *w_max = arena_.make<float>(T, false), *d_u = arena_.make<float>(T, false);
    uint32_t *period = arena_.make<uint32_t>(T, false);
    y.last_spike = arena_.make<unsigned long long>(T, false);
    y.flags = arena_.make<uint8_t>(T, false);
    uint8_t *delay = arena_.make<uint8_t>(T, false);
    y.w_min = w_min;
    y.w_max = w_max;
    y.d_u = d_u;
    y.period = period;
    y.delay = delay;
    std::vector<long long> col_ptr(static_cast<size_t>(q.n) + 1, 0);
    std::vector<std::vector<uint32_t>> inv(q.res_projs.size());  // loaded index -> CSR position
    uint64_t off = 0;
    for (size_t k = 0; k < q.res_projs.size(); ++k)
    {
        ProjectionSlot &p = *q.res_projs[k];
        const uint64_t S = p.n_syn;
        p.res_pop = &q;
        p.res_offset = off;
        if (S)
        {
            std::vector<uint32_t> perm(S);
            KNP_CUDA(cudaMemcpy(perm.data(), p.perm, S * 4, cudaMemcpyDeviceToHost));
            inv[k].resize(S);
            for (uint64_t e = 0; e < S; ++e) inv[k][perm[e]] = static_cast<uint32_t>(e);
            std::vector<float> res(S), lo(S), hi(S), du(S);
            std::vector<uint32_t> per(S);
            std::vector<unsigned long long> ls(S);
            std::vector<uint8_t> fl(S);
            for (uint64_t e = 0; e < S; ++e)
            {
                const knp_resource_synapse &r = p.rule[perm[e]];
                res[e] = r.synaptic_resource;
                lo[e] = r.w_min;
                hi[e] = r.w_max;
                du[e] = r.d_u;
                per[e] = r.dopamine_plasticity_period;
                ls[e] = r.last_spike_step;
                fl[e] = static_cast<uint8_t>((r.had_hebbian_update ? 1u : 0u) | (r.has_contributed ? 2u : 0u));
            }
            KNP_CUDA(cudaMemcpy(y.resource + off, res.data(), S * 4, cudaMemcpyHostToDevice));
            KNP_CUDA(cudaMemcpy(w_min + off, lo.data(), S * 4, cudaMemcpyHostToDevice));
            KNP_CUDA(cudaMemcpy(w_max + off, hi.data(), S * 4, cudaMemcpyHostToDevice));
            KNP_CUDA(cudaMemcpy(d_u + off, du.data(), S * 4, cudaMemcpyHostToDevice));
            KNP_CUDA(cudaMemcpy(period + off, per.data(), S * 4, cudaMemcpyHostToDevice));
            KNP_CUDA(cudaMemcpy(y.last_spike + off, ls.data(), S * 8, cudaMemcpyHostToDevice));
            KNP_CUDA(cudaMemcpy(y.flags + off, fl.data(), S, cudaMemcpyHostToDevice));
            KNP_CUDA(cudaMemcpy(y.w + off, p.w, S * 4, cudaMemcpyDeviceToDevice));
            KNP_CUDA(cudaMemcpy(delay + off, p.delay_d, S, cudaMemcpyDeviceToDevice));
            for (uint64_t i = 0; i < S; ++i) ++col_ptr[p.post[i] + 1];
        }
        arena_.release(p.w);
        arena_.release(p.delay_d);
        p.w = y.w + off;
        p.delay_d = delay + off;
        p.dev.w = p.w;
        p.dev.delay = p.delay_d;
        p.dev.last_spike = y.last_spike + off;
        off += S;
    }
    for (uint32_t i = 0; i < q.n; ++i) col_ptr[i + 1] += col_ptr[i];
    std::vector<unsigned long long> col_pos(T, 0);
    std::vector<long long> fill(col_ptr.begin(), col_ptr.end() - 1);
    for (size_t k = 0; k < q.res_projs.size(); ++k)
    {
        const ProjectionSlot &p = *q.res_projs[k];
        for (uint64_t i = 0; i < p.n_syn; ++i)
            col_pos[fill[p.post[i]]++] = (static_cast<unsigned long long>(k) << kResSlotShift) | (p.res_offset + inv[k][i]);
    }
    auto *cp = arena_.make<long long>(col_ptr.size(), false);
    auto *cpos = arena_.make<unsigned long long>(T, false);
    KNP_CUDA(cudaMemcpy(cp, col_ptr.data(), col_ptr.size() * 8, cudaMemcpyHostToDevice));
    KNP_CUDA(cudaMemcpy(cpos, col_pos.data(), T * 8, cudaMemcpyHostToDevice));
    y.col_ptr = cp;
    y.col_pos = cpos;
    q.res_locked_host.assign(q.res_projs.size(), 0u);
    q.res_locked = arena_.make<uint32_t>(q.res_projs.size());
    y.locked = q.res_locked;
    if (q.bdev.flags & kResSyn)
    {
        y.add_thr = q.bdev.syn.add_thr;
        y.work = q.bdev.syn.work;
        y.work_count = q.bdev.syn.work_count;
        q.bdev.syn = y;
    }
    if (q.kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF)
    {
        y.add_thr = q.adev.syn.add_thr;
        y.work = q.adev.syn.work;
        y.work_count = q.adev.syn.work_count;
        q.adev.syn = y;
    }
}

cudaError_t set_gather_smem(size_t bytes);

int Backend::gather_grid(const ProjectionSlot &p) const
{
    return static_cast<int>(std::max<uint32_t>(1, std::min<uint32_t>(p.dev.pull.n_windows, sm_count_)));
}

// The gather form is built for large delta projections fed by one population into an FP32 ring,
// when the device has room for a second (4, 6 or 8 B / synapse) copy of the synapses and the build's
// temporaries.
void Backend::build_pull(ProjectionSlot &p)
{
    PopulationSlot *post = find_pop(p.post_uid);
    if (p.pull_fraction < 0 || p.kind != KNP_SYNAPSE_DELTA || !post || p.n_syn < (1u << 20)) return;
    if (step_mode_ == KNP_GB300_STEP_FUSED) return;  // the fused step kernel scatters every step
    if (p.dev.n_src != 1 || p.dev.src[0].channel) return;
    const RingView &rg = post->ring;
    if (rg.fixed || (rg.forced && p.dev.forcing)) return;
    if (p.dev.type || (p.dev.uniform_type != KNP_OUT_EXCITATORY && p.dev.uniform_type != KNP_OUT_INHIBITORY_CURRENT))
        return;
    if (static_cast<uint64_t>(p.max_delay) * post->n >= 0xFFFFFFFFull) return;
    PullDev g{};
    g.words = round_up((p.n_rows + 31) / 32, 4);
    g.max_delay = p.max_delay;
    g.hist_slots = p.max_delay + 1;
    g.n_windows = (post->n + kPullWindow - 1) / kPullWindow;
    const int grid = static_cast<int>(std::max<uint32_t>(1, std::min<uint32_t>(g.n_windows, sm_count_)));
    const size_t smem = gather_smem_bytes(g, grid);
    int smem_max = 0;
    KNP_CUDA(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_));
    if (smem > static_cast<size_t>(smem_max)) return;
    size_t free_b = 0, total_b = 0;
    KNP_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (free_b < p.n_syn * 36 + static_cast<size_t>(p.max_delay) * post->n * 16 + (1ull << 30)) return;
    const bool negate = p.dev.uniform_type == KNP_OUT_INHIBITORY_CURRENT;
    PullBuffers bufs;
    KNP_CUDA(build_pull_layout(p.n_syn, p.n_rows, post->n, p.row_ptr, p.col, p.w, p.delay_d, negate, g, bufs, stream_));
    for (int i = 0; i < PullBuffers::kCount; ++i)
        if (bufs.ptr[i]) arena_.adopt(bufs.ptr[i], bufs.bytes[i]);
    g.bitmap = arena_.make<uint32_t>(static_cast<size_t>(g.hist_slots) * g.words);
    g.pulled = arena_.make<uint32_t>(g.hist_slots);
    g.threshold = static_cast<uint32_t>(std::max(1.0, std::ceil(p.pull_fraction * p.n_rows)));
    // 32 copies of the weight dictionary (one per bank) when shared memory has room for them.
    if (g.wtab && smem + static_cast<size_t>(g.n_tab) * 32 * 4 + 2048 <= static_cast<size_t>(smem_max)) g.tab_rep = 1;
    KNP_CUDA(set_gather_smem(std::max<size_t>(gather_smem_bytes(g, grid), 48 * 1024)));
    p.dev.pull = g;
    p.pull = true;
}

void Backend::set_pull_threshold(const Uid &proj, double fraction)
{
    ProjectionSlot *p = find_proj(proj);
    if (!p) throw Error(KNP_GB300_E_INVALID, "unknown projection");
    if (initialized_)
    {
        if (!p->pull)
        {
            if (fraction >= 0) throw Error(KNP_GB300_E_STATE, "this projection has no gather form");
            return;
        }
        KNP_CUDA(cudaStreamSynchronize(stream_));
        p->pull_fraction = fraction;
        // A negative fraction disables pulling: no step reaches a threshold above every spike count.
        p->dev.pull.threshold =
            fraction < 0 ? 0xFFFFFFFFu : static_cast<uint32_t>(std::max(1.0, std::ceil(fraction * p->n_rows)));
        capture_graphs();
        return;
    }
    p->pull_fraction = fraction;
}

void Backend::init()
{
    require_not_init("init");
    KNP_CUDA(cudaSetDevice(device_));
    if (step_mode_ == KNP_GB300_STEP_FUSED)
    {
        std::string why;
        if (!small_net_eligible(why))
            throw Error(KNP_GB300_E_INVALID, "the fused step kernel does not take this network: " + why);
    }
    for (auto &p : projs_)
    {
        if (!p->post_uid.is_null() && !find_pop(p->post_uid))
            throw Error(KNP_GB300_E_INVALID, "projection targets a population that is not loaded");
        PopulationSlot *post = find_pop(p->post_uid);
        if (post && post->is_altai())
            for (uint8_t t : p->type)
                if (t == KNP_OUT_INHIBITORY_CONDUCTANCE)
                    throw Error(KNP_GB300_E_INVALID, "AltAI-LIF neurons take no inhibitory-conductance impacts");
        if (post && post->kind == KNP_NEURON_LIF)
            for (uint8_t t : p->type)
                if (t > KNP_OUT_INHIBITORY_CURRENT)
                    throw Error(KNP_GB300_E_INVALID, "LIF neurons accept only excitatory and inhibitory-current impacts");
        if (p->generated)
        {
            p->max_delay = p->gen.d_hi;
            const double kmax = std::max(std::abs(p->gen.k_lo), std::abs(p->gen.k_hi));
            p->dyadic = static_cast<double>(p->gen.in_degree) * kmax / 256.0 < 32768.0;
            if (post && p->gen.n_post > post->n)
                throw Error(KNP_GB300_E_INVALID, "postsynaptic index out of the target population");
            continue;
        }
        uint32_t md = 1;
        for (uint32_t d : p->delay) md = std::max(md, d);
        p->max_delay = md;
        bool dy = true;
        for (float w : p->weight) dy = dy && is_dyadic(w);
        if (dy && post)
        {
            std::vector<double> colsum(post->n, 0.0);
            for (uint64_t i = 0; i < p->n_syn; ++i)
                if (p->post[i] < post->n) colsum[p->post[i]] += std::fabs(p->weight[i]);
            for (double v : colsum) dy = dy && v < 32768.0;
        }
        p->dyadic = dy && p->kind != KNP_SYNAPSE_RESOURCE_STDP_DELTA;  // resource-STDP weights change
        if (post)
            for (uint32_t v : p->post)
                if (v >= post->n) throw Error(KNP_GB300_E_INVALID, "postsynaptic index out of the target population");
    }
    if (projs_.size() > 62)
        for (auto &p : projs_)
            for (uint8_t ty : p->type)
                if (ty == KNP_OUT_BLOCKING)
                    throw Error(KNP_GB300_E_INVALID, "BLOCKING synapses need a backend of at most 62 projections");
    wire();
    // Per-step counters: population spike counts, then STDP touched counts.
    n_spike_counters_ = static_cast<uint32_t>(pops_.size());
    n_counters_ = n_spike_counters_;
    for (auto &p : projs_)
        if (p->kind == KNP_SYNAPSE_ADDITIVE_STDP_DELTA && p->n_syn) ++n_counters_;
    // Work-list counts of the resource-STDP training, one per population that may need one.
    for (auto &q : pops_)
        if (q->kind == KNP_NEURON_RESOURCE_STDP_BLIFAT || q->kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF)
            q->work_counter_index = n_counters_++;
    counters_ = arena_.make<uint32_t>(std::max<uint32_t>(n_counters_, 1));
    for (uint32_t i = 0; i < pops_.size(); ++i) pops_[i]->counter_index = i;
    neurons_total_ = 0;
    for (auto &q : pops_)
    {
        build_population(*q);
        neurons_total_ += q->n;
    }
    for (auto &p : projs_)
    {
        build_projection(*p);
        if (p->kind == KNP_SYNAPSE_ADDITIVE_STDP_DELTA && p->n_syn) build_stdp(*p);
        build_pull(*p);
    }
    for (auto &q : pops_) build_resource_synapses(*q);
    upload_locks();
    uint32_t ci = n_spike_counters_;
    for (auto &p : projs_)
        if (p->kind == KNP_SYNAPSE_ADDITIVE_STDP_DELTA && p->n_syn) p->stdp.touched_count = counters_ + ci++;
    // BLOCKING weight tables: entry k is the CSR weight array of the projection loaded k-th.
    for (auto &q : pops_)
    {
        if (!q->ring.blk) continue;
        std::vector<const float *> tab(std::max<size_t>(projs_.size(), 1), nullptr);
        for (size_t k = 0; k < projs_.size(); ++k)
            if (projs_[k]->post_uid == q->uid) tab[k] = projs_[k]->w;
        KNP_CUDA(cudaMemcpy(const_cast<const float **>(q->ring.blk_w), tab.data(), tab.size() * sizeof(const float *),
                            cudaMemcpyHostToDevice));
    }
    // Host copies of the synapse arrays are no longer needed, except what readback and STDP use.
    for (auto &p : projs_)
    {
        std::vector<uint32_t>().swap(p->pre);
        std::vector<uint32_t>().swap(p->delay);
        std::vector<float>().swap(p->weight);
        if (p->kind != KNP_SYNAPSE_ADDITIVE_STDP_DELTA) std::vector<uint32_t>().swap(p->post);
        if (p->res_pop) std::vector<knp_resource_synapse>().swap(p->rule);
    }
    std::string why;
    fused_ = step_mode_ == KNP_GB300_STEP_FUSED || (step_mode_ == KNP_GB300_STEP_AUTO && small_net_eligible(why));
    grid_ = false;
    if (!fused_ && (step_mode_ == KNP_GB300_STEP_GRID || step_mode_ == KNP_GB300_STEP_AUTO))
    {
        std::string why_grid;
        grid_ = grid_net_eligible(why_grid);
        if (!grid_ && step_mode_ == KNP_GB300_STEP_GRID)
            throw Error(KNP_GB300_E_INVALID, "the grid step kernel does not take this network: " + why_grid);
        if (grid_) setup_ring_window();
    }
    initialized_ = true;
    capture_graphs();
}

void Backend::set_step_mode(int mode)
{
    require_not_init("set_step_mode");
    if (mode != KNP_GB300_STEP_AUTO && mode != KNP_GB300_STEP_PHASES && mode != KNP_GB300_STEP_FUSED &&
        mode != KNP_GB300_STEP_GRID)
        throw Error(KNP_GB300_E_INVALID, "unknown step mode");
    step_mode_ = mode;
}

// The fused kernel is one cluster of at most 8 CTAs: it pays off while a step is a few microseconds
// of work, and it has no gather form (in AUTO mode a projection with a gather layout keeps the per-phase kernels; the
// FUSED mode builds no gather layout).
bool Backend::small_net_eligible(std::string &why) const
{
    uint64_t neurons = 0, syn = 0;
    for (auto &q : pops_) neurons += q->n;
    for (auto &q : pops_)
        if (q->is_altai())
        {
            why = "AltAI-LIF populations run on the per-phase kernels";
            return false;
        }
    for (auto &p : projs_)
    {
        syn += p->n_syn;
        if (p->kind == KNP_SYNAPSE_RESOURCE_STDP_DELTA)
        {
            why = "resource-STDP projections are trained between the per-phase kernels";
            return false;
        }
        if (p->pull)
        {
            why = "a projection has a gather layout";
            return false;
        }
        if (p->stdp_pops.size() > static_cast<size_t>(kMaxSources))
        {
            why = "a projection has more than " + std::to_string(kMaxSources) + " STDP populations";
            return false;
        }
    }
    if (neurons > kSmallMaxNeurons)
    {
        why = "more than " + std::to_string(kSmallMaxNeurons) + " neurons";
        return false;
    }
    if (syn > kSmallMaxSynapses)
    {
        why = "more than " + std::to_string(kSmallMaxSynapses) + " synapses";
        return false;
    }
    return true;
}

// The grid kernel runs any network of the per-phase path whose STDP projections have at most
// kMaxSources STDP populations, with at most kMaxGridPull gather-form projections, when one
// 1024-thread CTA per SM fits with the gather form's shared memory and the device takes
// cooperative launches.
bool Backend::grid_net_eligible(std::string &why)
{
    int coop = 0;
    KNP_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device_));
    if (!coop)
    {
        why = "the device does not take cooperative launches";
        return false;
    }
    size_t smem = 0;
    uint32_t n_pull = 0;
    for (auto &q : pops_)
        if (q->is_altai())
        {
            why = "AltAI-LIF populations run on the per-phase kernels";
            return false;
        }
    for (auto &p : projs_)
    {
        if (p->kind == KNP_SYNAPSE_RESOURCE_STDP_DELTA)
        {
            why = "resource-STDP projections are trained between the per-phase kernels";
            return false;
        }
        if (p->stdp_pops.size() > static_cast<size_t>(kMaxSources))
        {
            why = "a projection has more than " + std::to_string(kMaxSources) + " STDP populations";
            return false;
        }
        if (p->pull && p->dev.n_src)
        {
            ++n_pull;
            smem = std::max(smem, grid_net_smem(p->dev.pull, sm_count_));
        }
    }
    if (n_pull > static_cast<uint32_t>(kMaxGridPull))
    {
        why = "more than " + std::to_string(kMaxGridPull) + " gather-form projections";
        return false;
    }
    const int ctas = grid_net_ctas(smem);
    if (ctas <= 0)
    {
        why = "one CTA per SM does not fit (shared memory " + std::to_string(smem) + " B)";
        return false;
    }
    grid_ctas_ = ctas;
    grid_smem_ = smem;
    return true;
}

// Keeps the largest FP32 input ring in L2 during the grid kernel's launches: the scatter's atomics
// land there, while the synapse arrays stream through with evict-first loads. Uses the device's
// set-aside for persisting accesses (a limit of this process's context).
void Backend::setup_ring_window()
{
    ring_window_ = cudaAccessPolicyWindow{};
    const RingView *best = nullptr;
    size_t best_bytes = 0;
    for (auto &q : pops_)
    {
        const RingView &rg = q->input_ring();
        const size_t bytes = rg.v32 ? static_cast<size_t>(rg.slots) * rg.pitch * 4 : 0;
        if (bytes > best_bytes)
        {
            best_bytes = bytes;
            best = &rg;
        }
    }
    if (!best || best_bytes < (size_t(4) << 20)) return;
    int max_persist = 0, max_window = 0;
    if (cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, device_) != cudaSuccess ||
        cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, device_) != cudaSuccess ||
        max_persist <= 0 || max_window <= 0)
    {
        cudaGetLastError();
        return;
    }
    const size_t window = std::min(best_bytes, static_cast<size_t>(max_window));
    const size_t set_aside = std::min(window, static_cast<size_t>(max_persist));
    if (cudaDeviceGetLimit(&persisting_before_, cudaLimitPersistingL2CacheSize) != cudaSuccess ||
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, std::max(set_aside, persisting_before_)) != cudaSuccess)
    {
        cudaGetLastError();
        return;
    }
    persisting_l2_ = true;
    ring_window_.base_ptr = best->v32;
    ring_window_.num_bytes = window;
    ring_window_.hitRatio = static_cast<float>(static_cast<double>(set_aside) / static_cast<double>(window));
    ring_window_.hitProp = cudaAccessPropertyPersisting;
    ring_window_.missProp = cudaAccessPropertyStreaming;
}

// Uploads the device descriptors of the fused kernel (again after a change of recording): set 0
// with the per-step counters and spike lists of the per-phase kernels, set 1 the same with a second
// counter array and a second spike list per population.
void Backend::build_small_net()
{
    small_cluster_ = small_net_cluster();
    if (!counters_alt_)
    {
        counters_alt_ = arena_.make<uint32_t>(std::max<uint32_t>(n_counters_, 1));
        for (auto &q : pops_)
        {
            const uint32_t *list = q->spike_list();
            spikes_alt_.emplace_back(list, arena_.make<uint32_t>(std::max<uint32_t>(q->n_pad, 4), false));
        }
    }
    for (int set = 0; set < 2; ++set)
    {
        uint32_t *base = set ? counters_alt_ : counters_;
        auto cnt = [&](const uint32_t *c) -> uint32_t * {
            if (c >= counters_ && c < counters_ + n_counters_) return base + (c - counters_);
            return const_cast<uint32_t *>(c);
        };
        auto list = [&](const uint32_t *l) -> uint32_t * {
            if (set && l)
                for (auto &[a, b] : spikes_alt_)
                    if (a == l) return b;
            return const_cast<uint32_t *>(l);
        };
        std::vector<SmallPop> pops;
        for (auto &q : pops_)
        {
            SmallPop sp{};
            sp.kind = q->kind == KNP_NEURON_LIF ? kSmallLif : kSmallBlifat;
            sp.blifat = q->bdev;
            sp.lif = q->ldev;
            sp.blifat.spike_count = cnt(sp.blifat.spike_count);
            sp.lif.spike_count = cnt(sp.lif.spike_count);
            sp.blifat.spikes = list(sp.blifat.spikes);
            sp.lif.spikes = list(sp.lif.spikes);
            pops.push_back(sp);
        }
        std::vector<ProjectionDev> projs;
        std::vector<SmallStdp> rules;
        small_pull_.clear();
        for (auto &p : projs_)
        {
            if (p->dev.n_src)
            {
                if (p->pull) small_pull_.push_back(static_cast<uint32_t>(projs.size()));
                ProjectionDev d = p->dev;
                for (int k = 0; k < d.n_src; ++k)
                {
                    d.src[k].count = cnt(d.src[k].count);
                    d.src[k].idx = list(d.src[k].idx);
                }
                projs.push_back(d);
            }
            if (p->kind != KNP_SYNAPSE_ADDITIVE_STDP_DELTA || p->n_syn == 0 || p->stdp_sources.empty()) continue;
            if (p->stdp_sources.size() > static_cast<size_t>(kMaxSources))
                throw Error(KNP_GB300_E_INVALID, "too many STDP populations for one projection");
            SmallStdp r{};
            r.d = p->stdp;
            r.d.touched_count = cnt(r.d.touched_count);
            for (auto &[src, both] : p->stdp_sources)
            {
                r.src[r.n_src] = src;
                r.src[r.n_src].count = cnt(src.count);
                r.src[r.n_src].idx = list(src.idx);
                r.both[r.n_src] = both;
                ++r.n_src;
            }
            rules.push_back(r);
        }
        if (!small_.pops[0])
        {
            small_.n_pops = static_cast<uint32_t>(pops.size());
            small_.n_projs = static_cast<uint32_t>(projs.size());
            small_.n_stdp = static_cast<uint32_t>(rules.size());
            SmallPop *dp = arena_.make<SmallPop>(2 * std::max<size_t>(pops.size(), 1));
            ProjectionDev *dj = arena_.make<ProjectionDev>(2 * std::max<size_t>(projs.size(), 1));
            SmallStdp *ds = arena_.make<SmallStdp>(2 * std::max<size_t>(rules.size(), 1));
            for (int k = 0; k < 2; ++k)
            {
                small_.pops[k] = dp + k * std::max<size_t>(pops.size(), 1);
                small_.projs[k] = dj + k * std::max<size_t>(projs.size(), 1);
                small_.stdp[k] = ds + k * std::max<size_t>(rules.size(), 1);
            }
        }
        small_.end[set] = StepEnd{base, n_counters_, n_spike_counters_};
        KNP_CUDA(cudaMemcpy(const_cast<SmallPop *>(small_.pops[set]), pops.data(), pops.size() * sizeof(SmallPop),
                            cudaMemcpyHostToDevice));
        KNP_CUDA(cudaMemcpy(const_cast<ProjectionDev *>(small_.projs[set]), projs.data(),
                            projs.size() * sizeof(ProjectionDev), cudaMemcpyHostToDevice));
        KNP_CUDA(cudaMemcpy(const_cast<SmallStdp *>(small_.stdp[set]), rules.data(), rules.size() * sizeof(SmallStdp),
                            cudaMemcpyHostToDevice));
    }
}

// ------------------------------------------------------------------------------------ stepping

// One population's step: its kernel, then (resource-STDP populations with resource-STDP synapses)
// the training that ends the population's step in the reference (populations_old.h:207-209).
void Backend::launch_population(const PopulationSlot &q)
{
    if (q.kind == KNP_NEURON_LIF)
    {
        launch_lif(q.ldev, ctl_, stream_);
        return;
    }
    if (q.is_altai())
    {
        if (q.adev.ring.bev_key) launch_altai_blocking(q.adev, ctl_, stream_);
        launch_altai(q.adev, ctl_, stream_);
        if (q.adev.flags & kResource)
        {
            const uint64_t blocks = std::max<uint64_t>(1, std::min<uint64_t>((q.n + 7) / 8, 4ull * sm_count_));
            const TrainView v{q.adev.res, q.adev.syn, q.adev.dopa, q.adev.spikes, q.adev.spike_count};
            launch_resource_train(v, static_cast<int>(blocks), ctl_, stream_);
        }
        return;
    }
    launch_blifat(q.bdev, ctl_, stream_);
    if (q.bdev.flags & kResSyn)
    {
        const uint64_t blocks = std::max<uint64_t>(1, std::min<uint64_t>((q.n + 7) / 8, 4ull * sm_count_));
        const TrainView v{q.bdev.res, q.bdev.syn, q.bdev.dopa, q.bdev.spikes, q.bdev.spike_count};
        launch_resource_train(v, static_cast<int>(blocks), ctl_, stream_);
    }
}

void Backend::enqueue_step()
{
    for (auto &q : pops_) launch_population(*q);
    for (auto &p : projs_)
    {
        if (p->dev.n_src == 0) continue;
        uint64_t bound = 0;
        for (int k = 0; k < p->dev.n_src; ++k)
        {
            const SpikeSource &s = p->dev.src[k];
            bound += s.channel ? p->n_rows : p->n_rows;
        }
        const uint64_t blocks = std::max<uint64_t>(1, std::min<uint64_t>((bound + 7) / 8, 8ull * sm_count_));
        launch_projection(p->dev, ctl_, static_cast<int>(blocks), stream_);
    }
    for (auto &p : projs_)
        if (p->pull) launch_gather(p->dev, ctl_, gather_grid(*p), stream_);
    for (auto &p : projs_)
    {
        if (p->kind != KNP_SYNAPSE_ADDITIVE_STDP_DELTA || p->n_syn == 0 || p->stdp_sources.empty()) continue;
        for (auto &[src, both] : p->stdp_sources) launch_stdp_append(p->stdp, src, both, ctl_, stream_);
        launch_stdp_modify(p->stdp, ctl_, stream_);
    }
    StepEnd e{counters_, n_counters_, n_spike_counters_};
    launch_step_end(e, ctl_, stream_);
}

void Backend::capture_graphs()
{
    KNP_CUDA(cudaStreamSynchronize(stream_));
    if (graph1_) cudaGraphExecDestroy(graph1_);
    if (graphK_) cudaGraphExecDestroy(graphK_);
    graph1_ = graphK_ = nullptr;
    if (fused_ || grid_)
    {
        build_small_net();
        if (grid_)
        {
            grid_net_.net = small_;
            if (!grid_net_.barrier) grid_net_.barrier = arena_.make<unsigned long long>(1);
            grid_net_.n_pull = static_cast<uint32_t>(small_pull_.size());
            for (size_t k = 0; k < small_pull_.size(); ++k) grid_net_.pull[k] = small_pull_[k];
        }
        return;
    }
    for (int which = 0; which < 2; ++which)
    {
        cudaGraph_t g = nullptr;
        KNP_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        const uint64_t k = which ? kGraphSteps : 1;
        for (uint64_t i = 0; i < k; ++i) enqueue_step();
        KNP_CUDA(cudaStreamEndCapture(stream_, &g));
        cudaGraphExec_t ex = nullptr;
        KNP_CUDA(cudaGraphInstantiate(&ex, g, 0));
        cudaGraphDestroy(g);
        (which ? graphK_ : graph1_) = ex;
    }
}

uint64_t Backend::steps_before_drain() const
{
    uint64_t room = ~0ull;
    for (auto &q : pops_)
        if (q->record && q->rec_bits) room = std::min<uint64_t>(room, q->rec_slots - (step_ - drained_to_));
    return room;
}

void Backend::stage_host_inputs()
{
    // Pinned staging: wait until the previous staging copy has been consumed.
    KNP_CUDA(cudaEventSynchronize(pinned_free_));
    size_t need = 0;
    for (auto &c : channels_)
        if (c->has_pending) need += sizeof(ChannelDev) + 16 + c->pending.size() * 4 + 64;
    for (auto &m : pending_impacts_) need += m.post.size() * 9 + 64;
    if (need > pinned_bytes_)
    {
        if (pinned_) KNP_CUDA(cudaFreeHost(pinned_));
        pinned_bytes_ = std::max<size_t>(need * 2, 1 << 16);
        KNP_CUDA(cudaHostAlloc(&pinned_, pinned_bytes_, cudaHostAllocDefault));
    }
    char *hp = static_cast<char *>(pinned_);
    size_t off = 0;
    auto stage = [&](const void *src, size_t bytes) -> char *
    {
        off = (off + 15) & ~size_t(15);
        char *dst = hp + off;
        std::memcpy(dst, src, bytes);
        off += bytes;
        return dst;
    };
    for (auto &c : channels_)
    {
        if (!c->has_pending) continue;
        const uint64_t n = c->pending.size();
        if (n > c->cap_idx || c->cap_steps < 1 || c->scheduled || c->owns_generated)
        {
            KNP_CUDA(cudaStreamSynchronize(stream_));
            if (c->idx && !c->owns_generated) arena_.release(c->idx);
            if (c->idx && c->owns_generated) cudaFree(c->idx);
            if (c->offsets) arena_.release(c->offsets);
            c->cap_idx = std::max<uint64_t>(n * 2, 1024);
            c->cap_steps = 1;
            c->idx = arena_.make<uint32_t>(c->cap_idx, false);
            c->offsets = arena_.make<long long>(2);
            c->owns_generated = false;
        }
        const long long offs[2] = {0, static_cast<long long>(n)};
        c->host = ChannelDev{step_, 1, c->offsets, c->idx};
        c->scheduled = false;
        char *a = stage(offs, sizeof(offs));
        KNP_CUDA(cudaMemcpyAsync(c->offsets, a, sizeof(offs), cudaMemcpyHostToDevice, stream_));
        if (n)
        {
            char *b = stage(c->pending.data(), n * 4);
            KNP_CUDA(cudaMemcpyAsync(c->idx, b, n * 4, cudaMemcpyHostToDevice, stream_));
        }
        char *h = stage(&c->host, sizeof(ChannelDev));
        KNP_CUDA(cudaMemcpyAsync(c->dev, h, sizeof(ChannelDev), cudaMemcpyHostToDevice, stream_));
        c->pending.clear();
        c->has_pending = false;
    }
    std::map<PopulationSlot *, uint32_t> ext_seq;
    for (auto &m : pending_impacts_)
    {
        PopulationSlot *q = find_pop(m.receiver);
        const uint32_t n = static_cast<uint32_t>(m.post.size());
        if (!q || !n) continue;
        // Device staging for impacts: allocated per message batch and released after the step.
        uint32_t *dpost = arena_.make<uint32_t>(n, false);
        float *dval = arena_.make<float>(n, false);
        uint8_t *dtype = arena_.make<uint8_t>(n, false);
        KNP_CUDA(cudaMemcpyAsync(dpost, stage(m.post.data(), n * 4), n * 4, cudaMemcpyHostToDevice, stream_));
        KNP_CUDA(cudaMemcpyAsync(dval, stage(m.value.data(), n * 4), n * 4, cudaMemcpyHostToDevice, stream_));
        KNP_CUDA(cudaMemcpyAsync(dtype, stage(m.type.data(), n), n, cudaMemcpyHostToDevice, stream_));
        // External impacts on a population are numbered in message order within the step (the order of
        // an AltAI-LIF population's BLOCKING events).
        const uint32_t seq = ext_seq[q];
        ext_seq[q] += n;
        launch_apply_impacts(q->input_ring(), dpost, dval, dtype, m.forcing ? 1 : 0, n, seq, ctl_, stream_);
        KNP_CUDA(cudaGetLastError());
        KNP_CUDA(cudaStreamSynchronize(stream_));
        arena_.release(dpost);
        arena_.release(dval);
        arena_.release(dtype);
    }
    pending_impacts_.clear();
    KNP_CUDA(cudaEventRecord(pinned_free_, stream_));
}

void Backend::step(uint64_t n)
{
    require_init("step");
    KNP_CUDA(cudaSetDevice(device_));
    while (n > 0)
    {
        bool host_inputs = !pending_impacts_.empty();
        for (auto &c : channels_) host_inputs = host_inputs || c->has_pending;
        if (any_recording_ && steps_before_drain() == 0) drain_recordings();
        if (host_inputs)
        {
            stage_host_inputs();
            if (fused_ || grid_)
            {
                if (!small_.pops[0]) throw Error(KNP_GB300_E_STATE, "the fused step kernel was not set up");
                if (grid_)
                    KNP_CUDA(launch_grid_net(grid_net_, ctl_, 1, grid_ctas_, grid_smem_, &ring_window_, stream_));
                else
                    KNP_CUDA(launch_small_net(small_, ctl_, 1, small_cluster_, stream_));
            }
            else
                KNP_CUDA(cudaGraphLaunch(graph1_, stream_));
            KNP_CUDA(cudaGetLastError());
            if (any_recording_) record_step_event(step_);
            ++step_;
            --n;
            continue;
        }
        uint64_t k = n;
        if (any_recording_) k = std::min<uint64_t>(k, steps_before_drain());
        uint64_t done = 0;
        if ((fused_ || grid_) && !small_.pops[0]) throw Error(KNP_GB300_E_STATE, "the fused step kernel was not set up");
        while ((fused_ || grid_) && done < k)
        {
            const uint64_t m = std::min<uint64_t>(k - done, kSmallMaxStepsPerLaunch);
            if (grid_)
                KNP_CUDA(launch_grid_net(grid_net_, ctl_, static_cast<uint32_t>(m), grid_ctas_, grid_smem_, &ring_window_,
                                         stream_));
            else
                KNP_CUDA(launch_small_net(small_, ctl_, static_cast<uint32_t>(m), small_cluster_, stream_));
            KNP_CUDA(cudaGetLastError());
            done += m;
        }
        while (k - done >= kGraphSteps)
        {
            KNP_CUDA(cudaGraphLaunch(graphK_, stream_));
            done += kGraphSteps;
        }
        while (done < k)
        {
            KNP_CUDA(cudaGraphLaunch(graph1_, stream_));
            ++done;
        }
        if (any_recording_ && k) record_step_event(step_ + k - 1);
        step_ += k;
        n -= k;
    }
}

float Backend::step_timed(uint64_t n)
{
    cudaEvent_t a, b;
    KNP_CUDA(cudaEventCreate(&a));
    KNP_CUDA(cudaEventCreate(&b));
    KNP_CUDA(cudaEventRecord(a, stream_));
    step(n);
    KNP_CUDA(cudaEventRecord(b, stream_));
    KNP_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    KNP_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    check_device_error();
    return ms;
}

void Backend::profile_grid_phases(uint64_t n, double *us)
{
    require_init("profile_grid_phases");
    KNP_CUDA(cudaSetDevice(device_));
    if (!grid_) throw Error(KNP_GB300_E_STATE, "the backend does not step with the persistent grid kernel");
    bool host_inputs = !pending_impacts_.empty();
    for (auto &c : channels_) host_inputs = host_inputs || c->has_pending;
    if (host_inputs) throw Error(KNP_GB300_E_STATE, "profile_grid_phases does not stage host messages");
    unsigned long long *acc = nullptr;
    KNP_CUDA(cudaMalloc(&acc, 3 * sizeof(unsigned long long)));
    unsigned long long h[3] = {0, 0, 0};
    cudaError_t err = cudaMemsetAsync(acc, 0, sizeof(h), stream_);
    if (err == cudaSuccess)
    {
        grid_net_.phase_ns = acc;
        try
        {
            step(n);
        }
        catch (...)
        {
            grid_net_.phase_ns = nullptr;
            cudaStreamSynchronize(stream_);
            cudaFree(acc);
            throw;
        }
        grid_net_.phase_ns = nullptr;
        err = cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, stream_);
        if (err == cudaSuccess) err = cudaStreamSynchronize(stream_);
    }
    cudaFree(acc);
    KNP_CUDA(err);
    check_device_error();
    for (int k = 0; k < 3; ++k) us[k] = static_cast<double>(h[k]) * 1e-3;
}

void Backend::profile_phases(uint64_t n, float *ms)
{
    require_init("profile_phases");
    KNP_CUDA(cudaSetDevice(device_));
    if (any_recording_) drain_recordings();
    bool host_inputs = !pending_impacts_.empty();
    for (auto &c : channels_) host_inputs = host_inputs || c->has_pending;
    if (host_inputs) throw Error(KNP_GB300_E_STATE, "profile_phases does not stage host messages");
    cudaEvent_t ev[5];
    for (auto &e : ev) KNP_CUDA(cudaEventCreate(&e));
    double acc[4] = {0, 0, 0, 0};
    for (uint64_t i = 0; i < n; ++i)
    {
        if (any_recording_ && steps_before_drain() == 0) drain_recordings();
        KNP_CUDA(cudaEventRecord(ev[0], stream_));
        for (auto &q : pops_) launch_population(*q);
        KNP_CUDA(cudaEventRecord(ev[1], stream_));
        for (auto &p : projs_)
        {
            if (p->dev.n_src == 0) continue;
            const uint64_t bound = static_cast<uint64_t>(p->dev.n_src) * p->n_rows;
            const uint64_t blocks = std::max<uint64_t>(1, std::min<uint64_t>((bound + 7) / 8, 8ull * sm_count_));
            launch_projection(p->dev, ctl_, static_cast<int>(blocks), stream_);
        }
        for (auto &p : projs_)
            if (p->pull) launch_gather(p->dev, ctl_, gather_grid(*p), stream_);
        KNP_CUDA(cudaEventRecord(ev[2], stream_));
        for (auto &p : projs_)
        {
            if (p->kind != KNP_SYNAPSE_ADDITIVE_STDP_DELTA || p->n_syn == 0 || p->stdp_sources.empty()) continue;
            for (auto &[src, both] : p->stdp_sources) launch_stdp_append(p->stdp, src, both, ctl_, stream_);
            launch_stdp_modify(p->stdp, ctl_, stream_);
        }
        KNP_CUDA(cudaEventRecord(ev[3], stream_));
        StepEnd e{counters_, n_counters_, n_spike_counters_};
        launch_step_end(e, ctl_, stream_);
        KNP_CUDA(cudaEventRecord(ev[4], stream_));
        KNP_CUDA(cudaEventSynchronize(ev[4]));
        for (int k = 0; k < 4; ++k)
        {
            float m = 0.f;
            KNP_CUDA(cudaEventElapsedTime(&m, ev[k], ev[k + 1]));
            acc[k] += m;
        }
        ++step_;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (int k = 0; k < 4; ++k) ms[k] = static_cast<float>(acc[k]);
    check_device_error();
}

void Backend::check_device_error()
{
    Control c{};
    KNP_CUDA(cudaMemcpyAsync(&c, ctl_, sizeof(Control), cudaMemcpyDeviceToHost, stream_));
    KNP_CUDA(cudaStreamSynchronize(stream_));
    if (c.error)
        throw Error(KNP_GB300_E_DEVICE_FLAG, "device error flags 0x" + std::to_string(c.error));
}

void Backend::alloc_recording(PopulationSlot &p)
{
    // Up to 4096 steps between drains, at most 64 MB of bitmaps per population.
    p.rec_words = std::max<uint32_t>((p.n + 31) / 32, 1);
    p.rec_slots = static_cast<uint32_t>(std::max<uint64_t>(1, std::min<uint64_t>(4096, (16ull << 20) / p.rec_words)));
    p.rec_bits = arena_.make<uint32_t>(static_cast<size_t>(p.rec_words) * p.rec_slots);
    any_recording_ = true;
}

void Backend::record_step_event(uint64_t last_step)
{
    const uint64_t slot = last_step % kStepEvents;
    KNP_CUDA(cudaEventRecord(step_ev_[slot], stream_));
    step_ev_of_[slot] = last_step + 1;
}

// Copies the recorded bitmaps of steps [drained_to_, upto) to the host (per step: the bitmap and
// its spike count); read_spikes expands a step's bitmap into ascending spike indexes, the order of
// the reference's SpikeMessage (populations_old.h:104-118). When the completion event of step
// upto - 1 is at hand, the copy waits for that event only (on copy_stream_), so the steps queued
// after it keep running; otherwise it waits for the whole stream.
void Backend::drain_recordings(uint64_t upto)
{
    upto = std::min(upto, step_);
    if (upto <= drained_to_) return;
    const uint64_t steps = upto - drained_to_;
    const uint64_t ev = (upto - 1) % kStepEvents;
    const bool by_event = step_ev_of_[ev] == upto;
    cudaStream_t cs = by_event ? copy_stream_ : stream_;
    if (by_event) KNP_CUDA(cudaStreamWaitEvent(copy_stream_, step_ev_[ev], 0));
    // Every recorded population's bitmaps go to their own span of the pinned buffer, then the
    // control block; one wait for all of them.
    size_t need = 0;
    for (auto &q : pops_)
        if (q->record && q->rec_bits) need += static_cast<size_t>(steps) * q->rec_words;
    if (need > rec_host_words_)
    {
        KNP_CUDA(cudaStreamSynchronize(copy_stream_));
        if (rec_host_) KNP_CUDA(cudaFreeHost(rec_host_));
        rec_host_ = nullptr;
        size_t cap = 0;
        for (auto &q : pops_)
            if (q->rec_bits) cap += static_cast<size_t>(q->rec_slots) * q->rec_words;
        cap = std::max(cap, need);
        KNP_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&rec_host_), cap * 4, cudaHostAllocDefault));
        rec_host_words_ = cap;
    }
    size_t off = 0;
    for (auto &q : pops_)
    {
        if (!q->record || !q->rec_bits) continue;
        // The steps occupy ring slots drained_to_ % slots ... (upto - 1) % slots: one or two spans.
        const uint64_t first = drained_to_ % q->rec_slots;
        const uint64_t span1 = std::min<uint64_t>(steps, q->rec_slots - first);
        const size_t W = q->rec_words;
        KNP_CUDA(cudaMemcpyAsync(rec_host_ + off, q->rec_bits + first * W, span1 * W * 4, cudaMemcpyDeviceToHost, cs));
        if (span1 < steps)
            KNP_CUDA(cudaMemcpyAsync(rec_host_ + off + span1 * W, q->rec_bits, (steps - span1) * W * 4,
                                     cudaMemcpyDeviceToHost, cs));
        off += static_cast<size_t>(steps) * W;
    }
    // Device error flags as of the drained steps (read on the same stream as the bitmaps).
    KNP_CUDA(cudaMemcpyAsync(ctl_host_, ctl_, sizeof(Control), cudaMemcpyDeviceToHost, cs));
    KNP_CUDA(cudaStreamSynchronize(cs));
    off = 0;
    for (auto &q : pops_)
    {
        if (!q->record || !q->rec_bits) continue;
        const size_t W = q->rec_words;
        for (uint64_t k = 0; k < steps; ++k)
        {
            const uint64_t step = drained_to_ + k;
            if (step < q->record_from) continue;
            const uint32_t *bits = rec_host_ + off + k * W;
            RecordedStep &r = q->recorded[step];
            r.bits.assign(bits, bits + W);
            r.count = 0;
            r.block_prefix.resize((W + kExpandBlockWords - 1) / kExpandBlockWords);
            // Word pairs (kExpandBlockWords is even, so a block starts on a pair), then an odd last word.
            size_t w = 0;
            for (; w + 1 < W; w += 2)
            {
                if (w % kExpandBlockWords == 0) r.block_prefix[w / kExpandBlockWords] = r.count;
                uint64_t pair;
                std::memcpy(&pair, bits + w, sizeof(pair));
                r.count += static_cast<uint32_t>(__builtin_popcountll(pair));
            }
            if (w < W)
            {
                if (w % kExpandBlockWords == 0) r.block_prefix[w / kExpandBlockWords] = r.count;
                r.count += static_cast<uint32_t>(__builtin_popcount(bits[w]));
            }
        }
        off += static_cast<size_t>(steps) * W;
    }
    drained_to_ = upto;
    if (ctl_host_->error)
        throw Error(KNP_GB300_E_DEVICE_FLAG, "device error flags 0x" + std::to_string(ctl_host_->error));
}

namespace
{
// Per byte value: its set bits' positions (padded to 8) and their number, for the expansion below.
struct ByteBits
{
    uint8_t pos[256][8];
    uint8_t cnt[256];
    ByteBits()
    {
        for (int b = 0; b < 256; ++b)
        {
            cnt[b] = 0;
            for (int i = 0; i < 8; ++i) pos[b][i] = 0;
            for (int i = 0; i < 8; ++i)
                if (b >> i & 1) pos[b][cnt[b]++] = static_cast<uint8_t>(i);
        }
    }
};
const ByteBits kByteBits;

// Ascending indexes of the set bits of words [w0, w1) of `bits` into out[k0, end), end = min(the
// range's last index + 1, cap): full words are written as runs, other words a byte at a time from
// kByteBits (eight entries at once where they stay below `end`, so a range never writes into the
// next range's part of `out`).
void expand_bits(const uint32_t *bits, size_t w0, size_t w1, uint32_t k0, uint32_t end, uint32_t *out)
{
    uint32_t k = k0;
    for (size_t w = w0; w < w1 && k < end; ++w)
    {
        // Skip zero word pairs (most words are zero at low firing rates).
        if (!(w & 1u) && w + 1 < w1)
        {
            uint64_t pair;
            std::memcpy(&pair, bits + w, sizeof(pair));
            if (!pair)
            {
                ++w;
                continue;
            }
        }
        uint32_t x = bits[w];
        if (!x) continue;
        const uint32_t base = static_cast<uint32_t>(w * 32);
        if (x == 0xFFFFFFFFu && k + 32 <= end)
        {
            for (uint32_t i = 0; i < 32; ++i) out[k + i] = base + i;
            k += 32;
            continue;
        }
        if (__builtin_popcount(x) <= 4)
        {
            // Sparse word (the common case at low firing rates): lowest set bit first.
            for (; x && k < end; x &= x - 1) out[k++] = base + static_cast<uint32_t>(__builtin_ctz(x));
            continue;
        }
        for (uint32_t j = 0; j < 4; ++j)
        {
            const uint32_t byte = x >> (8 * j) & 0xFFu;
            if (!byte) continue;
            const uint32_t c = kByteBits.cnt[byte];
            if (k + 8 <= end)
            {
                for (uint32_t i = 0; i < 8; ++i) out[k + i] = base + 8 * j + kByteBits.pos[byte][i];
                k += c;
            }
            else
            {
                for (uint32_t i = 0; i < c && k < end; ++i) out[k++] = base + 8 * j + kByteBits.pos[byte][i];
            }
        }
    }
}
}  // namespace

ExpandPool::ExpandPool(unsigned workers)
{
    for (unsigned i = 0; i < workers; ++i) threads_.emplace_back([this] { work(); });
}

ExpandPool::~ExpandPool()
{
    {
        std::lock_guard<std::mutex> lk(m_);
        stop_ = true;
    }
    go_.notify_all();
    for (auto &t : threads_) t.join();
}

void ExpandPool::drain_tasks()
{
    for (unsigned i = next_.fetch_add(1); i < n_tasks_; i = next_.fetch_add(1)) (*fn_)(i);
}

void ExpandPool::work()
{
    uint64_t seen = 0;
    for (;;)
    {
        {
            std::unique_lock<std::mutex> lk(m_);
            go_.wait(lk, [&] { return stop_ || gen_ != seen; });
            if (stop_) return;
            seen = gen_;
        }
        drain_tasks();
        {
            std::lock_guard<std::mutex> lk(m_);
            if (--busy_ == 0) done_.notify_one();
        }
    }
}

void ExpandPool::run(unsigned n_tasks, const std::function<void(unsigned)> &fn)
{
    {
        std::lock_guard<std::mutex> lk(m_);
        fn_ = &fn;
        n_tasks_ = n_tasks;
        next_.store(0);
        busy_ = static_cast<unsigned>(threads_.size());
        ++gen_;
    }
    go_.notify_all();
    drain_tasks();
    std::unique_lock<std::mutex> lk(m_);
    done_.wait(lk, [&] { return busy_ == 0; });
}

void Backend::read_spikes(const Uid &pop, uint64_t step, uint32_t cap, uint32_t *out, uint32_t *n)
{
    require_init("read_spikes");
    PopulationSlot *q = find_pop(pop);
    if (!q) throw Error(KNP_GB300_E_INVALID, "unknown population");
    if (!q->record) throw Error(KNP_GB300_E_STATE, "spike recording is not enabled for this population");
    if (step >= step_) throw Error(KNP_GB300_E_INVALID, "step has not been run yet");
    if (step >= drained_to_) drain_recordings(step + 1);
    auto it = q->recorded.find(step);
    if (it == q->recorded.end()) throw Error(KNP_GB300_E_INVALID, "spikes of this step were not recorded or were discarded");
    // Ascending indexes straight from the step's bitmap into the caller's buffer.
    const RecordedStep &r = it->second;
    *n = r.count;
    const size_t W = r.bits.size();
    const unsigned blocks = static_cast<unsigned>(r.block_prefix.size());
    // Large steps are expanded in parallel, one block of words per task (its offset is known).
    if (r.count >= (1u << 16) && blocks > 1)
    {
        if (!expand_pool_)
        {
            const unsigned hc = std::max(1u, std::thread::hardware_concurrency());
            expand_pool_ = std::make_unique<ExpandPool>(std::min(7u, hc > 1 ? hc - 1 : 1u));
        }
        const std::function<void(unsigned)> task = [&](unsigned b)
        {
            const uint32_t k0 = r.block_prefix[b];
            const uint32_t k1 = b + 1 < blocks ? r.block_prefix[b + 1] : r.count;
            if (k0 >= cap) return;
            const size_t w0 = static_cast<size_t>(b) * kExpandBlockWords;
            expand_bits(r.bits.data(), w0, std::min(W, w0 + kExpandBlockWords), k0, std::min(k1, cap), out);
        };
        expand_pool_->run(blocks, task);
    }
    else
    {
        expand_bits(r.bits.data(), 0, W, 0, std::min(r.count, cap), out);
    }
}

void Backend::discard_spikes(uint64_t before)
{
    for (auto &q : pops_) q->recorded.erase(q->recorded.begin(), q->recorded.lower_bound(before));
}

// ------------------------------------------------------------------------------------ messages

void Backend::send_spikes(const Uid &sender, uint64_t, uint32_t n, const uint32_t *idx)
{
    require_init("send_spikes");
    Channel *c = find_channel(sender);
    if (!c)
    {
        // No projection subscribed to this sender: the message reaches nobody (as on the bus).
        return;
    }
    if (c->scheduled && step_ >= c->host.first_step && step_ - c->host.first_step < c->host.n_steps)
        throw Error(KNP_GB300_E_STATE, "this sender's device spike schedule covers the next step");
    c->pending.insert(c->pending.end(), idx, idx + n);
    c->has_pending = true;
}

void Backend::load_schedule(
    const Uid &sender, uint64_t first_step, uint64_t n_steps, const int64_t *offsets, const uint32_t *idx)
{
    require_init("load_spike_schedule");
    Channel *c = find_channel(sender);
    if (!c) throw Error(KNP_GB300_E_INVALID, "no projection is subscribed to this sender");
    if (offsets[0] != 0) throw Error(KNP_GB300_E_INVALID, "schedule offsets must start at 0");
    for (uint64_t t = 0; t < n_steps; ++t)
        if (offsets[t + 1] < offsets[t]) throw Error(KNP_GB300_E_INVALID, "schedule offsets must be non-decreasing");
    const uint64_t total = static_cast<uint64_t>(offsets[n_steps]);
    KNP_CUDA(cudaStreamSynchronize(stream_));
    if (c->idx && c->owns_generated) cudaFree(c->idx);
    else if (c->idx) arena_.release(c->idx);
    if (c->offsets) arena_.release(c->offsets);
    c->idx = arena_.make<uint32_t>(std::max<uint64_t>(total, 1), false);
    c->offsets = arena_.make<long long>(n_steps + 1, false);
    c->owns_generated = false;
    c->cap_idx = total;
    c->cap_steps = n_steps;
    KNP_CUDA(cudaMemcpy(c->offsets, offsets, (n_steps + 1) * 8, cudaMemcpyHostToDevice));
    if (total) KNP_CUDA(cudaMemcpy(c->idx, idx, total * 4, cudaMemcpyHostToDevice));
    c->host = ChannelDev{first_step, n_steps, c->offsets, c->idx};
    KNP_CUDA(cudaMemcpy(c->dev, &c->host, sizeof(ChannelDev), cudaMemcpyHostToDevice));
    c->scheduled = true;
}

void Backend::generate_bernoulli(
    const Uid &sender, uint32_t n_sources, double p, uint64_t first_step, uint64_t n_steps, uint64_t seed,
    uint64_t stream)
{
    require_init("generate_bernoulli_schedule");
    Channel *c = find_channel(sender);
    if (!c) throw Error(KNP_GB300_E_INVALID, "no projection is subscribed to this sender");
    if (n_steps > 65535) throw Error(KNP_GB300_E_INVALID, "at most 65535 steps per generated schedule");
    KNP_CUDA(cudaStreamSynchronize(stream_));
    if (c->idx && c->owns_generated) cudaFree(c->idx);
    else if (c->idx) arena_.release(c->idx);
    if (c->offsets) arena_.release(c->offsets);
    c->offsets = arena_.make<long long>(n_steps + 1, false);
    uint32_t *idx = nullptr;
    uint64_t total = 0;
    const double pc = std::min(std::max(p, 0.0), 1.0);
    const unsigned long long thr = static_cast<unsigned long long>(pc * 9007199254740992.0);
    KNP_CUDA(gen_bernoulli_schedule(n_sources, thr, stream_key(seed, stream), first_step, n_steps, c->offsets, &idx,
                                    &total, stream_));
    KNP_CUDA(cudaStreamSynchronize(stream_));
    c->idx = idx;
    c->owns_generated = true;
    c->cap_idx = total;
    c->cap_steps = n_steps;
    c->host = ChannelDev{first_step, n_steps, c->offsets, c->idx};
    KNP_CUDA(cudaMemcpy(c->dev, &c->host, sizeof(ChannelDev), cudaMemcpyHostToDevice));
    c->scheduled = true;
}

void Backend::send_impacts(
    const Uid &sender, const Uid &receiver, bool forcing, uint32_t n, const uint32_t *post, const float *value,
    const uint8_t *type)
{
    require_init("send_impacts");
    PopulationSlot *q = find_pop(receiver);
    if (!q) throw Error(KNP_GB300_E_INVALID, "unknown receiver population");
    if (!q->impact_senders.count(sender)) return;  // not subscribed: the message reaches nobody
    PendingImpacts m{receiver, forcing, {}, {}, {}};
    for (uint32_t i = 0; i < n; ++i)
    {
        if (post[i] >= q->n) throw Error(KNP_GB300_E_INVALID, "impact postsynaptic index out of range");
        const uint8_t t = type ? type[i] : 0;
        if (t > KNP_OUT_BLOCKING) throw Error(KNP_GB300_E_INVALID, "unhandled synapse type");
        if (q->kind == KNP_NEURON_LIF && t > KNP_OUT_INHIBITORY_CURRENT)
            throw Error(KNP_GB300_E_INVALID, "unhandled synapse type");
        if (q->is_altai() && t == KNP_OUT_INHIBITORY_CONDUCTANCE)
            throw Error(KNP_GB300_E_INVALID, "unhandled synapse type");
        m.post.push_back(post[i]);
        m.value.push_back(value[i]);
        m.type.push_back(t);
    }
    // Of several BLOCKING impacts on one neuron only the last one in the message counts
    // (blifat_impl.h:86): the earlier ones are dropped here, so the device writes each target once.
    // (AltAI-LIF neurons apply every BLOCKING impact in order: all are kept.)
    std::map<uint32_t, size_t> last_blk;
    for (size_t i = 0; i < m.type.size() && !q->is_altai(); ++i)
        if (m.type[i] == KNP_OUT_BLOCKING) last_blk[m.post[i]] = i;
    if (!last_blk.empty())
    {
        PendingImpacts r{receiver, forcing, {}, {}, {}};
        for (size_t i = 0; i < m.type.size(); ++i)
        {
            if (m.type[i] == KNP_OUT_BLOCKING && last_blk[m.post[i]] != i) continue;
            r.post.push_back(m.post[i]);
            r.value.push_back(m.value[i]);
            r.type.push_back(m.type[i]);
        }
        m = std::move(r);
    }
    pending_impacts_.push_back(std::move(m));
}

// ------------------------------------------------------------------------------------ readback

void Backend::read_blifat(const Uid &pop, knp_blifat_neuron *out, knp_resource_stdp_state *ext)
{
    PopulationSlot *q = find_pop(pop);
    if (!q || q->kind == KNP_NEURON_LIF || q->is_altai()) throw Error(KNP_GB300_E_INVALID, "unknown BLIFAT population");
    const uint32_t n = q->n;
    std::copy(q->init_blifat.begin(), q->init_blifat.end(), out);
    if (ext && !q->init_res.empty()) std::copy(q->init_res.begin(), q->init_res.end(), ext);
    if (!initialized_) return;
    KNP_CUDA(cudaStreamSynchronize(stream_));
    const BlifatDev &d = q->bdev;
    const uint32_t f = d.flags;
    const uint64_t T = step_;
    auto getf = [&](const float *p)
    {
        std::vector<float> v(n);
        if (n) KNP_CUDA(cudaMemcpy(v.data(), p, n * 4, cudaMemcpyDeviceToHost));
        return v;
    };
    auto getu = [&](const uint32_t *p)
    {
        std::vector<uint32_t> v(n);
        if (n) KNP_CUDA(cudaMemcpy(v.data(), p, n * 4, cudaMemcpyDeviceToHost));
        return v;
    };
    if (T == 0) return;
    auto V = getf(d.V);
    for (uint32_t i = 0; i < n; ++i) out[i].potential = V[i];
    if (f & kLiveVPre)
    {
        auto v = getf(d.V_pre);
        for (uint32_t i = 0; i < n; ++i) out[i].pre_impact_potential = v[i];
    }
    else
        for (uint32_t i = 0; i < n; ++i) out[i].pre_impact_potential = 0.0;
    if (f & kLiveThrDyn)
    {
        auto v = getf(d.thr_dyn);
        for (uint32_t i = 0; i < n; ++i) out[i].dynamic_threshold = v[i];
    }
    if (f & kLiveTrace)
    {
        auto v = getf(d.trace);
        for (uint32_t i = 0; i < n; ++i) out[i].postsynaptic_trace = v[i];
    }
    if (f & kLiveG)
    {
        auto v = getf(d.g);
        for (uint32_t i = 0; i < n; ++i) out[i].inhibitory_conductance = v[i];
    }
    if (d.dopa)
    {
        auto v = getf(d.dopa);
        for (uint32_t i = 0; i < n; ++i) out[i].dopamine_value = v[i];
    }
    if (f & kResSyn)
    {
        std::vector<double> v(n);
        if (n) KNP_CUDA(cudaMemcpy(v.data(), d.syn.add_thr, n * 8, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < n; ++i) out[i].additional_threshold = v[i];
    }
    else if (d.add_thr)
    {
        auto v = getf(d.add_thr);
        for (uint32_t i = 0; i < n; ++i) out[i].additional_threshold = v[i];
    }
    {
        auto v = getu(d.n_since);
        for (uint32_t i = 0; i < n; ++i)
        {
            if (f & kLiveRefract)
                out[i].n_time_steps_since_last_firing =
                    v[i] == 0xFFFFFFFFu ? std::numeric_limits<uint64_t>::max() : static_cast<uint64_t>(v[i]);
            else
                out[i].n_time_steps_since_last_firing = (T - 1) - v[i];
        }
    }
    if (f & kLiveBurst)
    {
        auto v = getu(d.burst_phase);
        for (uint32_t i = 0; i < n; ++i) out[i].bursting_phase = v[i];
    }
    if (f & kLiveBlock)
    {
        std::vector<long long> v(n);
        if (n) KNP_CUDA(cudaMemcpy(v.data(), d.blocking, n * 8, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < n; ++i) out[i].total_blocking_period = v[i];
    }
    else
        for (uint32_t i = 0; i < n; ++i) out[i].total_blocking_period = std::numeric_limits<int64_t>::max() - T;
    if (ext && (f & kResource))
    {
        const ResourceDev &r = d.res;
        auto st = getu(reinterpret_cast<const uint32_t *>(r.isi_status));
        auto stab = getf(r.stability);
        auto fr = getf(r.free_resource);
        std::vector<unsigned long long> ls(n), lss(n), fis(n);
        std::vector<uint8_t> forced(n);
        if (n)
        {
            KNP_CUDA(cudaMemcpy(ls.data(), r.last_step, n * 8, cudaMemcpyDeviceToHost));
            KNP_CUDA(cudaMemcpy(lss.data(), r.last_spike_step, n * 8, cudaMemcpyDeviceToHost));
            KNP_CUDA(cudaMemcpy(fis.data(), r.first_isi_spike, n * 8, cudaMemcpyDeviceToHost));
            KNP_CUDA(cudaMemcpy(forced.data(), r.is_forced, n, cudaMemcpyDeviceToHost));
        }
        for (uint32_t i = 0; i < n; ++i)
        {
            ext[i].isi_status = static_cast<int32_t>(st[i]);
            ext[i].stability = stab[i];
            ext[i].free_synaptic_resource = fr[i];
            ext[i].last_step = ls[i];
            ext[i].last_spike_step = lss[i];
            ext[i].first_isi_spike = fis[i];
            ext[i].is_being_forced = forced[i];
        }
    }
}

void Backend::read_lif(const Uid &pop, knp_lif_neuron *out)
{
    PopulationSlot *q = find_pop(pop);
    if (!q || q->kind != KNP_NEURON_LIF) throw Error(KNP_GB300_E_INVALID, "unknown LIF population");
    const uint32_t n = q->n;
    std::copy(q->init_lif.begin(), q->init_lif.end(), out);
    if (!initialized_ || n == 0) return;
    KNP_CUDA(cudaStreamSynchronize(stream_));
    std::vector<float> V(n);
    std::vector<uint32_t> rc(n);
    KNP_CUDA(cudaMemcpy(V.data(), q->ldev.V, n * 4, cudaMemcpyDeviceToHost));
    KNP_CUDA(cudaMemcpy(rc.data(), q->ldev.refract, n * 4, cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < n; ++i)
    {
        out[i].potential = V[i];
        out[i].refract_counter = rc[i];
    }
}

void Backend::read_weights(const Uid &proj, float *out)
{
    ProjectionSlot *p = find_proj(proj);
    if (!p) throw Error(KNP_GB300_E_INVALID, "unknown projection");
    if (!initialized_)
    {
        if (p->generated) throw Error(KNP_GB300_E_STATE, "generated projection weights exist only after init");
        std::copy(p->weight.begin(), p->weight.end(), out);
        return;
    }
    KNP_CUDA(cudaStreamSynchronize(stream_));
    std::vector<float> w(p->n_syn);
    if (p->n_syn) KNP_CUDA(cudaMemcpy(w.data(), p->w, p->n_syn * 4, cudaMemcpyDeviceToHost));
    if (p->generated)
    {
        // Generated projections are read back in CSR order (row by presynaptic neuron).
        std::copy(w.begin(), w.end(), out);
        return;
    }
    std::vector<uint32_t> perm(p->n_syn);
    if (p->n_syn) KNP_CUDA(cudaMemcpy(perm.data(), p->perm, p->n_syn * 4, cudaMemcpyDeviceToHost));
    for (uint64_t e = 0; e < p->n_syn; ++e) out[perm[e]] = w[e];
}

void Backend::read_altai(const Uid &pop, knp_altai_neuron *out, knp_resource_stdp_state *ext)
{
    PopulationSlot *q = find_pop(pop);
    if (!q || !q->is_altai()) throw Error(KNP_GB300_E_INVALID, "unknown AltAI-LIF population");
    const uint32_t n = q->n;
    std::copy(q->init_altai.begin(), q->init_altai.end(), out);
    if (ext && !q->init_res.empty()) std::copy(q->init_res.begin(), q->init_res.end(), ext);
    if (!initialized_ || step_ == 0 || n == 0) return;
    KNP_CUDA(cudaStreamSynchronize(stream_));
    const AltaiDev &d = q->adev;
    auto get = [&](const auto *p)
    {
        using V = std::remove_const_t<std::remove_pointer_t<decltype(p)>>;
        std::vector<V> v(n);
        KNP_CUDA(cudaMemcpy(v.data(), p, n * sizeof(V), cudaMemcpyDeviceToHost));
        return v;
    };
    auto V = get(d.V);
    auto Vp = get(d.V_pre);
    auto act = get(d.activity);
    auto add = get(d.add_thr);
    for (uint32_t i = 0; i < n; ++i)
    {
        out[i].potential = V[i];
        out[i].pre_impact_potential = Vp[i];
        out[i].activity_time = act[i];
        out[i].additional_threshold = add[i];
    }
    if (d.dopa)
    {
        auto v = get(d.dopa);
        for (uint32_t i = 0; i < n; ++i) out[i].dopamine_value = v[i];
    }
    if (ext && (d.flags & kResource))
    {
        const ResourceDev &r = d.res;
        auto st = get(r.isi_status);
        auto stab = get(r.stability);
        auto fr = get(r.free_resource);
        auto ls = get(r.last_step);
        auto lss = get(r.last_spike_step);
        auto fis = get(r.first_isi_spike);
        auto forced = get(r.is_forced);
        for (uint32_t i = 0; i < n; ++i)
        {
            ext[i].isi_status = st[i];
            ext[i].stability = stab[i];
            ext[i].free_synaptic_resource = fr[i];
            ext[i].last_step = ls[i];
            ext[i].last_spike_step = lss[i];
            ext[i].first_isi_spike = fis[i];
            ext[i].is_being_forced = forced[i];
        }
    }
}

void Backend::read_resource_synapses(const Uid &proj, knp_resource_synapse *out)
{
    ProjectionSlot *p = find_proj(proj);
    if (!p || p->kind != KNP_SYNAPSE_RESOURCE_STDP_DELTA)
        throw Error(KNP_GB300_E_INVALID, "unknown resource-STDP projection");
    const uint64_t S = p->n_syn;
    if (!initialized_ || !p->res_pop)
    {
        // Not trained and not scattered (no target population on this backend): the loaded state.
        std::copy(p->rule.begin(), p->rule.end(), out);
        return;
    }
    if (!S) return;
    KNP_CUDA(cudaStreamSynchronize(stream_));
    const ResSynDev &y = p->res_pop->res_syn;
    const uint64_t off = p->res_offset;
    std::vector<float> res(S), lo(S), hi(S), du(S);
    std::vector<uint32_t> per(S), perm(S);
    std::vector<unsigned long long> ls(S);
    std::vector<uint8_t> fl(S);
    KNP_CUDA(cudaMemcpy(res.data(), y.resource + off, S * 4, cudaMemcpyDeviceToHost));
    KNP_CUDA(cudaMemcpy(lo.data(), y.w_min + off, S * 4, cudaMemcpyDeviceToHost));
    KNP_CUDA(cudaMemcpy(hi.data(), y.w_max + off, S * 4, cudaMemcpyDeviceToHost));
    KNP_CUDA(cudaMemcpy(du.data(), y.d_u + off, S * 4, cudaMemcpyDeviceToHost));
    KNP_CUDA(cudaMemcpy(per.data(), y.period + off, S * 4, cudaMemcpyDeviceToHost));
    KNP_CUDA(cudaMemcpy(ls.data(), y.last_spike + off, S * 8, cudaMemcpyDeviceToHost));
    KNP_CUDA(cudaMemcpy(fl.data(), y.flags + off, S, cudaMemcpyDeviceToHost));
    KNP_CUDA(cudaMemcpy(perm.data(), p->perm, S * 4, cudaMemcpyDeviceToHost));
    for (uint64_t e = 0; e < S; ++e)
    {
        knp_resource_synapse r{};
        r.synaptic_resource = res[e];
        r.w_min = lo[e];
        r.w_max = hi[e];
        r.d_u = du[e];
        r.dopamine_plasticity_period = per[e];
        r.had_hebbian_update = fl[e] & 1u;
        r.last_spike_step = ls[e];
        r.has_contributed = (fl[e] >> 1) & 1u;
        out[perm[e]] = r;
    }
}

uint64_t Backend::projection_size(const Uid &proj) const
{
    const ProjectionSlot *p = find_proj(proj);
    if (!p) throw Error(KNP_GB300_E_INVALID, "unknown projection");
    return p->n_syn;
}

void Backend::counters(uint64_t *events, uint64_t *spikes, uint64_t *updates)
{
    Control c{};
    if (initialized_)
    {
        KNP_CUDA(cudaMemcpyAsync(&c, ctl_, sizeof(Control), cudaMemcpyDeviceToHost, stream_));
        KNP_CUDA(cudaStreamSynchronize(stream_));
    }
    if (events) *events = c.events_total;
    if (spikes) *spikes = c.spikes_total;
    if (updates) *updates = neurons_total_ * step_;
}

void Backend::synchronize()
{
    KNP_CUDA(cudaStreamSynchronize(stream_));
    check_device_error();
}

}  // namespace knp_gb300
