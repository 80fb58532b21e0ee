// tmc_serve.cu — a request server for the photon walk: continuous batching of
// simulation requests that each stop at a target relative standard error.
//
// A request is one set of params.h knobs (what tiny_mc.c:34-69 computes for
// one -D setting) plus a target relative standard error (RSE) of the heat in
// one probe shell and a photon cap.  The server:
//
//  * admits a request into a free slot (the slot is its device tally memory,
//    max_shells x 32 bytes) or refuses it with TMC_E_BUSY, so the caller
//    queues; the tally and RNG state never leave the device while it runs;
//  * walks a request in RSE batches of B photons (B a power of two chosen so
//    one batch is about `steps_per_batch` photon steps, at least two photons
//    per thread of a block).  A batch is one or more work items (consecutive
//    photon ranges, `steps_per_item`) of the batched kernel, each walked by one
//    block, which also reports the item's own 128-bit sum of w in the probe
//    shell;
//  * stops a request only at fixed batch counts (min_batches, then doubling):
//    there it computes the batch-means RSE of the probe shell in FP64 over
//    batches 0..k-1 in order (a batch's value is the exact integer sum of its
//    items'), and stops if RSE <= target or the cap is reached.  The decision
//    depends only on the request's own photons, so a request's result is the
//    same alone, in any mix and under any of the scheduling settings;
//  * runs work in waves: launches of the batched kernel over pending items,
//    taken least-attained-service first (requests with the fewest photon
//    steps issued so far go first, so a new request's first round does not
//    queue behind the large later rounds of long-running ones), with up to
//    `waves` (16, at most 64) launches in flight on their own streams and at
//    most `inflight_items` items launched and unfinished;
//  * takes each item as soon as it finishes: the kernel appends the item's
//    probe value to a completion ring in mapped host memory after a
//    system-scope fence, so a request's decision waits for its own items, not
//    for the slowest item of the launch they were in;
//  * or, with `persistent`, keeps one long-running launch of the batched
//    kernel (either form) busy instead of launching waves: pending items are published
//    (least attained service first) into a ring in mapped host memory that
//    the kernel's blocks claim from as they free up, and finished items are
//    appended to a completion ring the host reads from its head.  The blocks
//    wait for more work
//    while requests are active and end once none are; the next admission
//    launches the kernel again.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tmc_batch.cuh"
#include "tmc_internal.h"

using namespace tmc;

namespace {

constexpr int WAVES = 64;           // launch slots (streams, buffers)
constexpr uint32_t DEFAULT_WAVES = 16;
using Clock = std::chrono::steady_clock;

double now_s()
{
    return std::chrono::duration<double>(Clock::now().time_since_epoch()).count();
}

struct Req {
    uint64_t id = 0;
    tmc_request r{};
    Derived d{};
    int slot = -1;
    uint32_t batch = 0;             // photons per RSE batch
    uint32_t item_photons = 0;      // photons per work item
    uint32_t items_per_batch = 0;
    double est_steps = 0.0;         // expected photon steps per photon
    uint64_t max_batches = 0;
    uint64_t issued = 0, done = 0;  // work items
    uint64_t next_decision = 0;     // in batches
    std::vector<unsigned long long> probe;   // per item: 128-bit sum of w in the probe shell
                                             // (2^-40 units), lo and hi
    double t_submit = 0.0;
};

struct Wave {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    BatchItemDev *d_items = nullptr;
    unsigned long long *d_counter = nullptr;   // item counter, error flag, ring tail
    BatchItemDev *h_items = nullptr;           // pinned
    unsigned long long *h_ring = nullptr;      // mapped: completion ring [items][4]
    unsigned long long *d_ring = nullptr;      // its device address
    unsigned long long *h_err = nullptr;       // pinned: the wave's error flag
    uint32_t n_items = 0;
    uint32_t head = 0;                         // ring entries taken
    bool busy = false;
};

struct Done {
    tmc_request_result res{};
    std::vector<tmc_tally> tally;
};

// The work queue of the persistent mode (mapped host memory unless noted).
// Items live in a pool of `cap` slots, freed as each item finishes (in any
// order); the queue proper is a ring of 2 x cap slot numbers in publishing
// order, which the kernel's blocks claim from.
struct Queue {
    uint32_t cap = 0;                          // pool slots (and completion entries), a power of two
    BatchItemDev *h_items = nullptr, *d_items = nullptr;     // the pool
    uint32_t *h_order = nullptr, *d_order = nullptr;         // queue: pool slot per position [2 cap]
    unsigned long long *h_pub = nullptr, *d_pub = nullptr;   // positions published
    unsigned *h_mode = nullptr, *d_mode = nullptr;           // QUEUE_HOLD / DRAIN / STOP
    unsigned long long *h_ring = nullptr, *d_ring = nullptr; // completions [cap][4], finishing order
    BatchProblemDev *h_problems = nullptr, *d_problems = nullptr;
    unsigned long long *d_counter = nullptr;   // device: claim counter, error flag, live blocks,
                                               // completion count
    unsigned *d_done = nullptr;                // device: per launch slot, blocks that ended
    unsigned *h_end = nullptr, *d_end = nullptr;   // per launch slot: {ended, error}
    uint64_t published = 0;                    // queue positions published
    uint64_t done_head = 0;                    // completions taken from the ring
    std::vector<uint32_t> free_slots;          // free pool slots
    std::vector<uint64_t> req;                 // per pool slot: request id of the item
    std::vector<uint64_t> g;                   // per pool slot: item index within its request
    std::vector<uint8_t> state;                // per pool slot: 0 free, 1 published
    unsigned mode = QUEUE_DRAIN;
    bool drained = true;                       // mode was DRAIN since the last launch
};

}  // namespace

struct tmc_server {
    tmc_server_config cfg{};
    int device = -1, sms = 0, grid = 0;
    uint32_t items_cap = 0;
    BatchProblemDev *d_problems = nullptr;
    unsigned long long *d_tally = nullptr;   // [slots][max_shells][4]
    unsigned long long *d_steps = nullptr;   // [slots]
    cudaStream_t admin = nullptr;
    Wave waves[WAVES];
    std::vector<int> free_slots;
    std::unordered_map<uint64_t, Req> active;
    std::deque<uint64_t> order;              // admission order of active requests
    std::vector<uint64_t> slot_req;          // slot -> request id
    uint32_t wave_cap = 0;                   // items per wave
    uint64_t inflight = 0;                   // work items launched, not harvested
    std::unordered_map<uint64_t, Done> finished;
    uint64_t next_id = 1;
    uint64_t photons = 0, steps = 0, n_waves = 0;
    PhiloxKeys keys{};
    Queue q;                                 // persistent mode
    // pinned zeros: a new request's device tally is cleared by a copy from
    // here, which runs on a copy engine; a memset kernel could wait for SM
    // room that the persistent launch's waiting blocks hold
    unsigned char *h_zero = nullptr;
};

namespace {

void destroy_server(tmc_server *s)
{
    if (!s)
        return;
    if (s->q.h_mode)   // running persistent blocks finish their items and end
        __atomic_store_n(s->q.h_mode, QUEUE_STOP, __ATOMIC_RELEASE);
    for (Wave &w : s->waves) {
        if (w.stream)
            cudaStreamSynchronize(w.stream);
        if (w.done)
            cudaEventDestroy(w.done);
        if (w.stream)
            cudaStreamDestroy(w.stream);
        cudaFree(w.d_items);
        cudaFree(w.d_counter);
        cudaFreeHost(w.h_items);
        cudaFreeHost(w.h_ring);
        cudaFreeHost(w.h_err);
    }
    if (s->admin)
        cudaStreamDestroy(s->admin);
    cudaFreeHost(s->h_zero);
    cudaFreeHost(s->q.h_items);
    cudaFreeHost(s->q.h_order);
    cudaFreeHost(s->q.h_pub);
    cudaFreeHost(s->q.h_mode);
    cudaFreeHost(s->q.h_ring);
    cudaFreeHost(s->q.h_problems);
    cudaFree(s->q.d_counter);
    cudaFree(s->q.d_done);
    cudaFreeHost(s->q.h_end);
    cudaFree(s->d_problems);
    cudaFree(s->d_tally);
    cudaFree(s->d_steps);
    delete s;
}

// Photons per RSE batch: a power of two near steps_per_batch / E[steps], in
// [lo, 65536].  lo is two photons per thread of the block for the kernel with
// per-item barriers (fewer would idle the block at the barrier), and one
// warp's claim (BATCH_CHUNK) for the barrier-free kernel, whose lanes move on
// to the next item.
uint32_t batch_photons(const tmc_server_config &cfg, double est_steps)
{
    const double want = cfg.steps_per_batch / std::max(1.0, est_steps);
    uint32_t b = cfg.stream ? (uint32_t)BATCH_CHUNK : 2 * cfg.block;
    while (b < 65536 && 2.0 * b <= want)
        b *= 2;
    return b;
}

// Work items per RSE batch: a power of two (batch is one too) so that an item
// is about steps_per_item photon steps, but no smaller than the kernel's
// smallest item (batch_photons' lower bound).  A batch's items are
// consecutive photon ranges walked by different blocks at once, so a decision
// round takes the time of one item, not of one batch; the batch's probe value
// is the exact sum of its items', so results do not depend on the split.
uint32_t items_per_batch(const tmc_server_config &cfg, uint32_t batch, double est_steps)
{
    const uint32_t lo = cfg.stream ? (uint32_t)BATCH_CHUNK : 2 * cfg.block;
    uint32_t k = 1;
    if (cfg.steps_per_item > 0.0)
        while (batch / (2 * k) >= lo && (double)(batch / k) * est_steps > 2.0 * cfg.steps_per_item)
            k *= 2;
    return k;
}

double expected_steps_host(float albedo)
{
    if (!(albedo > 0.0f))
        return 1.0 / 0.9;
    const double la = std::log((double)albedo);
    double w = 1.0, e = 0.0, p = 1.0;
    for (int stage = 0; stage < 12 && p > 1e-12; ++stage) {
        double k = std::max(1.0, std::ceil(std::log(0.001 / w) / la));
        e += p * k;
        w = w * std::pow((double)albedo, k) / 0.1;
        p *= 0.1;
    }
    return e;
}

// batch-means RSE over batches 0..k-1; batch j's value is the sum of its
// items' probes, in item order
double batch_rse(const std::vector<unsigned long long> &probe, uint32_t ipb, uint64_t k,
                 double *mean_out)
{
    // a batch's value: the exact 128-bit sum of its items' probes (low and
    // high 64-bit words), converted to weight units once, so it does not
    // depend on how many items the batch was split into
    std::vector<double> x(k, 0.0);
    for (uint64_t j = 0; j < k; ++j) {
        unsigned __int128 v = 0;
        for (uint32_t i = 0; i < ipb; ++i) {
            const uint64_t g = j * ipb + i;
            v += ((unsigned __int128)probe[2 * g + 1] << 64) + probe[2 * g];
        }
        x[j] = (double)(unsigned long long)(v >> 64) * 0x1p24 + (double)(unsigned long long)v * 0x1p-40;
    }
    double sum = 0.0;
    for (uint64_t j = 0; j < k; ++j)
        sum += x[j];
    const double m = sum / (double)k;
    double ss = 0.0;
    for (uint64_t j = 0; j < k; ++j)
        ss += (x[j] - m) * (x[j] - m);
    *mean_out = m;
    if (!(m > 0.0) || k < 2)
        return NAN;
    return std::sqrt(ss / (double)(k - 1) / (double)k) / m;
}

int finish(tmc_server *s, Req &q, bool reached, double rse)
{
    Done dn;
    dn.tally.resize(q.r.shells);
    unsigned long long st = 0;
    cudaError_t e = cudaMemcpy(dn.tally.data(), s->d_tally + 4ull * q.slot * s->cfg.max_shells,
                               sizeof(tmc_tally) * q.r.shells, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(&st, s->d_steps + q.slot, sizeof st, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return set_cuda_error(e, "server result copy");
    dn.res.photons = q.done * (uint64_t)q.item_photons;
    dn.res.photon_steps = st;
    dn.res.batches = (uint32_t)(q.done / q.items_per_batch);
    dn.res.batch_photons = q.batch;
    dn.res.rse = rse;
    dn.res.reached_target = reached ? 1 : 0;
    dn.res.latency_s = now_s() - q.t_submit;
    s->photons += dn.res.photons;
    s->steps += st;
    s->finished[q.id] = std::move(dn);
    s->free_slots.push_back(q.slot);
    return TMC_OK;
}

// Decide a request whose items up to its decision point are all back.
int decide(tmc_server *s, uint64_t id)
{
    auto f = s->active.find(id);
    if (f == s->active.end())
        return TMC_OK;
    Req &q = f->second;
    if (q.done != q.next_decision * q.items_per_batch)
        return TMC_OK;
    tmc::NvtxRange nvtx_range("tmc_server decision");
    double m = 0.0;
    const double rse = batch_rse(q.probe, q.items_per_batch, q.next_decision, &m);
    const bool reached = (rse == rse) && rse <= q.r.target_rse;
    if (reached || q.next_decision >= q.max_batches) {
        int st = finish(s, q, reached, rse);
        if (st)
            return st;
        s->order.erase(std::find(s->order.begin(), s->order.end(), id));
        s->active.erase(f);
    } else {
        q.next_decision = std::min(2 * q.next_decision, q.max_batches);
    }
    return TMC_OK;
}

// Take the items of a wave that have finished (its completion ring, in
// finishing order), store their probe values and decide where possible.
// ended: the wave's launch and its error-flag copy are complete, so every
// item is in the ring unless a bounded device wait ran out.
int harvest(tmc_server *s, Wave &w, bool ended)
{
    if (ended && *w.h_err) {
        set_error_text("server wave: a bounded device wait ran out");
        return TMC_E_TIMEOUT;
    }
    std::vector<uint64_t> touched;
    while (w.head < w.n_items) {
        unsigned long long *e = w.h_ring + 4 * (size_t)w.head;
        if (__atomic_load_n(&e[3], __ATOMIC_ACQUIRE) == 0)
            break;
        const uint64_t i = e[2];
        if (i >= w.n_items) {
            set_error_text("server wave: bad completion-ring entry");
            return TMC_E_STATE;
        }
        const BatchItemDev &it = w.h_items[i];
        const uint64_t id = s->slot_req[it.problem];
        auto f = s->active.find(id);
        if (f == s->active.end() || f->second.item_photons == 0 ||
            2 * (it.first / f->second.item_photons) + 1 >= f->second.probe.size()) {
            set_error_text("server wave: a finished item matches no running request");
            return TMC_E_STATE;
        }
        Req &q = f->second;
        const uint64_t g = it.first / q.item_photons;
        q.probe[2 * g] = e[0];
        q.probe[2 * g + 1] = e[1];
        ++q.done;
        --s->inflight;
        touched.push_back(id);
        ++w.head;
    }
    std::sort(touched.begin(), touched.end());
    touched.erase(std::unique(touched.begin(), touched.end()), touched.end());
    for (uint64_t id : touched) {
        int st = decide(s, id);
        if (st)
            return st;
    }
    if (ended) {
        if (w.head != w.n_items) {
            set_error_text("server wave: finished items missing from the completion ring");
            return TMC_E_STATE;
        }
        w.busy = false;
        w.n_items = 0;
    }
    return TMC_OK;
}

// Take up to cap_n pending items: least attained service first (requests
// with the fewest photon steps issued so far, i.e. new requests' first rounds,
// go ahead of the later, larger rounds of long-running ones; ties in
// admission order), at most `quota` items per request.  put(item, request id,
// item index within the request) receives them in order.
template <class Put>
uint32_t take_pending(tmc_server *s, uint64_t cap_n, uint64_t quota_base, Put put)
{
    uint32_t n = 0;
    std::vector<std::pair<double, uint64_t>> pend;
    for (uint64_t id : s->order) {
        auto f = s->active.find(id);
        if (f == s->active.end())
            continue;
        const Req &q = f->second;
        if (q.issued < q.next_decision * q.items_per_batch)
            pend.push_back({(double)q.issued * q.item_photons * q.est_steps, id});
    }
    if (pend.empty() || cap_n == 0)
        return 0;
    const uint64_t quota = std::max<uint64_t>(
        16, std::min<uint64_t>(s->cfg.max_items_per_request, quota_base / pend.size()));
    std::stable_sort(pend.begin(), pend.end(),
                     [](const auto &x, const auto &y) { return x.first < y.first; });
    for (size_t c = 0; c < pend.size() && n < cap_n; ++c) {
        Req &q = s->active.find(pend[c].second)->second;   // present: collected above
        const uint64_t limit = q.next_decision * q.items_per_batch;
        const uint64_t k = std::min<uint64_t>({limit - q.issued, quota, cap_n - n});
        for (uint64_t j = 0; j < k; ++j) {
            BatchItemDev it;
            it.problem = (uint32_t)q.slot;
            it.count = q.item_photons;
            it.first = (q.issued + j) * (uint64_t)q.item_photons;
            put(it, q.id, q.issued + j);
            ++n;
        }
        q.issued += k;
        if (q.probe.size() < 2 * q.issued)
            q.probe.resize(2 * q.issued, 0ull);
    }
    return n;
}

// Fill a wave with pending items (take_pending's order) and launch it.
int launch_wave(tmc_server *s, Wave &w)
{
    tmc::NvtxRange nvtx_range("tmc_server wave launch");
    const uint64_t room = s->cfg.inflight_items
                              ? (s->inflight < s->cfg.inflight_items ? s->cfg.inflight_items - s->inflight : 0)
                              : ~0ull;
    const uint64_t cap_n = std::min<uint64_t>(s->wave_cap, room);
    uint32_t n = 0;
    take_pending(s, cap_n, s->wave_cap,
                 [&](const BatchItemDev &it, uint64_t, uint64_t) { w.h_items[n++] = it; });
    if (n == 0)
        return TMC_OK;
    w.n_items = n;
    w.head = 0;
    s->inflight += n;
    std::memset(w.h_ring, 0, 4 * sizeof(unsigned long long) * n);   // the wave is idle
    cudaError_t e = cudaMemcpyAsync(w.d_items, w.h_items, sizeof(BatchItemDev) * n,
                                    cudaMemcpyHostToDevice, w.stream);
    if (e == cudaSuccess)   // item counter, error flag, ring tail
        e = cudaMemsetAsync(w.d_counter, 0, 3 * sizeof(unsigned long long), w.stream);
    if (e == cudaSuccess) {
        BatchArgs a{};
        a.keys = s->keys;
        a.problems = s->d_problems;
        a.items = w.d_items;
        a.n_items = n;
        a.max_shells = s->cfg.max_shells;
        a.probe_shell = s->cfg.probe_shell;
        a.tally = s->d_tally;
        a.steps = s->d_steps;
        a.item_counter = w.d_counter;
        a.item_probe = nullptr;
        a.error = reinterpret_cast<unsigned *>(w.d_counter + 1);
        a.done_ring = w.d_ring;
        a.done_tail = reinterpret_cast<unsigned *>(w.d_counter + 2);
        a.wait_limit_ns = 0;
        a.hold_buffers = nullptr;
        if (s->cfg.stream)
            e = walk_stream_launch(a, (int)s->cfg.block, s->cfg.math,
                                   std::max(1, std::min<int>(s->grid, (int)n)), w.stream);
        else
            e = walk_batch_launch(a, (int)s->cfg.block, s->cfg.math,
                                  std::max(1, std::min<int>(s->grid, (int)n)), w.stream);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(w.h_err, w.d_counter + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                            w.stream);
    if (e == cudaSuccess)
        e = cudaEventRecord(w.done, w.stream);
    if (e != cudaSuccess)
        return set_cuda_error(e, "server wave launch");
    w.busy = true;
    ++s->n_waves;
    return TMC_OK;
}

// ------------------------------------------------------- persistent mode

// Take the finished queue items from the completion ring (in finishing
// order: only new entries are read), store their probes, free their pool
// slots, decide.
int harvest_queue(tmc_server *s)
{
    Queue &Q = s->q;
    std::vector<uint64_t> touched;
    for (;;) {
        unsigned long long *e = Q.h_ring + 4 * (size_t)(Q.done_head & (Q.cap - 1));
        if (__atomic_load_n(&e[3], __ATOMIC_ACQUIRE) == 0)
            break;
        const uint64_t slot = e[2];
        if (slot >= Q.cap || Q.state[slot] != 1) {
            set_error_text("server queue: completion entry for an item not in flight");
            return TMC_E_STATE;
        }
        auto f = s->active.find(Q.req[slot]);
        if (f == s->active.end() || 2 * Q.g[slot] + 1 >= f->second.probe.size()) {
            set_error_text("server queue: a finished item matches no running request");
            return TMC_E_STATE;
        }
        Req &q = f->second;
        q.probe[2 * Q.g[slot]] = e[0];
        q.probe[2 * Q.g[slot] + 1] = e[1];
        ++q.done;
        --s->inflight;
        // free for a later completion, which comes only after more publishing
        __atomic_store_n(&e[3], 0ull, __ATOMIC_RELAXED);
        ++Q.done_head;
        Q.state[slot] = 0;
        Q.free_slots.push_back((uint32_t)slot);
        touched.push_back(q.id);
    }
    std::sort(touched.begin(), touched.end());
    touched.erase(std::unique(touched.begin(), touched.end()), touched.end());
    for (uint64_t id : touched) {
        int st = decide(s, id);
        if (st)
            return st;
    }
    return TMC_OK;
}

// Publish pending items into free pool slots, keeping at most
// inflight_items published and unfinished (so a new request's first round
// waits behind at most that many items), then release the new count.  A
// queue position is reused 2 x cap positions later, when at least cap more
// items have finished, all claimed after it.
void publish_queue(tmc_server *s)
{
    Queue &Q = s->q;
    const uint64_t budget = std::min<uint64_t>(
        Q.cap, s->cfg.inflight_items ? s->cfg.inflight_items : 2ull * (uint64_t)s->grid);
    const uint64_t room = s->inflight < budget ? std::min<uint64_t>(budget - s->inflight, Q.free_slots.size()) : 0;
    const uint32_t n = take_pending(s, room, budget, [&](const BatchItemDev &it, uint64_t id, uint64_t g) {
        const uint32_t slot = Q.free_slots.back();
        Q.free_slots.pop_back();
        Q.h_items[slot] = it;
        Q.req[slot] = id;
        Q.g[slot] = g;
        Q.state[slot] = 1;
        Q.h_order[Q.published & (2 * Q.cap - 1)] = slot;
        ++Q.published;
    });
    if (n) {
        s->inflight += n;
        __atomic_store_n(Q.h_pub, (unsigned long long)Q.published, __ATOMIC_RELEASE);
    }
}

int launch_persistent(tmc_server *s, Wave &w)
{
    tmc::NvtxRange nvtx_range("tmc_server persistent launch");
    Queue &Q = s->q;
    BatchArgs a{};
    a.keys = s->keys;
    a.problems = Q.d_problems;
    a.max_shells = s->cfg.max_shells;
    a.probe_shell = s->cfg.probe_shell;
    a.tally = s->d_tally;
    a.steps = s->d_steps;
    a.item_counter = Q.d_counter;
    a.error = reinterpret_cast<unsigned *>(Q.d_counter + 1);
    a.done_ring = Q.d_ring;
    a.q_items = Q.d_items;
    a.q_order = Q.d_order;
    a.q_published = Q.d_pub;
    a.q_mode = Q.d_mode;
    a.q_live = reinterpret_cast<unsigned *>(Q.d_counter + 2);
    a.done_tail = reinterpret_cast<unsigned *>(Q.d_counter + 3);
    a.q_cap = Q.cap;
    a.idle_limit_ns = 20ull * 1000000ull;   // with no request active, blocks end after 20 ms
    // the launch's end record; nothing goes on the stream after the kernel
    const size_t k = (size_t)(&w - s->waves);
    __atomic_store_n(&Q.h_end[2 * k], 0u, __ATOMIC_RELAXED);
    Q.h_end[2 * k + 1] = 0u;
    a.q_done_blocks = Q.d_done + k;
    a.q_ended = Q.d_end + 2 * k;
    cudaError_t e = cudaMemcpyAsync(Q.d_done + k, s->h_zero, sizeof(unsigned), cudaMemcpyHostToDevice, w.stream);
    if (e == cudaSuccess)
        e = s->cfg.stream ? walk_stream_launch(a, (int)s->cfg.block, s->cfg.math, s->grid, w.stream)
                          : walk_batch_launch(a, (int)s->cfg.block, s->cfg.math, s->grid, w.stream);
    if (e != cudaSuccess)
        return set_cuda_error(e, "server persistent launch");
    w.busy = true;
    w.n_items = 0;
    ++s->n_waves;
    Q.drained = false;
    return TMC_OK;
}

int progress_persistent(tmc_server *s)
{
    Queue &Q = s->q;
    uint32_t running = 0;
    for (Wave &w : s->waves) {
        if (!w.busy)
            continue;
        const size_t k = (size_t)(&w - s->waves);
        if (__atomic_load_n(&Q.h_end[2 * k], __ATOMIC_ACQUIRE) == 0) {
            ++running;
            continue;
        }
        w.busy = false;
        if (Q.h_end[2 * k + 1]) {
            set_error_text("server persistent launch: a bounded device wait ran out");
            return TMC_E_TIMEOUT;
        }
    }
    int st = harvest_queue(s);
    if (st)
        return st;
    // blocks wait for work while requests are active, and end once none are
    const unsigned mode = s->active.empty() ? QUEUE_DRAIN : QUEUE_HOLD;
    if (mode != Q.mode) {
        Q.mode = mode;
        __atomic_store_n(Q.h_mode, mode, __ATOMIC_RELEASE);
        if (mode == QUEUE_DRAIN)
            Q.drained = true;
    }
    publish_queue(s);
    // a launch is needed when work is queued and no launch runs, or when the
    // running ones may be ending (the mode was DRAIN since they started)
    if (s->inflight > 0 && (running == 0 || (Q.drained && mode == QUEUE_HOLD))) {
        const uint32_t cap = s->cfg.waves ? s->cfg.waves : DEFAULT_WAVES;
        for (Wave &w : s->waves) {
            if (running >= cap)
                break;
            if (w.busy)
                continue;
            return launch_persistent(s, w);
        }
    }
    return TMC_OK;
}

int progress_locked(tmc_server *s)
{
    if (s->cfg.persistent)
        return progress_persistent(s);
    for (Wave &w : s->waves) {
        if (!w.busy)
            continue;
        const cudaError_t e = cudaEventQuery(w.done);
        if (e != cudaSuccess && e != cudaErrorNotReady)
            return set_cuda_error(e, "server wave");
        int st = harvest(s, w, e == cudaSuccess);
        if (st)
            return st;
    }
    const uint32_t cap = s->cfg.waves ? s->cfg.waves : DEFAULT_WAVES;
    uint32_t busy = 0;
    for (const Wave &w : s->waves)
        busy += w.busy ? 1u : 0u;
    for (Wave &w : s->waves) {
        if (busy >= cap || (s->cfg.inflight_items && s->inflight >= s->cfg.inflight_items))
            break;
        if (w.busy)
            continue;
        int st = launch_wave(s, w);
        if (st)
            return st;
        busy += w.busy ? 1u : 0u;
    }
    return TMC_OK;
}

bool config_valid(const tmc_server_config &c)
{
    return c.slots > 0 && c.slots <= (1u << 20) && c.max_shells > 0 && c.max_shells <= (1u << 16) &&
           c.min_batches >= 2 && c.max_items_per_request > 0 && c.steps_per_batch > 0.0 &&
           c.steps_per_item >= 0.0 && c.waves <= (uint32_t)WAVES &&
           (c.math == TMC_MATH_EXACT || c.math == TMC_MATH_FAST) &&
           (c.block == 128 || c.block == 256 || c.block == 512) && c.persistent <= 1;
}

// The request's knobs as tmc_params checks them, plus the server's own limits.
int request_valid(const tmc_server_config &c, const tmc_request &r)
{
    tmc_params p;
    tmc_params_default(&p);
    p.shells = r.shells;
    p.microns_per_shell = r.microns_per_shell;
    p.mu_a = r.mu_a;
    p.mu_s = r.mu_s;
    int st = validate(&p);
    if (st)
        return st;
    if (r.shells > c.max_shells || !(r.target_rse > 0.0) || r.max_photons == 0 ||
        r.max_photons > (1ull << 40) || r.photon_id_base > ~0ull - r.max_photons)
        return TMC_E_INVALID;
    return TMC_OK;
}

}  // namespace

extern "C" {

void tmc_server_config_default(tmc_server_config *c)
{
    if (!c)
        return;
    std::memset(c, 0, sizeof *c);
    c->slots = 1024;
    c->max_shells = 501;
    c->probe_shell = 10;
    c->min_batches = 16;
    c->seed = 1;
    c->math = TMC_MATH_FAST;
    c->block = 128;
    c->max_items_per_request = 1024;
    c->steps_per_batch = 8388608.0;
}

int tmc_server_create(tmc_server **out, const tmc_server_config *cfg)
{
    if (!out || !cfg)
        return TMC_E_INVALID;
    *out = nullptr;
    if (!config_valid(*cfg))
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    int st = TMC_OK;
    DeviceCtx *c = current_ctx(&st);
    if (!c)
        return st;
    std::unique_ptr<tmc_server, void (*)(tmc_server *)> s(new tmc_server, destroy_server);
    s->cfg = *cfg;
    cfg = &s->cfg;
    s->device = c->device;
    s->sms = c->sms;
    s->keys = make_philox_keys(cfg->seed);
    const size_t smem = cfg->stream ? walk_stream_smem(cfg->max_shells, (int)cfg->block)
                                    : walk_batch_smem(cfg->max_shells, (int)cfg->block);
    if (smem > c->smem_optin) {
        set_error_text("tmc_server_create: max_shells too large for the shared-memory histograms");
        return TMC_E_INVALID;
    }
    cudaError_t e = cfg->stream ? walk_stream_prepare((int)cfg->block, cfg->math, cfg->max_shells, c->sms, &s->grid,
                                                      cfg->persistent != 0)
                                : walk_batch_prepare((int)cfg->block, cfg->math, cfg->max_shells, c->sms, &s->grid,
                                                     cfg->persistent != 0);
    if (e != cudaSuccess)
        return set_cuda_error(e, "server kernel config");
    const size_t slots = cfg->slots;
    s->slot_req.assign(slots, 0);
    s->wave_cap = (uint32_t)std::max(1024, 4 * s->grid);
    s->items_cap = s->wave_cap;
    e = cudaMalloc(&s->d_problems, sizeof(BatchProblemDev) * slots);
    if (e == cudaSuccess)
        e = cudaMalloc(&s->d_tally, sizeof(tmc_tally) * slots * cfg->max_shells);
    if (e == cudaSuccess)
        e = cudaMalloc(&s->d_steps, sizeof(unsigned long long) * slots);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&s->admin, cudaStreamNonBlocking);
    for (Wave &w : s->waves) {
        if (e == cudaSuccess)
            e = cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming);
        if (e == cudaSuccess)
            e = cudaMalloc(&w.d_items, sizeof(BatchItemDev) * s->items_cap);
        if (e == cudaSuccess)
            e = cudaMalloc(&w.d_counter, 3 * sizeof(unsigned long long));
        if (e == cudaSuccess)
            e = cudaMallocHost(&w.h_err, sizeof(unsigned long long));
        if (e == cudaSuccess)
            e = cudaMallocHost(&w.h_items, sizeof(BatchItemDev) * s->items_cap);
        if (e == cudaSuccess)
            e = cudaHostAlloc(&w.h_ring, 4 * sizeof(unsigned long long) * s->items_cap, cudaHostAllocMapped);
        if (e == cudaSuccess)
            e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&w.d_ring), w.h_ring, 0);
    }
    if (e == cudaSuccess)
        e = cudaMallocHost(&s->h_zero, sizeof(tmc_tally) * cfg->max_shells);
    if (e == cudaSuccess)
        std::memset(s->h_zero, 0, sizeof(tmc_tally) * cfg->max_shells);
    if (e == cudaSuccess && cfg->persistent) {
        Queue &Q = s->q;
        Q.cap = 1;
        while (Q.cap < std::max<uint32_t>(4096, 4 * (uint32_t)s->grid))
            Q.cap *= 2;
        Q.req.assign(Q.cap, 0);
        Q.g.assign(Q.cap, 0);
        Q.state.assign(Q.cap, 0);
        Q.free_slots.resize(Q.cap);
        for (uint32_t i = 0; i < Q.cap; ++i)
            Q.free_slots[i] = Q.cap - 1 - i;
        auto mapped = [&](auto **h, auto **d, size_t bytes) {
            cudaError_t r = cudaHostAlloc(reinterpret_cast<void **>(h), bytes, cudaHostAllocMapped);
            if (r == cudaSuccess) {
                std::memset(*h, 0, bytes);
                r = cudaHostGetDevicePointer(reinterpret_cast<void **>(d), *h, 0);
            }
            return r;
        };
        e = mapped(&Q.h_items, &Q.d_items, sizeof(BatchItemDev) * Q.cap);
        if (e == cudaSuccess)
            e = mapped(&Q.h_order, &Q.d_order, sizeof(uint32_t) * 2 * Q.cap);
        if (e == cudaSuccess)
            e = mapped(&Q.h_pub, &Q.d_pub, sizeof(unsigned long long));
        if (e == cudaSuccess)
            e = mapped(&Q.h_mode, &Q.d_mode, sizeof(unsigned));
        if (e == cudaSuccess)
            e = mapped(&Q.h_ring, &Q.d_ring, 4 * sizeof(unsigned long long) * Q.cap);
        if (e == cudaSuccess)
            e = mapped(&Q.h_problems, &Q.d_problems, sizeof(BatchProblemDev) * slots);
        if (e == cudaSuccess)
            e = mapped(&Q.h_end, &Q.d_end, 2 * sizeof(unsigned) * WAVES);
        if (e == cudaSuccess)
            e = cudaMalloc(&Q.d_done, sizeof(unsigned) * WAVES);
        if (e == cudaSuccess)
            e = cudaMalloc(&Q.d_counter, 4 * sizeof(unsigned long long));
        if (e == cudaSuccess)
            e = cudaMemset(Q.d_counter, 0, 4 * sizeof(unsigned long long));
        if (e == cudaSuccess)
            *Q.h_mode = QUEUE_DRAIN;
    }
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_server_create");
    for (int i = (int)slots - 1; i >= 0; --i)
        s->free_slots.push_back(i);
    *out = s.release();
    return TMC_OK;
}

int tmc_server_submit(tmc_server *s, const tmc_request *r, uint64_t *id)
{
    tmc::NvtxRange nvtx_range("tmc_server_submit");
    if (!s || !r)
        return TMC_E_INVALID;
    int st = request_valid(s->cfg, *r);
    if (st)
        return st;
    std::lock_guard<std::mutex> lk(api_mutex());
    if (s->free_slots.empty())
        return TMC_E_BUSY;
    Req q;
    q.id = s->next_id++;
    q.r = *r;
    q.d = derive(r->mu_a, r->mu_s, r->microns_per_shell, r->shells);
    const double est = expected_steps_host(q.d.albedo);
    q.est_steps = est;
    q.batch = batch_photons(s->cfg, est);
    q.items_per_batch = items_per_batch(s->cfg, q.batch, est);
    q.item_photons = q.batch / q.items_per_batch;
    q.max_batches = std::max<uint64_t>(1, (r->max_photons + q.batch - 1) / q.batch);
    q.next_decision = std::min<uint64_t>(s->cfg.min_batches, q.max_batches);
    q.slot = s->free_slots.back();
    q.t_submit = now_s();
    BatchProblemDev pd;
    pd.c.albedo = q.d.albedo;
    pd.c.spm = q.d.spm;
    pd.c.last = q.d.last;
    pd.c.shells = q.d.shells;
    pd.id_base = r->photon_id_base;
    pd.tally_offset = (unsigned long long)q.slot * s->cfg.max_shells;
    cudaError_t e = cudaSuccess;
    if (s->cfg.persistent)   // read by the kernel only after the request's items are published
        s->q.h_problems[q.slot] = pd;
    else
        e = cudaMemcpyAsync(s->d_problems + q.slot, &pd, sizeof pd, cudaMemcpyHostToDevice, s->admin);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_tally + 4ull * q.slot * s->cfg.max_shells, s->h_zero,
                            sizeof(tmc_tally) * s->cfg.max_shells, cudaMemcpyHostToDevice, s->admin);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_steps + q.slot, s->h_zero, sizeof(unsigned long long), cudaMemcpyHostToDevice,
                            s->admin);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s->admin);
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_server_submit");
    s->free_slots.pop_back();
    s->slot_req[q.slot] = q.id;
    if (id)
        *id = q.id;
    s->order.push_back(q.id);
    s->active.emplace(q.id, std::move(q));
    return TMC_OK;
}

int tmc_server_progress(tmc_server *s, uint32_t *waves_in_flight, uint32_t *active_requests)
{
    if (!s)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    int st = progress_locked(s);
    if (waves_in_flight) {
        uint32_t n = 0;
        for (const Wave &w : s->waves)
            n += w.busy ? 1 : 0;
        *waves_in_flight = n;
    }
    if (active_requests)
        *active_requests = (uint32_t)s->active.size();
    return st;
}

int tmc_server_poll(tmc_server *s, uint64_t id, int *done)
{
    if (!s || !done)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    if (s->finished.count(id)) {
        *done = 1;
        return TMC_OK;
    }
    if (s->active.count(id)) {
        *done = 0;
        return TMC_OK;
    }
    return TMC_E_STATE;
}

int tmc_server_result(tmc_server *s, uint64_t id, tmc_tally *tally, tmc_request_result *res)
{
    if (!s)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    auto f = s->finished.find(id);
    if (f == s->finished.end())
        return TMC_E_STATE;
    if (tally)
        std::memcpy(tally, f->second.tally.data(), sizeof(tmc_tally) * f->second.tally.size());
    if (res)
        *res = f->second.res;
    s->finished.erase(f);
    return TMC_OK;
}

int tmc_server_stats(tmc_server *s, uint64_t *photons, uint64_t *photon_steps, uint64_t *waves)
{
    if (!s)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    if (photons)
        *photons = s->photons;
    if (photon_steps)
        *photon_steps = s->steps;
    if (waves)
        *waves = s->n_waves;
    return TMC_OK;
}

int tmc_server_work(tmc_server *s, uint64_t *photon_steps)
{
    if (!s || !photon_steps)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    // finished requests plus the device counters of the running ones (a wave
    // adds to them as its blocks finish items)
    std::vector<unsigned long long> cur(s->cfg.slots, 0);
    cudaError_t e = cudaMemcpyAsync(cur.data(), s->d_steps, sizeof(unsigned long long) * s->cfg.slots,
                                    cudaMemcpyDeviceToHost, s->admin);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s->admin);
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_server_work");
    uint64_t t = s->steps;
    for (const auto &kv : s->active)
        t += cur[kv.second.slot];
    *photon_steps = t;
    return TMC_OK;
}

int tmc_server_run_trace(tmc_server *s, const tmc_request *reqs, const double *arrival_s, uint32_t n,
                         double time_limit_s, tmc_request_result *results, uint32_t *completed)
{
    if (!s || (n && (!reqs || !arrival_s || !results)))
        return TMC_E_INVALID;
    for (uint32_t i = 1; i < n; ++i)
        if (arrival_s[i] < arrival_s[i - 1])
            return TMC_E_INVALID;
    std::vector<uint64_t> ids(n, 0);
    std::unordered_map<uint64_t, uint32_t> index;
    std::unordered_map<uint64_t, double> submit_t;
    for (uint32_t i = 0; i < n; ++i)
        std::memset(&results[i], 0, sizeof results[i]);
    const double t0 = now_s();
    uint32_t next = 0, done = 0;
    int st = TMC_OK;
    while (done < n) {
        const double t = now_s() - t0;
        if (time_limit_s > 0.0 && t > time_limit_s)
            break;
        // admit everything that has arrived, in order, while slots are free
        while (next < n && arrival_s[next] <= t) {
            uint64_t id = 0;
            st = tmc_server_submit(s, &reqs[next], &id);
            if (st == TMC_E_BUSY)
                break;
            if (st)
                return st;
            ids[next] = id;
            index[id] = next;
            submit_t[id] = s->active.count(id) ? s->active[id].t_submit : now_s();
            ++next;
        }
        uint32_t in_flight = 0, act = 0;
        if ((st = tmc_server_progress(s, &in_flight, &act)))
            return st;
        // collect completions
        std::vector<uint64_t> fin;
        {
            std::lock_guard<std::mutex> lk(api_mutex());
            for (auto &kv : s->finished)
                if (index.count(kv.first))
                    fin.push_back(kv.first);
        }
        for (uint64_t id : fin) {
            const uint32_t i = index[id];
            tmc_request_result r;
            if ((st = tmc_server_result(s, id, nullptr, &r)))
                return st;
            // latency from arrival, not from admission: completion time is
            // submission time + the server's latency
            const double t_sub = (double)(submit_t.count(id) ? submit_t[id] : t0);
            r.latency_s = (t_sub + r.latency_s) - (t0 + arrival_s[i]);
            submit_t.erase(id);
            results[i] = r;
            index.erase(id);
            ++done;
        }
        if (fin.empty())
            std::this_thread::sleep_for(std::chrono::microseconds(in_flight ? 20 : 200));
    }
    if (completed)
        *completed = done;
    return TMC_OK;
}

int tmc_server_plan(const tmc_server_config *cfg, const tmc_request *r, uint32_t *batch,
                    uint32_t *items_per_batch_out, double *steps_per_photon)
{
    if (!cfg || !r || !config_valid(*cfg))
        return TMC_E_INVALID;
    const int st = request_valid(*cfg, *r);
    if (st)
        return st;
    const Derived d = derive(r->mu_a, r->mu_s, r->microns_per_shell, r->shells);
    const double est = expected_steps_host(d.albedo);
    const uint32_t b = batch_photons(*cfg, est);
    if (batch)
        *batch = b;
    if (items_per_batch_out)
        *items_per_batch_out = items_per_batch(*cfg, b, est);
    if (steps_per_photon)
        *steps_per_photon = est;
    return TMC_OK;
}

int tmc_batch_means_rse(const uint64_t *probes, uint32_t items_per_batch_in, uint64_t n_batches,
                        double *rse, double *mean)
{
    if (!probes || items_per_batch_in == 0 || n_batches == 0 || !rse)
        return TMC_E_INVALID;
    std::vector<unsigned long long> v(probes, probes + 2 * (size_t)items_per_batch_in * n_batches);
    double m = 0.0;
    *rse = batch_rse(v, items_per_batch_in, n_batches, &m);
    if (mean)
        *mean = m;
    return TMC_OK;
}

int tmc_server_destroy(tmc_server *s)
{
    if (!s)
        return TMC_OK;
    std::lock_guard<std::mutex> lk(api_mutex());
    destroy_server(s);
    return TMC_OK;
}

}  // extern "C"
