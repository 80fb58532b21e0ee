// tmc_batch.cu — many independent walks (problems of different optics, shell
// counts and photon counts) in ONE persistent launch.
//
// Reference: each problem is what tiny_mc.c:34-69 computes for one set of
// params.h knobs; the reference runs one problem per process.  Here:
//
//  * the host splits every problem into work items (photon-id ranges) of
//    roughly equal estimated photon steps — the expected steps per photon of
//    photon.c's weight recursion times the photon count — so a problem of
//    6e5 steps per photon is spread over many blocks while a problem of a few
//    steps per photon stays one item; items are ordered heaviest first;
//  * each resident block takes the next item from a global counter, zeroes
//    its shared-memory histogram for that problem's shells, walks the item's
//    photons with the same loop as the plain kernel (warps claim photons from
//    a shared-memory counter; a warp whose lane reaches a multiple of
//    flush_steps(BLOCK) steps swaps the histogram into the problem's global
//    tally), then adds what is left to the problem's 128-bit global tally and
//    takes the next item;
//  * results are integer tallies keyed by photon id, so each problem's tally
//    is bit-identical to the plain kernel's for the same photons, whatever
//    the item split, block size or order;
//  * a batch can be replayed through a captured CUDA graph (zeroing + walk),
//    and an autotuner picks block size and item granularity by timing a
//    reduced copy of the batch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "tmc_batch.cuh"
#include "tmc_internal.h"
#include "tmc_walk.cuh"

namespace tmc {

// QUEUE: the request server's persistent launch (BatchArgs, queue mode):
// thread 0 claims each item from the ring in mapped host memory, waiting with
// back-off while nothing is published (bounded: see queue_idle_verdict), and
// each finished item's completion is appended to the completion ring.
template <int BLOCK, class M, bool QUEUE>
__global__ void __launch_bounds__(BLOCK) walk_batch(const BatchArgs a)
{
    constexpr uint32_t END = 0xffffffffu;
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ uint32_t sh_item, sh_next, sh_probe_hi;
    __shared__ unsigned long long sh_probe_acc;
    __shared__ BatchItemDev sh_itm;
    __shared__ BatchProblemDev sh_pr;
    __shared__ unsigned long long sh_qidx;
    uint32_t *my = smem + 4 * a.max_shells + threadIdx.x;
    if (QUEUE && threadIdx.x == 0 && a.q_live)
        atomicAdd(a.q_live, 1u);

    for (;;) {
        if (threadIdx.x == 0) {
            if constexpr (QUEUE) {
                unsigned long long idle_since = 0;
                sh_item = END;
                for (;;) {
                    BatchItemDev itm;
                    BatchProblemDev pr;
                    unsigned long long c = 0;
                    if (queue_try_claim(a, itm, pr, c)) {
                        sh_itm = itm;
                        sh_pr = pr;
                        sh_qidx = c;
                        sh_item = (uint32_t)(c & (a.q_cap - 1));
                        break;
                    }
                    const unsigned long long now = global_ns();
                    if (idle_since == 0)
                        idle_since = now;
                    if (queue_idle_verdict(a, now - idle_since))
                        break;
                    __nanosleep(256u + (unsigned)min((now - idle_since) >> 4, 16384ull));
                }
            } else {
                sh_item = (uint32_t)min(atomicAdd(a.item_counter, 1ull), 0xffffffffull);
            }
            sh_next = 0;
            sh_probe_hi = 0;
            sh_probe_acc = 0;
        }
        __syncthreads();
        const uint32_t it = sh_item;
        if (QUEUE ? it == END : it >= a.n_items)
            break;
        const BatchItemDev item = QUEUE ? sh_itm : a.items[it];
        const BatchProblemDev pr = QUEUE ? sh_pr : a.problems[item.problem];
        const uint32_t S = pr.c.shells;
        for (uint32_t s = threadIdx.x; s < 4 * S; s += BLOCK)
            smem[s] = 0;
        __syncthreads();

        SharedSource<BATCH_CHUNK> src;
        src.counter = &sh_next;
        src.count = item.count;
        src.first = pr.id_base + item.first;
        unsigned long long *g = a.tally + 4 * pr.tally_offset;
        const uint32_t ps = min(a.probe_shell, S - 1);
        const bool probe = a.item_probe || a.done_ring;
        const uint32_t steps = walk_loop<BLOCK, M, SharedSource<BATCH_CHUNK>, Hist::Block>(
            pr.c, src, a.keys, smem, g, my, probe ? &sh_probe_acc : nullptr,
            probe ? &sh_probe_hi : nullptr, ps);

        __syncthreads();
        flush_tally<BLOCK>(smem, S, g);
        // this item's own sum of w in the probe shell, 128-bit: what the
        // walk's flushes took from the shell plus what is left in it
        const unsigned long long rest = ((unsigned long long)smem[S + ps] << 32) | smem[ps];
        const unsigned long long probe_lo = sh_probe_acc + rest;
        const uint32_t probe_hi = sh_probe_hi + (probe_lo < rest ? 1u : 0u);
        if (a.item_probe && threadIdx.x == 0) {
            a.item_probe[2 * (size_t)it] = probe_lo;
            a.item_probe[2 * (size_t)it + 1] = probe_hi;
        }
        const unsigned long long tot = warp_sum_u64(steps);
        if ((threadIdx.x & 31u) == 0 && tot)
            atomicAdd(&a.steps[item.problem], tot);
        if (a.done_ring)
            __threadfence();
        __syncthreads();
        if (a.done_ring && threadIdx.x == 0) {
            if constexpr (QUEUE)
                publish_item_at(a, sh_qidx, probe_lo, probe_hi);
            else
                publish_item(a, it, probe_lo, probe_hi);
        }
    }
    if (QUEUE && threadIdx.x == 0)
        queue_block_end(a);
}

template <int BLOCK, class M, bool QUEUE>
static cudaError_t walk_batch_config(int sms, size_t smem, int *grid)
{
    auto kern = walk_batch<BLOCK, M, QUEUE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BLOCK, smem);
    if (e != cudaSuccess)
        return e;
    if (per_sm < 1)
        return cudaErrorInvalidConfiguration;
    *grid = sms * per_sm;
    return cudaSuccess;
}

size_t walk_batch_smem(uint32_t max_shells, int block)
{
    return (size_t)16 * max_shells + (size_t)4 * SLOTS * block;
}

template <bool QUEUE>
static cudaError_t batch_prepare(int block, bool fast, size_t smem, int sms, int *grid)
{
    switch (block) {
    case 128: return fast ? walk_batch_config<128, FastMath, QUEUE>(sms, smem, grid)
                          : walk_batch_config<128, ExactMath, QUEUE>(sms, smem, grid);
    case 256: return fast ? walk_batch_config<256, FastMath, QUEUE>(sms, smem, grid)
                          : walk_batch_config<256, ExactMath, QUEUE>(sms, smem, grid);
    case 512: return fast ? walk_batch_config<512, FastMath, QUEUE>(sms, smem, grid)
                          : walk_batch_config<512, ExactMath, QUEUE>(sms, smem, grid);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t walk_batch_prepare(int block, uint32_t math, uint32_t max_shells, int sms, int *grid, bool queue)
{
    const size_t smem = walk_batch_smem(max_shells, block);
    const bool fast = math == TMC_MATH_FAST;
    return queue ? batch_prepare<true>(block, fast, smem, sms, grid)
                 : batch_prepare<false>(block, fast, smem, sms, grid);
}

template <int BLOCK>
static void batch_launch_b(const BatchArgs &a, bool fast, int grid, size_t smem, cudaStream_t s)
{
    if (a.q_items) {
        if (fast) walk_batch<BLOCK, FastMath, true><<<grid, BLOCK, smem, s>>>(a);
        else walk_batch<BLOCK, ExactMath, true><<<grid, BLOCK, smem, s>>>(a);
    } else {
        if (fast) walk_batch<BLOCK, FastMath, false><<<grid, BLOCK, smem, s>>>(a);
        else walk_batch<BLOCK, ExactMath, false><<<grid, BLOCK, smem, s>>>(a);
    }
}

cudaError_t walk_batch_launch(const BatchArgs &a, int block, uint32_t math, int grid, cudaStream_t s)
{
    const size_t smem = walk_batch_smem(a.max_shells, block);
    const bool fast = math == TMC_MATH_FAST;
    switch (block) {
    case 128: batch_launch_b<128>(a, fast, grid, smem, s); break;
    case 256: batch_launch_b<256>(a, fast, grid, smem, s); break;
    case 512: batch_launch_b<512>(a, fast, grid, smem, s); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

namespace {

// Expected photon steps per photon of photon.c's weight recursion: after k
// steps the weight is albedo^k; the first time it drops below 0.001 the
// photon survives with probability 0.1 and its weight is multiplied by 10.
double expected_steps(float albedo)
{
    if (!(albedo > 0.0f))
        return 1.0 / 0.9;
    const double la = std::log((double)albedo);
    double w = 1.0, e = 0.0, p = 1.0;
    for (int stage = 0; stage < 12 && p > 1e-12; ++stage) {
        double k = std::ceil(std::log(0.001 / w) / la);
        if (k < 1.0)
            k = 1.0;
        e += p * k;
        w = w * std::pow((double)albedo, k) / 0.1;
        p *= 0.1;
    }
    return e;
}

}  // namespace

}  // namespace tmc

using namespace tmc;

struct tmc_batch {
    std::vector<tmc_problem> problems;
    std::vector<Derived> derived;
    std::vector<double> est_steps;
    std::vector<unsigned long long> offsets;   // [n + 1] shell offsets
    uint64_t seed = 0;
    uint32_t math = TMC_MATH_EXACT;
    uint32_t max_shells = 0;
    tmc_batch_config cfg{256, 8, 0, 0};
    int device = -1;
    int sms = 0;
    int grid = 0;            // resident blocks for the current config (set by plan)
    size_t smem_optin = 0;
    // device buffers
    BatchProblemDev *d_problems = nullptr;
    BatchItemDev *d_items = nullptr;
    uint32_t n_items = 0;
    size_t items_cap = 0;
    unsigned long long *d_tally = nullptr;
    unsigned long long *d_steps = nullptr;
    unsigned long long *d_counter = nullptr;
    unsigned *d_hold = nullptr;          // test hook of walk_stream's waits (tmc_batch_test_wait)
    unsigned long long wait_limit_ns = 0;
    // graph
    cudaGraphExec_t graph = nullptr;
    cudaStream_t capture_stream = nullptr;
    cudaStream_t last_stream = nullptr;
    bool planned = false;
    // configurations timed by the last autotune on the reduced copy (ms, config)
    std::vector<std::pair<double, tmc_batch_config>> tuned;
};

namespace {

size_t batch_smem(const tmc_batch *b, int block)
{
    return b->cfg.stream ? walk_stream_smem(b->max_shells, block) : walk_batch_smem(b->max_shells, block);
}

cudaError_t grid_for(const tmc_batch *b, int *grid)
{
    return b->cfg.stream ? walk_stream_prepare(b->cfg.block, b->math, b->max_shells, b->sms, grid)
                         : walk_batch_prepare(b->cfg.block, b->math, b->max_shells, b->sms, grid);
}

// Split problems into items of about equal estimated photon steps.
// Split problems into work items (photon-id ranges) of about equal
// estimated photon steps for `grid` resident blocks of `block` threads with
// `items_per_block` items each, heaviest first.  Host only.
std::vector<BatchItemDev> plan_items(const std::vector<tmc_problem> &problems,
                                     const std::vector<double> &est_steps, int grid, int block,
                                     int items_per_block)
{
    double total = 0.0;
    for (size_t i = 0; i < problems.size(); ++i)
        total += est_steps[i] * (double)problems[i].n_photons;
    const double target = std::max(1.0, total / ((double)grid * std::max(1, items_per_block)));
    // Smallest item: two photons per thread of the block (a lane whose first
    // photon dies early takes a second one), or one photon per thread for a
    // problem whose photons are so long (high albedo: up to ~1e6 steps, each
    // walked serially by one lane) that two of them in a row would reach the
    // launch's expected steps per lane: spread one per lane, such photons
    // start in the first items and do not set the end of the launch.
    const double lane_steps = total / ((double)grid * block);
    std::vector<std::pair<double, BatchItemDev>> items;
    for (size_t i = 0; i < problems.size(); ++i) {
        const unsigned long long n = problems[i].n_photons;
        if (n == 0)
            continue;
        const unsigned long long min_item =
            (unsigned long long)block * (2.0 * est_steps[i] <= lane_steps ? 2 : 1);
        const double work = est_steps[i] * (double)n;
        unsigned long long k = (unsigned long long)std::ceil(work / target);
        k = std::max(1ull, std::min(k, (n + min_item - 1) / min_item));
        k = std::max(k, (n + 0x3fffffffull) / 0x40000000ull);   // counts stay below 2^30
        const unsigned long long per = n / k, extra = n % k;
        unsigned long long at = 0;
        for (unsigned long long j = 0; j < k; ++j) {
            const unsigned long long c = per + (j < extra ? 1 : 0);
            BatchItemDev it;
            it.problem = (uint32_t)i;
            it.count = (uint32_t)c;
            it.first = at;
            at += c;
            items.push_back({est_steps[i] * (double)c, it});
        }
    }
    std::stable_sort(items.begin(), items.end(),
                     [](const auto &x, const auto &y) { return x.first > y.first; });
    std::vector<BatchItemDev> h(items.size());
    for (size_t i = 0; i < items.size(); ++i)
        h[i] = items[i].second;
    return h;
}

int plan(tmc_batch *b)
{
    int grid = 0;
    cudaError_t e = grid_for(b, &grid);   // also sets the kernel's shared-memory limit
    if (e != cudaSuccess)
        return set_cuda_error(e, "batch kernel config");
    b->grid = grid;
    const std::vector<BatchItemDev> h =
        plan_items(b->problems, b->est_steps, grid, b->cfg.block, b->cfg.items_per_block);
    if (h.size() > b->items_cap) {
        if (b->d_items)
            cudaFree(b->d_items);
        b->d_items = nullptr;
        b->items_cap = 0;
        e = cudaMalloc(&b->d_items, sizeof(BatchItemDev) * std::max<size_t>(1, h.size()));
        if (e != cudaSuccess)
            return set_cuda_error(e, "cudaMalloc(batch items)");
        b->items_cap = std::max<size_t>(1, h.size());
    }
    if (!h.empty()) {
        e = cudaMemcpy(b->d_items, h.data(), sizeof(BatchItemDev) * h.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess)
            return set_cuda_error(e, "cudaMemcpy(batch items)");
    }
    b->n_items = (uint32_t)h.size();
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->planned = true;
    return TMC_OK;
}

cudaError_t enqueue(const tmc_batch *b, cudaStream_t s)
{
    const size_t n = b->problems.size();
    cudaError_t e = cudaMemsetAsync(b->d_tally, 0, sizeof(tmc_tally) * b->offsets[n], s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(b->d_steps, 0, sizeof(unsigned long long) * std::max<size_t>(1, n), s);
    if (e == cudaSuccess)   // item counter and error flag
        e = cudaMemsetAsync(b->d_counter, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess || b->n_items == 0)
        return e;
    // launch only (no attribute calls, so it can be captured): plan() has set
    // the kernel's shared-memory limit and the resident grid
    BatchArgs a{};
    a.keys = make_philox_keys(b->seed);
    a.problems = b->d_problems;
    a.items = b->d_items;
    a.n_items = b->n_items;
    a.max_shells = b->max_shells;
    a.probe_shell = 0;
    a.tally = b->d_tally;
    a.steps = b->d_steps;
    a.item_counter = b->d_counter;
    a.item_probe = nullptr;
    a.error = reinterpret_cast<unsigned *>(b->d_counter + 1);
    a.done_ring = nullptr;
    a.done_tail = nullptr;
    a.wait_limit_ns = b->wait_limit_ns;
    a.hold_buffers = b->d_hold;
    if (b->cfg.stream) {
        // up to two items open per block, the second claimed when needed
        const int grid = std::max(1, std::min<int>(b->grid, (int)b->n_items));
        return walk_stream_launch(a, b->cfg.block, b->math, grid, s);
    }
    const int grid = std::max(1, std::min<int>(b->grid, (int)b->n_items));
    return walk_batch_launch(a, b->cfg.block, b->math, grid, s);
}

int check_batch_device(const tmc_batch *b)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return set_cuda_error(e, "cudaGetDevice");
    if (dev != b->device) {
        set_error_text("tmc_batch used on a different device than it was created on");
        return TMC_E_STATE;
    }
    return TMC_OK;
}

void free_batch(tmc_batch *b)
{
    if (!b)
        return;
    if (b->graph)
        cudaGraphExecDestroy(b->graph);
    if (b->capture_stream)
        cudaStreamDestroy(b->capture_stream);
    cudaFree(b->d_problems);
    cudaFree(b->d_items);
    cudaFree(b->d_tally);
    cudaFree(b->d_steps);
    cudaFree(b->d_counter);
    cudaFree(b->d_hold);
    delete b;
}

int run_locked(tmc_batch *b, void *stream)
{
    int st = check_batch_device(b);
    if (st)
        return st;
    if (!b->planned && (st = plan(b)))
        return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (b->cfg.use_graph) {
        if (!b->graph) {
            if (!b->capture_stream &&
                (e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking)) != cudaSuccess)
                return set_cuda_error(e, "cudaStreamCreate(capture)");
            cudaGraph_t g = nullptr;
            e = cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess)
                return set_cuda_error(e, "cudaStreamBeginCapture");
            cudaError_t e1 = enqueue(b, b->capture_stream);
            e = cudaStreamEndCapture(b->capture_stream, &g);
            if (e1 != cudaSuccess || e != cudaSuccess) {
                if (g)
                    cudaGraphDestroy(g);
                return set_cuda_error(e1 != cudaSuccess ? e1 : e, "batch graph capture");
            }
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                b->graph = nullptr;
                return set_cuda_error(e, "cudaGraphInstantiate");
            }
        }
        e = cudaGraphLaunch(b->graph, s);
    } else {
        e = enqueue(b, s);
    }
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_batch_run");
    b->last_stream = s;
    return TMC_OK;
}

}  // namespace

extern "C" {

int tmc_batch_create(tmc_batch **out, const tmc_problem *problems, uint32_t n_problems, uint64_t seed,
                     uint32_t math)
{
    if (!out || (n_problems && !problems))
        return TMC_E_INVALID;
    if (math != TMC_MATH_EXACT && math != TMC_MATH_FAST)
        return TMC_E_INVALID;
    *out = nullptr;
    unsigned long long total_shells = 0;
    uint32_t max_shells = 1;
    for (uint32_t i = 0; i < n_problems; ++i) {
        tmc_params p;
        tmc_params_default(&p);
        p.shells = problems[i].shells;
        p.microns_per_shell = problems[i].microns_per_shell;
        p.mu_a = problems[i].mu_a;
        p.mu_s = problems[i].mu_s;
        p.math = math;
        int st = validate(&p);
        if (st)
            return st;
        if (problems[i].n_photons > (1ull << 62) ||
            problems[i].photon_id_base > ~0ull - problems[i].n_photons)
            return TMC_E_OVERFLOW;
        total_shells += problems[i].shells;
        max_shells = std::max(max_shells, problems[i].shells);
    }
    std::lock_guard<std::mutex> lk(api_mutex());
    int st = TMC_OK;
    DeviceCtx *c = current_ctx(&st);
    if (!c)
        return st;
    std::unique_ptr<tmc_batch> b(new tmc_batch);
    b->problems.assign(problems, problems + n_problems);
    b->seed = seed;
    b->math = math;
    b->max_shells = max_shells;
    b->device = c->device;
    b->sms = c->sms;
    b->smem_optin = c->smem_optin;
    if (batch_smem(b.get(), 512) > b->smem_optin) {
        b->cfg.block = 256;
        if (batch_smem(b.get(), 256) > b->smem_optin) {
            set_error_text("tmc_batch_create: too many shells for the shared-memory histogram");
            return TMC_E_INVALID;
        }
    }
    b->offsets.resize(n_problems + 1);
    std::vector<BatchProblemDev> hp(n_problems);
    b->offsets[0] = 0;
    for (uint32_t i = 0; i < n_problems; ++i) {
        const tmc_problem &q = problems[i];
        const Derived d = derive(q.mu_a, q.mu_s, q.microns_per_shell, q.shells);
        b->derived.push_back(d);
        b->est_steps.push_back(expected_steps(d.albedo));
        hp[i].c.albedo = d.albedo;
        hp[i].c.spm = d.spm;
        hp[i].c.last = d.last;
        hp[i].c.shells = d.shells;
        hp[i].id_base = q.photon_id_base;
        hp[i].tally_offset = b->offsets[i];
        b->offsets[i + 1] = b->offsets[i] + q.shells;
    }
    cudaError_t e = cudaMalloc(&b->d_problems, sizeof(BatchProblemDev) * std::max<size_t>(1, n_problems));
    if (e == cudaSuccess && n_problems)
        e = cudaMemcpy(b->d_problems, hp.data(), sizeof(BatchProblemDev) * n_problems, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMalloc(&b->d_tally, sizeof(tmc_tally) * std::max<unsigned long long>(1, total_shells));
    if (e == cudaSuccess)
        e = cudaMalloc(&b->d_steps, sizeof(unsigned long long) * std::max<size_t>(1, n_problems));
    if (e == cudaSuccess)
        e = cudaMalloc(&b->d_counter, 2 * sizeof(unsigned long long));
    if (e != cudaSuccess) {
        int r = set_cuda_error(e, "tmc_batch_create");
        free_batch(b.release());
        return r;
    }
    *out = b.release();
    return TMC_OK;
}

int tmc_batch_set_config(tmc_batch *b, const tmc_batch_config *cfg)
{
    if (!b || !cfg)
        return TMC_E_INVALID;
    const int block = cfg->block ? cfg->block : 256;
    if (block != 128 && block != 256 && block != 512)
        return TMC_E_INVALID;
    if (cfg->items_per_block < 0 || cfg->items_per_block > 1024)
        return TMC_E_INVALID;
    const size_t need = cfg->stream ? walk_stream_smem(b->max_shells, block)
                                    : walk_batch_smem(b->max_shells, block);
    if (need > b->smem_optin)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    bool replan = block != b->cfg.block || (cfg->items_per_block ? cfg->items_per_block : 8) !=
                                                    b->cfg.items_per_block;
    b->cfg.block = block;
    b->cfg.items_per_block = cfg->items_per_block ? cfg->items_per_block : 8;
    if (b->cfg.use_graph != (cfg->use_graph ? 1 : 0) && b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->cfg.use_graph = cfg->use_graph ? 1 : 0;
    if (b->cfg.stream != (cfg->stream ? 1 : 0)) {
        b->cfg.stream = cfg->stream ? 1 : 0;
        replan = true;
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
    }
    if (replan)
        b->planned = false;
    return TMC_OK;
}

int tmc_batch_get_config(const tmc_batch *b, tmc_batch_config *cfg)
{
    if (!b || !cfg)
        return TMC_E_INVALID;
    *cfg = b->cfg;
    return TMC_OK;
}

int tmc_batch_run(tmc_batch *b, void *stream)
{
    tmc::NvtxRange nvtx_range("tmc_batch_run");
    if (!b)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    return run_locked(b, stream);
}

int tmc_batch_read(tmc_batch *b, tmc_tally *tallies, uint64_t *steps_per_problem)
{
    if (!b)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    int st = check_batch_device(b);
    if (st)
        return st;
    cudaError_t e = cudaStreamSynchronize(b->last_stream);
    const size_t n = b->problems.size();
    unsigned long long err = 0;
    if (e == cudaSuccess)
        e = cudaMemcpy(&err, b->d_counter + 1, sizeof err, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && err) {
        set_error_text("tmc_batch_read: a bounded device wait ran out");
        return TMC_E_TIMEOUT;
    }
    if (e == cudaSuccess && tallies)
        e = cudaMemcpy(tallies, b->d_tally, sizeof(tmc_tally) * b->offsets[n], cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && steps_per_problem && n)
        e = cudaMemcpy(steps_per_problem, b->d_steps, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_batch_read");
    return TMC_OK;
}

int tmc_batch_tally_offsets(const tmc_batch *b, uint64_t *offsets)
{
    if (!b || !offsets)
        return TMC_E_INVALID;
    for (size_t i = 0; i < b->offsets.size(); ++i)
        offsets[i] = b->offsets[i];
    return TMC_OK;
}

int tmc_batch_info(const tmc_batch *b, uint32_t *n_items, double *est_photon_steps)
{
    if (!b)
        return TMC_E_INVALID;
    if (n_items)
        *n_items = b->n_items;
    if (est_photon_steps) {
        double t = 0.0;
        for (size_t i = 0; i < b->problems.size(); ++i)
            t += b->est_steps[i] * (double)b->problems[i].n_photons;
        *est_photon_steps = t;
    }
    return TMC_OK;
}

const void *tmc_batch_device_tallies(const tmc_batch *b) { return b ? b->d_tally : nullptr; }

int tmc_batch_plan_items(const tmc_problem *problems, uint32_t n_problems, int grid, int block,
                         int items_per_block, uint64_t *items_out, uint64_t capacity, uint64_t *n_items)
{
    if ((n_problems && !problems) || !n_items || grid < 1 || block < 32 || items_per_block < 1 ||
        (capacity && !items_out))
        return TMC_E_INVALID;
    std::vector<tmc_problem> pr(problems, problems + n_problems);
    std::vector<double> est(n_problems);
    for (uint32_t i = 0; i < n_problems; ++i) {
        tmc_params p;
        tmc_params_default(&p);
        p.shells = pr[i].shells;
        p.microns_per_shell = pr[i].microns_per_shell;
        p.mu_a = pr[i].mu_a;
        p.mu_s = pr[i].mu_s;
        const int st = validate(&p);
        if (st)
            return st;
        est[i] = expected_steps(derive(p.mu_a, p.mu_s, p.microns_per_shell, p.shells).albedo);
    }
    const std::vector<BatchItemDev> h = plan_items(pr, est, grid, block, items_per_block);
    *n_items = h.size();
    if (h.size() > capacity)
        return capacity ? TMC_E_OVERFLOW : TMC_OK;
    for (size_t i = 0; i < h.size(); ++i) {
        items_out[3 * i] = h[i].problem;
        items_out[3 * i + 1] = h[i].first;
        items_out[3 * i + 2] = h[i].count;
    }
    return TMC_OK;
}

int tmc_expected_steps(float mu_a, float mu_s, double *steps_per_photon)
{
    if (!steps_per_photon)
        return TMC_E_INVALID;
    tmc_params p;
    tmc_params_default(&p);
    p.mu_a = mu_a;
    p.mu_s = mu_s;
    int st = validate(&p);
    if (st)
        return st;
    *steps_per_photon = expected_steps(derive(mu_a, mu_s, 50.0f, 1).albedo);
    return TMC_OK;
}

int tmc_batch_autotune(tmc_batch *b, double scale, double max_steps_per_photon, double *best_ms)
{
    tmc::NvtxRange nvtx_range("tmc_batch_autotune");
    if (!b || !(scale > 0.0) || scale > 1.0)
        return TMC_E_INVALID;
    // a reduced copy: photon counts scaled, problems with very long walks left
    // out (a single photon of those would dominate every timing)
    std::vector<tmc_problem> red;
    for (size_t i = 0; i < b->problems.size(); ++i) {
        if (max_steps_per_photon > 0.0 && b->est_steps[i] > max_steps_per_photon)
            continue;
        tmc_problem q = b->problems[i];
        q.n_photons = std::max<uint64_t>(64, (uint64_t)std::ceil((double)q.n_photons * scale));
        red.push_back(q);
    }
    if (red.empty())
        return TMC_OK;
    tmc_batch *t = nullptr;
    int st = tmc_batch_create(&t, red.data(), (uint32_t)red.size(), b->seed, b->math);
    if (st)
        return st;
    static const int blocks[3] = {128, 256, 512};
    static const int ipb[4] = {4, 8, 16, 64};
    static const int streams[2] = {0, 1};
    double best = 1e300;
    tmc_batch_config best_cfg = b->cfg;
    b->tuned.clear();
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    for (int k = 0; k < 24 && e == cudaSuccess && st == TMC_OK; ++k) {
        {
            const int bi = k % 3, ii = (k / 3) % 4, si = k / 12;
            tmc_batch_config c{blocks[bi], ipb[ii], 0, streams[si]};
            if (tmc_batch_set_config(t, &c) != TMC_OK)
                continue;
            st = tmc_batch_run(t, nullptr);          // warm-up and planning
            if (st)
                break;
            e = cudaEventRecord(e0, nullptr);
            if (e == cudaSuccess)
                st = tmc_batch_run(t, nullptr);
            if (e == cudaSuccess)
                e = cudaEventRecord(e1, nullptr);
            if (e == cudaSuccess)
                e = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (e == cudaSuccess)
                e = cudaEventElapsedTime(&ms, e0, e1);
            if (e == cudaSuccess && st == TMC_OK)
                st = tmc_batch_read(t, nullptr, nullptr);   // error flag of the run
            if (e == cudaSuccess && st == TMC_OK)
                b->tuned.push_back({(double)ms, c});
            if (e == cudaSuccess && st == TMC_OK && ms < best) {
                best = ms;
                best_cfg = c;
            }
        }
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    free_batch(t);
    if (st)
        return st;
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_batch_autotune");
    best_cfg.use_graph = b->cfg.use_graph;
    st = tmc_batch_set_config(b, &best_cfg);
    if (best_ms)
        *best_ms = best;
    return st;
}

int tmc_batch_refine(tmc_batch *b, uint32_t max_candidates, double *best_ms)
{
    tmc::NvtxRange nvtx_range("tmc_batch_refine");
    if (!b || max_candidates == 0)
        return TMC_E_INVALID;
    if (b->tuned.empty())
        return TMC_E_STATE;
    // the fastest reduced-copy configuration of each (kernel, block size):
    // first the fastest of each kernel, so that both kernels are timed on
    // the batch itself however the reduced copy ranked them, then the rest
    // in order
    std::vector<std::pair<double, tmc_batch_config>> cand(b->tuned);
    std::stable_sort(cand.begin(), cand.end(),
                     [](const auto &x, const auto &y) { return x.first < y.first; });
    std::vector<tmc_batch_config> pick;
    auto add = [&](const tmc_batch_config &c) {
        for (const auto &q : pick)
            if (q.block == c.block && q.stream == c.stream)
                return;
        if (pick.size() < max_candidates)
            pick.push_back(c);
    };
    for (uint32_t kernel = 0; kernel < 2; ++kernel)
        for (const auto &c : cand)
            if (c.second.stream == kernel) {
                add(c.second);
                break;
            }
    for (const auto &c : cand)
        add(c.second);
    const int use_graph = b->cfg.use_graph;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    int st = TMC_OK;
    double best = 1e300;
    tmc_batch_config best_cfg = b->cfg;
    for (size_t k = 0; k < pick.size() && e == cudaSuccess && st == TMC_OK; ++k) {
        tmc_batch_config c = pick[k];
        c.use_graph = 0;
        st = tmc_batch_set_config(b, &c);
        if (st)
            break;
        e = cudaEventRecord(e0, nullptr);
        if (e == cudaSuccess)
            st = tmc_batch_run(b, nullptr);
        if (e == cudaSuccess)
            e = cudaEventRecord(e1, nullptr);
        if (e == cudaSuccess)
            e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess)
            e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && st == TMC_OK)
            st = tmc_batch_read(b, nullptr, nullptr);
        if (e == cudaSuccess && st == TMC_OK && ms < best) {
            best = ms;
            best_cfg = c;
        }
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    if (st)
        return st;
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_batch_refine");
    best_cfg.use_graph = use_graph;
    st = tmc_batch_set_config(b, &best_cfg);
    if (best_ms)
        *best_ms = best;
    return st;
}

int tmc_batch_test_wait(tmc_batch *b, int hold_buffers, double wait_limit_s)
{
    if (!b || !(wait_limit_s >= 0.0) || wait_limit_s > 3600.0)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    cudaError_t e = cudaSuccess;
    if (!b->d_hold)
        e = cudaMalloc(&b->d_hold, sizeof(unsigned));
    if (e == cudaSuccess)
        e = cudaMemset(b->d_hold, hold_buffers ? 1 : 0, sizeof(unsigned));
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_batch_test_wait");
    b->wait_limit_ns = (unsigned long long)(wait_limit_s * 1e9);
    if (b->graph) {   // the captured launch holds the old limit
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return TMC_OK;
}

int tmc_batch_destroy(tmc_batch *b)
{
    if (!b)
        return TMC_OK;
    std::lock_guard<std::mutex> lk(api_mutex());
    free_batch(b);
    return TMC_OK;
}

}  // extern "C"
