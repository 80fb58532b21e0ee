// tmc_stream.cu — the batched walk without per-item barriers.
//
// walk_batch (tmc_batch.cu) walks one work item per block at a time: every
// warp of the block waits at a barrier for the slowest lane of the item before
// the block takes the next one.  With heavy-tailed walk lengths those waits
// idle a large part of the block.  walk_stream keeps up to TWO items open per
// block, each in a buffer with its own shared-memory histogram:
//
//  * a warp claims photons from its current item j; when j has no photons
//    left, lanes that need a photon take them from item j+1, which the first
//    warp to get there claims from the global queue (so a block never holds
//    an item it has not started), while the other lanes finish their photons
//    of j.  Each lane deposits into the histogram of its own photon's item,
//    so a warp spans at most two items;
//  * a warp reports an item done when the item has no photons left and none
//    of its lanes still walks one; the last warp of the block to report item
//    j flushes j's histogram into the problem's 128-bit tally, writes the
//    item's probe value and step count, zeroes the histogram and frees the
//    buffer for item j+2;
//  * the item's optics, tally pointer and photon ids live in the buffer's
//    shared record, not in registers, so the kernel keeps the plain walk's
//    occupancy; photon steps are added to the record when a photon dies;
//  * waits (a warp with nothing to walk until the block frees a buffer) are
//    bounded by wall time through %globaltimer (120 s unless the launch
//    says otherwise): past the limit the warp sets the error flag and
//    leaves; the host reports TMC_E_TIMEOUT.
// Queue mode (the request server's persistent launch): the items come from a
// ring in mapped host memory that the host keeps filling while the kernel
// runs.  A block claims an item only once the host has published it (a
// compare-and-swap on the claim counter below the published count, read with
// acquire semantics), polls the published count with back-off when the ring
// is empty, and ends when the host says stop, or says drain and nothing has
// been published for the idle limit; while the host says hold, an empty ring
// is waited on up to the wait limit.
// Results are bit-identical to walk_batch and the plain kernel: the same
// photons, integer sums.
#include <algorithm>

#include "tmc_batch.cuh"
#include "tmc_internal.h"
#include "tmc_walk.cuh"

namespace tmc {

namespace {

constexpr uint32_t END_ITEM = 0xffffffffu;
constexpr unsigned long long DEFAULT_WAIT_LIMIT_NS = QUEUE_DEFAULT_WAIT_LIMIT_NS;
constexpr uint32_t BUF_FREE = 0, BUF_CLAIMING = 1, BUF_OPEN = 2;

struct __align__(16) OpenItem {    // per buffer, in shared memory
    WalkConsts c;                  // optics of the item's problem
    unsigned long long *g;         // the problem's 128-bit global tally
    unsigned long long id_first;   // photon id of the item's first photon
    unsigned long long qidx;       // queue mode: the item's pool slot
    unsigned long long idle_since; // queue mode: first failed claim of this sequence (ns)
    unsigned long long next_poll;  // queue mode: no poll of the published count before (ns)
    uint32_t problem;              // the item's problem
    uint32_t item;                 // global item index, or END_ITEM
    uint32_t count;                // photons in the item
    uint32_t ps;                   // probe shell, clamped to the problem
    uint32_t next;                 // photon counter within the item
    uint32_t done;                 // warps that reported the item
    uint32_t wraps;                // 2^64 wraps of the probe shell's sum
    uint32_t steps_lo, steps_hi;   // photon steps walked on the item
    uint32_t gen;                  // item sequence number the buffer is for
    uint32_t state;                // BUF_FREE / BUF_CLAIMING / BUF_OPEN
};

__device__ __forceinline__ void fill_item(const BatchArgs &a, OpenItem *o, const BatchItemDev &itm,
                                          const BatchProblemDev &pr)
{
    o->c = pr.c;
    o->g = a.tally + 4 * pr.tally_offset;
    o->id_first = pr.id_base + itm.first;
    o->count = itm.count;
    o->problem = itm.problem;
    o->ps = min(a.probe_shell, pr.c.shells - 1);
    o->next = 0;
    o->done = 0;
    o->wraps = 0;
    o->steps_lo = 0;
    o->steps_hi = 0;
}

// Claim the next item into buffer o (one thread).  Returns false only in
// queue mode when nothing is published yet (try again later); otherwise o
// holds the item, or END_ITEM when there is no more work.
template <bool QUEUE>
__device__ __forceinline__ bool open_item(const BatchArgs &a, OpenItem *o)
{
    if constexpr (!QUEUE) {
        const unsigned long long it = atomicAdd(a.item_counter, 1ull);
        o->item = it < a.n_items ? (uint32_t)it : END_ITEM;
        if (it < a.n_items)
            fill_item(a, o, a.items[it], a.problems[a.items[it].problem]);
        return true;
    }
    const unsigned long long now = global_ns();
    if (now < o->next_poll)
        return false;
    BatchItemDev itm;
    BatchProblemDev pr;
    unsigned long long c = 0;
    if (queue_try_claim(a, itm, pr, c)) {
        fill_item(a, o, itm, pr);
        o->item = (uint32_t)(c & (a.q_cap - 1));
        o->qidx = c;
        o->idle_since = 0;
        o->next_poll = 0;
        return true;
    }
    if (o->idle_since == 0)
        o->idle_since = now;
    const unsigned long long waited = now - o->idle_since;
    if (queue_idle_verdict(a, waited)) {
        o->item = END_ITEM;
        return true;
    }
    o->next_poll = now + 256ull + min(waited >> 4, 16384ull);
    return false;
}

}  // namespace

template <int BLOCK, class M, bool QUEUE>
__global__ void __launch_bounds__(BLOCK) walk_stream(const BatchArgs a)
{
    constexpr unsigned NWARPS = BLOCK / 32;
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ OpenItem open[2];
    const uint32_t HS = 4 * a.max_shells;          // words per histogram
    uint32_t *my = smem + 2 * HS + threadIdx.x;    // ring slot k: my[k * BLOCK]
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;

    for (uint32_t s = threadIdx.x; s < 2 * HS; s += BLOCK)
        smem[s] = 0;
    if (threadIdx.x == 0) {
        if (QUEUE && a.q_live)
            atomicAdd(a.q_live, 1u);
        for (int b = 0; b < 2; ++b) {
            open[b].idle_since = 0;
            open[b].next_poll = 0;
        }
        // queue mode: wait (bounded inside open_item) for the first item
        while (!open_item<QUEUE>(a, &open[0]))
            __nanosleep(256);
        open[0].gen = 0;
        open[0].state = BUF_OPEN;
        open[1].gen = 1;
        open[1].state = BUF_FREE;
    }
    __syncthreads();
    volatile OpenItem *vopen = open;

    // ---- warp-uniform state
    uint32_t jc = 0;          // item sequence the warp claims photons from
    uint32_t rep = 0;         // lowest item sequence this warp has not reported
    bool exh = false;         // item jc has no photons left
    uint32_t cn = 0, ce = 0;  // current chunk of photon indices within item jc
    uint32_t it_c = open[0].item;

    // ---- lane state
    bool alive = false, want = true, pending = false;
    uint32_t pid_lo = 0, pid_hi = 0, blk = 0, prod = 0, cur = 0;
    float x = 0.f, y = 0.f, z = 0.f, u = 0.f, v = 0.f, w = 1.f, weight = 1.f;
    uint32_t lb = 0;                          // buffer of this lane's photon
    uint32_t steps = 0;                       // steps of this lane's photon
    // the constants of this lane's photon's item, read from the buffer's
    // record once when the photon starts (the record cannot change while
    // the photon lives: its warp has not reported the item yet)
    WalkConsts pc{};
    unsigned long long *pg = nullptr;
    uint32_t pps = 0;
    unsigned long long wait_start = 0;

    for (;;) {
        // -------- report items this warp is finished with (oldest first)
        for (;;) {
            if (rep > jc || (rep == jc && !exh))
                break;
            const uint32_t rb = rep & 1u;
            if (vopen[rb].item == END_ITEM)
                break;
            if (__any_sync(FULL_MASK, alive && lb == rb))
                break;
            // the done count, after this warp's deposits into the item
            unsigned last = 0;
            __syncwarp();
            __threadfence_block();
            if (lane == 0)
                last = (atomicAdd((unsigned *)&open[rb].done, 1u) == NWARPS - 1) ? 1u : 0u;
            last = __shfl_sync(FULL_MASK, last, 0);
            if (last) {
                // every warp is done with item `rep`: flush, probe, reset, free
                __threadfence_block();
                const uint32_t it = vopen[rb].item;
                const uint32_t S = vopen[rb].c.shells;
                uint32_t *hist = smem + rb * HS;
                unsigned long long *gg = open[rb].g;
                for (uint32_t s = lane; s < S; s += 32) {
                    flush128(&gg[4 * s + 0], &gg[4 * s + 1],
                             ((unsigned long long)hist[S + s] << 32) | hist[s]);
                    flush128(&gg[4 * s + 2], &gg[4 * s + 3],
                             ((unsigned long long)hist[3 * S + s] << 32) | hist[2 * S + s]);
                }
                const uint32_t p = vopen[rb].ps;
                const unsigned long long probe_lo = ((unsigned long long)hist[S + p] << 32) | hist[p];
                const unsigned long long probe_hi = vopen[rb].wraps;
                if (lane == 0) {
                    const unsigned long long st =
                        ((unsigned long long)vopen[rb].steps_hi << 32) | vopen[rb].steps_lo;
                    if (st)
                        atomicAdd(&a.steps[vopen[rb].problem], st);
                    if (a.item_probe) {
                        a.item_probe[2 * (size_t)it] = probe_lo;
                        a.item_probe[2 * (size_t)it + 1] = probe_hi;
                    }
                }
                if (a.done_ring) {
                    __threadfence();
                    __syncwarp();
                    if (lane == 0) {
                        if constexpr (QUEUE)
                            publish_item_at(a, vopen[rb].qidx, probe_lo, probe_hi);
                        else
                            publish_item(a, it, probe_lo, probe_hi);
                    }
                }
                __syncwarp();
                for (uint32_t s = lane; s < 4 * S; s += 32)
                    hist[s] = 0;
                __threadfence_block();
                __syncwarp();
                unsigned hold = 0;
                if (lane == 0 && a.hold_buffers)
                    hold = *(volatile const unsigned *)a.hold_buffers;
                hold = __shfl_sync(FULL_MASK, hold, 0);
                if (lane == 0 && !hold) {
                    vopen[rb].state = BUF_FREE;
                    __threadfence_block();
                    vopen[rb].gen = rep + 2;
                }
                __syncwarp();
            }
            ++rep;
        }

        // -------- hand photons to lanes that want one
        unsigned need = __ballot_sync(FULL_MASK, want);
        while (need) {
            if (it_c == END_ITEM)
                break;
            const uint32_t cb = jc & 1u;
            if (!exh) {
                const unsigned n_need = __popc(need);
                const unsigned rank = __popc(need & lt_mask);
                uint32_t k = min((uint32_t)n_need, ce - cn);
                if (k == 0) {
                    uint32_t base = 0;
                    if (lane == 0)
                        base = atomicAdd((unsigned *)&open[cb].next, (uint32_t)BATCH_CHUNK);
                    base = __shfl_sync(FULL_MASK, base, 0);
                    const uint32_t count = open[cb].count;
                    if (base >= count) {
                        exh = true;
                        continue;
                    }
                    cn = base;
                    ce = min(base + (uint32_t)BATCH_CHUNK, count);
                    k = min((uint32_t)n_need, ce - cn);
                }
                const bool mine = ((need >> lane) & 1u) && rank < k;
                if (mine) {
                    // launch, photon.c:12-18
                    const unsigned long long pid = open[cb].id_first + (cn + rank);
                    pid_lo = (uint32_t)pid;
                    pid_hi = (uint32_t)(pid >> 32);
                    want = false;
                    alive = true;
                    blk = 0;
                    cur = prod;
                    pending = false;
                    x = y = z = 0.f;
                    u = v = 0.f;
                    w = 1.f;
                    weight = 1.f;
                    lb = cb;
                    steps = 0;
                    pc = open[cb].c;
                    pg = open[cb].g;
                    pps = open[cb].ps;
                }
                cn += k;
                need = __ballot_sync(FULL_MASK, want);
                continue;
            }
            // item jc is used up: move on to sequence jc+1 once its buffer is
            // free, claiming its item if no warp of the block has yet
            const uint32_t nb = cb ^ 1u;
            uint32_t st = BUF_FREE;
            if (lane == 0 && vopen[nb].gen == jc + 1) {
                __threadfence_block();
                st = vopen[nb].state;
                if (st == BUF_FREE &&
                    atomicCAS((unsigned *)&open[nb].state, BUF_FREE, BUF_CLAIMING) == BUF_FREE) {
                    const bool got = open_item<QUEUE>(a, &open[nb]);
                    __threadfence_block();
                    st = got ? BUF_OPEN : BUF_FREE;   // queue empty: free again, retry later
                    vopen[nb].state = st;
                }
            }
            st = __shfl_sync(FULL_MASK, st, 0);
            if (st != BUF_OPEN)
                break;
            __threadfence_block();
            ++jc;
            exh = false;
            cn = ce = 0;
            it_c = vopen[nb].item;
        }
        if (it_c == END_ITEM && need) {
            // no more work for lanes that want a photon
            want = false;
        }

        const bool any_alive = __any_sync(FULL_MASK, alive);
        if (!any_alive) {
            if (it_c == END_ITEM && rep >= jc)
                break;   // all photons walked, all items reported
            // nothing to walk until the block frees a buffer: sleep about an
            // eighth of the time waited so far (64 ns .. 16 us), so waiting
            // warps leave the issue slots to the block's walking warps
            const unsigned long long now = global_ns();
            if (wait_start == 0)
                wait_start = now;
            else if (now - wait_start > (a.wait_limit_ns ? a.wait_limit_ns : DEFAULT_WAIT_LIMIT_NS)) {
                if (lane == 0)
                    atomicExch(a.error, 1u);
                break;
            }
            __nanosleep(64u + (unsigned)min((now - wait_start) >> 3, 16384ull));
            continue;
        }
        wait_start = 0;

        // -------- refill once REFILL_MIN_SHORT_ITEMS walking lanes are short of the
        // 6 words an iteration may use (or every walking lane is), as walk_loop
        for (;;) {
            const unsigned low = __ballot_sync(FULL_MASK, alive && (prod - cur) < 6u);
            if (low == 0 ||
                (__popc(low) < REFILL_MIN_SHORT_ITEMS && low != __ballot_sync(FULL_MASK, alive)))
                break;
            if (alive && (prod - cur) <= (uint32_t)(RING - 4)) {
                const uint4 r = philox4x32_10(blk, 0u, pid_lo, pid_hi, a.keys);
                ++blk;
                const uint32_t p = prod & (RING - 1);
                uint32_t *dst = my + p * BLOCK;
                dst[0 * BLOCK] = r.x;
                dst[1 * BLOCK] = r.y;
                dst[2 * BLOCK] = r.z;
                dst[3 * BLOCK] = r.w;
                uint32_t *mir = dst + RING * BLOCK;
                if (p <= 4u) {
                    mir[0 * BLOCK] = r.x;
                    mir[1 * BLOCK] = r.y;
                }
                if (p == 0u) {
                    mir[2 * BLOCK] = r.z;
                    mir[3 * BLOCK] = r.w;
                }
                prod += 4;
            }
        }

        if (alive && (prod - cur) >= 6u) {   // a short lane waits for the next refill
            const uint32_t *rd = my + (cur & (RING - 1)) * BLOCK;
            if (!pending) {
                // move, photon.c:21-24
                const float U = uniform01(rd[0]);
                rd += BLOCK;
                ++cur;
                const float t = M::step_length(U);
                x = M::move(x, t, u);
                y = M::move(y, t, v);
                z = M::move(z, t, w);
                // absorb, photon.c:26-32
                const WalkConsts c = pc;
                const float rr = M::radius_shells(x, y, z, c.spm);
                const uint32_t shell = __float2uint_rz(fminf(rr, c.last));
                const uint32_t S = c.shells;
                uint32_t *t0 = smem + lb * HS + shell;
                unsigned long long *g = pg;
                uint32_t lo, hi;
                fx40_split(weight, lo, hi);
                tally_add(t0, t0 + S, &g[4 * shell + 1], lo, hi,
                          shell == pps ? (uint32_t *)&open[lb].wraps : nullptr);
                fx40_split(__fmul_rn(weight, weight), lo, hi);
                tally_add(t0 + 2 * S, t0 + 3 * S, &g[4 * shell + 3], lo, hi);
                weight = M::mul(weight, c.albedo);
                ++steps;
            }
            // the next two tries of the rejection method, photon.c:36-40
            const float xa1 = uniform_pm1(rd[0 * BLOCK]);
            const float xa2 = uniform_pm1(rd[1 * BLOCK]);
            const float xb1 = uniform_pm1(rd[2 * BLOCK]);
            const float xb2 = uniform_pm1(rd[3 * BLOCK]);
            const float ta = M::norm2(xa1, xa2);
            const float tb = M::norm2(xb1, xb2);
            const bool first = !(1.0f < ta);
            const float xi1 = first ? xa1 : xb1;
            const float xi2 = first ? xa2 : xb2;
            const float tt = first ? ta : tb;
            rd += first ? 2 * BLOCK : 4 * BLOCK;
            cur += first ? 2u : 4u;
            pending = (1.0f < tt);
            if (!pending) {
                // new direction, photon.c:41-43
                u = fmaf(2.0f, tt, -1.0f);
                const float sc = M::dir_scale(tt, u);
                v = M::mul(xi1, sc);
                w = M::mul(xi2, sc);
                // roulette, photon.c:45-49
                if (weight < 0.001f) {
                    const float U = uniform01(rd[0]);
                    ++cur;
                    if (U > 0.1f) {
                        alive = false;
                        want = true;
                        // the photon's steps into its item's 64-bit count
                        uint32_t *sl = (uint32_t *)&open[lb].steps_lo;
                        const uint32_t old = atomicAdd(sl, steps);
                        if (old + steps < old)
                            atomicAdd((uint32_t *)&open[lb].steps_hi, 1u);
                    } else {
                        weight = __fdiv_rn(weight, 0.1f);
                    }
                }
            }
        }
    }
    // every warp has left the loop (their waits are bounded)
    __syncthreads();
    if (QUEUE && threadIdx.x == 0)
        queue_block_end(a);
}

size_t walk_stream_smem(uint32_t max_shells, int block)
{
    return (size_t)32 * max_shells + (size_t)4 * SLOTS * block;
}

template <int BLOCK, class M, bool QUEUE>
static cudaError_t stream_config(int sms, size_t smem, int *grid)
{
    auto kern = walk_stream<BLOCK, M, QUEUE>;
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

template <bool QUEUE>
static cudaError_t stream_prepare(int block, bool fast, size_t smem, int sms, int *grid)
{
    switch (block) {
    case 128: return fast ? stream_config<128, FastMath, QUEUE>(sms, smem, grid)
                          : stream_config<128, ExactMath, QUEUE>(sms, smem, grid);
    case 256: return fast ? stream_config<256, FastMath, QUEUE>(sms, smem, grid)
                          : stream_config<256, ExactMath, QUEUE>(sms, smem, grid);
    case 512: return fast ? stream_config<512, FastMath, QUEUE>(sms, smem, grid)
                          : stream_config<512, ExactMath, QUEUE>(sms, smem, grid);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t walk_stream_prepare(int block, uint32_t math, uint32_t max_shells, int sms, int *grid,
                                bool queue)
{
    const size_t smem = walk_stream_smem(max_shells, block);
    const bool fast = math == TMC_MATH_FAST;
    return queue ? stream_prepare<true>(block, fast, smem, sms, grid)
                 : stream_prepare<false>(block, fast, smem, sms, grid);
}

template <int BLOCK>
static void stream_launch_b(const BatchArgs &a, bool fast, int grid, size_t smem, cudaStream_t s)
{
    if (a.q_items) {
        if (fast) walk_stream<BLOCK, FastMath, true><<<grid, BLOCK, smem, s>>>(a);
        else walk_stream<BLOCK, ExactMath, true><<<grid, BLOCK, smem, s>>>(a);
    } else {
        if (fast) walk_stream<BLOCK, FastMath, false><<<grid, BLOCK, smem, s>>>(a);
        else walk_stream<BLOCK, ExactMath, false><<<grid, BLOCK, smem, s>>>(a);
    }
}

cudaError_t walk_stream_launch(const BatchArgs &a, int block, uint32_t math, int grid, cudaStream_t s)
{
    const size_t smem = walk_stream_smem(a.max_shells, block);
    const bool fast = math == TMC_MATH_FAST;
    switch (block) {
    case 128: stream_launch_b<128>(a, fast, grid, smem, s); break;
    case 256: stream_launch_b<256>(a, fast, grid, smem, s); break;
    case 512: stream_launch_b<512>(a, fast, grid, smem, s); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace tmc
