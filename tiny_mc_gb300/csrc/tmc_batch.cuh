// tmc_batch.cuh — the batched walk kernel's tables and launch helpers, shared
// by the batch plan (tmc_batch.cu) and the request server (tmc_serve.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tmc_walk.cuh"

namespace tmc {

constexpr int BATCH_CHUNK = 32;   // photon ids a warp claims from its item at once

// The queue-mode control word (BatchArgs::q_mode), written by the host.
constexpr unsigned QUEUE_HOLD = 0, QUEUE_DRAIN = 1, QUEUE_STOP = 2;

struct BatchProblemDev {
    WalkConsts c;
    unsigned long long id_base;
    unsigned long long tally_offset;   // in shells
};

struct BatchItemDev {
    uint32_t problem;
    uint32_t count;
    unsigned long long first;          // first photon of the item, relative to the problem
};

struct BatchArgs {
    PhiloxKeys keys;
    const BatchProblemDev *problems;
    const BatchItemDev *items;
    uint32_t n_items;
    uint32_t max_shells;
    uint32_t probe_shell;              // shell whose per-item sum goes to item_probe
    unsigned long long *tally;         // [total shells][4]
    unsigned long long *steps;         // [problems]
    unsigned long long *item_counter;  // zero at launch
    unsigned long long *item_probe;    // [n_items][2] (128-bit, lo then hi) or null
    unsigned *error;                   // walk_stream: set to 1 when a bounded wait ran out
    // Completion ring or null: [n_items][4] in mapped host memory.  Each
    // finished item takes the next entry (done_tail, zero at launch) and
    // writes its probe value (lo, hi), its index, then 1 into the entry's
    // last word, so the host can take items as they finish.
    unsigned long long *done_ring;
    unsigned *done_tail;
    // walk_stream's bounded waits: wall-time limit (0 = 120 s), and a test
    // hook (null in normal runs): while *hold_buffers is nonzero, finished
    // items' buffers are not freed, so waiting warps run into the limit.
    unsigned long long wait_limit_ns;
    const unsigned *hold_buffers;
    // Queue mode (the request server's persistent launch), when q_items is
    // not null: items sit in a pool of q_cap slots (a power of two) in mapped
    // host memory, and the queue is a ring of 2 q_cap pool slot numbers
    // (q_order) in publishing order that the host keeps filling while the
    // kernel runs; `problems` is mapped host memory too.  *q_published
    // (host-written, release) counts the positions published so far and
    // *item_counter (device) those claimed; a block claims only published
    // positions, and each finished item's completion is appended to done_ring
    // (done_tail, device, counts them) with the item's pool slot in its third
    // word.  *q_mode (host-written) says what a block does when
    // nothing is published: QUEUE_HOLD waits (up to the wait limit),
    // QUEUE_DRAIN ends after idle_limit_ns, QUEUE_STOP ends at once.
    // *q_live (device) counts the blocks still running.  Nothing is queued on
    // the launch's stream behind the kernel (work waiting there could hold up
    // other streams' copies in a shared hardware queue while the kernel waits
    // for the host): the last block to end counts itself in *q_done_blocks
    // (device, zero at launch) and writes {1, error flag} to q_ended (mapped).
    const BatchItemDev *q_items;        // the item pool [q_cap]
    const uint32_t *q_order;            // queue: pool slot per position [2 q_cap]
    const unsigned long long *q_published;
    const unsigned *q_mode;
    unsigned *q_live;
    unsigned *q_done_blocks;
    unsigned *q_ended;
    uint32_t q_cap;
    unsigned long long idle_limit_ns;
};

// Publish a finished item into the completion ring (one thread).  The
// caller's block (or warp) has flushed the item's tally and added its steps,
// each thread then fenced at device scope and synchronised with the caller:
// the system-scope fence here orders all of that before the entry's ready
// word, which the host reads with acquire semantics.
__device__ __forceinline__ void publish_item(const BatchArgs &a, uint32_t it, unsigned long long lo,
                                             unsigned long long hi)
{
    const unsigned slot = atomicAdd(a.done_tail, 1u);
    volatile unsigned long long *e = a.done_ring + 4 * (size_t)slot;
    e[0] = lo;
    e[1] = hi;
    e[2] = it;
    __threadfence_system();
    e[3] = 1ull;
}

// Queue mode: the completion of the item in pool slot `index`, appended to the
// completion ring in finishing order (entry done_tail % q_cap), so the host
// reads only new completions.  The host keeps at most q_cap items published
// and unfinished, and clears an entry before publishing the item whose
// completion could reuse it.
__device__ __forceinline__ void publish_item_at(const BatchArgs &a, unsigned long long index,
                                                unsigned long long lo, unsigned long long hi)
{
    const unsigned t = atomicAdd(a.done_tail, 1u);
    volatile unsigned long long *e = a.done_ring + 4 * (size_t)(t & (a.q_cap - 1));
    e[0] = lo;
    e[1] = hi;
    e[2] = index;
    __threadfence_system();
    e[3] = 1ull;
}

// -------------------------------------------- queue mode (persistent server)
constexpr unsigned long long QUEUE_DEFAULT_WAIT_LIMIT_NS = 120ull * 1000000000ull;

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned long long load_acquire_sys(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Claim the next published queue position, if any (one thread): the
// position's pool slot is read from mapped host memory (written by the host
// before it published the position), then a compare-and-swap on the claim
// counter below the published count takes the position.  Reading the slot
// before the swap makes it valid when the swap succeeds: the host rewrites a
// position's entry 2 q_cap positions later, only after at least q_cap items
// claimed after it have finished.  The item and its problem are then read from
// the pool slot, which stays the item's until its completion is harvested.
// qidx receives the pool slot, which identifies the item's completion.
// Returns false when nothing is published.
__device__ __forceinline__ bool queue_try_claim(const BatchArgs &a, BatchItemDev &itm, BatchProblemDev &pr,
                                                unsigned long long &qidx)
{
    const unsigned long long pub = load_acquire_sys(a.q_published);
    unsigned long long c = *(volatile unsigned long long *)a.item_counter;
    uint32_t slot = 0;
    while (c < pub) {
        slot = *(const volatile uint32_t *)(a.q_order + (c & (2 * a.q_cap - 1)));
        __threadfence();
        const unsigned long long prev = atomicCAS(a.item_counter, c, c + 1);
        if (prev == c)
            break;
        c = prev;
    }
    if (c >= pub)
        return false;
    const volatile BatchItemDev *vi = a.q_items + slot;
    itm.problem = vi->problem;
    itm.count = vi->count;
    itm.first = vi->first;
    const volatile BatchProblemDev *vp = a.problems + itm.problem;
    pr.c.albedo = vp->c.albedo;
    pr.c.spm = vp->c.spm;
    pr.c.last = vp->c.last;
    pr.c.shells = vp->c.shells;
    pr.id_base = vp->id_base;
    pr.tally_offset = vp->tally_offset;
    qidx = slot;
    return true;
}

// What a block with nothing claimed does after waiting `waited` ns (one
// thread): 1 = end (STOP, or DRAIN past the idle limit), 2 = end with the
// error flag set (the wait limit ran out), 0 = keep waiting.
__device__ __forceinline__ int queue_idle_verdict(const BatchArgs &a, unsigned long long waited)
{
    const unsigned mode = *(volatile const unsigned *)a.q_mode;
    if (mode == QUEUE_STOP)
        return 1;
    if (mode == QUEUE_DRAIN && waited > a.idle_limit_ns)
        return 1;
    if (waited > (a.wait_limit_ns ? a.wait_limit_ns : QUEUE_DEFAULT_WAIT_LIMIT_NS)) {
        atomicExch(a.error, 1u);
        return 2;
    }
    return 0;
}

// The end of a queue-mode block (thread 0, after the block's last flush):
// count the block out, and the launch's last block writes the end record.
__device__ __forceinline__ void queue_block_end(const BatchArgs &a)
{
    if (a.q_live)
        atomicSub(a.q_live, 1u);
    __threadfence();
    if (atomicAdd(a.q_done_blocks, 1u) == gridDim.x - 1) {
        __threadfence();
        volatile unsigned *e = a.q_ended;
        e[1] = *(volatile const unsigned *)a.error;
        __threadfence_system();
        e[0] = 1u;
    }
}

size_t walk_batch_smem(uint32_t max_shells, int block);
// Sets the shared-memory limit of the list form (queue = false) or the queue
// form and returns its resident grid.
cudaError_t walk_batch_prepare(int block, uint32_t math, uint32_t max_shells, int sms, int *grid,
                               bool queue = false);
// Launch only (capturable); walk_batch_prepare must have run for this shape.
cudaError_t walk_batch_launch(const BatchArgs &a, int block, uint32_t math, int grid, cudaStream_t s);

// The barrier-free variant (tmc_stream.cu): up to two items open per block.
size_t walk_stream_smem(uint32_t max_shells, int block);
// Sets the shared-memory limit of the list form (queue = false) or the queue
// form and returns its resident grid.
cudaError_t walk_stream_prepare(int block, uint32_t math, uint32_t max_shells, int sms, int *grid,
                                bool queue = false);
cudaError_t walk_stream_launch(const BatchArgs &a, int block, uint32_t math, int grid, cudaStream_t s);

}  // namespace tmc
