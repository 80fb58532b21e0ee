// tmc_walk.cuh — the photon-walk loop shared by the plain and batched kernels.
//
// Reference path: tiny_mc.c:47-49 calls photon() (photon.c:6-51) once per
// photon.  Here every thread of a persistent grid carries one photon at a
// time and warps refill dead lanes with new photon ids:
//
//  * when a photon dies in the roulette (photon.c:45-49) its lane takes the
//    next photon id from a chunk its warp claimed from a PhotonSource (a
//    global counter for the plain kernel, a shared-memory counter over one
//    work item for the batched kernel), so lanes never idle while work
//    remains;
//  * the rejection loop of photon.c:36-40 is folded into the main loop: each
//    iteration evaluates the next two rejection tries from the buffered
//    stream and consumes only the words photon.c would (two if the first try
//    is accepted, four otherwise).  A photon whose two tries both failed
//    (p = 0.046) skips the move/absorb part on the next iteration, so lanes
//    of a warp stay in lock-step instead of waiting for the lane with the
//    most retries;
//  * random words come from a per-thread ring of 16 words in shared memory,
//    refilled four at a time from Philox; slots 16..21 mirror 0..5 so the
//    <= 6 words one iteration reads are fixed offsets from one base.  An
//    iteration needs >= 6 buffered words (it consumes at most six: step,
//    four for two tries, roulette); the refill at the top runs once at least
//    four walking lanes are short (a short lane waits an iteration or two
//    rather than make the whole warp pay for a Philox block few lanes use),
//    and then every lane with room refills, so Philox runs with most lanes
//    active;
//  * the two tallies of photon.c:30-31 go into a shared-memory histogram of
//    64-bit fixed-point sums (sum of w and of w^2, 2^-40 units), each kept as
//    two 32-bit words updated with native 32-bit shared atomics (a 64-bit
//    shared atomicAdd is a compare-and-swap loop, 4x slower here).  The
//    histogram is one per warp (the plain kernel, where that fits) or one per
//    block; either way it is added into the 128-bit global tally and cleared
//    each time one of its lanes' step count reaches a multiple of a bound
//    (flush_steps), which keeps its 64-bit sums from wrapping, so a deposit
//    needs no wrap check.
#pragma once

#include "tmc_device.cuh"

namespace tmc {

constexpr int RING = 16;        // random words buffered per thread
constexpr int MIRROR = 6;       // slots 16..21 repeat slots 0..5
constexpr int SLOTS = RING + MIRROR;
// The warp runs a Philox refill pass once this many walking lanes are short
// of words (or every walking lane is).  Measured on the plain walk, 2^30
// photons of params.h optics: 1 lane 716 ms, 2 lanes 683, 4 lanes 673, 8
// lanes 681, 16 lanes 709.
constexpr int REFILL_MIN_SHORT = 4;
// The same for the batched kernels, whose warps run short of photons at the
// end of every work item.  Measured on the 4096-problem sweep at 1/64 photon
// scale: walk_batch (128 threads, 16 items) 1.04e11 photon-steps/s with 2
// against 1.00e11 with 4; walk_stream (256, 16) 1.006e11 against 0.993e11.
constexpr int REFILL_MIN_SHORT_ITEMS = 2;

// Where a walk keeps its tallies.  Warp: one shared histogram per warp.
// Block: one per block, shared by its warps.  Global: none; every deposit is
// a 64-bit atomic add into the 128-bit global tally (shell counts whose
// histogram does not fit in shared memory).
enum class Hist { Warp, Block, Global };

// A shared histogram written by `lanes` lanes is added into the global tally
// and cleared each time one of those lanes' step count reaches a multiple of
// flush_steps(lanes), checked at the top of every iteration (in which a lane
// steps at most once) for every lane that walks a photon or has just lost one
// (a block's histogram skips lanes left without a photon at the end of a
// small work item, which would otherwise flush on every iteration).  A lane's
// count changes only while it walks, so every lane is checked at every
// multiple it reaches and deposits at most flush_steps + 1 times between two
// flushes.  A deposit adds at most 2^8 + 1 to a high word (w <= 1, plus the
// low word's carry), so a high word stays below
// lanes * 257 * (2^23 / lanes + 1) < 2^32: the 64-bit sums never wrap.
__host__ __device__ constexpr uint32_t flush_steps(uint32_t lanes)
{
    return (1u << 23) / lanes;
}
static_assert(512ull * 257ull * ((1ull << 23) / 512 + 1) < (1ull << 32), "high word bound");
static_assert(32ull * 257ull * ((1ull << 23) / 32 + 1) < (1ull << 32), "high word bound");

// Add a warp's own histogram (4 * S words) into the 128-bit global tally and
// clear it.  Warp-collective.
__device__ __forceinline__ void warp_flush_tally(uint32_t *tally, uint32_t S, unsigned long long *g)
{
    __syncwarp();
    for (uint32_t s = threadIdx.x & 31u; s < S; s += 32) {
        flush128(&g[4 * s + 0], &g[4 * s + 1], ((unsigned long long)tally[S + s] << 32) | tally[s]);
        flush128(&g[4 * s + 2], &g[4 * s + 3],
                 ((unsigned long long)tally[3 * S + s] << 32) | tally[2 * S + s]);
        tally[s] = 0;
        tally[S + s] = 0;
        tally[2 * S + s] = 0;
        tally[3 * S + s] = 0;
    }
    __syncwarp();
}

// Add a block's histogram into the 128-bit global tally and clear it, by one
// warp while the others keep depositing: every word is taken with an atomic
// exchange against zero.  Sums stay exact: a deposit's low-word overflow is
// carried into a high word by the depositing lane, whichever side of an
// exchange either add lands on, and every word's content reaches the global
// tally at one flush or the next.  probe_acc / probe_hi (shared, may be
// null): the 128-bit running sum of the w words taken from shell
// probe_shell.  Warp-collective.
__device__ __forceinline__ void swap_flush_tally(uint32_t *tally, uint32_t S, unsigned long long *g,
                                                 unsigned long long *probe_acc, uint32_t *probe_hi,
                                                 uint32_t probe_shell)
{
    for (uint32_t s = threadIdx.x & 31u; s < S; s += 32) {
        const uint32_t lo = atomicExch(&tally[s], 0u);
        const uint32_t hi = atomicExch(&tally[S + s], 0u);
        const unsigned long long v = ((unsigned long long)hi << 32) | lo;
        flush128(&g[4 * s + 0], &g[4 * s + 1], v);
        if (probe_acc && s == probe_shell && v) {
            const unsigned long long old = atomicAdd(probe_acc, v);
            if (old + v < old)
                atomicAdd(probe_hi, 1u);
        }
        const uint32_t lo2 = atomicExch(&tally[2 * S + s], 0u);
        const uint32_t hi2 = atomicExch(&tally[3 * S + s], 0u);
        flush128(&g[4 * s + 2], &g[4 * s + 3], ((unsigned long long)hi2 << 32) | lo2);
    }
}

// Per-problem constants of photon.c:8-9 (computed on the host in float,
// exactly as photon.c does) plus the shell count.
struct WalkConsts {
    float albedo;
    float spm;     // shells_per_mfp
    float last;    // (float)(shells - 1)
    uint32_t shells;
};

// Photon ids from a global 64-bit counter over [0, n): each warp claims
// CHUNK ids per atomic.
template <int CHUNK>
struct GlobalSource {
    unsigned long long *counter;
    unsigned long long n;
    unsigned long long id_base;
    unsigned long long cnext = 0, cend = 0;
    bool exhausted = false;

    // Warp-collective.  need = ballot of lanes wanting a photon, rank = this
    // lane's index among them.  Returns true and the photon id if this lane
    // got one (only meaningful for wanting lanes).
    __device__ __forceinline__ bool next(unsigned need, unsigned rank, unsigned lane,
                                         unsigned long long &pid)
    {
        const unsigned n_need = __popc(need);
        unsigned long long id = cnext + rank;
        bool got = rank < cend - cnext;
        if (n_need > cend - cnext) {
            const unsigned take0 = (unsigned)(cend - cnext);
            unsigned long long base = 0;
            if (!exhausted) {
                if (lane == 0)
                    base = atomicAdd(counter, (unsigned long long)CHUNK);
                base = __shfl_sync(FULL_MASK, base, 0);
                exhausted = base >= n;
            }
            if (exhausted) {
                cnext = cend;
            } else {
                cend = min(base + (unsigned long long)CHUNK, n);
                if (!got) {
                    id = base + (rank - take0);
                    got = id < cend;
                }
                cnext = min(base + (n_need - take0), cend);
            }
        } else {
            cnext += n_need;
        }
        pid = id_base + id;
        return got;
    }
};

// Photon ids from a shared-memory 32-bit counter over one work item of
// `count` photons starting at id `first`.
template <int CHUNK>
struct SharedSource {
    uint32_t *counter;   // shared memory, zero at the start of the item
    uint32_t count;
    unsigned long long first;
    uint32_t cnext = 0, cend = 0;
    bool exhausted = false;

    __device__ __forceinline__ bool next(unsigned need, unsigned rank, unsigned lane,
                                         unsigned long long &pid)
    {
        const unsigned n_need = __popc(need);
        uint32_t id = cnext + rank;
        bool got = rank < cend - cnext;
        if (n_need > cend - cnext) {
            const unsigned take0 = cend - cnext;
            uint32_t base = 0;
            if (!exhausted) {
                if (lane == 0)
                    base = atomicAdd(counter, (uint32_t)CHUNK);
                base = __shfl_sync(FULL_MASK, base, 0);
                exhausted = base >= count;
            }
            if (exhausted) {
                cnext = cend;
            } else {
                cend = min(base + (uint32_t)CHUNK, count);
                if (!got) {
                    id = base + (rank - take0);
                    got = id < cend;
                }
                cnext = min(base + (n_need - take0), cend);
            }
        } else {
            cnext += n_need;
        }
        pid = first + id;
        return got;
    }
};

// Walk photons from `src` until it is exhausted and every lane's photon has
// died.  Warp-collective: all 32 lanes of every warp call it.  tally: the
// shared histogram (H = Warp: this warp's; Block: the block's), 4 * shells
// words (low and high of sum w, then of sum w^2), flushed into g, the
// problem's global 128-bit tally [shells][4], every flush_steps lane steps;
// the caller flushes what is left.  probe_acc / probe_hi (Block only, may be
// null): receive the w sums those flushes take from shell probe_shell.
// Returns this thread's photon steps.
template <int BLOCK, class M, class Source, Hist H, int MIN_SHORT = REFILL_MIN_SHORT_ITEMS>
__device__ __forceinline__ uint32_t walk_loop(const WalkConsts c, Source &src,
                                              const PhiloxKeys &keys, uint32_t *tally,
                                              unsigned long long *g, uint32_t *my,
                                              unsigned long long *probe_acc = nullptr,
                                              uint32_t *probe_hi = nullptr,
                                              uint32_t probe_shell = 0)
{
    const uint32_t S = c.shells;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;

    bool alive = false, want = true, pending = false;
    uint32_t pid_lo = 0, pid_hi = 0, blk = 0, prod = 0, cur = 0;
    float x = 0.f, y = 0.f, z = 0.f, u = 0.f, v = 0.f, w = 1.f, weight = 1.f;
    uint32_t steps = 0;

    for (;;) {
        // -------- hand new photon ids to lanes whose photon died (shared
        // histograms: also flush it when a lane's step count reaches a
        // multiple of the flush bound)
        constexpr bool SHARED = H != Hist::Global;
        constexpr uint32_t FLUSH_MASK = flush_steps(H == Hist::Warp ? 32u : (uint32_t)BLOCK) - 1u;
        const bool at_bound = (steps & FLUSH_MASK) == 0u && (H == Hist::Warp || alive || want);
        const unsigned need = __ballot_sync(FULL_MASK, want || (SHARED && at_bound));
        if (need) {
            unsigned want_mask = need;
            if constexpr (SHARED) {
                if (__any_sync(FULL_MASK, at_bound)) {
                    if constexpr (H == Hist::Warp)
                        warp_flush_tally(tally, S, g);
                    else
                        swap_flush_tally(tally, S, g, probe_acc, probe_hi, probe_shell);
                }
                want_mask = __ballot_sync(FULL_MASK, want);
            }
            unsigned long long pid = 0;
            const bool got = want_mask ? src.next(want_mask, __popc(want_mask & lt_mask), lane, pid)
                                       : false;
            if (want) {
                want = false;
                alive = got;
                // launch, photon.c:12-18
                pid_lo = (uint32_t)pid;
                pid_hi = (uint32_t)(pid >> 32);
                blk = 0;
                cur = prod;   // drop words buffered for the previous photon
                pending = false;
                x = y = z = 0.f;
                u = v = 0.f;
                w = 1.f;
                weight = 1.f;
            }
            // lanes change from alive to idle only here
            if (__ballot_sync(FULL_MASK, alive) == 0)
                break;
        }

        // -------- refill: an iteration needs >= 6 buffered words (it uses
        // <= 6).  The warp runs Philox only once MIN_SHORT walking lanes
        // are short (or every walking lane is): a refill costs the
        // whole warp the same issue slots however many lanes take part, so a
        // short lane waits instead (the others, using >= 2 words each per
        // iteration, soon join it).  A fresh photon starts empty and needs two
        // passes.
        for (;;) {
            const unsigned low = __ballot_sync(FULL_MASK, alive && (prod - cur) < 6u);
            if (low == 0 ||
                (__popc(low) < MIN_SHORT && low != __ballot_sync(FULL_MASK, alive)))
                break;
            if (alive && (prod - cur) <= (uint32_t)(RING - 4)) {
                const uint4 r = philox4x32_10(blk, 0u, pid_lo, pid_hi, keys);
                ++blk;
                const uint32_t p = prod & (RING - 1);
                uint32_t *dst = my + p * BLOCK;
                dst[0 * BLOCK] = r.x;
                dst[1 * BLOCK] = r.y;
                dst[2 * BLOCK] = r.z;
                dst[3 * BLOCK] = r.w;
                // mirror: slots 16..19 repeat 0..3, slots 20..21 repeat 4..5
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
            // the <= 6 words this iteration may read, from one base
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
                // absorb, photon.c:26-32 (clamp in float: same shell for every
                // radius below 2^32 shells, and a NaN radius lands last)
                const float rr = M::radius_shells(x, y, z, c.spm);
                const uint32_t shell = __float2uint_rz(fminf(rr, c.last));
                uint32_t lo, hi;
                if constexpr (H == Hist::Global) {
                    fx40_split(weight, lo, hi);
                    flush128(&g[4 * shell + 0], &g[4 * shell + 1], ((unsigned long long)hi << 32) | lo);
                    fx40_split(__fmul_rn(weight, weight), lo, hi);
                    flush128(&g[4 * shell + 2], &g[4 * shell + 3], ((unsigned long long)hi << 32) | lo);
                } else {
                    uint32_t *t0 = tally + shell;
                    fx40_split(weight, lo, hi);
                    tally_add_nowrap(t0, t0 + S, lo, hi);
                    fx40_split(__fmul_rn(weight, weight), lo, hi);
                    tally_add_nowrap(t0 + 2 * S, t0 + 3 * S, lo, hi);
                }
                weight = M::mul(weight, c.albedo);
                ++steps;
            }
            // the next two tries of the rejection method, photon.c:36-40; the
            // second one's words are consumed only if the first is rejected
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
                    } else {
                        weight = __fdiv_rn(weight, 0.1f);
                    }
                }
            }
        }
    }
    return steps;
}

// Add a block's shared histogram (4 * shells words) into a 128-bit global
// tally [shells][4].  Block-collective, after a barrier.
template <int BLOCK>
__device__ __forceinline__ void flush_tally(const uint32_t *tally, uint32_t S, unsigned long long *g)
{
    for (uint32_t s = threadIdx.x; s < S; s += BLOCK) {
        flush128(&g[4 * s + 0], &g[4 * s + 1], ((unsigned long long)tally[S + s] << 32) | tally[s]);
        flush128(&g[4 * s + 2], &g[4 * s + 3],
                 ((unsigned long long)tally[3 * S + s] << 32) | tally[2 * S + s]);
    }
}

}  // namespace tmc
