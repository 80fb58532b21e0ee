// tmc_plain.cu — the plain photon-walk kernel: one problem, n photons.
//
// Reference path: tiny_mc.c:47-49 calls photon() (photon.c:6-51) once per
// photon.  Here a persistent grid of warps walks all n photons:
//
//  * one photon per thread at a time; when a photon dies in the roulette
//    (photon.c:45-49) its lane takes the next photon id from a chunk its warp
//    claimed from a global counter, so lanes never idle while work remains;
//  * the rejection loop of photon.c:36-40 is folded into the main loop: each
//    iteration evaluates the next two rejection tries from the buffered
//    stream and consumes only the words photon.c would (two if the first try
//    is accepted, four otherwise).  A photon whose two tries both failed
//    (p = 0.046) skips the move/absorb part on the next iteration.  Lanes of a
//    warp thus stay in lock-step instead of waiting for the lane with the
//    most retries;
//  * random words come from a per-thread ring of RING words in shared memory,
//    refilled four at a time from Philox.  One iteration consumes at most six
//    words (step, four for two tries, roulette), and the refill at the top
//    keeps at least six buffered, so no draw inside the iteration needs a
//    refill.  The refill runs only when some lane of the warp is short, and
//    then every lane with room refills, so Philox runs with most lanes active;
//  * the two tallies of photon.c:30-31 go into a per-block shared-memory
//    histogram of 64-bit fixed-point sums (sum of w and of w^2 in 2^-40
//    units), each kept as two 32-bit words updated with native 32-bit shared
//    atomics (a 64-bit shared atomicAdd is a compare-and-swap loop); a wrap
//    of a 64-bit shared sum carries 2^64 into the 128-bit global tally, and
//    each block flushes its histogram once at the end.
#include <algorithm>

#include "tmc_device.cuh"
#include "tmc_internal.h"

namespace tmc {

constexpr int RING = 16;        // random words buffered per thread
constexpr int MIRROR = 6;       // slots 16..21 repeat slots 0..5: the <= 6 words
                                // one iteration reads never wrap around
constexpr int SLOTS = RING + MIRROR;
constexpr int CHUNK = 256;      // photon ids a warp claims per atomic

struct PlainArgs {
    PhiloxKeys keys;
    float albedo;
    float spm;
    float last;
    uint32_t shells;
    unsigned long long n_photons;
    unsigned long long id_base;
    unsigned long long *tally;   // [shells][4]: w lo, w hi, w2 lo, w2 hi
    unsigned long long *work;    // photon claim counter, zero at launch
    unsigned long long *steps;   // += photon steps, may be null
};

template <int BLOCK, class M>
__global__ void __launch_bounds__(BLOCK) walk_plain(const PlainArgs a)
{
    extern __shared__ __align__(16) uint32_t smem[];
    // tallies, [shells] each: low and high words of sum w, then of sum w^2
    const uint32_t S = a.shells;
    uint32_t *ring = smem + 4 * S;

    for (uint32_t s = threadIdx.x; s < 4 * S; s += BLOCK)
        smem[s] = 0;
    __syncthreads();

    uint32_t *my = ring + threadIdx.x;   // slot k of this thread's ring: my[k * BLOCK]
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;
    unsigned long long *g = a.tally;

    // warp-uniform chunk of photon ids
    unsigned long long cnext = 0, cend = 0;
    bool exhausted = false;

    // lane state
    bool alive = false, want = true, pending = false;
    uint32_t pid_lo = 0, pid_hi = 0, blk = 0, prod = 0, cur = 0;
    float x = 0.f, y = 0.f, z = 0.f, u = 0.f, v = 0.f, w = 1.f, weight = 1.f;
    uint32_t steps = 0;   // < 2^32 per thread for any launch this library makes

    for (;;) {
        // -------- hand new photon ids to lanes whose photon died
        const unsigned need = __ballot_sync(FULL_MASK, want);
        if (need) {
            const unsigned n = __popc(need);
            const unsigned rank = __popc(need & lt_mask);
            unsigned long long id = cnext + rank;
            bool got = rank < cend - cnext;
            if (n > cend - cnext) {
                // the current chunk runs out: claim the next one
                const unsigned take0 = (unsigned)(cend - cnext);
                unsigned long long base = 0;
                if (!exhausted) {
                    if (lane == 0)
                        base = atomicAdd(a.work, (unsigned long long)CHUNK);
                    base = __shfl_sync(FULL_MASK, base, 0);
                    exhausted = base >= a.n_photons;
                }
                if (exhausted) {
                    cnext = cend;
                } else {
                    cend = min(base + (unsigned long long)CHUNK, a.n_photons);
                    if (!got) {
                        id = base + (rank - take0);
                        got = id < cend;
                    }
                    cnext = min(base + (n - take0), cend);
                }
            } else {
                cnext += n;
            }
            if (want) {
                want = false;
                alive = got;
                // launch, photon.c:12-18
                const unsigned long long pid = a.id_base + id;
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

        // -------- keep >= 6 random words buffered (one iteration uses <= 6);
        // a fresh photon starts empty and needs two passes
        while (__any_sync(FULL_MASK, alive && (prod - cur) < 6u)) {
            if (alive && (prod - cur) <= (uint32_t)(RING - 4)) {
                const uint4 r = philox4x32_10(blk, 0u, pid_lo, pid_hi, a.keys);
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

        if (alive) {
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
                const float rr = M::radius_shells(x, y, z, a.spm);
                const uint32_t shell = __float2uint_rz(fminf(rr, a.last));
                uint32_t *t0 = smem + shell;
                uint32_t lo, hi;
                fx40_split(weight, lo, hi);
                tally_add(t0, t0 + S, &g[4 * shell + 1], lo, hi);
                fx40_split(__fmul_rn(weight, weight), lo, hi);
                tally_add(t0 + 2 * S, t0 + 3 * S, &g[4 * shell + 3], lo, hi);
                weight = M::mul(weight, a.albedo);
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

    __syncthreads();
    for (uint32_t s = threadIdx.x; s < S; s += BLOCK) {
        flush128(&g[4 * s + 0], &g[4 * s + 1], ((unsigned long long)smem[S + s] << 32) | smem[s]);
        flush128(&g[4 * s + 2], &g[4 * s + 3],
                 ((unsigned long long)smem[3 * S + s] << 32) | smem[2 * S + s]);
    }
    if (a.steps) {
        const unsigned long long tot = warp_sum_u64(steps);
        if (lane == 0 && tot)
            atomicAdd(a.steps, tot);
    }
}

size_t plain_smem_bytes(uint32_t shells, int block)
{
    return (size_t)16 * shells + (size_t)4 * SLOTS * block;
}

int plain_max_shells(const DeviceCtx &ctx)
{
    const size_t cap = ctx.smem_optin ? ctx.smem_optin : 48 * 1024;
    const size_t ring = (size_t)4 * SLOTS * 256;
    return cap > ring ? (int)((cap - ring) / 16) : 0;
}

template <int BLOCK, class M>
static cudaError_t launch_t(const PlainLaunch &L, const DeviceCtx &ctx, cudaStream_t stream)
{
    const size_t smem = plain_smem_bytes(L.d.shells, BLOCK);
    auto kern = walk_plain<BLOCK, M>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BLOCK, smem);
    if (e != cudaSuccess)
        return e;
    if (per_sm < 1)
        return cudaErrorInvalidConfiguration;
    if (L.blocks_per_sm > 0)
        per_sm = std::min(per_sm, L.blocks_per_sm);
    unsigned long long grid = (unsigned long long)ctx.sms * per_sm;
    // no more blocks than there are photon chunks to hand out
    const unsigned long long warps_needed = (L.n_photons + CHUNK - 1) / CHUNK;
    const unsigned long long blocks_needed = (warps_needed + BLOCK / 32 - 1) / (BLOCK / 32);
    grid = std::max(1ull, std::min(grid, blocks_needed));
    if (L.max_blocks > 0)
        grid = std::min(grid, (unsigned long long)L.max_blocks);

    PlainArgs a;
    a.keys = make_philox_keys(L.p->seed);
    a.albedo = L.d.albedo;
    a.spm = L.d.spm;
    a.last = L.d.last;
    a.shells = L.d.shells;
    a.n_photons = L.n_photons;
    a.id_base = L.p->photon_id_base;
    a.tally = reinterpret_cast<unsigned long long *>(L.d_tally);
    a.work = L.d_work;
    a.steps = L.d_steps;
    kern<<<(unsigned)grid, BLOCK, smem, stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_plain(const PlainLaunch &L, const DeviceCtx &ctx, cudaStream_t stream)
{
    const int block = L.block ? L.block : 256;
    const bool fast = L.p->math == TMC_MATH_FAST;
    switch (block) {
    case 128:
        return fast ? launch_t<128, FastMath>(L, ctx, stream) : launch_t<128, ExactMath>(L, ctx, stream);
    case 256:
        return fast ? launch_t<256, FastMath>(L, ctx, stream) : launch_t<256, ExactMath>(L, ctx, stream);
    case 512:
        return fast ? launch_t<512, FastMath>(L, ctx, stream) : launch_t<512, ExactMath>(L, ctx, stream);
    default:
        return cudaErrorInvalidValue;
    }
}

}  // namespace tmc
