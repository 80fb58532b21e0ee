// tmc_plain.cu — the plain photon-walk kernel: one problem, n photons.
//
// Reference path: tiny_mc.c:47-49 calls photon() (photon.c:6-51) once per
// photon.  Here a persistent grid of warps walks all n photons:
//
//  * one photon per thread at a time; when a photon dies in the roulette
//    (photon.c:45-49) its lane takes the next photon id from a chunk its warp
//    claimed from a global counter, so lanes never idle while work remains;
//  * the rejection loop of photon.c:36-40 is unrolled into the main loop: each
//    iteration makes exactly one rejection try, and a photon whose try failed
//    skips the move/absorb part on the next iteration.  Lanes of a warp thus
//    stay in lock-step instead of waiting for the lane with the most retries;
//  * random words come from a per-thread ring of RING words in shared memory,
//    refilled four at a time from Philox.  One iteration consumes at most four
//    words (step, two for the try, roulette), and the refill at the top keeps
//    at least four buffered, so no draw inside the iteration needs a refill.
//    The refill runs only when some lane of the warp is short, and then every
//    lane with room refills, so Philox runs with most lanes active;
//  * the two tallies of photon.c:30-31 go into a per-block shared-memory
//    histogram of 64-bit fixed-point sums (sum of w and of w^2 in 2^-40
//    units); a wrap of a 64-bit shared sum carries 2^64 into the 128-bit
//    global tally, and each block flushes its histogram once at the end.
#include <algorithm>

#include "tmc_device.cuh"
#include "tmc_internal.h"

namespace tmc {

constexpr int RING = 16;        // random words buffered per thread
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
    extern __shared__ __align__(16) unsigned long long smem[];
    unsigned long long *sh_w = smem;
    unsigned long long *sh_w2 = smem + a.shells;
    uint32_t *ring = reinterpret_cast<uint32_t *>(smem + 2 * a.shells);

    for (uint32_t s = threadIdx.x; s < a.shells; s += BLOCK) {
        sh_w[s] = 0;
        sh_w2[s] = 0;
    }
    __syncthreads();

    uint32_t *my = ring + threadIdx.x;   // word k of the ring: my[k * BLOCK]
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
    unsigned long long steps = 0;

    for (;;) {
        // -------- hand new photon ids to lanes whose photon died
        const unsigned need = __ballot_sync(FULL_MASK, want);
        if (need) {
            const unsigned n = __popc(need);
            const unsigned rank = __popc(need & lt_mask);
            unsigned long long id = 0;
            bool got = false;
            const unsigned take0 = (unsigned)min((unsigned long long)n, cend - cnext);
            if (want && rank < take0) {
                id = cnext + rank;
                got = true;
            }
            cnext += take0;
            if (n > take0 && !exhausted) {
                unsigned long long base = 0;
                if (lane == 0)
                    base = atomicAdd(a.work, (unsigned long long)CHUNK);
                base = __shfl_sync(FULL_MASK, base, 0);
                if (base >= a.n_photons) {
                    exhausted = true;
                } else {
                    cnext = base;
                    cend = min(base + (unsigned long long)CHUNK, a.n_photons);
                    const unsigned take1 =
                        (unsigned)min((unsigned long long)(n - take0), cend - cnext);
                    if (want && rank >= take0 && rank - take0 < take1) {
                        id = cnext + (rank - take0);
                        got = true;
                    }
                    cnext += take1;
                }
            }
            if (want) {
                want = false;
                alive = got;
                if (got) {   // launch, photon.c:12-18
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
            }
        }
        if (__ballot_sync(FULL_MASK, alive) == 0)
            break;

        // -------- keep >= 4 random words buffered (one iteration uses <= 4)
        if (__any_sync(FULL_MASK, alive && (prod - cur) < 4u)) {
            if (alive && (prod - cur) <= (uint32_t)(RING - 4)) {
                const uint4 r = philox4x32_10(blk, 0u, pid_lo, pid_hi, a.keys);
                ++blk;
                uint32_t *dst = my + (prod & (RING - 1)) * BLOCK;
                dst[0 * BLOCK] = r.x;
                dst[1 * BLOCK] = r.y;
                dst[2 * BLOCK] = r.z;
                dst[3 * BLOCK] = r.w;
                prod += 4;
            }
        }

        if (alive) {
            if (!pending) {
                // move, photon.c:21-24
                const float U = uniform01(my[(cur & (RING - 1)) * BLOCK]);
                ++cur;
                const float t = M::step_length(U);
                x = M::move(x, t, u);
                y = M::move(y, t, v);
                z = M::move(z, t, w);
                // absorb, photon.c:26-32 (clamp in float: same shell for every
                // radius below 2^32 shells, and a NaN radius lands last)
                const float rr = M::radius_shells(x, y, z, a.spm);
                const uint32_t shell = __float2uint_rz(fminf(rr, a.last));
                add_carry(&sh_w[shell], &g[4 * shell + 1], fx40(weight));
                add_carry(&sh_w2[shell], &g[4 * shell + 3], fx40(__fmul_rn(weight, weight)));
                weight = M::mul(weight, a.albedo);
                ++steps;
            }
            // one try of the rejection method, photon.c:36-40
            const float xi1 = uniform_pm1(my[(cur & (RING - 1)) * BLOCK]);
            const float xi2 = uniform_pm1(my[((cur + 1) & (RING - 1)) * BLOCK]);
            cur += 2;
            const float tt = M::norm2(xi1, xi2);
            pending = (1.0f < tt);
            if (!pending) {
                // new direction, photon.c:41-43
                u = fmaf(2.0f, tt, -1.0f);
                const float sc = M::dir_scale(tt, u);
                v = M::mul(xi1, sc);
                w = M::mul(xi2, sc);
                // roulette, photon.c:45-49
                if (weight < 0.001f) {
                    const float U = uniform01(my[(cur & (RING - 1)) * BLOCK]);
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
    for (uint32_t s = threadIdx.x; s < a.shells; s += BLOCK) {
        flush128(&g[4 * s + 0], &g[4 * s + 1], sh_w[s]);
        flush128(&g[4 * s + 2], &g[4 * s + 3], sh_w2[s]);
    }
    if (a.steps) {
        steps = warp_sum_u64(steps);
        if (lane == 0 && steps)
            atomicAdd(a.steps, steps);
    }
}

size_t plain_smem_bytes(uint32_t shells, int block)
{
    return (size_t)16 * shells + (size_t)4 * RING * block;
}

int plain_max_shells(const DeviceCtx &ctx)
{
    const size_t cap = ctx.smem_optin ? ctx.smem_optin : 48 * 1024;
    const size_t ring = (size_t)4 * RING * 256;
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
