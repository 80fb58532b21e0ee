// tmc_plain.cu — the plain photon-walk kernel: one problem, n photons.
//
// Reference path: tiny_mc.c:47-49 calls photon() (photon.c:6-51) once per
// photon.  Here a persistent grid walks all n photons with the loop in
// tmc_walk.cuh; each block owns a shared-memory histogram of the problem's
// shells and adds it to the 128-bit global tally once at the end.  Shell
// counts whose histogram does not fit in shared memory (params.h's SHELLS is
// any size in the reference) take the WIDE form: deposits go straight into the
// 128-bit global tally with 64-bit atomics; the sums are the same integers.
#include <algorithm>

#include "tmc_internal.h"
#include "tmc_walk.cuh"

namespace tmc {

constexpr int CHUNK = 256;      // photon ids a warp claims per atomic

struct PlainArgs {
    PhiloxKeys keys;
    WalkConsts c;
    unsigned long long n_photons;
    unsigned long long id_base;
    unsigned long long *tally;   // [shells][4]: w lo, w hi, w2 lo, w2 hi
    unsigned long long *work;    // photon claim counter, zero at launch
    unsigned long long *steps;   // += photon steps, may be null
};

template <int BLOCK, class M, bool WIDE>
__global__ void __launch_bounds__(BLOCK) walk_plain(const PlainArgs a)
{
    extern __shared__ __align__(16) uint32_t smem[];
    const uint32_t S = WIDE ? 0u : a.c.shells;   // histogram words / 4
    for (uint32_t s = threadIdx.x; s < 4 * S; s += BLOCK)
        smem[s] = 0;
    __syncthreads();

    GlobalSource<CHUNK> src;
    src.counter = a.work;
    src.n = a.n_photons;
    src.id_base = a.id_base;
    uint32_t *my = smem + 4 * S + threadIdx.x;   // ring slot k: my[k * BLOCK]
    const uint32_t steps =
        walk_loop<BLOCK, M, GlobalSource<CHUNK>, WIDE>(a.c, src, a.keys, smem, a.tally, my);

    if constexpr (!WIDE) {
        __syncthreads();
        flush_tally<BLOCK>(smem, S, a.tally);
    }
    if (a.steps) {
        const unsigned long long tot = warp_sum_u64(steps);
        if ((threadIdx.x & 31u) == 0 && tot)
            atomicAdd(a.steps, tot);
    }
}

size_t plain_smem_bytes(uint32_t shells, int block)
{
    return (size_t)16 * shells + (size_t)4 * SLOTS * block;
}

// Largest shell count whose histogram fits beside a block's ring buffers.
static uint32_t histogram_max_shells(const DeviceCtx &ctx, int block)
{
    const size_t cap = ctx.smem_optin ? ctx.smem_optin : 48 * 1024;
    const size_t ring = (size_t)4 * SLOTS * block;
    return cap > ring ? (uint32_t)((cap - ring) / 16) : 0u;
}

template <int BLOCK, class M, bool WIDE>
static cudaError_t launch_t(const PlainLaunch &L, const DeviceCtx &ctx, cudaStream_t stream)
{
    const size_t smem = plain_smem_bytes(WIDE ? 0u : L.d.shells, BLOCK);
    auto kern = walk_plain<BLOCK, M, WIDE>;
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
    a.c.albedo = L.d.albedo;
    a.c.spm = L.d.spm;
    a.c.last = L.d.last;
    a.c.shells = L.d.shells;
    a.n_photons = L.n_photons;
    a.id_base = L.p->photon_id_base;
    a.tally = reinterpret_cast<unsigned long long *>(L.d_tally);
    a.work = L.d_work;
    a.steps = L.d_steps;
    kern<<<(unsigned)grid, BLOCK, smem, stream>>>(a);
    return cudaGetLastError();
}

template <int BLOCK>
static cudaError_t launch_b(const PlainLaunch &L, const DeviceCtx &ctx, cudaStream_t stream)
{
    const bool fast = L.p->math == TMC_MATH_FAST;
    if (L.d.shells <= histogram_max_shells(ctx, BLOCK))
        return fast ? launch_t<BLOCK, FastMath, false>(L, ctx, stream)
                    : launch_t<BLOCK, ExactMath, false>(L, ctx, stream);
    return fast ? launch_t<BLOCK, FastMath, true>(L, ctx, stream)
                : launch_t<BLOCK, ExactMath, true>(L, ctx, stream);
}

cudaError_t launch_plain(const PlainLaunch &L, const DeviceCtx &ctx, cudaStream_t stream)
{
    // 512 threads by default: 3 blocks of 512 and 6 of 256 both fill the SM's
    // 1536 threads at 40 registers, and 512 measured 0.8% faster
    switch (L.block ? L.block : 512) {
    case 128: return launch_b<128>(L, ctx, stream);
    case 256: return launch_b<256>(L, ctx, stream);
    case 512: return launch_b<512>(L, ctx, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace tmc
