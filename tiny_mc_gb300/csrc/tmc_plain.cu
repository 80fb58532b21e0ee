// tmc_plain.cu — the plain photon-walk kernel: one problem, n photons.
//
// Reference path: tiny_mc.c:47-49 calls photon() (photon.c:6-51) once per
// photon.  Here a persistent grid walks all n photons with the loop in
// tmc_walk.cuh; each block owns a shared-memory histogram of the problem's
// shells and adds it to the 128-bit global tally once at the end.
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

template <int BLOCK, class M>
__global__ void __launch_bounds__(BLOCK) walk_plain(const PlainArgs a)
{
    extern __shared__ __align__(16) uint32_t smem[];
    const uint32_t S = a.c.shells;
    for (uint32_t s = threadIdx.x; s < 4 * S; s += BLOCK)
        smem[s] = 0;
    __syncthreads();

    GlobalSource<CHUNK> src;
    src.counter = a.work;
    src.n = a.n_photons;
    src.id_base = a.id_base;
    uint32_t *my = smem + 4 * S + threadIdx.x;   // ring slot k: my[k * BLOCK]
    const uint32_t steps = walk_loop<BLOCK, M>(a.c, src, a.keys, smem, a.tally, my);

    __syncthreads();
    flush_tally<BLOCK>(smem, S, a.tally);
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
