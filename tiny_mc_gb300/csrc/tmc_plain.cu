// tmc_plain.cu — the plain photon-walk kernel: one problem, n photons.
//
// Reference path: tiny_mc.c:47-49 calls photon() (photon.c:6-51) once per
// photon.  Here a persistent grid walks all n photons with the loop in
// tmc_walk.cuh.  Deposits go into shared-memory histograms of the problem's
// shells: one per warp where that fits without costing occupancy, else one
// per block; each is added into the 128-bit global tally every flush_steps
// lane steps (2^18 for a warp's, 2^23 / threads for a block's) and at the
// end.
// Shell counts whose histogram does not fit in shared memory at all
// (params.h's SHELLS is any size in the reference) take the global form:
// deposits go straight into the 128-bit global tally with 64-bit atomics.  The
// sums are the same integers in every form.
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

template <int BLOCK, class M, Hist H>
__global__ void __launch_bounds__(BLOCK) walk_plain(const PlainArgs a)
{
    extern __shared__ __align__(16) uint32_t smem[];
    constexpr bool PER_WARP = H == Hist::Warp;
    const uint32_t S = H == Hist::Global ? 0u : a.c.shells;   // words per histogram / 4
    const uint32_t words = (PER_WARP ? BLOCK / 32 : 1) * 4 * S;
    for (uint32_t s = threadIdx.x; s < words; s += BLOCK)
        smem[s] = 0;
    __syncthreads();

    GlobalSource<CHUNK> src;
    src.counter = a.work;
    src.n = a.n_photons;
    src.id_base = a.id_base;
    uint32_t *my = smem + words + threadIdx.x;   // ring slot k: my[k * BLOCK]
    uint32_t *tally = PER_WARP ? smem + (threadIdx.x / 32) * 4 * S : smem;
    const uint32_t steps = walk_loop<BLOCK, M, GlobalSource<CHUNK>, H, REFILL_MIN_SHORT>(
        a.c, src, a.keys, tally, a.tally, my);

    if constexpr (PER_WARP) {
        warp_flush_tally(tally, S, a.tally);
    } else if constexpr (H == Hist::Block) {
        __syncthreads();
        flush_tally<BLOCK>(smem, S, a.tally);
    }
    if (a.steps) {
        const unsigned long long tot = warp_sum_u64(steps);
        if ((threadIdx.x & 31u) == 0 && tot)
            atomicAdd(a.steps, tot);
    }
}

static size_t plain_smem_bytes(uint32_t shells, int block, Hist h)
{
    const size_t hist = h == Hist::Global ? 0 : (size_t)16 * shells * (h == Hist::Warp ? block / 32 : 1);
    return hist + (size_t)4 * SLOTS * block;
}

template <int BLOCK, class M, Hist H>
static cudaError_t set_smem(size_t smem)
{
    return cudaFuncSetAttribute(walk_plain<BLOCK, M, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// Blocks of walk_plain<BLOCK, M, H> resident per SM with `smem` bytes (0 if
// it does not fit).
template <int BLOCK, class M, Hist H>
static cudaError_t occupancy(const DeviceCtx &ctx, size_t smem, int &per_sm)
{
    per_sm = 0;
    const size_t cap = ctx.smem_optin ? ctx.smem_optin : 48 * 1024;
    if (smem > cap)
        return cudaSuccess;
    cudaError_t e = set_smem<BLOCK, M, H>(smem);
    if (e != cudaSuccess)
        return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, walk_plain<BLOCK, M, H>, BLOCK, smem);
}

template <int BLOCK, class M, Hist H>
static cudaError_t launch_t(const PlainLaunch &L, const DeviceCtx &ctx, int per_sm, cudaStream_t stream)
{
    const size_t smem = plain_smem_bytes(L.d.shells, BLOCK, H);
    cudaError_t e = set_smem<BLOCK, M, H>(smem);
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
    walk_plain<BLOCK, M, H><<<(unsigned)grid, BLOCK, smem, stream>>>(a);
    return cudaGetLastError();
}

// Per-warp histograms where they fit at the occupancy a per-block histogram
// would get, else a per-block histogram where it fits, else the global form.
template <int BLOCK, class M>
static cudaError_t launch_m(const PlainLaunch &L, const DeviceCtx &ctx, cudaStream_t stream)
{
    const uint32_t S = L.d.shells;
    int warp_sm = 0, block_sm = 0;
    cudaError_t e = occupancy<BLOCK, M, Hist::Warp>(ctx, plain_smem_bytes(S, BLOCK, Hist::Warp), warp_sm);
    if (e == cudaSuccess)
        e = occupancy<BLOCK, M, Hist::Block>(ctx, plain_smem_bytes(S, BLOCK, Hist::Block), block_sm);
    if (e != cudaSuccess)
        return e;
    if (warp_sm >= 1 && warp_sm >= block_sm)
        return launch_t<BLOCK, M, Hist::Warp>(L, ctx, warp_sm, stream);
    if (block_sm >= 1)
        return launch_t<BLOCK, M, Hist::Block>(L, ctx, block_sm, stream);
    int global_sm = 0;
    e = occupancy<BLOCK, M, Hist::Global>(ctx, plain_smem_bytes(S, BLOCK, Hist::Global), global_sm);
    if (e != cudaSuccess)
        return e;
    return launch_t<BLOCK, M, Hist::Global>(L, ctx, global_sm, stream);
}

template <int BLOCK>
static cudaError_t launch_b(const PlainLaunch &L, const DeviceCtx &ctx, cudaStream_t stream)
{
    return L.p->math == TMC_MATH_FAST ? launch_m<BLOCK, FastMath>(L, ctx, stream)
                                      : launch_m<BLOCK, ExactMath>(L, ctx, stream);
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
