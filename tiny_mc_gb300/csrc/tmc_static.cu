// tmc_static.cu — tmc_photon_batch_static: the host-array photon walk without
// any device allocation.
//
// tmc_photon_batch allocates its device scratch (the per-shell tallies, the
// FP64 results and the photon claim counter) the first time it runs on a
// device.  Some callers cannot let a library allocate device memory: a host
// program whose device memory belongs to another allocator (a framework's
// caching pool that must see every byte), a real-time loop that forbids
// allocation after start-up, or a plugin host that hands out memory itself.
// This entry point keeps that scratch in a fixed file-scope __device__ array
// instead.  The array belongs to the library's module: a GPU holds it from the
// moment the module is loaded on it until the process exits.  Under lazy
// module loading (the CUDA default) that moment is the first call of this
// entry point on that device, so the first call itself makes the driver load
// the module (and the walk and finalisation kernels it launches): make it
// during start-up, before any stream capture; a call with n_photons = 0 does
// exactly that set-up and walks nothing.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side stand-in), so the first call on each device, with that
// device current, looks the address up with cudaGetSymbolAddress and keeps
// it.  The kept address belongs to the device's primary context: after
// cudaDeviceReset, or when the caller makes another context current on the
// device, it is stale, and that use is not supported.  Every call shares the
// one array and it keeps the last call's contents: each call clears the claim
// counter and the tallies it uses before its walk.  Calls are serialised by
// the library's lock and wait for their own work, so calls through this entry
// point never overlap; work that ran two of them at once on the GPU would race
// on the shared array.
#include <cstring>

#include "tmc_device.cuh"
#include "tmc_internal.h"

namespace tmc {
namespace {

constexpr size_t STATIC_COUNTERS = 256;   // photon claim counter at offset 0
constexpr size_t STATIC_TALLY_BYTES = sizeof(tmc_tally) * TMC_STATIC_MAX_SHELLS;
constexpr size_t STATIC_HEAT_BYTES = 2 * sizeof(double) * TMC_STATIC_MAX_SHELLS;
constexpr size_t STATIC_BYTES = STATIC_COUNTERS + STATIC_TALLY_BYTES + STATIC_HEAT_BYTES;
static_assert(STATIC_BYTES == TMC_STATIC_SCRATCH_BYTES, "scratch size in tmc.h");

// device address of g_static_scratch on each device, looked up once
void *g_static_addr[64];
// FP64 results copied back before they are added to the caller's floats
double g_static_host[2 * TMC_STATIC_MAX_SHELLS];

}  // namespace

static __device__ __align__(256) unsigned char g_static_scratch[STATIC_BYTES];

}  // namespace tmc

using namespace tmc;

extern "C" int tmc_photon_batch_static(float *heat, float *heat2, uint64_t n_photons,
                                       const tmc_params *p, void *stream)
{
    int st = validate(p);
    if (st)
        return st;
    if (!heat || !heat2) {
        set_error_text("tmc_photon_batch_static: heat or heat2 is NULL");
        return TMC_E_INVALID;
    }
    if (p->shells > TMC_STATIC_MAX_SHELLS) {
        set_error_text("tmc_photon_batch_static: shells > TMC_STATIC_MAX_SHELLS (4096)");
        return TMC_E_INVALID;
    }
    if (n_photons > (1ull << 62) || p->photon_id_base > ~0ull - n_photons) {
        set_error_text("tmc_photon_batch_static: photon count or photon_id_base + count overflows "
                       "64-bit photon ids");
        return TMC_E_OVERFLOW;
    }
    std::lock_guard<std::mutex> lk(api_mutex());

    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return set_cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) {
        set_error_text("tmc_photon_batch_static: device ordinal outside 0..63");
        return TMC_E_NODEVICE;
    }
    if (!g_static_addr[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_static_scratch);
        if (e != cudaSuccess)
            return set_cuda_error(e, "cudaGetSymbolAddress(static scratch)");
        g_static_addr[dev] = ptr;
    }
    DeviceCtx c;   // launch limits only; nothing here is allocated
    int sms = 0, optin = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess)
        return set_cuda_error(e, "cudaDeviceGetAttribute");
    c.device = dev;
    c.sms = sms;
    c.smem_optin = (size_t)optin;

    unsigned char *base = static_cast<unsigned char *>(g_static_addr[dev]);
    unsigned long long *work = reinterpret_cast<unsigned long long *>(base);
    tmc_tally *tally = reinterpret_cast<tmc_tally *>(base + STATIC_COUNTERS);
    double *heat_out = reinterpret_cast<double *>(base + STATIC_COUNTERS + STATIC_TALLY_BYTES);
    const uint32_t S = p->shells;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);

    // the array keeps the previous call's contents: clear counter and tallies
    e = cudaMemsetAsync(base, 0, STATIC_COUNTERS + sizeof(tmc_tally) * S, s);
    if (e != cudaSuccess)
        return set_cuda_error(e, "cudaMemsetAsync(static scratch)");
    const Derived d = derive(p->mu_a, p->mu_s, p->microns_per_shell, S);
    // launched even for zero photons (one block that walks nothing), so that a
    // zero-photon first call also loads the walk kernel
    PlainLaunch L{};
    L.p = p;
    L.d = d;
    L.n_photons = n_photons;
    L.d_tally = tally;
    L.d_work = work;
    L.d_steps = nullptr;
    e = launch_plain(L, c, s);
    if (e != cudaSuccess)
        return set_cuda_error(e, "walk_plain launch (static)");
    e = launch_tally_to_heat(tally, S, (double)d.c, heat_out, heat_out + S, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(g_static_host, heat_out, sizeof(double) * 2 * S, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_photon_batch_static");
    for (uint32_t i = 0; i < S; ++i) {
        heat[i] = (float)((double)heat[i] + g_static_host[i]);
        heat2[i] = (float)((double)heat2[i] + g_static_host[S + i]);
    }
    return TMC_OK;
}
