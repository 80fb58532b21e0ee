// tmc_api.cu — the C ABI (include/tmc.h): validation, per-device resources,
// the drop-in photon_batch entry points and the FP64 finalisation kernel.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "tmc_device.cuh"
#include "tmc_internal.h"

namespace tmc {

namespace {
std::mutex g_mutex;
thread_local std::string g_error;   // per thread, like errno
DeviceCtx g_ctx[64];
int g_plain_block = 0;
int g_plain_blocks_per_sm = 0;
int g_plain_max_blocks = 0;
}  // namespace

std::mutex &api_mutex() { return g_mutex; }

void set_error_text(const std::string &s) { g_error = s; }

int set_cuda_error(cudaError_t e, const char *where)
{
    char buf[256];
    std::snprintf(buf, sizeof buf, "%s: %s (%s)", where, cudaGetErrorString(e), cudaGetErrorName(e));
    g_error = buf;
    if (e == cudaErrorMemoryAllocation)
        return TMC_E_NOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ||
        e == cudaErrorNoKernelImageForDevice)
        return TMC_E_NODEVICE;
    return TMC_E_CUDA;
}

int validate(const tmc_params *p)
{
    auto invalid = [](const char *why) {
        set_error_text(std::string("invalid parameters: ") + why);
        return TMC_E_INVALID;
    };
    if (!p)
        return invalid("null tmc_params");
    if (p->shells == 0 || p->shells > (1u << 24))
        return invalid("shells must be 1 .. 2^24");
    // MU_A "!!non-zero!!" (params.h:14): with mu_a = 0 the weight never
    // decays and a photon never dies.
    if (!(p->mu_a > 0.0f) || !std::isfinite(p->mu_a))
        return invalid("mu_a must be finite and > 0");
    if (!(p->mu_s >= 0.0f) || !std::isfinite(p->mu_s))
        return invalid("mu_s must be finite and >= 0");
    if (!(p->microns_per_shell > 0.0f) || !std::isfinite(p->microns_per_shell))
        return invalid("microns_per_shell must be finite and > 0");
    if (p->math != TMC_MATH_EXACT && p->math != TMC_MATH_FAST)
        return invalid("math must be TMC_MATH_EXACT or TMC_MATH_FAST");
    if (p->reserved != 0)
        return invalid("reserved must be 0");
    // If mu_a is so small against mu_s that the float albedo rounds to 1, the
    // weight never decays (photon.c:32) and no photon would ever die.
    if (!(p->mu_s / (p->mu_s + p->mu_a) < 1.0f))
        return invalid("mu_a too small against mu_s: the float albedo rounds to 1");
    return TMC_OK;
}

Derived derive(float mu_a, float mu_s, float microns_per_shell, uint32_t shells)
{
    Derived d;
    d.albedo = mu_s / (mu_s + mu_a);                                      // photon.c:8
    d.spm = (float)(1e4 / (double)microns_per_shell / (double)(mu_a + mu_s));  // photon.c:9
    d.c = 1.0f - d.albedo;
    d.last = (float)(shells - 1);
    d.shells = shells;
    return d;
}

DeviceCtx *current_ctx(int *status)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        *status = set_cuda_error(e, "cudaGetDevice");
        return nullptr;
    }
    if (dev < 0 || dev >= 64) {
        *status = TMC_E_NODEVICE;
        return nullptr;
    }
    DeviceCtx &c = g_ctx[dev];
    if (c.device < 0) {
        cudaDeviceProp prop;
        e = cudaGetDeviceProperties(&prop, dev);
        if (e != cudaSuccess) {
            *status = set_cuda_error(e, "cudaGetDeviceProperties");
            return nullptr;
        }
        c.sms = prop.multiProcessorCount;
        c.cc_major = prop.major;
        c.cc_minor = prop.minor;
        c.smem_optin = prop.sharedMemPerBlockOptin;
        e = cudaMalloc(&c.workspace, WORKSPACE_BYTES);
        if (e != cudaSuccess) {
            *status = set_cuda_error(e, "cudaMalloc(workspace)");
            return nullptr;
        }
        e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            *status = set_cuda_error(e, "cudaStreamCreate");
            return nullptr;
        }
        e = cudaEventCreateWithFlags(&c.ws_done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            *status = set_cuda_error(e, "cudaEventCreate");
            return nullptr;
        }
        c.device = dev;
    }
    *status = TMC_OK;
    return &c;
}

static bool capturing(cudaStream_t stream)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

cudaError_t ws_acquire(DeviceCtx &c, cudaStream_t stream)
{
    if (capturing(stream))
        return cudaSuccess;
    return cudaStreamWaitEvent(stream, c.ws_done, 0);
}

cudaError_t ws_release(DeviceCtx &c, cudaStream_t stream)
{
    if (capturing(stream))
        return cudaSuccess;
    return cudaEventRecord(c.ws_done, stream);
}

static int ensure_buffers(DeviceCtx &c, uint32_t shells)
{
    if (c.tally_cap < shells) {
        if (c.tally)
            cudaFree(c.tally);
        c.tally = nullptr;
        c.tally_cap = 0;
        cudaError_t e = cudaMalloc(&c.tally, sizeof(tmc_tally) * shells);
        if (e != cudaSuccess)
            return set_cuda_error(e, "cudaMalloc(tally)");
        c.tally_cap = shells;
    }
    if (c.out_cap < shells) {
        if (c.heat_out)
            cudaFree(c.heat_out);
        c.heat_out = nullptr;
        c.out_cap = 0;
        cudaError_t e = cudaMalloc(&c.heat_out, sizeof(double) * 2 * shells);
        if (e != cudaSuccess)
            return set_cuda_error(e, "cudaMalloc(heat)");
        c.out_cap = shells;
    }
    return TMC_OK;
}

__global__ void tally_to_heat_kernel(const tmc_tally *t, uint32_t shells, double c, double *heat,
                                     double *heat2)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= shells)
        return;
    const tmc_tally q = t[s];
    const double sw = (double)q.w_hi * 0x1p24 + (double)q.w_lo * 0x1p-40;
    const double sw2 = (double)q.w2_hi * 0x1p24 + (double)q.w2_lo * 0x1p-40;
    heat[s] = c * sw;
    heat2[s] = (c * c) * sw2;
}

// tiny_mc.c:60-66 in FP64 from exact tallies: t = 4 pi MPS^3 N / 1e12 (cm^3),
// density[i] = heat[i] / t / (i^2 + i + 1/3), error[i] = sqrt(heat2[i] -
// heat[i]^2 / N) / t / (i^2 + i + 1/3) (NaN where the per-deposit variance
// estimate goes negative, as the reference's does), extra = heat[S-1] / N.
__global__ void report_fp64_kernel(const tmc_tally *t, uint32_t shells, double c, double mps,
                                   double photons, double *density, double *error, double *extra)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= shells)
        return;
    const tmc_tally q = t[i];
    const double heat = c * ((double)q.w_hi * 0x1p24 + (double)q.w_lo * 0x1p-40);
    const double heat2 = (c * c) * ((double)q.w2_hi * 0x1p24 + (double)q.w2_lo * 0x1p-40);
    const double vol = 4.0 * 3.14159265358979323846 * mps * mps * mps * photons / 1e12;
    const double shell = (double)i * (double)i + (double)i + 1.0 / 3.0;
    if (i + 1 < shells) {
        density[i] = heat / vol / shell;
        error[i] = sqrt(heat2 - heat * heat / photons) / vol / shell;
    } else {
        *extra = heat / photons;
    }
}

cudaError_t launch_report_fp64(const tmc_tally *d_tally, uint32_t shells, double c, double mps,
                               double photons, double *d_out, cudaStream_t stream)
{
    report_fp64_kernel<<<(shells + 255) / 256, 256, 0, stream>>>(d_tally, shells, c, mps, photons, d_out,
                                                                  d_out + shells, d_out + 2 * shells);
    return cudaGetLastError();
}

cudaError_t launch_tally_to_heat(const tmc_tally *d_tally, uint32_t shells, double c,
                                 double *d_heat, double *d_heat2, cudaStream_t stream)
{
    const int bs = 256;
    tally_to_heat_kernel<<<(shells + bs - 1) / bs, bs, 0, stream>>>(d_tally, shells, c, d_heat,
                                                                   d_heat2);
    return cudaGetLastError();
}

// Shared part of the host-array entry points: walk into ctx.tally.
static int run_into_ctx_tally(DeviceCtx &c, uint64_t n, const tmc_params *p, const Derived &d,
                              unsigned long long *d_steps)
{
    int st = ensure_buffers(c, p->shells);
    if (st)
        return st;
    cudaError_t e = cudaMemsetAsync(c.tally, 0, sizeof(tmc_tally) * p->shells, c.stream);
    if (e == cudaSuccess)
        e = ws_acquire(c, c.stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(c.workspace, 0, WORKSPACE_BYTES, c.stream);
    if (e != cudaSuccess)
        return set_cuda_error(e, "cudaMemsetAsync");
    if (n == 0)
        return TMC_OK;
    PlainLaunch L{};
    L.p = p;
    L.d = d;
    L.n_photons = n;
    L.d_tally = c.tally;
    L.d_work = reinterpret_cast<unsigned long long *>(c.workspace);
    L.d_steps = d_steps;
    L.block = g_plain_block;
    L.blocks_per_sm = g_plain_blocks_per_sm;
    L.max_blocks = g_plain_max_blocks;
    e = launch_plain(L, c, c.stream);
    if (e != cudaSuccess)
        return set_cuda_error(e, "walk_plain launch");
    return TMC_OK;
}

// After the host-array calls' reads of the step counter.
static int release_ctx_workspace(DeviceCtx &c)
{
    const cudaError_t e = ws_release(c, c.stream);
    return e == cudaSuccess ? TMC_OK : set_cuda_error(e, "cudaEventRecord(workspace)");
}

static int check_sizes(uint64_t n, const tmc_params *p)
{
    if (n > (1ull << 62) || p->photon_id_base > ~0ull - n) {
        set_error_text("photon count or photon_id_base + count overflows 64-bit photon ids");
        return TMC_E_OVERFLOW;
    }
    return TMC_OK;
}

__global__ void debug_rand_kernel(PhiloxKeys keys, uint32_t pid_lo, uint32_t pid_hi, uint32_t n,
                                  int32_t *out)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;   // Philox block index
    if (4 * b >= n)
        return;
    const uint4 r = philox4x32_10(b, 0u, pid_lo, pid_hi, keys);
    const uint32_t w[4] = {r.x, r.y, r.z, r.w};
    for (uint32_t j = 0; j < 4 && 4 * b + j < n; ++j)
        out[4 * b + j] = (int32_t)rand31(w[j]);
}

}  // namespace tmc

using namespace tmc;

extern "C" {

void tmc_params_default(tmc_params *p)
{
    if (!p)
        return;
    std::memset(p, 0, sizeof *p);
    p->shells = 101;             // params.h:6
    p->microns_per_shell = 50;   // params.h:22
    p->mu_a = 2.0f;              // params.h:14
    p->mu_s = 20.0f;             // params.h:18
    p->seed = 1;
    p->photon_id_base = 0;
    p->math = TMC_MATH_EXACT;
}

size_t tmc_workspace_bytes(void) { return WORKSPACE_BYTES; }

int tmc_photon_batch_fx(tmc_tally *tally, uint64_t n_photons, const tmc_params *p,
                        uint64_t *photon_steps)
{
    tmc::NvtxRange nvtx_range("tmc_photon_batch_fx");
    int st = validate(p);
    if (st)
        return st;
    if (!tally)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    DeviceCtx *c = current_ctx(&st);
    if (!c)
        return st;
    if ((st = check_sizes(n_photons, p)))
        return st;
    const Derived d = derive(p->mu_a, p->mu_s, p->microns_per_shell, p->shells);
    unsigned long long *d_steps = reinterpret_cast<unsigned long long *>(c->workspace) + 1;
    if ((st = run_into_ctx_tally(*c, n_photons, p, d, d_steps)))
        return st;
    std::vector<tmc_tally> h(p->shells);
    unsigned long long steps = 0;
    cudaError_t e = cudaMemcpyAsync(h.data(), c->tally, sizeof(tmc_tally) * p->shells,
                                    cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&steps, d_steps, sizeof steps, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && (st = release_ctx_workspace(*c)))
        return st;
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_photon_batch_fx");
    for (uint32_t s = 0; s < p->shells; ++s) {
        unsigned __int128 a = ((unsigned __int128)tally[s].w_hi << 64) | tally[s].w_lo;
        unsigned __int128 b = ((unsigned __int128)tally[s].w2_hi << 64) | tally[s].w2_lo;
        a += ((unsigned __int128)h[s].w_hi << 64) | h[s].w_lo;
        b += ((unsigned __int128)h[s].w2_hi << 64) | h[s].w2_lo;
        tally[s].w_lo = (uint64_t)a;
        tally[s].w_hi = (uint64_t)(a >> 64);
        tally[s].w2_lo = (uint64_t)b;
        tally[s].w2_hi = (uint64_t)(b >> 64);
    }
    if (photon_steps)
        *photon_steps += steps;
    return TMC_OK;
}

int tmc_photon_batch(float *heat, float *heat2, uint64_t n_photons, const tmc_params *p)
{
    tmc::NvtxRange nvtx_range("tmc_photon_batch");
    int st = validate(p);
    if (st)
        return st;
    if (!heat || !heat2)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    DeviceCtx *c = current_ctx(&st);
    if (!c)
        return st;
    if ((st = check_sizes(n_photons, p)))
        return st;
    const Derived d = derive(p->mu_a, p->mu_s, p->microns_per_shell, p->shells);
    if ((st = run_into_ctx_tally(*c, n_photons, p, d, nullptr)))
        return st;
    if ((st = release_ctx_workspace(*c)))
        return st;
    const uint32_t S = p->shells;
    cudaError_t e = launch_tally_to_heat(c->tally, S, (double)d.c, c->heat_out, c->heat_out + S,
                                         c->stream);
    std::vector<double> h(2 * (size_t)S);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h.data(), c->heat_out, sizeof(double) * 2 * S, cudaMemcpyDeviceToHost,
                            c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_photon_batch");
    for (uint32_t s = 0; s < S; ++s) {
        heat[s] = (float)((double)heat[s] + h[s]);
        heat2[s] = (float)((double)heat2[s] + h[S + s]);
    }
    return TMC_OK;
}

int tmc_photon_batch_device(tmc_tally *d_tally, uint64_t n_photons, const tmc_params *p,
                            uint64_t *d_steps, void *d_workspace, void *stream)
{
    tmc::NvtxRange nvtx_range("tmc_photon_batch_device");
    int st = validate(p);
    if (st)
        return st;
    if (!d_tally)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    DeviceCtx *c = current_ctx(&st);
    if (!c)
        return st;
    if ((st = check_sizes(n_photons, p)))
        return st;
    if (n_photons == 0)
        return TMC_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    void *ws = d_workspace ? d_workspace : c->workspace;
    cudaError_t e = d_workspace ? cudaSuccess : ws_acquire(*c, s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(ws, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess)
        return set_cuda_error(e, "cudaMemsetAsync(workspace)");
    PlainLaunch L{};
    L.p = p;
    L.d = derive(p->mu_a, p->mu_s, p->microns_per_shell, p->shells);
    L.n_photons = n_photons;
    L.d_tally = d_tally;
    L.d_work = reinterpret_cast<unsigned long long *>(ws);
    L.d_steps = reinterpret_cast<unsigned long long *>(d_steps);
    L.block = g_plain_block;
    L.blocks_per_sm = g_plain_blocks_per_sm;
    L.max_blocks = g_plain_max_blocks;
    e = launch_plain(L, *c, s);
    if (e == cudaSuccess && !d_workspace)
        e = ws_release(*c, s);
    if (e != cudaSuccess)
        return set_cuda_error(e, "walk_plain launch");
    return TMC_OK;
}

int tmc_report_fp64_device(const tmc_tally *d_tally, const tmc_params *p, uint64_t photons, double *d_out,
                           void *stream)
{
    int st = validate(p);
    if (st)
        return st;
    if (!d_tally || !d_out || photons == 0)
        return TMC_E_INVALID;
    const Derived d = derive(p->mu_a, p->mu_s, p->microns_per_shell, p->shells);
    cudaError_t e = launch_report_fp64(d_tally, p->shells, (double)d.c, (double)p->microns_per_shell,
                                       (double)photons, d_out, reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TMC_OK : set_cuda_error(e, "tmc_report_fp64_device");
}

int tmc_report_fp64(const tmc_tally *tally, const tmc_params *p, uint64_t photons, double *density,
                    double *error, double *extra)
{
    int st = validate(p);
    if (st)
        return st;
    if (!tally || !density || !error || !extra || photons == 0)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    DeviceCtx *c = current_ctx(&st);
    if (!c)
        return st;
    if ((st = ensure_buffers(*c, p->shells)))
        return st;
    const uint32_t S = p->shells;
    double *d_out = nullptr;
    cudaError_t e = cudaMallocAsync(&d_out, sizeof(double) * (2 * S + 1), c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->tally, tally, sizeof(tmc_tally) * S, cudaMemcpyHostToDevice, c->stream);
    const Derived d = derive(p->mu_a, p->mu_s, p->microns_per_shell, S);
    if (e == cudaSuccess)
        e = launch_report_fp64(c->tally, S, (double)d.c, (double)p->microns_per_shell, (double)photons,
                               d_out, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(density, d_out, sizeof(double) * (S - 1), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(error, d_out + S, sizeof(double) * (S - 1), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(extra, d_out + 2 * S, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (d_out)
        cudaFreeAsync(d_out, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? TMC_OK : set_cuda_error(e, "tmc_report_fp64");
}

int tmc_tally_to_heat(const tmc_tally *tally, const tmc_params *p, double *heat, double *heat2)
{
    int st = validate(p);
    if (st)
        return st;
    if (!tally)
        return TMC_E_INVALID;
    const Derived d = derive(p->mu_a, p->mu_s, p->microns_per_shell, p->shells);
    const double c = (double)d.c;
    for (uint32_t s = 0; s < p->shells; ++s) {
        const double sw = (double)tally[s].w_hi * 0x1p24 + (double)tally[s].w_lo * 0x1p-40;
        const double sw2 = (double)tally[s].w2_hi * 0x1p24 + (double)tally[s].w2_lo * 0x1p-40;
        if (heat)
            heat[s] = c * sw;
        if (heat2)
            heat2[s] = (c * c) * sw2;
    }
    return TMC_OK;
}

int tmc_set_plain_launch(int block, int blocks_per_sm, int max_blocks)
{
    if (block != 0 && block != 128 && block != 256 && block != 512)
        return TMC_E_INVALID;
    if (blocks_per_sm < 0 || blocks_per_sm > 32 || max_blocks < 0)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    g_plain_block = block;
    g_plain_blocks_per_sm = blocks_per_sm;
    g_plain_max_blocks = max_blocks;
    return TMC_OK;
}

int tmc_debug_rand(uint64_t seed, uint64_t photon, uint32_t n, int32_t *out)
{
    if (!out || n == 0 || n > (1u << 24))
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    int st = TMC_OK;
    DeviceCtx *c = current_ctx(&st);
    if (!c)
        return st;
    int32_t *d = nullptr;
    cudaError_t e = cudaMallocAsync(&d, sizeof(int32_t) * n, c->stream);
    if (e != cudaSuccess)
        return set_cuda_error(e, "cudaMallocAsync(debug)");
    const uint32_t blocks = (n + 3) / 4;
    debug_rand_kernel<<<(blocks + 127) / 128, 128, 0, c->stream>>>(
        make_philox_keys(seed), (uint32_t)photon, (uint32_t)(photon >> 32), n, d);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, d, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaFreeAsync(d, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_debug_rand");
    return TMC_OK;
}

const char *tmc_strerror(int status)
{
    switch (status) {
    case TMC_OK: return "ok";
    case TMC_E_INVALID: return "invalid parameter";
    case TMC_E_CUDA: return "CUDA error";
    case TMC_E_NOMEM: return "out of memory";
    case TMC_E_TIMEOUT: return "wait timed out";
    case TMC_E_OVERFLOW: return "count overflow";
    case TMC_E_NODEVICE: return "no usable CUDA device";
    case TMC_E_BUSY: return "admission refused";
    case TMC_E_STATE: return "invalid state";
    default: return "unknown status";
    }
}

const char *tmc_last_error(void) { return g_error.c_str(); }

}  // extern "C"
