// tmc_view.cu — the viewer's two jobs without a graphics stack.
//
// The reference's OpenGL viewer (cg_mc.c) walks up to 20 photons per frame
// into a float `heats` array, uploads it to a shader storage buffer
// (cg_mc.c:71-87) and colours every pixel by the heat of the shell at its
// radius (fragment shader, cg_mc.c:38-67).  Here:
//
//  * tmc_progressive: a walk advanced frame by frame (each frame continues the
//    photon-id sequence, so after k photons the tallies are exactly those of
//    one k-photon call), with an asynchronous snapshot of the running heat
//    after every frame that the host reads without waiting for the walk;
//  * tmc_colormap: the fragment shader's arithmetic as a CUDA kernel writing a
//    device RGBA8 (and float red) image instead of a window.
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "tmc_device.cuh"
#include "tmc_internal.h"

using namespace tmc;

namespace {

// cg_mc.c:45-64, one thread per pixel.  gl_FragCoord = (px + 0.5, py + 0.5)
// (row 0 is the bottom row); uv = gl_FragCoord / 800 (the shader's literal);
// shell = int(|uv - 0.5| / 0.7071067811865476 * (shells - 1)), clamped to the
// last shell for targets wider than 800; red = 2 / (1 + exp(-0.004 heat)) - 1.
__global__ void colormap_kernel(const float *heats, uint32_t shells, uint32_t width, uint32_t height,
                                float *red, uchar4 *rgba)
{
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= width || py >= height)
        return;
    const float mc = 0.7071067811865476f;
    const float ux = __fsub_rn(__fdiv_rn(__fadd_rn((float)px, 0.5f), 800.0f), 0.5f);
    const float uy = __fsub_rn(__fdiv_rn(__fadd_rn((float)py, 0.5f), 800.0f), 0.5f);
    const float dr = __fsqrt_rn(__fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy)));
    int id = __float2int_rz(__fmul_rn(__fdiv_rn(dr, mc), (float)(shells - 1)));
    id = min(id, (int)shells - 1);
    const float heat = heats[id];
    const float fit = __fsub_rn(__fdiv_rn(2.0f, __fadd_rn(1.0f, expf(__fmul_rn(-0.004f, heat)))), 1.0f);
    const size_t k = (size_t)py * width + px;
    if (red)
        red[k] = fit;
    if (rgba) {
        const float c = fminf(fmaxf(fit, 0.0f), 1.0f);
        rgba[k] = make_uchar4((unsigned char)__float2int_rn(c * 255.0f), 0, 0, 255);
    }
}

__global__ void heat_to_float_kernel(const double *heat, const double *heat2, uint32_t shells,
                                     float *fheat, float *fheat2)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < shells) {
        fheat[s] = (float)heat[s];
        fheat2[s] = (float)heat2[s];
    }
}

cudaError_t launch_colormap(const float *d_heats, uint32_t shells, uint32_t width, uint32_t height,
                            float *d_red, uint8_t *d_rgba, cudaStream_t s)
{
    const dim3 blk(32, 8);
    const dim3 grd((width + blk.x - 1) / blk.x, (height + blk.y - 1) / blk.y);
    colormap_kernel<<<grd, blk, 0, s>>>(d_heats, shells, width, height, d_red,
                                        reinterpret_cast<uchar4 *>(d_rgba));
    return cudaGetLastError();
}

}  // namespace

struct tmc_progressive {
    tmc_params p{};
    Derived d{};
    int device = -1;
    DeviceCtx launch_ctx;             // launch limits (SM count, shared memory)
    cudaStream_t stream = nullptr;
    tmc_tally *d_tally = nullptr;
    unsigned long long *d_work = nullptr;
    double *d_heat = nullptr;         // 2 x shells
    float *d_fheat = nullptr;         // 2 x shells, the latest snapshot on the device
    uint8_t *d_image = nullptr;       // render target
    size_t image_cap = 0;
    // two pinned host snapshot buffers, alternating
    float *h_snap[2] = {nullptr, nullptr};
    uint64_t snap_photons[2] = {0, 0};
    cudaEvent_t snap_done[2] = {nullptr, nullptr};
    bool snap_pending[2] = {false, false};
    int next_snap = 0;
    uint64_t photons = 0;             // photons enqueued so far
    uint64_t latest_photons = 0;      // photons of the newest snapshot handed out
};

namespace {

void destroy_progressive(tmc_progressive *g)
{
    if (!g)
        return;
    if (g->stream)
        cudaStreamSynchronize(g->stream);
    for (int i = 0; i < 2; ++i) {
        if (g->snap_done[i])
            cudaEventDestroy(g->snap_done[i]);
        cudaFreeHost(g->h_snap[i]);
    }
    cudaFree(g->d_tally);
    cudaFree(g->d_work);
    cudaFree(g->d_heat);
    cudaFree(g->d_fheat);
    cudaFree(g->d_image);
    if (g->stream)
        cudaStreamDestroy(g->stream);
    delete g;
}

}  // namespace

extern "C" {

int tmc_colormap(const float *d_heats, uint32_t shells, uint32_t width, uint32_t height, float *d_red,
                 uint8_t *d_rgba, void *stream)
{
    if (!d_heats || shells == 0 || width == 0 || height == 0 || width > 16384 || height > 16384 ||
        (!d_red && !d_rgba))
        return TMC_E_INVALID;
    cudaError_t e = launch_colormap(d_heats, shells, width, height, d_red, d_rgba,
                                    reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TMC_OK : set_cuda_error(e, "tmc_colormap");
}

int tmc_colormap_host(const float *heats, uint32_t shells, uint32_t width, uint32_t height, float *red,
                      uint8_t *rgba)
{
    if (!heats || shells == 0 || width == 0 || height == 0 || width > 16384 || height > 16384 ||
        (!red && !rgba))
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    int st = TMC_OK;
    DeviceCtx *c = current_ctx(&st);
    if (!c)
        return st;
    const size_t px = (size_t)width * height;
    float *d_h = nullptr, *d_red = nullptr;
    uint8_t *d_rgba = nullptr;
    cudaError_t e = cudaMallocAsync(&d_h, sizeof(float) * shells, c->stream);
    if (e == cudaSuccess && red)
        e = cudaMallocAsync(&d_red, sizeof(float) * px, c->stream);
    if (e == cudaSuccess && rgba)
        e = cudaMallocAsync(&d_rgba, 4 * px, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_h, heats, sizeof(float) * shells, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = launch_colormap(d_h, shells, width, height, d_red, d_rgba, c->stream);
    if (e == cudaSuccess && red)
        e = cudaMemcpyAsync(red, d_red, sizeof(float) * px, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && rgba)
        e = cudaMemcpyAsync(rgba, d_rgba, 4 * px, cudaMemcpyDeviceToHost, c->stream);
    cudaFreeAsync(d_h, c->stream);
    if (d_red)
        cudaFreeAsync(d_red, c->stream);
    if (d_rgba)
        cudaFreeAsync(d_rgba, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? TMC_OK : set_cuda_error(e, "tmc_colormap_host");
}

int tmc_progressive_create(tmc_progressive **out, const tmc_params *p)
{
    if (!out)
        return TMC_E_INVALID;
    *out = nullptr;
    int st = validate(p);
    if (st)
        return st;
    std::lock_guard<std::mutex> lk(api_mutex());
    DeviceCtx *c = current_ctx(&st);
    if (!c)
        return st;
    std::unique_ptr<tmc_progressive, void (*)(tmc_progressive *)> g(new tmc_progressive,
                                                                    destroy_progressive);
    g->p = *p;
    g->d = derive(p->mu_a, p->mu_s, p->microns_per_shell, p->shells);
    g->device = c->device;
    g->launch_ctx.device = c->device;
    g->launch_ctx.sms = c->sms;
    g->launch_ctx.smem_optin = c->smem_optin;
    const uint32_t S = p->shells;
    cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMalloc(&g->d_tally, sizeof(tmc_tally) * S);
    if (e == cudaSuccess)
        e = cudaMalloc(&g->d_work, WORKSPACE_BYTES);
    if (e == cudaSuccess)
        e = cudaMalloc(&g->d_heat, 2 * sizeof(double) * S);
    if (e == cudaSuccess)
        e = cudaMalloc(&g->d_fheat, 2 * sizeof(float) * S);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = cudaMallocHost(&g->h_snap[i], 2 * sizeof(float) * S);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&g->snap_done[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess)
        e = cudaMemsetAsync(g->d_tally, 0, sizeof(tmc_tally) * S, g->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(g->d_fheat, 0, 2 * sizeof(float) * S, g->stream);
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_progressive_create");
    *out = g.release();
    return TMC_OK;
}

int tmc_progressive_advance(tmc_progressive *g, uint64_t n_photons)
{
    if (!g)
        return TMC_E_INVALID;
    if (n_photons > (1ull << 62) || g->p.photon_id_base + g->photons > ~0ull - n_photons)
        return TMC_E_OVERFLOW;
    std::lock_guard<std::mutex> lk(api_mutex());
    const uint32_t S = g->p.shells;
    cudaError_t e = cudaSuccess;
    if (n_photons) {
        tmc_params q = g->p;
        q.photon_id_base = g->p.photon_id_base + g->photons;
        e = cudaMemsetAsync(g->d_work, 0, sizeof(unsigned long long), g->stream);
        if (e == cudaSuccess) {
            PlainLaunch L{};
            L.p = &q;
            L.d = g->d;
            L.n_photons = n_photons;
            L.d_tally = g->d_tally;
            L.d_work = g->d_work;
            e = launch_plain(L, g->launch_ctx, g->stream);
        }
        g->photons += n_photons;
    }
    // snapshot: FP64 heat of the running tallies, as floats on the device and
    // in one of two pinned host buffers
    const int k = g->next_snap;
    if (e == cudaSuccess)
        e = launch_tally_to_heat(g->d_tally, S, (double)g->d.c, g->d_heat, g->d_heat + S, g->stream);
    if (e == cudaSuccess) {
        heat_to_float_kernel<<<(S + 255) / 256, 256, 0, g->stream>>>(g->d_heat, g->d_heat + S, S,
                                                                   g->d_fheat, g->d_fheat + S);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(g->h_snap[k], g->d_fheat, 2 * sizeof(float) * S, cudaMemcpyDeviceToHost,
                            g->stream);
    if (e == cudaSuccess)
        e = cudaEventRecord(g->snap_done[k], g->stream);
    if (e != cudaSuccess)
        return set_cuda_error(e, "tmc_progressive_advance");
    g->snap_photons[k] = g->photons;
    g->snap_pending[k] = true;
    g->next_snap ^= 1;
    return TMC_OK;
}

// Copies the newest finished snapshot.  Returns 1 if it is newer than the one
// handed out before, 0 if not (or none has finished yet and wait == 0).
int tmc_progressive_snapshot(tmc_progressive *g, float *heat, float *heat2, uint64_t *photons, int wait)
{
    if (!g)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    const uint32_t S = g->p.shells;
    if (wait) {
        cudaError_t e = cudaStreamSynchronize(g->stream);
        if (e != cudaSuccess)
            return set_cuda_error(e, "tmc_progressive_snapshot");
    }
    int best = -1;
    for (int i = 0; i < 2; ++i) {
        if (!g->snap_pending[i])
            continue;
        cudaError_t e = cudaEventQuery(g->snap_done[i]);
        if (e == cudaErrorNotReady)
            continue;
        if (e != cudaSuccess)
            return set_cuda_error(e, "tmc_progressive_snapshot");
        if (best < 0 || g->snap_photons[i] > g->snap_photons[best])
            best = i;
    }
    if (best < 0 || g->snap_photons[best] < g->latest_photons ||
        (g->snap_photons[best] == g->latest_photons && g->latest_photons != 0))
        return 0;
    if (heat)
        std::memcpy(heat, g->h_snap[best], sizeof(float) * S);
    if (heat2)
        std::memcpy(heat2, g->h_snap[best] + S, sizeof(float) * S);
    if (photons)
        *photons = g->snap_photons[best];
    g->latest_photons = g->snap_photons[best];
    return 1;
}

// The viewer's colour map of the newest device snapshot into host RGBA8
// [height][width] (row 0 = bottom); waits for the work enqueued so far.
int tmc_progressive_render(tmc_progressive *g, uint32_t width, uint32_t height, uint8_t *rgba)
{
    if (!g || !rgba || width == 0 || height == 0 || width > 16384 || height > 16384)
        return TMC_E_INVALID;
    std::lock_guard<std::mutex> lk(api_mutex());
    const size_t bytes = 4ull * width * height;
    cudaError_t e = cudaSuccess;
    if (g->image_cap < bytes) {
        cudaFree(g->d_image);
        g->d_image = nullptr;
        g->image_cap = 0;
        e = cudaMalloc(&g->d_image, bytes);
        if (e == cudaSuccess)
            g->image_cap = bytes;
    }
    if (e == cudaSuccess)
        e = launch_colormap(g->d_fheat, g->p.shells, width, height, nullptr, g->d_image, g->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(rgba, g->d_image, bytes, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(g->stream);
    return e == cudaSuccess ? TMC_OK : set_cuda_error(e, "tmc_progressive_render");
}

int tmc_progressive_destroy(tmc_progressive *g)
{
    std::lock_guard<std::mutex> lk(api_mutex());
    destroy_progressive(g);
    return TMC_OK;
}

}  // extern "C"
