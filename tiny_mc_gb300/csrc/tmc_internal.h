// tmc_internal.h — host-side declarations shared by the library's .cu files.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <mutex>
#include <nvtx3/nvToolsExt.h>
#include <string>

#include "tmc.h"

namespace tmc {

// An NVTX range for the duration of a scope: the host-side phases (walk
// calls, batch runs and tuning, server waves and harvests) show up named on a
// profiler's timeline.  NVTX v3 is header-only and costs a few nanoseconds
// when no tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};


// Per-problem constants exactly as photon.c:8-9 computes them in float.
struct Derived {
    float albedo;   // MU_S / (MU_S + MU_A), photon.c:8
    float c;        // 1.0f - albedo, photon.c:30
    float spm;      // shells_per_mfp, photon.c:9 (double quotient stored to float)
    float last;     // (float)(shells - 1)
    uint32_t shells;
};

int validate(const tmc_params *p);
Derived derive(float mu_a, float mu_s, float microns_per_shell, uint32_t shells);

// One device's cached resources.
struct DeviceCtx {
    int device = -1;
    int sms = 0;
    int cc_major = 0, cc_minor = 0;
    size_t smem_optin = 0;
    void *workspace = nullptr;          // tmc_workspace_bytes()
    tmc_tally *tally = nullptr;         // tally_cap shells
    size_t tally_cap = 0;
    double *heat_out = nullptr;         // 2 * out_cap doubles
    size_t out_cap = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ws_done = nullptr;      // recorded after the last use of workspace
};

// Returns the context of the current device (creating it), or nullptr with
// *status set.
DeviceCtx *current_ctx(int *status);
std::mutex &api_mutex();
int set_cuda_error(cudaError_t e, const char *where);
void set_error_text(const std::string &s);

constexpr size_t WORKSPACE_BYTES = 256;

// The context's workspace (photon claim counter, step counter) is shared by
// the host-array calls and by device-form calls that bring no workspace of
// their own, on whatever stream each uses.  ws_acquire makes `stream` wait on
// the GPU until the previous use has finished; ws_release marks the end of
// this use.  A stream under capture is left alone (the ordering would not be
// part of the graph; callers that capture pass their own workspace).
cudaError_t ws_acquire(DeviceCtx &c, cudaStream_t stream);
cudaError_t ws_release(DeviceCtx &c, cudaStream_t stream);

// Plain walk launch (tmc_plain.cu).  d_work points at a zeroed 64-bit photon
// claim counter.
struct PlainLaunch {
    const tmc_params *p;
    Derived d;
    uint64_t n_photons;
    tmc_tally *d_tally;
    unsigned long long *d_work;
    unsigned long long *d_steps;
    int block;          // threads per block (0 = default)
    int blocks_per_sm;  // 0 = occupancy limit
    int max_blocks;     // 0 = no cap on the grid
};
cudaError_t launch_plain(const PlainLaunch &L, const DeviceCtx &ctx, cudaStream_t stream);

// FP64 finalisation on the device (tmc_api.cu).
cudaError_t launch_tally_to_heat(const tmc_tally *d_tally, uint32_t shells, double c,
                                 double *d_heat, double *d_heat2, cudaStream_t stream);

}  // namespace tmc
