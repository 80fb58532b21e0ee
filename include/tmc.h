/*
 * tmc.h — C ABI of libtmc_gb300.so, the GB300 (sm_103a) photon walk of
 * Tiny Monte Carlo (computacionparalela/tiny_mc).
 *
 * The reference's boundary is one call per photon,
 *     void photon(float *heats, float *heats_squared);        photon.h:3
 * with compile-time knobs (params.h:5-27) and the global libc rand() seeded by
 * the caller (tiny_mc.c:43).  This library replaces the caller's photon loop
 * (tiny_mc.c:47-49) by ONE call that walks n photons on the GPU and
 * accumulates (+=) into the same two caller-owned float arrays.
 *
 * Plain pointers and sizes only; no CUDA or torch types in the signatures
 * (streams are passed as void*, a cudaStream_t or NULL for the default
 * stream).  All entry points return TMC_OK (0) or a negative tmc_status.
 *
 * Thread safety: like photon() (global rand, unsynchronised +=), the library
 * is meant to be driven by one host thread at a time per process; calls are
 * serialised by an internal lock so concurrent calls are safe but not
 * concurrent.  Device scratch the library owns is ordered on the GPU as well:
 * an asynchronous call that uses it (tmc_photon_batch_device with no
 * workspace) finishes on the GPU before any later call touches it.
 */
#ifndef TMC_H
#define TMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TMC_ABI_VERSION 1

typedef enum tmc_status {
    TMC_OK = 0,
    TMC_E_INVALID = -1,   /* a parameter is out of range (e.g. mu_a <= 0, shells == 0) */
    TMC_E_CUDA = -2,      /* a CUDA runtime call failed; tmc_last_error() has the text */
    TMC_E_NOMEM = -3,     /* device or host allocation failed */
    TMC_E_TIMEOUT = -4,   /* a bounded device-side or host-side wait ran out */
    TMC_E_OVERFLOW = -5,  /* a count would overflow its integer type */
    TMC_E_NODEVICE = -6,  /* no CUDA device, or not an sm_103 device */
    TMC_E_BUSY = -7,      /* admission refused (served mode: no slot or tally memory) */
    TMC_E_STATE = -8      /* call not valid in the current state (e.g. unknown request id) */
} tmc_status;

/* Arithmetic of the walk. */
typedef enum tmc_math {
    /* Every float operation of photon.c:21-49 IEEE-rounded in photon.c's
     * order (no FMA contraction), sqrtf and divisions correctly rounded, and
     * the step-length logarithm evaluated by the library's own fixed sequence
     * of float operations.  Integer tallies are bit-identical to the CPU
     * restatement of photon.c driven by the same Philox streams. */
    TMC_MATH_EXACT = 0,
    /* Hardware approximations: lg2.approx for the logarithm, sqrt.approx,
     * contracted multiply-adds and (1-u^2)/t rewritten as 4(1-t).  Same draws
     * and branch decisions; tallies agree with the exact form statistically
     * (per-shell relative differences far below 1e-4 at params.h optics). */
    TMC_MATH_FAST = 1
} tmc_math;

/* Runtime form of params.h's knobs. */
typedef struct tmc_params {
    uint32_t shells;            /* SHELLS            (params.h:5-7),   1 .. 2^24 */
    float microns_per_shell;    /* MICRONS_PER_SHELL (params.h:21-23), > 0       */
    float mu_a;                 /* MU_A, 1/cm        (params.h:13-15), > 0       */
    float mu_s;                 /* MU_S, 1/cm        (params.h:17-19), >= 0      */
    uint64_t seed;              /* SEED (params.h:25-27): the Philox key          */
    uint64_t photon_id_base;    /* photon ids of this call: base .. base+n-1      */
    uint32_t math;              /* tmc_math                                        */
    uint32_t reserved;          /* must be 0                                       */
} tmc_params;

/*
 * Exact per-shell tallies.  A deposit of weight w (photon.c:30-31 deposits
 * (1-albedo)*w) adds rint(w * 2^40) to sum_w and rint(fl(w*w) * 2^40) to
 * sum_w2, as 128-bit unsigned integers split in 64-bit halves.  Integer sums
 * make results independent of thread order: runs are bit-reproducible.
 *   heat[s]  = (1-albedo)   * sum_w  * 2^-40
 *   heat2[s] = (1-albedo)^2 * sum_w2 * 2^-40
 */
typedef struct tmc_tally {
    uint64_t w_lo, w_hi;
    uint64_t w2_lo, w2_hi;
} tmc_tally;

/* params.h defaults: SHELLS 101, MICRONS_PER_SHELL 50, MU_A 2, MU_S 20;
 * seed 1, photon_id_base 0, TMC_MATH_EXACT. */
void tmc_params_default(tmc_params *p);

/*
 * The drop-in for the photon loop of tiny_mc.c:47-49 (one photon() call per
 * photon, photon.c:6).  Walks photons photon_id_base .. +n_photons-1 and
 * ACCUMULATES into caller-owned host arrays of length p->shells:
 *     heat[s]  += (1-albedo) * sum of w      over deposits in shell s
 *     heat2[s] += (1-albedo)^2 * sum of w^2  over deposits in shell s
 * heat2 keeps photon.c:31's per-deposit-square meaning.  Synchronous.
 */
int tmc_photon_batch(float *heat, float *heat2, uint64_t n_photons, const tmc_params *p);

/* Same walk; adds the exact integer tallies into host `tally` [p->shells].
 * photon_steps (may be NULL) += number of deposits (= photon steps). */
int tmc_photon_batch_fx(tmc_tally *tally, uint64_t n_photons, const tmc_params *p,
                        uint64_t *photon_steps);

/* Bytes of device scratch the device-pointer entry points need. */
size_t tmc_workspace_bytes(void);

/*
 * Device-resident form: d_tally is DEVICE memory [p->shells] and is added to
 * (+=).  d_steps (device, may be NULL) += photon steps.  d_workspace is
 * device scratch of tmc_workspace_bytes() bytes, or NULL to use a buffer the
 * library allocates once per device.  That shared buffer is also the one the
 * host-array calls use: every use of it, on any stream, first waits on the
 * GPU for the previous use to end, so calls with NULL on different streams
 * run one after another (bring a workspace per stream to overlap them).
 * Under stream capture that ordering is not recorded: pass a workspace when
 * capturing.  stream is a cudaStream_t (NULL = legacy default stream).
 * Asynchronous: returns after the launch.
 */
int tmc_photon_batch_device(tmc_tally *d_tally, uint64_t n_photons, const tmc_params *p,
                            uint64_t *d_steps, void *d_workspace, void *stream);

/*
 * Allocation-free form of tmc_photon_batch (same walk, same result, host
 * arrays).  No counterpart in the reference: photon() never touches device
 * memory.  For callers that cannot let a library call cudaMalloc — device
 * memory owned by another allocator, or a loop that forbids allocation after
 * start-up.  Its device scratch (claim counter, tallies, FP64 results) is a
 * fixed array of TMC_STATIC_SCRATCH_BYTES inside the library's module, held
 * by a GPU from the moment the module is loaded on it until the process
 * exits.  shells above TMC_STATIC_MAX_SHELLS return TMC_E_INVALID.  The first
 * call on a device loads the module there (under CUDA's default lazy loading
 * this is a driver allocation) and looks up the array's device address: make
 * that call during start-up and before any stream capture; n_photons = 0 does
 * only this set-up.  The address is kept for the device's primary context:
 * not supported after cudaDeviceReset or under another current context.
 * All calls share the array (each clears what it uses first); calls are
 * serialised and synchronous, and two of them running at once on the GPU
 * would race.  stream: a cudaStream_t or NULL.
 */
#define TMC_STATIC_MAX_SHELLS 4096
#define TMC_STATIC_SCRATCH_BYTES (256 + 32 * TMC_STATIC_MAX_SHELLS + 16 * TMC_STATIC_MAX_SHELLS)
int tmc_photon_batch_static(float *heat, float *heat2, uint64_t n_photons, const tmc_params *p,
                            void *stream);

/* FP64 conversion of exact tallies (host arrays): heat/heat2 as defined at
 * tmc_tally.  Either output may be NULL. */
int tmc_tally_to_heat(const tmc_tally *tally, const tmc_params *p, double *heat, double *heat2);

/*
 * The report of tiny_mc.c:58-66, from float heat/heat2 of `photons` photons:
 * the two column-title lines, one line per shell but the last, and the
 * "# extra" line, with the same printf formats and the same float/double
 * arithmetic.  Writes at most cap bytes (NUL-terminated); returns the length
 * it needed (excluding NUL), or a negative tmc_status.
 */
int tmc_format_report(char *buf, size_t cap, const float *heat, const float *heat2,
                      uint64_t photons, const tmc_params *p);

/*
 * The numbers of that report computed in FP64 on the GPU from exact tallies
 * (tiny_mc.c:60-66 in double precision): density[i] (W/cm^3) and error[i]
 * for i < shells-1, and extra = heat[shells-1] / photons.
 *   tmc_report_fp64_device: d_tally and d_out are device memory; d_out gets
 *     [density (shells) | error (shells) | extra], asynchronous on stream.
 *   tmc_report_fp64: host tallies in, host arrays out (density and error of
 *     shells-1 entries), synchronous.
 * tmc_format_report_fp64 prints them with the report's printf formats.
 */
int tmc_report_fp64_device(const tmc_tally *d_tally, const tmc_params *p, uint64_t photons, double *d_out,
                           void *stream);
int tmc_report_fp64(const tmc_tally *tally, const tmc_params *p, uint64_t photons, double *density,
                    double *error, double *extra);
int tmc_format_report_fp64(char *buf, size_t cap, const double *density, const double *error,
                           double extra, const tmc_params *p);

/* ----------------------------------------------------------------- viewer
 * The viewer's jobs (cg_mc.c) without a graphics stack.  No window, no GL:
 * a device image buffer.
 *
 * tmc_colormap: the fragment shader's arithmetic (cg_mc.c:45-64) per pixel of
 * a width x height target, row 0 = bottom: shell = int(|uv - 0.5| / 0.7071 *
 * (shells-1)) with uv = (pixel + 0.5) / 800, red = 2 / (1 + exp(-0.004 *
 * heats[shell])) - 1.  d_heats (device, float [shells], the viewer's raw
 * heats array), outputs d_red (float [h][w]) and/or d_rgba (uint8 [h][w][4]).
 */
int tmc_colormap(const float *d_heats, uint32_t shells, uint32_t width, uint32_t height, float *d_red,
                 uint8_t *d_rgba, void *stream);
/* Same with host arrays (synchronous). */
int tmc_colormap_host(const float *heats, uint32_t shells, uint32_t width, uint32_t height, float *red,
                      uint8_t *rgba);

/*
 * Progressive walk: the viewer's loop (cg_mc.c:71-87, a few photons per frame
 * into heats, uploaded every frame) as frames that continue the photon-id
 * sequence, so after k photons the tallies equal one k-photon call.  Each
 * advance enqueues the frame's walk and an asynchronous snapshot of the
 * running heat/heat2 (float, like the viewer's arrays); snapshot() copies the
 * newest finished one without waiting (wait = 0) and returns 1 if it is newer
 * than the last one returned, else 0.  render() colours the newest device
 * snapshot into host RGBA8.
 */
typedef struct tmc_progressive tmc_progressive;
int tmc_progressive_create(tmc_progressive **out, const tmc_params *p);
int tmc_progressive_advance(tmc_progressive *g, uint64_t n_photons);
int tmc_progressive_snapshot(tmc_progressive *g, float *heat, float *heat2, uint64_t *photons, int wait);
int tmc_progressive_render(tmc_progressive *g, uint32_t width, uint32_t height, uint8_t *rgba);
int tmc_progressive_destroy(tmc_progressive *g);

/* ------------------------------------------------------------------ batch
 * Many independent walks in one persistent launch.  Each problem is what the
 * reference computes for one set of params.h knobs (tiny_mc.c:34-69 run with
 * one -D setting); the reference runs one problem per process.  All problems
 * of a batch share one seed and arithmetic mode; give problems disjoint
 * photon-id ranges for independent streams.  A problem's tally is
 * bit-identical to tmc_photon_batch_fx on the same photons.
 */
typedef struct tmc_problem {
    uint32_t shells;            /* SHELLS            */
    float microns_per_shell;    /* MICRONS_PER_SHELL */
    float mu_a;                 /* MU_A, 1/cm        */
    float mu_s;                 /* MU_S, 1/cm        */
    uint64_t n_photons;
    uint64_t photon_id_base;
} tmc_problem;

typedef struct tmc_batch tmc_batch;   /* opaque plan with device buffers */

typedef struct tmc_batch_config {
    int block;            /* threads per block: 128, 256 or 512 (0 = 256) */
    int items_per_block;  /* work items per resident block: load-balance granularity (0 = 8) */
    int use_graph;        /* 1: run through a captured CUDA graph, replayed on later runs */
    int stream;           /* 1: up to two items open per block, lanes flow into the next item
                             instead of waiting at a barrier for the slowest lane */
} tmc_batch_config;

int tmc_batch_create(tmc_batch **out, const tmc_problem *problems, uint32_t n_problems,
                     uint64_t seed, uint32_t math);
int tmc_batch_set_config(tmc_batch *b, const tmc_batch_config *cfg);
int tmc_batch_get_config(const tmc_batch *b, tmc_batch_config *cfg);
/* Times block size x items-per-block x kernel (stream 0/1) candidates on a
 * reduced copy of the batch
 * (photon counts x scale, problems above max_steps_per_photon expected steps
 * left out; 0 = keep all) and keeps the fastest.  best_ms may be NULL. */
int tmc_batch_autotune(tmc_batch *b, double scale, double max_steps_per_photon, double *best_ms);
/* Second tuning stage, on the batch itself: takes the fastest configuration
 * of each (kernel, block size) from the last tmc_batch_autotune, at most
 * max_candidates of them (the fastest of each kernel first, then the rest in
 * order), times one full run of each and keeps the fastest (a reduced copy cannot rank them: how much the longest single
 * photons weigh depends on the batch's size).  Costs max_candidates runs;
 * results do not depend on the configuration.  TMC_E_STATE if autotune has
 * not run.  Not in the reference (it has no batched form). */
int tmc_batch_refine(tmc_batch *b, uint32_t max_candidates, double *best_ms);
/* Test hook of the barrier-free kernel's bounded waits (stream = 1): its
 * waits give up after wait_limit_s seconds of wall time (0 = 120 s), set the
 * batch's error flag and return, and tmc_batch_read then reports
 * TMC_E_TIMEOUT.  hold_buffers != 0 stops finished items from freeing their
 * buffers, so waiting warps run into that limit; the kernel still ends and the
 * context stays usable.  Not in the reference. */
int tmc_batch_test_wait(tmc_batch *b, int hold_buffers, double wait_limit_s);
/* Zeroes the batch's device tallies and walks every problem (asynchronous on
 * stream, a cudaStream_t or NULL). */
int tmc_batch_run(tmc_batch *b, void *stream);
/* Waits for the last run and copies tallies [total shells] (problem i's shells
 * start at offsets[i]) and photon steps per problem; either may be NULL. */
int tmc_batch_read(tmc_batch *b, tmc_tally *tallies, uint64_t *steps_per_problem);
int tmc_batch_tally_offsets(const tmc_batch *b, uint64_t *offsets /* [n_problems + 1] */);
int tmc_batch_info(const tmc_batch *b, uint32_t *n_items, double *est_photon_steps);
/* Expected photon steps per photon for optics (mu_a, mu_s): photon.c's weight
 * recursion (albedo^k, roulette at 0.001 with survival 0.1, photon.c:32,45-49)
 * evaluated on the host.  The batch planner splits work with it. */
int tmc_expected_steps(float mu_a, float mu_s, double *steps_per_photon);
/* The batch planner on the host, for a given resident grid: the work items
 * (problem, first photon, photon count) a batch would walk, heaviest first,
 * as items_out[3 i .. 3 i + 2].  *n_items receives the count; with capacity
 * 0 only the count is computed, a smaller nonzero capacity returns
 * TMC_E_OVERFLOW.  No device needed.  Not in the reference. */
int tmc_batch_plan_items(const tmc_problem *problems, uint32_t n_problems, int grid, int block,
                         int items_per_block, uint64_t *items_out, uint64_t capacity, uint64_t *n_items);
/* Device address of the batch's tallies (valid until destroy). */
const void *tmc_batch_device_tallies(const tmc_batch *b);
int tmc_batch_destroy(tmc_batch *b);

/* ----------------------------------------------------------------- server
 * Continuous batching of simulation requests, each stopped at a target
 * relative standard error.  No counterpart in the reference (one run per
 * process); each request is one tiny_mc.c run with its own knobs.  A request
 * is walked in RSE batches; at fixed batch counts (min_batches, then
 * doubling) the batch-means RSE of the heat in `probe_shell` is computed in
 * FP64 and the request stops when it is <= target_rse or max_photons is
 * reached.  Results depend only on the request (optics, photon_id_base,
 * server seed and arithmetic), not on what else runs.
 */
typedef struct tmc_request {
    uint32_t shells;
    float microns_per_shell;
    float mu_a;
    float mu_s;
    double target_rse;          /* e.g. 0.01 for 1 % */
    uint64_t max_photons;       /* cap */
    uint64_t photon_id_base;    /* first photon id of this request's streams */
} tmc_request;

typedef struct tmc_request_result {
    uint64_t photons;           /* photons walked (batches x batch_photons) */
    uint64_t photon_steps;
    uint32_t batches;
    uint32_t batch_photons;
    double rse;                 /* batch-means RSE at the stop (NaN if the shell got nothing) */
    int32_t reached_target;     /* 1: rse <= target; 0: stopped at the cap */
    int32_t reserved;
    double latency_s;           /* completion - submission (run_trace: - arrival) */
} tmc_request_result;

typedef struct tmc_server_config {
    uint32_t slots;                 /* requests resident at once (tally memory) */
    uint32_t max_shells;            /* tally memory per slot: max_shells x 32 bytes */
    uint32_t probe_shell;           /* shell of the RSE (10 = 500-550 um at 50 um shells) */
    uint32_t min_batches;           /* first stop decision */
    uint64_t seed;
    uint32_t math;
    uint32_t block;                 /* 128, 256 or 512 */
    uint32_t max_items_per_request; /* RSE batches of one request in one wave */
    uint32_t stream;                /* 1: barrier-free kernel (up to two items open per block) */
    double steps_per_batch;         /* target photon steps per RSE batch */
    double steps_per_item;          /* target photon steps per work item: a batch is split
                                       into 2^k items walked by different blocks (0 = one
                                       item per batch); results do not depend on it */
    uint32_t waves;                 /* launches in flight at once, 1..64 (0 = 16) */
    uint32_t inflight_items;        /* work items launched and not yet finished: no new
                                       items above it, so new requests do not queue behind
                                       long-running ones (0 = unbounded; with persistent,
                                       0 = twice the resident blocks) */
    uint32_t persistent;            /* 1: instead of launches per wave, a long-running
                                       launch of the batched kernel (per-item barriers, or
                                       barrier-free with stream = 1) takes items from a
                                       work queue in mapped host memory that the server
                                       keeps filling (least attained service first); its
                                       blocks wait for work while requests are active and
                                       end once none are (waves does not apply).  Higher
                                       capacity and lower latency than waves, but while
                                       requests are active it holds the SMs: other work on
                                       the GPU waits for it (the default, 0, leaves room
                                       between launches) */
} tmc_server_config;

typedef struct tmc_server tmc_server;

void tmc_server_config_default(tmc_server_config *c);
int tmc_server_create(tmc_server **out, const tmc_server_config *cfg);
/* TMC_E_BUSY when no slot is free (the caller queues the request). */
int tmc_server_submit(tmc_server *s, const tmc_request *r, uint64_t *request_id);
/* Non-blocking: harvests finished waves (persistent: the items finished
 * since the last call), makes stop decisions, and launches the next wave on a
 * free stream (persistent: publishes the next items to the running launch,
 * relaunching it if it ended). */
int tmc_server_progress(tmc_server *s, uint32_t *waves_in_flight, uint32_t *active_requests);
int tmc_server_poll(tmc_server *s, uint64_t request_id, int *done);
/* Result of a finished request (then forgotten); tally [shells] may be NULL. */
int tmc_server_result(tmc_server *s, uint64_t request_id, tmc_tally *tally, tmc_request_result *res);
int tmc_server_stats(tmc_server *s, uint64_t *photons, uint64_t *photon_steps, uint64_t *waves);
/* Photon steps walked so far, including those of requests still running. */
int tmc_server_work(tmc_server *s, uint64_t *photon_steps);
/* Replays an arrival trace in real time (arrival_s sorted, seconds from the
 * start): admits requests as they arrive and slots free up, drives the server
 * until all complete or time_limit_s (0 = none) passes.  results[i] is zero
 * for requests not completed; latency is completion - arrival. */
int tmc_server_run_trace(tmc_server *s, const tmc_request *reqs, const double *arrival_s, uint32_t n,
                         double time_limit_s, tmc_request_result *results, uint32_t *completed);
int tmc_server_destroy(tmc_server *s);

/* The server's plan for a request, computed on the host without a device:
 * photons per RSE batch, work items per batch and the expected photon steps
 * per photon it was sized from.  Not in the reference. */
int tmc_server_plan(const tmc_server_config *cfg, const tmc_request *r, uint32_t *batch_photons,
                    uint32_t *items_per_batch, double *steps_per_photon);
/* The server's stop statistic, on the host: batch-means relative standard
 * error of n_batches batches, batch j's value being the exact 128-bit sum of
 * its items' probes probes[2 i] (low 64 bits) and probes[2 i + 1] (high),
 * i = j * items_per_batch .. + items_per_batch - 1, converted to weight units
 * (2^-40) once; NaN when the mean is not positive.  Not in the reference. */
int tmc_batch_means_rse(const uint64_t *probes, uint32_t items_per_batch, uint64_t n_batches,
                        double *rse, double *mean);

/*
 * Launch shape of the plain walk: threads per block (128, 256 or 512; 0 =
 * default, 512), resident blocks per SM (0 = occupancy limit) and a cap on the
 * grid (0 = none).  Results do not depend on it (integer tallies,
 * photon-keyed streams); only speed does.
 */
int tmc_set_plain_launch(int block, int blocks_per_sm, int max_blocks);

/* The first n rand() values of photon `photon` under `seed`, produced by the
 * device's Philox path (one small kernel); out is a host array of n int32. */
int tmc_debug_rand(uint64_t seed, uint64_t photon, uint32_t n, int32_t *out);

/* Measured throughput of the special-function unit on the current device
 * (lg2/sqrt/rcp approximations, MUFU ops per second over all SMs): the
 * denominator of the walk's SFU roofline.  No reference counterpart. */
int tmc_probe_sfu_rate(double *mufu_ops_per_s);

/* Text of a status code, and the detail of the calling thread's last
 * failed call (kept per thread, like errno; valid until that thread's next
 * failure). */
const char *tmc_strerror(int status);
const char *tmc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* TMC_H */
