/*
 * tmc_oracle.h — CPU oracle for the tiny_mc photon walk.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
 * this code; the tests, the smoke check and the CPU-baseline leg of the bench
 * compare against it.
 *
 * What it restates (reference = computacionparalela/tiny_mc):
 *   photon.c:6-51   the walk of one photon (launch, move, absorb, re-direct,
 *                   roulette), in three arithmetic forms:
 *                     - FP32, in photon.c's exact evaluation order with no FMA
 *                       contraction (the "oracle32" restatement);
 *                     - FP64, the same draws in double precision ("oracle64");
 *                     - FP32 driven by glibc rand() exactly as tiny_mc.c:43-49
 *                       does (the "native" replay).
 *   params.h:5-27   the knobs, as runtime fields of tmo_params.
 *   tiny_mc.c:26-27 float tallies heat/heat2 (per-photon float arrays here).
 *
 * Random numbers: the reference calls rand() (photon.c:21, :37-38, :46).  The
 * oracle replaces it by a per-photon Philox-4x32-10 stream (Salmon et al.,
 * "Parallel random numbers: as easy as 1, 2, 3", SC'11) so that the GPU can
 * consume the identical sequence:
 *     word n of photon p = Philox4x32_10(ctr = {n/4 lo, n/4 hi, p lo, p hi},
 *                                        key = {seed lo, seed hi})[n % 4]
 *     rand()  = word >> 1, with 0 mapped to 1  (RAND_MAX stays 2^31-1)
 * The 0 -> 1 mapping removes the reference's undefined -logf(0) case.
 *
 * Logarithm: photon.c:21 calls logf().  LOG_NATIVE uses the C library's logf;
 * LOG_TMC uses tmo_logf below, a fixed sequence of IEEE-rounded float
 * operations that the GPU kernel evaluates identically, which makes the GPU's
 * integer tallies bit-identical to this oracle's.
 */
#ifndef TMC_ORACLE_H
#define TMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tmo_params {
    uint32_t shells;            /* SHELLS            params.h:5-7   */
    float microns_per_shell;    /* MICRONS_PER_SHELL params.h:21-23 */
    float mu_a;                 /* MU_A              params.h:13-15 */
    float mu_s;                 /* MU_S              params.h:17-19 */
    uint64_t seed;              /* Philox key (SEED  params.h:25-27) */
} tmo_params;

enum { TMO_LOG_TMC = 0, TMO_LOG_NATIVE = 1 };

/* Philox-4x32-10 block function. */
void tmo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* The logarithm shared bit-for-bit with the GPU kernel's exact mode. */
float tmo_logf(float x);
/* Its largest error in ulps (against the C library's double log) over every
 * stride-th float of [lo, hi], and the share of them correctly rounded. */
double tmo_logf_max_ulp(float lo, float hi, uint32_t stride, double *correct_share);

/* Per-photon rand() stream (what the injected rand() returns). */
typedef struct tmo_stream {
    uint64_t photon;
    uint64_t seed;
    uint64_t n;        /* words consumed */
    uint32_t buf[4];
} tmo_stream;
void tmo_stream_init(tmo_stream *s, uint64_t seed, uint64_t photon);
int tmo_stream_rand(tmo_stream *s);

/* First n rand() values of photon p (for known-answer checks). */
void tmo_stream_dump(uint64_t seed, uint64_t photon, uint32_t n, int32_t *out);

/*
 * FP32 restatement, exact integer tallies.  Photons id_base .. id_base+n-1.
 * tally[4*s + 0..3] += {sum_w lo, sum_w hi, sum_w2 lo, sum_w2 hi}, where a
 * deposit of weight w adds rint(w * 2^40) to sum_w and rint(fl(w*w) * 2^40) to
 * sum_w2 (128-bit sums).  deposits[s] += number of deposits (may be NULL).
 * steps (may be NULL) += total deposits.  nthreads > 1 splits the photon range.
 * Returns 0, or -1 on invalid parameters.
 */
int tmo_walk_fx(const tmo_params *p, uint64_t id_base, uint64_t n, int log_mode,
                uint64_t *tally, uint64_t *deposits, uint64_t *steps, int nthreads);

/*
 * FP32 restatement of ONE photon into float arrays exactly as photon.c:30-31
 * accumulates them (heats[s] += (1-a)*w; heats_squared[s] += (1-a)*(1-a)*w*w).
 */
int tmo_walk_photon_f32(const tmo_params *p, uint64_t photon, int log_mode,
                        float *heats, float *heats_squared);

/* Per-photon 64-bit FNV-1a hash of the float arrays that one photon fills. */
int tmo_photon_hashes(const tmo_params *p, uint64_t id_base, uint32_t n, int log_mode,
                      uint64_t *hashes, double *heat_sum, double *heat2_sum);

/*
 * FP64 oracle: the same draws, every operation in double precision.
 * heat[s] += (1-a)*w ; heat2[s] += ((1-a)*w)^2 ; deposits[s] += 1.
 */
int tmo_walk_f64(const tmo_params *p, uint64_t id_base, uint64_t n, double *heat,
                 double *heat2, uint64_t *deposits, int nthreads);

/*
 * Native replay: srand(seed) then n photons drawing from the C library's
 * global rand() and logf, accumulating into float heat/heat2 in the order
 * tiny_mc.c:47-49 does.  batch > 0 additionally writes the per-batch float
 * tallies of consecutive groups of `batch` photons into batch_heat /
 * batch_heat2 ([n/batch][shells]).
 */
int tmo_native_run(const tmo_params *p, uint64_t n, uint32_t seed, float *heat, float *heat2,
                   uint32_t batch, float *batch_heat, float *batch_heat2);

/* Wall-clock throughput probe for the CPU baseline: photons/s of the native
 * replay over n photons (single thread, global rand). */
double tmo_native_rate(const tmo_params *p, uint64_t n, uint32_t seed, uint64_t *steps);

/* The viewer's fragment-shader colour map (cg_mc.c:38-67) on the CPU:
 * red[height][width] float and rgba[height][width][4] (either may be NULL),
 * row 0 = the bottom row (gl_FragCoord.y = 0.5). */
void tmo_colormap(const float *heats, uint32_t shells, uint32_t width, uint32_t height, float *red,
                  unsigned char *rgba);

#ifdef __cplusplus
}
#endif
#endif
