/*
 * ref_native.c — driver for the reference's unmodified photon.c with the C
 * library's own rand() and logf().  TEST INFRASTRUCTURE ONLY: linked into
 * oracle/_ref/ shared objects to produce native-RNG fixtures and CPU timings.
 */
#define _POSIX_C_SOURCE 200809L
#include <stdint.h>
#include <stdlib.h>
#include <time.h>

void photon(float *heats, float *heats_squared); /* photon.h:3 */

unsigned ref_shells(void) { return SHELLS; }

/* tiny_mc.c:43-49: srand(seed), then n photons into the same float arrays. */
int ref_native_run(uint64_t n, unsigned seed, float *heat, float *heat2)
{
    srand(seed);
    for (uint64_t i = 0; i < n; ++i)
        photon(heat, heat2);
    return 0;
}

/* The same rand() sequence, but photon i accumulates into batch i/batch. */
int ref_native_batches(uint64_t n, unsigned seed, unsigned batch, float *bh, float *bh2)
{
    srand(seed);
    for (uint64_t i = 0; i < n; ++i)
        photon(bh + (i / batch) * SHELLS, bh2 + (i / batch) * SHELLS);
    return 0;
}

/* Photons per second of the reference walk on this core. */
double ref_native_rate(uint64_t n, unsigned seed)
{
    static float h[SHELLS], h2[SHELLS];
    struct timespec a, b;
    srand(seed);
    clock_gettime(CLOCK_MONOTONIC, &a);
    for (uint64_t i = 0; i < n; ++i)
        photon(h, h2);
    clock_gettime(CLOCK_MONOTONIC, &b);
    double dt = (double)(b.tv_sec - a.tv_sec) + 1e-9 * (double)(b.tv_nsec - a.tv_nsec);
    return dt > 0 ? (double)n / dt : 0.0;
}
