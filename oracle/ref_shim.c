/*
 * ref_shim.c — driver for the reference's unmodified photon.c compiled with
 * ref_inject.h.  TEST INFRASTRUCTURE ONLY: linked into oracle/_ref/ shared objects.
 *
 * photon() (photon.c:6, declared at photon.h:3) is called once per photon
 * with freshly zeroed float arrays, exactly as tiny_mc.c:48 calls it but one
 * photon at a time, so that each photon's float deposits can be compared bit
 * for bit with the oracle's restatement.
 */
#include "tmc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

void photon(float *heats, float *heats_squared); /* photon.h:3 */

static tmo_stream g_stream;
static int g_log_mode = TMO_LOG_NATIVE;

int tmo_ref_rand(void) { return tmo_stream_rand(&g_stream); }

float tmo_ref_logf(float x) { return g_log_mode == TMO_LOG_TMC ? tmo_logf(x) : logf(x); }

unsigned ref_shells(void) { return SHELLS; }

static unsigned long long fnv1a(unsigned long long h, const void *data, size_t n)
{
    const unsigned char *b = (const unsigned char *)data;
    for (size_t i = 0; i < n; ++i) {
        h ^= b[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

/* Same contract as tmo_photon_hashes (tmc_oracle.h), but the walk is the
 * reference's photon(). */
int ref_photon_hashes(uint64_t seed, uint64_t id_base, uint32_t n, int log_mode,
                      uint64_t *hashes, double *heat_sum, double *heat2_sum)
{
    static float h[SHELLS], h2[SHELLS];
    g_log_mode = log_mode;
    for (uint32_t i = 0; i < n; ++i) {
        memset(h, 0, sizeof h);
        memset(h2, 0, sizeof h2);
        tmo_stream_init(&g_stream, seed, id_base + i);
        photon(h, h2);
        uint64_t hv = fnv1a(0xcbf29ce484222325ull, h, sizeof h);
        hashes[i] = fnv1a(hv, h2, sizeof h2);
        for (unsigned s = 0; s < SHELLS; ++s) {
            heat_sum[s] += h[s];
            heat2_sum[s] += h2[s];
        }
    }
    return 0;
}
