/*
 * ref_inject.h — force-included (gcc -include) ahead of the reference's
 * UNMODIFIED photon.c when oracle/Makefile builds oracle/_ref/.  TEST
 * INFRASTRUCTURE ONLY.
 *
 * After the system headers are in, the two library calls photon.c makes
 * (rand() at photon.c:21,37,38,46 and logf() at photon.c:21) are renamed to
 * the oracle's injection points in ref_shim.c, so the reference's own walk
 * consumes the per-photon Philox stream and, optionally, the oracle's
 * logarithm.  RAND_MAX keeps its value (2^31-1).
 */
#include <math.h>
#include <stdlib.h>

int tmo_ref_rand(void);
float tmo_ref_logf(float);

#define rand tmo_ref_rand
#define logf tmo_ref_logf
