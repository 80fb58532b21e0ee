/*
 * tmc_oracle.c — CPU oracle for the tiny_mc photon walk.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle, never the product): the product
 * library does not link, load or call anything in oracle/.
 *
 * Must be compiled with -std=c11 -ffp-contract=off (the Makefile does): the
 * FP32 restatement relies on every float operation being rounded on its own,
 * exactly like the reference built with `gcc -std=c11` (Makefile:5), where
 * ISO C mode leaves FMA contraction off.
 */
#define _POSIX_C_SOURCE 200809L
#include "tmc_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ---------------------------------------------------------------- Philox */
/* Philox-4x32-10 from its published description (Salmon, Moraes, Dror and
 * Shaw, SC'11): ten rounds of two 32x32->64 multiplies, key bumped by the
 * Weyl constants between rounds. */
#define TMO_PHILOX_M0 0xD2511F53u
#define TMO_PHILOX_M1 0xCD9E8D57u
#define TMO_PHILOX_W0 0x9E3779B9u
#define TMO_PHILOX_W1 0xBB67AE85u

void tmo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)TMO_PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)TMO_PHILOX_M1 * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += TMO_PHILOX_W0;
        k1 += TMO_PHILOX_W1;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

void tmo_stream_init(tmo_stream *s, uint64_t seed, uint64_t photon)
{
    s->photon = photon;
    s->seed = seed;
    s->n = 0;
}

int tmo_stream_rand(tmo_stream *s)
{
    uint32_t j = (uint32_t)(s->n & 3u);
    if (j == 0) {
        uint64_t b = s->n >> 2;
        uint32_t ctr[4] = {(uint32_t)b, (uint32_t)(b >> 32), (uint32_t)s->photon,
                           (uint32_t)(s->photon >> 32)};
        uint32_t key[2] = {(uint32_t)s->seed, (uint32_t)(s->seed >> 32)};
        tmo_philox4x32_10(ctr, key, s->buf);
    }
    s->n++;
    uint32_t r = s->buf[j] >> 1;
    return r ? (int)r : 1;
}

void tmo_stream_dump(uint64_t seed, uint64_t photon, uint32_t n, int32_t *out)
{
    tmo_stream s;
    tmo_stream_init(&s, seed, photon);
    for (uint32_t i = 0; i < n; ++i)
        out[i] = tmo_stream_rand(&s);
}

/* ------------------------------------------------------------------- log */
static inline float f_of(uint32_t u)
{
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
}
static inline uint32_t u_of(float f)
{
    uint32_t u;
    memcpy(&u, &f, sizeof u);
    return u;
}

/*
 * Natural logarithm for positive normal floats (the walk only asks for
 * x in [2^-31, 1]): the library's own division-free sequence, the one the
 * GPU's exact arithmetic evaluates.  x = 2^k * m with m in [sqrt(1/2),
 * sqrt(2)), f = m - 1 (exact), log(m) = f + f^2 R(f) with R the degree-8
 * polynomial oracle/logfit.py derives (Chebyshev interpolant of log1p(f)/f,
 * coefficients rounded to float) evaluated by Horner with fmaf, and
 * log(x) = k*ln2_hi + (k*ln2_lo + log(m)) with ln2 split so k*ln2_hi is exact.
 * Every operation is one IEEE-rounded op (fmaf rounds once); the GPU kernel
 * evaluates the same sequence with __fmul_rn/__fmaf_rn and gets the same bits.
 */
float tmo_logf(float x)
{
    uint32_t ix = u_of(x);
    int32_t k = (int32_t)((ix + 0x004afb0du) >> 23) - 127;
    float m = f_of(ix - ((uint32_t)k << 23));
    float f = m - 1.0f;
    float f2 = f * f;
    float r = -0x1.31335ap-4f;
    r = fmaf(r, f, 0x1.064786p-3f);
    r = fmaf(r, f, -0x1.0fb036p-3f);
    r = fmaf(r, f, 0x1.22cf10p-3f);
    r = fmaf(r, f, -0x1.5423b0p-3f);
    r = fmaf(r, f, 0x1.999e86p-3f);
    r = fmaf(r, f, -0x1.000424p-2f);
    r = fmaf(r, f, 0x1.55555ep-2f);
    r = fmaf(r, f, -0x1.fffff8p-2f);
    float lm = fmaf(f2, r, f);
    float kf = (float)k;
    return fmaf(kf, 0.693145751953125f, fmaf(kf, 1.42860682e-6f, lm));
}

/* Largest error of tmo_logf in ulps against the C library's double log over
 * the floats from lo to hi (bit patterns, every `stride`-th), and the share of
 * them that tmo_logf rounds correctly. */
double tmo_logf_max_ulp(float lo, float hi, uint32_t stride, double *correct_share)
{
    double worst = 0.0;
    uint64_t n = 0, exact = 0;
    if (stride == 0)
        stride = 1;
    for (uint64_t u = u_of(lo); u <= u_of(hi); u += stride) {
        const float x = f_of((uint32_t)u);
        const float y = tmo_logf(x);
        const double t = log((double)x);
        const float ft = (float)fabs(t);
        const double spacing = (double)nextafterf(ft, INFINITY) - (double)ft;
        const double e = t == 0.0 ? fabs((double)y) : fabs((double)y - t) / spacing;
        if ((float)t == y)
            ++exact;
        if (e > worst)
            worst = e;
        ++n;
    }
    if (correct_share)
        *correct_share = n ? (double)exact / (double)n : 0.0;
    return worst;
}

/* ------------------------------------------------------ derived constants */
typedef struct {
    float albedo;   /* photon.c:8 */
    float c;        /* 1.0f - albedo, photon.c:30 */
    float spm;      /* shells_per_mfp, photon.c:9 */
    uint32_t shells;
} derived32;

static int derive32(const tmo_params *p, derived32 *d)
{
    if (!p || p->shells == 0 || !(p->mu_a > 0.0f) || !(p->mu_s >= 0.0f) ||
        !(p->microns_per_shell > 0.0f))
        return -1;
    d->albedo = p->mu_s / (p->mu_s + p->mu_a);
    d->spm = (float)(1e4 / (double)p->microns_per_shell / (double)(p->mu_a + p->mu_s));
    d->c = 1.0f - d->albedo;
    d->shells = p->shells;
    if (!(d->albedo < 1.0f))   /* weight would never decay: no photon would die */
        return -1;
    return 0;
}

/* ------------------------------------------------------------ rand source */
typedef struct {
    int native;      /* 1: the C library's global rand() */
    tmo_stream s;
} rsrc;

static inline int rs_rand(rsrc *r) { return r->native ? rand() : tmo_stream_rand(&r->s); }

/* ----------------------------------------------------------- deposit sink */
typedef unsigned __int128 u128;

typedef struct {
    int kind;               /* 0: fixed point, 1: float arrays */
    u128 *sw, *sw2;         /* kind 0 */
    uint64_t *dep;          /* kind 0, may be NULL */
    uint64_t steps;
    float *h, *h2;          /* kind 1 */
    float *bh, *bh2;        /* kind 1, second pair or NULL */
} sink;

static inline uint64_t fx40(float v) { return (uint64_t)llrintf(v * 1099511627776.0f); }

static inline void deposit(sink *k, uint32_t shell, float weight, float c)
{
    k->steps++;
    if (k->kind == 0) {
        k->sw[shell] += fx40(weight);
        k->sw2[shell] += fx40(weight * weight);
        if (k->dep)
            k->dep[shell]++;
    } else {
        /* photon.c:30-31, same expressions, same rounding */
        k->h[shell] += c * weight;
        k->h2[shell] += c * c * weight * weight;
        if (k->bh) {
            k->bh[shell] += c * weight;
            k->bh2[shell] += c * c * weight * weight;
        }
    }
}

/* ------------------------------------------------------- the FP32 walk */
/* photon.c:6-51 restated with runtime parameters.  Shell clamp: the value is
 * clamped in float before the conversion (identical to photon.c:26-29 for
 * every radius below 2^32 shells; a NaN radius lands in the last shell). */
static void walk32(const derived32 *d, rsrc *rs, int log_mode, sink *k)
{
    const float last = (float)(d->shells - 1);
    float x = 0.0f, y = 0.0f, z = 0.0f;
    float u = 0.0f, v = 0.0f, w = 1.0f;
    float weight = 1.0f;
    for (;;) {
        float U = (float)rs_rand(rs) / 2147483648.0f;
        float t = -(log_mode == TMO_LOG_TMC ? tmo_logf(U) : logf(U));
        x += t * u;
        y += t * v;
        z += t * w;

        float rr = sqrtf(x * x + y * y + z * z) * d->spm;
        uint32_t shell = (rr < last) ? (uint32_t)rr : d->shells - 1;
        deposit(k, shell, weight, d->c);
        weight *= d->albedo;

        float xi1, xi2;
        do {
            xi1 = 2.0f * (float)rs_rand(rs) / 2147483648.0f - 1.0f;
            xi2 = 2.0f * (float)rs_rand(rs) / 2147483648.0f - 1.0f;
            t = xi1 * xi1 + xi2 * xi2;
        } while (1.0f < t);
        u = 2.0f * t - 1.0f;
        v = xi1 * sqrtf((1.0f - u * u) / t);
        w = xi2 * sqrtf((1.0f - u * u) / t);

        if (weight < 0.001f) {
            if ((float)rs_rand(rs) / 2147483648.0f > 0.1f)
                break;
            weight /= 0.1f;
        }
    }
}

/* ------------------------------------------------------- the FP64 walk */
typedef struct {
    double albedo, c, spm;
    uint32_t shells;
} derived64;

static void walk64(const derived64 *d, rsrc *rs, double *heat, double *heat2, uint64_t *dep)
{
    /* the literals of photon.c:45-48 keep their float values so that the
     * roulette decisions consume the same draws */
    const double wmin = (double)0.001f, psurv = (double)0.1f;
    const double last = (double)(d->shells - 1);
    double x = 0.0, y = 0.0, z = 0.0, u = 0.0, v = 0.0, w = 1.0, weight = 1.0;
    for (;;) {
        double U = (double)rs_rand(rs) * 0x1p-31;
        double t = -log(U);
        x += t * u;
        y += t * v;
        z += t * w;
        double rr = sqrt(x * x + y * y + z * z) * d->spm;
        uint32_t shell = (rr < last) ? (uint32_t)rr : d->shells - 1;
        double dq = d->c * weight;
        heat[shell] += dq;
        heat2[shell] += dq * dq;
        if (dep)
            dep[shell]++;
        weight *= d->albedo;
        double xi1, xi2;
        do {
            xi1 = 2.0 * (double)rs_rand(rs) * 0x1p-31 - 1.0;
            xi2 = 2.0 * (double)rs_rand(rs) * 0x1p-31 - 1.0;
            t = xi1 * xi1 + xi2 * xi2;
        } while (1.0 < t);
        u = 2.0 * t - 1.0;
        v = xi1 * sqrt((1.0 - u * u) / t);
        w = xi2 * sqrt((1.0 - u * u) / t);
        if (weight < wmin) {
            if ((double)rs_rand(rs) * 0x1p-31 > psurv)
                break;
            weight /= psurv;
        }
    }
}

/* ------------------------------------------------------------ threading */
typedef struct {
    const tmo_params *p;
    uint64_t id0, n;
    int log_mode;
    int f64;
    /* fx outputs */
    u128 *sw, *sw2;
    uint64_t *dep;
    uint64_t steps;
    /* f64 outputs */
    double *heat, *heat2;
} job;

static void *run_job(void *arg)
{
    job *j = (job *)arg;
    rsrc rs;
    rs.native = 0;
    if (!j->f64) {
        derived32 d;
        derive32(j->p, &d);
        sink k = {0};
        k.kind = 0;
        k.sw = j->sw;
        k.sw2 = j->sw2;
        k.dep = j->dep;
        for (uint64_t i = 0; i < j->n; ++i) {
            tmo_stream_init(&rs.s, j->p->seed, j->id0 + i);
            walk32(&d, &rs, j->log_mode, &k);
        }
        j->steps = k.steps;
    } else {
        derived64 d;
        d.albedo = (double)j->p->mu_s / ((double)j->p->mu_s + (double)j->p->mu_a);
        d.c = 1.0 - d.albedo;
        d.spm = 1e4 / (double)j->p->microns_per_shell / ((double)j->p->mu_a + (double)j->p->mu_s);
        d.shells = j->p->shells;
        for (uint64_t i = 0; i < j->n; ++i) {
            tmo_stream_init(&rs.s, j->p->seed, j->id0 + i);
            walk64(&d, &rs, j->heat, j->heat2, j->dep);
        }
    }
    return NULL;
}

static int run_jobs(const tmo_params *p, uint64_t id_base, uint64_t n, int log_mode, int f64,
                    int nthreads, job **out_jobs)
{
    if (nthreads < 1)
        nthreads = 1;
    if ((uint64_t)nthreads > n && n > 0)
        nthreads = (int)n;
    if (n == 0)
        nthreads = 1;
    uint32_t S = p->shells;
    job *jobs = (job *)calloc((size_t)nthreads, sizeof(job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th)
        return -2;
    uint64_t per = n / (uint64_t)nthreads, extra = n % (uint64_t)nthreads, at = id_base;
    for (int t = 0; t < nthreads; ++t) {
        job *j = &jobs[t];
        j->p = p;
        j->id0 = at;
        j->n = per + ((uint64_t)t < extra ? 1 : 0);
        at += j->n;
        j->log_mode = log_mode;
        j->f64 = f64;
        j->dep = (uint64_t *)calloc(S, sizeof(uint64_t));
        if (f64) {
            j->heat = (double *)calloc(S, sizeof(double));
            j->heat2 = (double *)calloc(S, sizeof(double));
        } else {
            j->sw = (u128 *)calloc(S, sizeof(u128));
            j->sw2 = (u128 *)calloc(S, sizeof(u128));
        }
    }
    for (int t = 1; t < nthreads; ++t)
        pthread_create(&th[t], NULL, run_job, &jobs[t]);
    run_job(&jobs[0]);
    for (int t = 1; t < nthreads; ++t)
        pthread_join(th[t], NULL);
    free(th);
    *out_jobs = jobs;
    return nthreads;
}

int tmo_walk_fx(const tmo_params *p, uint64_t id_base, uint64_t n, int log_mode,
                uint64_t *tally, uint64_t *deposits, uint64_t *steps, int nthreads)
{
    derived32 d;
    if (derive32(p, &d) != 0 || !tally)
        return -1;
    job *jobs = NULL;
    int nt = run_jobs(p, id_base, n, log_mode, 0, nthreads, &jobs);
    if (nt < 0)
        return -2;
    uint32_t S = p->shells;
    for (uint32_t s = 0; s < S; ++s) {
        u128 a = (u128)tally[4 * s + 0] | ((u128)tally[4 * s + 1] << 64);
        u128 b = (u128)tally[4 * s + 2] | ((u128)tally[4 * s + 3] << 64);
        for (int t = 0; t < nt; ++t) {
            a += jobs[t].sw[s];
            b += jobs[t].sw2[s];
            if (deposits)
                deposits[s] += jobs[t].dep[s];
        }
        tally[4 * s + 0] = (uint64_t)a;
        tally[4 * s + 1] = (uint64_t)(a >> 64);
        tally[4 * s + 2] = (uint64_t)b;
        tally[4 * s + 3] = (uint64_t)(b >> 64);
    }
    for (int t = 0; t < nt; ++t) {
        if (steps)
            *steps += jobs[t].steps;
        free(jobs[t].sw);
        free(jobs[t].sw2);
        free(jobs[t].dep);
    }
    free(jobs);
    return 0;
}

int tmo_walk_f64(const tmo_params *p, uint64_t id_base, uint64_t n, double *heat,
                 double *heat2, uint64_t *deposits, int nthreads)
{
    derived32 d;
    if (derive32(p, &d) != 0 || !heat || !heat2)
        return -1;
    job *jobs = NULL;
    int nt = run_jobs(p, id_base, n, TMO_LOG_NATIVE, 1, nthreads, &jobs);
    if (nt < 0)
        return -2;
    for (uint32_t s = 0; s < p->shells; ++s) {
        for (int t = 0; t < nt; ++t) {
            heat[s] += jobs[t].heat[s];
            heat2[s] += jobs[t].heat2[s];
            if (deposits)
                deposits[s] += jobs[t].dep[s];
        }
    }
    for (int t = 0; t < nt; ++t) {
        free(jobs[t].heat);
        free(jobs[t].heat2);
        free(jobs[t].dep);
    }
    free(jobs);
    return 0;
}

int tmo_walk_photon_f32(const tmo_params *p, uint64_t photon, int log_mode, float *heats,
                        float *heats_squared)
{
    derived32 d;
    if (derive32(p, &d) != 0)
        return -1;
    rsrc rs;
    rs.native = 0;
    tmo_stream_init(&rs.s, p->seed, photon);
    sink k = {0};
    k.kind = 1;
    k.h = heats;
    k.h2 = heats_squared;
    walk32(&d, &rs, log_mode, &k);
    return 0;
}

static uint64_t fnv1a(uint64_t h, const void *data, size_t n)
{
    const unsigned char *b = (const unsigned char *)data;
    for (size_t i = 0; i < n; ++i) {
        h ^= b[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

int tmo_photon_hashes(const tmo_params *p, uint64_t id_base, uint32_t n, int log_mode,
                      uint64_t *hashes, double *heat_sum, double *heat2_sum)
{
    uint32_t S = p->shells;
    float *h = (float *)malloc(S * sizeof(float)), *h2 = (float *)malloc(S * sizeof(float));
    if (!h || !h2)
        return -2;
    for (uint32_t i = 0; i < n; ++i) {
        memset(h, 0, S * sizeof(float));
        memset(h2, 0, S * sizeof(float));
        if (tmo_walk_photon_f32(p, id_base + i, log_mode, h, h2) != 0) {
            free(h);
            free(h2);
            return -1;
        }
        uint64_t hv = fnv1a(0xcbf29ce484222325ull, h, S * sizeof(float));
        hashes[i] = fnv1a(hv, h2, S * sizeof(float));
        for (uint32_t s = 0; s < S; ++s) {
            heat_sum[s] += h[s];
            heat2_sum[s] += h2[s];
        }
    }
    free(h);
    free(h2);
    return 0;
}

int tmo_native_run(const tmo_params *p, uint64_t n, uint32_t seed, float *heat, float *heat2,
                   uint32_t batch, float *batch_heat, float *batch_heat2)
{
    derived32 d;
    if (derive32(p, &d) != 0)
        return -1;
    rsrc rs;
    rs.native = 1;
    srand(seed);   /* tiny_mc.c:43 */
    sink k = {0};
    k.kind = 1;
    k.h = heat;
    k.h2 = heat2;
    for (uint64_t i = 0; i < n; ++i) {   /* tiny_mc.c:47-49 */
        if (batch) {
            uint64_t b = i / batch;
            k.bh = batch_heat + b * d.shells;
            k.bh2 = batch_heat2 + b * d.shells;
        }
        walk32(&d, &rs, TMO_LOG_NATIVE, &k);
    }
    return 0;
}

double tmo_native_rate(const tmo_params *p, uint64_t n, uint32_t seed, uint64_t *steps)
{
    derived32 d;
    if (derive32(p, &d) != 0)
        return -1.0;
    float *h = (float *)calloc(d.shells, sizeof(float));
    float *h2 = (float *)calloc(d.shells, sizeof(float));
    if (!h || !h2)
        return -2.0;
    rsrc rs;
    rs.native = 1;
    srand(seed);
    sink k = {0};
    k.kind = 1;
    k.h = h;
    k.h2 = h2;
    struct timespec a, b;
    clock_gettime(CLOCK_MONOTONIC, &a);
    for (uint64_t i = 0; i < n; ++i)
        walk32(&d, &rs, TMO_LOG_NATIVE, &k);
    clock_gettime(CLOCK_MONOTONIC, &b);
    double dt = (double)(b.tv_sec - a.tv_sec) + 1e-9 * (double)(b.tv_nsec - a.tv_nsec);
    if (steps)
        *steps = k.steps;
    free(h);
    free(h2);
    return dt > 0 ? (double)n / dt : 0.0;
}

/* ------------------------------------------------------ viewer colour map */
/* cg_mc.c:38-67 (fragment shader FSHADER) restated in C: pixel (px, py) of a
 * width x height target has gl_FragCoord = (px + 0.5, py + 0.5); uv = that /
 * 800 (the shader divides by the literal 800, cg_mc.c:50); dr = |uv - 0.5|;
 * shell = int(dr / 0.7071067811865476 * (shells - 1)) (truncation), clamped
 * to the last shell for targets larger than 800; red = 2 / (1 + exp(-0.004
 * heat)) - 1 (L = 2, b = 1, k = 0.004, cg_mc.c:58-62).  rgba8 is the usual
 * UNORM conversion of (red, 0, 0, 1). */
void tmo_colormap(const float *heats, uint32_t shells, uint32_t width, uint32_t height, float *red,
                  unsigned char *rgba)
{
    const float mc = 0.7071067811865476f;
    for (uint32_t py = 0; py < height; ++py) {
        for (uint32_t px = 0; px < width; ++px) {
            float ux = ((float)px + 0.5f) / 800.0f - 0.5f;
            float uy = ((float)py + 0.5f) / 800.0f - 0.5f;
            float dr = sqrtf(ux * ux + uy * uy);
            int id = (int)((dr / mc) * (float)(shells - 1));
            if (id > (int)shells - 1)
                id = (int)shells - 1;
            float heat = heats[id];
            float fit = 2.0f / (1.0f + 1.0f * expf(-0.004f * heat)) - 1.0f;
            size_t k = (size_t)py * width + px;
            if (red)
                red[k] = fit;
            if (rgba) {
                float c = fit < 0.0f ? 0.0f : (fit > 1.0f ? 1.0f : fit);
                rgba[4 * k + 0] = (unsigned char)lrintf(c * 255.0f);
                rgba[4 * k + 1] = 0;
                rgba[4 * k + 2] = 0;
                rgba[4 * k + 3] = 255;
            }
        }
    }
}
