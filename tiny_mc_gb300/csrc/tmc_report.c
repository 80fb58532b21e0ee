/*
 * tmc_report.c — the results table of tiny_mc.c:58-66, written from the float
 * heat/heat2 arrays with the same printf formats and the same mixture of
 * float and double arithmetic, so that the drop-in driver's table is
 * byte-for-byte what the reference prints for the same arrays.
 *
 * Compiled with -std=c11 -ffp-contract=off (every float operation rounded on
 * its own, as in the reference's ISO C build).
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>

#include "tmc.h"

static const double TMC_PI = 3.14159265358979323846; /* M_PI */

typedef struct {
    char *buf;
    size_t cap;
    size_t len;
} out_t;

static void put(out_t *o, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    char *dst = (o->buf && o->len < o->cap) ? o->buf + o->len : NULL;
    size_t room = dst ? o->cap - o->len : 0;
    int n = vsnprintf(dst, room, fmt, ap);
    va_end(ap);
    if (n > 0)
        o->len += (size_t)n;
}

int tmc_format_report(char *buf, size_t cap, const float *heat, const float *heat2,
                      uint64_t photons, const tmc_params *p)
{
    if (!heat || !heat2 || !p || p->shells == 0 || photons == 0)
        return TMC_E_INVALID;
    if (buf && cap)
        buf[0] = '\0';
    out_t o = {buf, cap, 0};
    const unsigned shells = p->shells;
    const float mps = p->microns_per_shell;
    const float nf = (float)photons;   /* PHOTONS as a float operand */

    put(&o, "# Radius\tHeat\n");
    put(&o, "# [microns]\t[W/cm^3]\tError\n");
    /* tiny_mc.c:60: float t = 4.0f * M_PI * powf(MPS, 3.0f) * PHOTONS / 1e12; */
    float t = (float)((4.0 * TMC_PI) * (double)powf(mps, 3.0f) * (double)photons / 1e12);
    for (unsigned i = 0; i < shells - 1; ++i) {
        /* tiny_mc.c:62-64 */
        float radius = (float)i * mps;
        double h = (double)(heat[i] / t) / ((double)(i * i + i) + 1.0 / 3.0);
        float var = heat2[i] - heat[i] * heat[i] / nf;
        double err = sqrt((double)var) / (double)t / (double)((float)(i * i + i) + 1.0f / 3.0f);
        put(&o, "%6.0f\t%12.5f\t%12.5f\n", (double)radius, h, err);
    }
    put(&o, "# extra\t%12.5f\n", (double)(heat[shells - 1] / nf)); /* tiny_mc.c:66 */
    if (buf && cap && o.len >= cap)
        buf[cap - 1] = '\0';
    return o.len > 0x7fffffff ? TMC_E_OVERFLOW : (int)o.len;
}

/* The same table from FP64 values (tmc_report_fp64_device): radius column in
 * float as tiny_mc.c:62 prints it, heat and error columns from the doubles. */
int tmc_format_report_fp64(char *buf, size_t cap, const double *density, const double *error,
                           double extra, const tmc_params *p)
{
    if (!density || !error || !p || p->shells == 0)
        return TMC_E_INVALID;
    if (buf && cap)
        buf[0] = '\0';
    out_t o = {buf, cap, 0};
    put(&o, "# Radius\tHeat\n");
    put(&o, "# [microns]\t[W/cm^3]\tError\n");
    for (unsigned i = 0; i < p->shells - 1; ++i)
        put(&o, "%6.0f\t%12.5f\t%12.5f\n", (double)((float)i * p->microns_per_shell), density[i],
            error[i]);
    put(&o, "# extra\t%12.5f\n", extra);
    if (buf && cap && o.len >= cap)
        buf[cap - 1] = '\0';
    return o.len > 0x7fffffff ? TMC_E_OVERFLOW : (int)o.len;
}
