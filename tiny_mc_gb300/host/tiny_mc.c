/*
 * tiny_mc.c (drop-in driver) — the headless program of the reference
 * (tiny_mc.c:34-69) on top of libtmc_gb300: same compile-time knobs
 * (SHELLS, PHOTONS, MU_A, MU_S, MICRONS_PER_SHELL, SEED as -D macros with the
 * params.h:5-27 defaults), same stdout layout, but the photon loop of
 * tiny_mc.c:47-49 is ONE tmc_photon_batch() call on the GPU.
 *
 * Optional arguments override the macros at run time:
 *     tiny_mc [photons [seed [exact|fast [float|fp64 [image.ppm]]]]]
 * "fp64" prints the table from the GPU's FP64 normalisation of the exact
 * tallies instead of the float arrays; image.ppm writes the viewer's colour
 * map of the heat array (cg_mc.c:38-67) as an 800x800 binary PPM.
 */
#define _POSIX_C_SOURCE 199309L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "tmc.h"

#ifndef SHELLS
#define SHELLS 101
#endif
#ifndef PHOTONS
#define PHOTONS 32768
#endif
#ifndef MU_A
#define MU_A 2.0f
#endif
#ifndef MU_S
#define MU_S 20.0f
#endif
#ifndef MICRONS_PER_SHELL
#define MICRONS_PER_SHELL 50
#endif
#ifndef SEED
#define SEED (time(NULL))
#endif

static double wall_seconds(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return 1e-9 * ts.tv_nsec + (double)ts.tv_sec;
}

static float heat[SHELLS];
static float heat2[SHELLS];

int main(int argc, char **argv)
{
    unsigned long long photons = PHOTONS;
    unsigned long long seed = (unsigned long long)(SEED);
    tmc_params p;
    tmc_params_default(&p);
    p.shells = SHELLS;
    p.microns_per_shell = MICRONS_PER_SHELL;
    p.mu_a = MU_A;
    p.mu_s = MU_S;
    if (argc > 1)
        photons = strtoull(argv[1], NULL, 10);
    if (argc > 2)
        seed = strtoull(argv[2], NULL, 10);
    if (argc > 3 && strcmp(argv[3], "fast") == 0)
        p.math = TMC_MATH_FAST;
    const int fp64 = argc > 4 && strcmp(argv[4], "fp64") == 0;
    const char *ppm = argc > 5 ? argv[5] : NULL;
    p.seed = seed;

    printf("# %s\n# %s\n# %s\n", "Tiny Monte Carlo by Scott Prahl (http://omlc.ogi.edu)",
           "1 W Point Source Heating in Infinite Isotropic Scattering Medium",
           "GB300 (sm_103a) version on libtmc_gb300");
    printf("# Scattering = %8.3f/cm\n", (double)p.mu_s);
    printf("# Absorption = %8.3f/cm\n", (double)p.mu_a);
    printf("# Photons    = %8llu\n#\n", photons);

    static tmc_tally tally[SHELLS];
    double start = wall_seconds();
    int st = fp64 ? tmc_photon_batch_fx(tally, photons, &p, NULL)
                  : tmc_photon_batch(heat, heat2, photons, &p);
    double end = wall_seconds();
    if (st != TMC_OK) {
        fprintf(stderr, "tmc_photon_batch: %s (%s)\n", tmc_strerror(st), tmc_last_error());
        return 1;
    }
    double elapsed = end - start;
    printf("# %lf seconds\n", elapsed);
    printf("# %lf K photons per second\n", 1e-3 * (double)photons / elapsed);

    int need;
    char *buf;
    if (fp64) {
        static double density[SHELLS], error[SHELLS], h[SHELLS], h2[SHELLS];
        double extra = 0.0;
        if (tmc_report_fp64(tally, &p, photons, density, error, &extra) != TMC_OK)
            return 1;
        tmc_tally_to_heat(tally, &p, h, h2);
        for (int i = 0; i < SHELLS; ++i) {
            heat[i] = (float)h[i];
            heat2[i] = (float)h2[i];
        }
        need = tmc_format_report_fp64(NULL, 0, density, error, extra, &p);
        if (need < 0 || !(buf = (char *)malloc((size_t)need + 1)))
            return 1;
        tmc_format_report_fp64(buf, (size_t)need + 1, density, error, extra, &p);
    } else {
        need = tmc_format_report(NULL, 0, heat, heat2, photons, &p);
        if (need < 0 || !(buf = (char *)malloc((size_t)need + 1)))
            return 1;
        tmc_format_report(buf, (size_t)need + 1, heat, heat2, photons, &p);
    }
    fputs(buf, stdout);
    free(buf);
    if (ppm) {
        static unsigned char rgba[800 * 800 * 4];
        if (tmc_colormap_host(heat, SHELLS, 800, 800, NULL, rgba) != TMC_OK)
            return 1;
        FILE *f = fopen(ppm, "wb");
        if (!f)
            return 1;
        fprintf(f, "P6\n800 800\n255\n");
        for (int y = 799; y >= 0; --y)          /* top row first; row 0 is the bottom */
            for (int x = 0; x < 800; ++x)
                fwrite(&rgba[4 * (y * 800 + x)], 1, 3, f);
        fclose(f);
    }
    return 0;
}
