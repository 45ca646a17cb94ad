/*
 * synth_host.c -- seeded 2D Brownian-motion imaging-FCS stack simulator on
 * the host (C, OpenMP), used to make the benchmark and test stacks that both
 * the GPU engine and the CPU baseline read.
 *
 * Semantics follow simulateACF2D (Imaging_FCS_1_52.java:13854-14409): particles
 * on a periodic square larger than the detector by `margin` on every side,
 * Gaussian steps of variance 2 D dt per axis (steps_per_frame steps per
 * frame), Poisson photon emission per step at rate cps, each photon displaced
 * by the Gaussian PSF (sigma = 1/e^2 radius / 2) and counted in the pixel it
 * lands in, irreversible bleaching with time constant tau_bleach, camera
 * offset.  D may be given per 16 x 16 pixel tile (the particle's current
 * tile sets its step).
 *
 * Every particle owns a counter-based random stream (splitmix64), and photon
 * counts are integer sums, so the stack depends only on the seed, never on
 * the number of threads.
 */
#include <math.h>

#define SYNTH_PI 3.14159265358979323846
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double x, y;
    int bleached, species;
    uint64_t rng;
} particle;

static uint64_t splitmix(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static double urand(uint64_t *s) { return ((double)(splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

static void nrand2(uint64_t *s, double *a, double *b)
{
    const double u1 = urand(s), u2 = urand(s);
    const double r = sqrt(-2.0 * log(u1));
    *a = r * cos(2.0 * SYNTH_PI * u2);
    *b = r * sin(2.0 * SYNTH_PI * u2);
}

static int poisson(uint64_t *s, double lambda)
{
    if (lambda > 30.0) {
        double a, b;
        nrand2(s, &a, &b);
        long k = lround(lambda + sqrt(lambda) * a);
        return k < 0 ? 0 : (int)k;
    }
    const double L = exp(-lambda);
    double p = 1.0;
    int k = 0;
    do { k++; p *= urand(s); } while (p > L && k < 1000);
    return k - 1;
}

/* out: uint16 [frames][height][width].  d_tile_map (optional):
 * [ceil(h/16)][ceil(w/16)] um^2/s.  Returns 0 on success. */
int synth_brownian(int width, int height, int frames, double frametime, int steps_per_frame,
                   double pixel_um, double psf_um, double density, double d1, double d2,
                   double fraction2, double cps, double tau_bleach, int offset, double margin,
                   uint64_t seed, const float *d_tile_map, uint16_t *out)
{
    if (width <= 0 || height <= 0 || frames <= 0 || steps_per_frame <= 0 || !(pixel_um > 0) || !out) return 1;
    const double lx = width * pixel_um + 2 * margin, ly = height * pixel_um + 2 * margin;
    long np = lround(density * lx * ly);
    if (np < 1) np = 1;
    const double dt = frametime / steps_per_frame, sig = psf_um / 2.0;
    const double ph_step = cps * dt;
    const double p_bleach = tau_bleach > 0 ? 1.0 - exp(-dt / tau_bleach) : 0.0;
    const int tx_n = (width + 15) / 16, ty_n = (height + 15) / 16;
    particle *pt = (particle *)malloc(sizeof(particle) * np);
    if (!pt) return 1;
    for (long i = 0; i < np; i++) {
        uint64_t s = seed ^ (0xD1B54A32D192ED03ull * (uint64_t)(i + 1));
        splitmix(&s);
        pt[i].x = urand(&s) * lx;
        pt[i].y = urand(&s) * ly;
        pt[i].bleached = 0;
        pt[i].species = urand(&s) < fraction2;
        pt[i].rng = s;
    }
    const size_t fsz = (size_t)width * height;
    const int block = 64;
    uint32_t *acc = (uint32_t *)malloc(sizeof(uint32_t) * fsz * block);
    if (!acc) { free(pt); return 1; }
    int rc = 0;
#pragma omp parallel
    {
        uint32_t *cnt = (uint32_t *)malloc(sizeof(uint32_t) * fsz * block);
        if (!cnt) {
#pragma omp atomic write
            rc = 1;
        }
        for (int f0 = 0; f0 < frames; f0 += block) {
            const int nf = frames - f0 < block ? frames - f0 : block;
            if (cnt) memset(cnt, 0, sizeof(uint32_t) * fsz * nf);
#pragma omp for schedule(static)
            for (long i = 0; i < np; i++) {
                particle p = pt[i];
                for (int f = 0; f < nf && cnt; f++) {
                    uint32_t *cf = cnt + (size_t)f * fsz;
                    for (int k = 0; k < steps_per_frame; k++) {
                        double d = p.species ? d2 : d1;
                        if (d_tile_map) {
                            int tx = (int)floor((p.x - margin) / pixel_um) / 16;
                            int ty = (int)floor((p.y - margin) / pixel_um) / 16;
                            tx = tx < 0 ? 0 : (tx >= tx_n ? tx_n - 1 : tx);
                            ty = ty < 0 ? 0 : (ty >= ty_n ? ty_n - 1 : ty);
                            d = d_tile_map[ty * tx_n + tx];
                        }
                        const double sd = sqrt(2.0 * d * dt);
                        double g1, g2;
                        nrand2(&p.rng, &g1, &g2);
                        p.x += sd * g1;
                        p.y += sd * g2;
                        p.x -= lx * floor(p.x / lx);
                        p.y -= ly * floor(p.y / ly);
                        if (p_bleach > 0 && !p.bleached && urand(&p.rng) < p_bleach) p.bleached = 1;
                        if (p.bleached) continue;
                        const int nph = poisson(&p.rng, ph_step);
                        for (int q = 0; q < nph; q++) {
                            double e1, e2;
                            nrand2(&p.rng, &e1, &e2);
                            const int px = (int)floor((p.x + sig * e1 - margin) / pixel_um);
                            const int py = (int)floor((p.y + sig * e2 - margin) / pixel_um);
                            if (px >= 0 && px < width && py >= 0 && py < height) cf[(size_t)py * width + px] += 1u;
                        }
                    }
                }
                pt[i] = p;
            }
            /* implicit barrier of the omp for: every particle's photons of this
             * block are in the threads' buffers; integer sums in any order */
#pragma omp for schedule(static)
            for (long i = 0; i < (long)(fsz * nf); i++) acc[i] = 0;
#pragma omp critical
            {
                if (cnt)
                    for (size_t i = 0; i < fsz * nf; i++) acc[i] += cnt[i];
            }
#pragma omp barrier
#pragma omp for schedule(static)
            for (long i = 0; i < (long)(fsz * nf); i++) {
                const uint32_t v = acc[i] + (uint32_t)offset;
                out[(size_t)f0 * fsz + i] = (uint16_t)(v > 65535u ? 65535u : v);
            }
        }
        free(cnt);
    }
    free(acc);
    free(pt);
    return rc;
}
