// imfcs_sim.cu -- seeded 2D Brownian-motion stack simulator on the GPU.
//
// Semantics follow simulateACF2D (Imaging_FCS_1_52.java:13854-14409):
// particles on a periodic square larger than the detector, Gaussian steps of
// variance 2 D dt per axis (steps_per_frame steps per frame), Poisson photon
// emission per step (rate cps), each photon displaced by the Gaussian PSF
// (sigma = 1/e^2 radius / 2) and counted in the pixel it lands in, optional
// irreversible bleaching with time constant tau, camera offset plus Gaussian
// read noise.  The random streams are counter-based (splitmix64 per particle),
// so a seed gives the same stack on every run.
#include <math.h>

#include "imfcs_gb300.h"
#include "imfcs_host.h"

namespace imfcs {

struct SimState {
    float x, y;
    uint32_t bleached;
    uint32_t species;
    uint64_t rng;
};

__device__ __forceinline__ uint64_t splitmix(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ float urand(uint64_t &s)
{
    return ((splitmix(s) >> 40) + 0.5f) * (1.0f / 16777216.0f);   // (0, 1)
}
__device__ __forceinline__ void nrand2(uint64_t &s, float &a, float &b)
{
    float u1 = urand(s), u2 = urand(s);
    float r = sqrtf(-2.f * logf(u1));
    float sn, cs;
    sincospif(2.f * u2, &sn, &cs);
    a = r * cs;
    b = r * sn;
}
__device__ __forceinline__ int poisson_small(uint64_t &s, float lambda)
{
    if (lambda > 30.f) {
        float a, b;
        nrand2(s, a, b);
        int k = (int)lrintf(lambda + sqrtf(lambda) * a);
        return k < 0 ? 0 : k;
    }
    float L = __expf(-lambda), p = 1.f;
    int k = 0;
    do { k++; p *= urand(s); } while (p > L && k < 1000);
    return k - 1;
}

struct SimArgs {
    int w, h, frames, steps;
    float dt_step, pixel, sig_psf, lx, ly, margin;
    float d1, d2, photons_per_step, bleach_p;
    int nparticles;
    const float *dmap;  // per 16x16 tile, or nullptr
    int tiles_x, tiles_y;
};

__global__ void sim_init_kernel(SimArgs a, SimState *st, uint64_t seed, float fraction2)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nparticles) return;
    uint64_t s = seed ^ (0xD1B54A32D192ED03ull * (uint64_t)(i + 1));
    splitmix(s);
    SimState p;
    p.x = urand(s) * a.lx;
    p.y = urand(s) * a.ly;
    p.bleached = 0;
    p.species = urand(s) < fraction2 ? 1u : 0u;
    p.rng = s;
    st[i] = p;
}

__global__ void sim_frames_kernel(SimArgs a, SimState *st, int f0, int nf, unsigned int *counts)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nparticles) return;
    SimState p = st[i];
    const float inv_px = 1.f / a.pixel;
    for (int f = 0; f < nf; f++) {
        unsigned int *cf = counts + (size_t)f * a.w * a.h;
        for (int k = 0; k < a.steps; k++) {
            float d = p.species ? a.d2 : a.d1;
            if (a.dmap) {
                int tx = (int)floorf((p.x - a.margin) * inv_px) / 16, ty = (int)floorf((p.y - a.margin) * inv_px) / 16;
                tx = min(max(tx, 0), a.tiles_x - 1);
                ty = min(max(ty, 0), a.tiles_y - 1);
                d = a.dmap[ty * a.tiles_x + tx];
            }
            float sd = sqrtf(2.f * d * a.dt_step), g1, g2;
            nrand2(p.rng, g1, g2);
            p.x += sd * g1;
            p.y += sd * g2;
            p.x -= a.lx * floorf(p.x / a.lx);
            p.y -= a.ly * floorf(p.y / a.ly);
            if (a.bleach_p > 0.f && !p.bleached && urand(p.rng) < a.bleach_p) p.bleached = 1;
            if (p.bleached) continue;
            int nph = poisson_small(p.rng, a.photons_per_step);
            for (int q = 0; q < nph; q += 2) {
                float e1, e2;
                nrand2(p.rng, e1, e2);
                for (int r = 0; r < 2 && q + r < nph; r++) {
                    float ex = p.x + a.sig_psf * (r ? e2 : e1);
                    float e3, e4;
                    nrand2(p.rng, e3, e4);
                    float ey = p.y + a.sig_psf * e3;
                    int px = (int)floorf((ex - a.margin) * inv_px);
                    int py = (int)floorf((ey - a.margin) * inv_px);
                    if (px >= 0 && px < a.w && py >= 0 && py < a.h) atomicAdd(&cf[py * a.w + px], 1u);
                }
            }
        }
    }
    st[i] = p;
}

__global__ void sim_camera_kernel(const unsigned int *counts, uint16_t *out, size_t n, size_t base,
                                  int offset, float read_noise, uint64_t seed)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v = (float)counts[i] + (float)offset;
    if (read_noise > 0.f) {
        uint64_t s = seed ^ (0x9E3779B97F4A7C15ull * (base + i + 1));
        float a, b;
        nrand2(s, a, b);
        v += read_noise * a;
    }
    v = rintf(v);
    v = fminf(fmaxf(v, 0.f), 65535.f);
    out[i] = (uint16_t)v;
}

}  // namespace imfcs

using namespace imfcs;

extern "C" int imfcs_simulate(const imfcs_sim_params *sp, const float *dev_d_tile_map, uint16_t *dev_stack,
                              void *stream)
{
    if (!sp || !dev_stack || sp->width <= 0 || sp->height <= 0 || sp->frames <= 0 ||
        sp->steps_per_frame <= 0 || !(sp->pixel_size > 0) || !(sp->frametime > 0)) {
        set_error("invalid simulation parameters");
        return 1;
    }
    cudaStream_t s = (cudaStream_t)stream;
    SimArgs a;
    a.w = sp->width;
    a.h = sp->height;
    a.frames = sp->frames;
    a.steps = sp->steps_per_frame;
    a.dt_step = (float)(sp->frametime / sp->steps_per_frame);
    a.pixel = (float)sp->pixel_size;
    a.sig_psf = (float)(sp->psf_radius / 2.0);
    a.margin = (float)sp->margin;
    a.lx = (float)(sp->width * sp->pixel_size + 2 * sp->margin);
    a.ly = (float)(sp->height * sp->pixel_size + 2 * sp->margin);
    a.d1 = (float)sp->d1;
    a.d2 = (float)sp->d2;
    a.photons_per_step = (float)(sp->cps * a.dt_step);
    a.bleach_p = sp->tau_bleach > 0 ? (float)(1.0 - exp(-(double)a.dt_step / sp->tau_bleach)) : 0.f;
    a.nparticles = (int)lround(sp->density * a.lx * a.ly);
    if (a.nparticles < 1) a.nparticles = 1;
    a.dmap = dev_d_tile_map;
    a.tiles_x = (sp->width + 15) / 16;
    a.tiles_y = (sp->height + 15) / 16;
    SimState *st = nullptr;
    unsigned int *counts = nullptr;
    const int chunk = 256;
    const size_t fsz = (size_t)sp->width * sp->height;
    cudaError_t e = cudaMalloc(&st, sizeof(SimState) * a.nparticles);
    if (e == cudaSuccess) e = cudaMalloc(&counts, sizeof(unsigned int) * fsz * chunk);
    if (e != cudaSuccess) {
        cudaFree(st);
        set_error(cuda_msg(e, "simulator allocation"));
        return 1;
    }
    int tb = 128;
    sim_init_kernel<<<(a.nparticles + tb - 1) / tb, tb, 0, s>>>(a, st, sp->seed, (float)sp->fraction2);
    for (int f0 = 0; f0 < sp->frames && e == cudaSuccess; f0 += chunk) {
        int nf = sp->frames - f0 < chunk ? sp->frames - f0 : chunk;
        e = cudaMemsetAsync(counts, 0, sizeof(unsigned int) * fsz * nf, s);
        if (e != cudaSuccess) break;
        sim_frames_kernel<<<(a.nparticles + tb - 1) / tb, tb, 0, s>>>(a, st, f0, nf, counts);
        size_t n = fsz * nf;
        sim_camera_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(counts, dev_stack + fsz * f0, n, fsz * f0,
                                                                     sp->offset, (float)sp->read_noise,
                                                                     sp->seed * 31 + 7);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(st);
    cudaFree(counts);
    if (e != cudaSuccess) { set_error(cuda_msg(e, "simulator")); return 1; }
    return 0;
}
