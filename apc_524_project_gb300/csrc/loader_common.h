// loader_common.h - deterministic, platform-independent particle sampling.
//
// The same inline code runs on the host (C++) and on the device (CUDA), so a
// species loaded on the GPU is bit-identical to the arrays generated on the
// host for the CPU oracle. Only IEEE-754 add, multiply, divide, sqrt, frexp
// and ldexp are used, always separately rounded (host: -ffp-contract=off,
// device: --fmad=false), so x86-64 and aarch64 hosts and the GPU agree.
//
// Per particle p of species s the random stream is a SplitMix64 sequence
// seeded from (seed, s, p); positions are uniform in the box (optionally with
// a cosine density modulation along x by rejection), velocities are Maxwellian
// by Marsaglia's polar method. This replaces the reference's Numerical Recipes
// ran2 + Box-Muller loader (src/particles/particle_handler.cpp:47-84,
// src/utils/RNG.cpp:68-141), whose sequential state cannot be split across
// GPU threads; the distributions are the same.
#ifndef EMOO_LOADER_COMMON_H
#define EMOO_LOADER_COMMON_H

#include <stdint.h>
#include <math.h>

#include "emoo.h"

#ifdef __CUDACC__
#define EMOO_HD __host__ __device__ __forceinline__
#else
#define EMOO_HD static inline
#endif

EMOO_HD uint64_t emoo_splitmix(uint64_t *s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// Uniform double in [0, 1) with 53 random bits.
EMOO_HD double emoo_uniform(uint64_t *s) { return (double)(emoo_splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

EMOO_HD uint64_t emoo_stream_seed(uint64_t seed, int species, int64_t p) {
    uint64_t s = seed ^ (0xD1B54A32D192ED03ULL * (uint64_t)(species + 1));
    uint64_t t = s + 0x9E3779B97F4A7C15ULL * (uint64_t)p;
    (void)emoo_splitmix(&t);
    return t;
}

// Natural log for x > 0 from basic operations: x = m 2^e with m in
// [1/sqrt2, sqrt2), log m = 2 atanh(u), u = (m-1)/(m+1), |u| < 0.172, by its
// odd power series (12 terms, truncation < 1e-19 relative).
EMOO_HD double emoo_log(double x) {
    int e;
    double m = frexp(x, &e);  // m in [0.5, 1)
    if (m < 0.70710678118654752440) {
        m = m * 2.0;
        e = e - 1;
    }
    double u = (m - 1.0) / (m + 1.0);
    double u2 = u * u;
    double term = u, sum = 0.0;
    for (int k = 0; k < 12; k++) {
        sum = sum + term / (double)(2 * k + 1);
        term = term * u2;
    }
    const double ln2_hi = 6.93147180369123816490e-01;  // high bits of ln 2
    const double ln2_lo = 1.90821492927058770002e-10;  // ln 2 - ln2_hi
    return (double)e * ln2_hi + ((double)e * ln2_lo + 2.0 * sum);
}

// cos(2 pi f) for any finite f, from basic operations: reduce f to [0, 1),
// fold by symmetry to an angle in [0, pi/4] and sum Taylor series.
EMOO_HD double emoo_cos2pi(double f) {
    f = f - floor(f);                  // [0,1)
    double g = f > 0.5 ? 1.0 - f : f;  // cos symmetric: [0, 0.5]
    double sgn = 1.0;
    if (g > 0.25) {  // cos(2pi g) = -cos(2pi (0.5-g))
        g = 0.5 - g;
        sgn = -1.0;
    }
    // g in [0, 0.25]; use sin for g > 0.125: cos(2 pi g) = sin(2 pi (0.25 - g))
    const double twopi = 6.28318530717958647692;
    int use_sin = g > 0.125;
    double a = use_sin ? twopi * (0.25 - g) : twopi * g;  // [0, pi/4]
    double a2 = a * a;
    double term, sum;
    if (use_sin) {
        term = a;
        sum = 0.0;
        for (int k = 0; k < 11; k++) {
            sum = sum + term;
            term = -term * a2 / (double)((2 * k + 2) * (2 * k + 3));
        }
    } else {
        term = 1.0;
        sum = 0.0;
        for (int k = 0; k < 11; k++) {
            sum = sum + term;
            term = -term * a2 / (double)((2 * k + 1) * (2 * k + 2));
        }
    }
    return sgn * sum;
}

// Two independent standard normals (Marsaglia polar method).
EMOO_HD void emoo_normal2(uint64_t *s, double *z0, double *z1) {
    double u1, u2, r;
    do {
        u1 = 2.0 * emoo_uniform(s) - 1.0;
        u2 = 2.0 * emoo_uniform(s) - 1.0;
        r = u1 * u1 + u2 * u2;
    } while (r >= 1.0 || r == 0.0);
    double f = sqrt(-2.0 * emoo_log(r) / r);
    *z0 = u1 * f;
    *z1 = u2 * f;
}

// Samples particle p of the species into out[7] = {x, y, z, vx, vy, vz, gamma}.
EMOO_HD void emoo_sample_particle(const emoo_gen_params *g, int64_t p, double *out) {
    uint64_t s = emoo_stream_seed(g->seed, g->species, p);
    double x;
    if (g->dens_amp != 0.0) {
        double amax = 1.0 + fabs(g->dens_amp);
        for (;;) {
            double ux = emoo_uniform(&s);
            double ua = emoo_uniform(&s);
            double w = 1.0 + g->dens_amp * emoo_cos2pi(g->dens_k * ux);
            if (ua * amax < w) {
                x = ux;
                break;
            }
        }
    } else {
        x = emoo_uniform(&s);
    }
    double y = emoo_uniform(&s);
    double z = emoo_uniform(&s);
    out[0] = x * g->L[0] + g->x0[0];
    out[1] = y * g->L[1] + g->x0[1];
    out[2] = z * g->L[2] + g->x0[2];
    double n0, n1, n2, n3;
    emoo_normal2(&s, &n0, &n1);
    emoo_normal2(&s, &n2, &n3);
    (void)n3;
    out[3] = g->vdrift[0] + g->vth[0] * n0;
    out[4] = g->vdrift[1] + g->vth[1] * n1;
    out[5] = g->vdrift[2] + g->vth[2] * n2;
    if (g->relativistic_gamma)
        out[6] = sqrt(1 - out[3] * out[3] - out[4] * out[4] - out[5] * out[5]);
    else
        out[6] = 0.0;
}

#endif
