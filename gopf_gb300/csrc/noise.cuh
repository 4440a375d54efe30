// noise.cuh -- counter-based Gaussian noise in k space (pf/noise.go).
//
// The reference draws real-space white noise N(0, 2S) per cell and step from
// Go's global math/rand (WhiteNoise.Generate, pf/noise.go:20-23), FFTs it as
// a derived field, and ConservativeNoise (pf/noise.go:60-99) combines D such
// fields as sum_d 2i sin(pi f_d) j_d(k), skipping |f_d| = 1/2.  The FFT of
// real white noise of variance s2 over N cells is a Hermitian complex
// Gaussian field with E|x(k)|^2 = N s2: independent complex values off the
// self-conjugate planes, conjugate pairs on them and real values at
// self-conjugate points.  The device draws that field directly in k space,
// keyed on (seed, step, canonical mode, component) with Philox-4x32-10
// (Salmon, Moraes, Dror & Shaw, SC'11) and the Box-Muller transform, so the
// statistics match the reference's while no real-space noise array exists.
// The noise is checked statistically, not sample for sample.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "gopf_types.h"

namespace gopf {

struct Philox4 {
    uint32_t v[4];
};

__device__ __forceinline__ Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                                  uint32_t k1)
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(M0, c0), lo0 = M0 * c0;
        const uint32_t hi1 = __umulhi(M1, c2), lo1 = M1 * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += W0;
        k1 += W1;
    }
    Philox4 o;
    o.v[0] = c0;
    o.v[1] = c1;
    o.v[2] = c2;
    o.v[3] = c3;
    return o;
}

// two independent standard normals from two 32-bit words (Box-Muller)
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, double &g1, double &g2)
{
    const double u1 = ((double)a + 1.0) * (1.0 / 4294967296.0); // (0, 1]
    const double u2 = (double)b * (1.0 / 4294967296.0);        // [0, 1)
    const double r = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    g1 = r * c;
    g2 = r * s;
}


// fold an index into (-n/2, n/2]
__device__ __forceinline__ long long fold_i(long long i, long long n) { return (2 * i > n) ? i - n : i; }

// Hermitian Gaussian of mode (kx, y, z) of component comp (half spectrum: kx in [0, X/2])
__device__ __forceinline__ void hermitian_gauss(const NoiseParams &np, long long X, long long Y, long long Z, long long kx,
                                                long long y, long long z, int comp, double &re, double &im)
{
    const long long yp = (Y - y) % Y, zp = (Z - z) % Z;
    const bool plane = (kx == 0) || (2 * kx == X);
    bool conj = false;
    long long cy = y, cz = z;
    if (plane) {
        if (yp == y && zp == z) { // self-conjugate point: real, variance N s2
            const unsigned long long st = *np.step;
            const Philox4 r = philox4x32_10((uint32_t)(kx * 4 + comp), (uint32_t)(y + Y * z), (uint32_t)st,
                                            (uint32_t)(st >> 32), np.seed_lo, np.seed_hi);
            double g1, g2;
            box_muller(r.v[0], r.v[1], g1, g2);
            re = np.amp * g1;
            im = 0.0;
            return;
        }
        if (z * Y + y > zp * Y + yp) { // draw from the canonical member of the pair and conjugate
            cy = yp;
            cz = zp;
            conj = true;
        }
    }
    const unsigned long long st = *np.step;
    const Philox4 r =
        philox4x32_10((uint32_t)(kx * 4 + comp), (uint32_t)(cy + Y * cz), (uint32_t)st, (uint32_t)(st >> 32), np.seed_lo,
                      np.seed_hi);
    double g1, g2;
    box_muller(r.v[0], r.v[1], g1, g2);
    const double s = np.amp * 0.70710678118654752440;
    re = s * g1;
    im = conj ? -s * g2 : s * g2;
}

// The noise term's contribution N_noise(k) to the explicit RHS (before dt), as
// complex (re, im).  m = -k^2 for the term's LAP power.
__device__ __forceinline__ void noise_term(const NoiseParams &np, long long X, long long Y, long long Z, long long kx,
                                           long long y, long long z, double mk, double &re, double &im)
{
    re = 0.0;
    im = 0.0;
    if (np.kind == 1) {
        hermitian_gauss(np, X, Y, Z, kx, y, z, 0, re, im);
    } else if (np.kind == 2) {
        // sum_d 2i sin(pi f_d) j_d, skipping |f_d| = 1/2 (pf/noise.go:85-99);
        // reference order f[0] = row (y), f[1] = col (kx), f[2] = depth (z)
        const double f[3] = {(double)fold_i(y, Y) / (double)Y, (double)kx / (double)X,
                             (double)fold_i(z, Z) / (double)Z};
        for (int d = 0; d < np.ndim; ++d) {
            if (fabs(fabs(f[d]) - 0.5) <= 1e-6) continue;
            double jr, ji;
            hermitian_gauss(np, X, Y, Z, kx, y, z, d, jr, ji);
            const double s2 = 2.0 * sinpi(f[d]);
            re += -s2 * ji; // (i * s2) * (jr + i ji)
            im += s2 * jr;
        }
    }
    double fac = np.coef;
    for (int q = 0; q < np.lap; ++q) fac *= mk;
    re *= fac;
    im *= fac;
}

} // namespace gopf
