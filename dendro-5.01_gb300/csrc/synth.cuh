// Seeded synthetic initial data shared by host and device code.
//
// Brill-Lindquist two-puncture data, the zero-momentum / zero-spin case of
// the reference's punctureData (BSSN_GR/src/grUtils.cpp:398-712):
//   psi = 1 + sum_i m_i / (2 r_i),  chi = psi^-4,  alpha = psi^-2,
//   gt = delta,  K = At = Gt = beta = B = 0,  chi, alpha >= chi_floor,
// masses 0.5 at (+-1, 0, 0.00123) (the z offset keeps grid points off the
// punctures, as BSSN_GR/pars/bbh.par.json does), plus U(-1,1)*noise on every
// field from a counter-based SplitMix64 keyed by (seed, block, var, point).
//
// Every operation is an IEEE-rounded add/sub/mul/div/sqrt with no
// contraction (device: explicit _rn intrinsics; host: -ffp-contract=off), so
// the host and device fills are bit-identical.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define DGB_HD __host__ __device__ __forceinline__
#else
#define DGB_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define SY_ADD(a, b) __dadd_rn((a), (b))
#define SY_SUB(a, b) __dsub_rn((a), (b))
#define SY_MUL(a, b) __dmul_rn((a), (b))
#define SY_DIV(a, b) __ddiv_rn((a), (b))
#define SY_SQRT(a) __dsqrt_rn((a))
#else
#include <math.h>
#define SY_ADD(a, b) ((a) + (b))
#define SY_SUB(a, b) ((a) - (b))
#define SY_MUL(a, b) ((a) * (b))
#define SY_DIV(a, b) ((a) / (b))
#define SY_SQRT(a) sqrt((a))
#endif

#define DGB_SYNTH_CHI_FLOOR 1e-4
#define DGB_SYNTH_PUNCTURE_Z 0.00123

DGB_HD uint64_t dgb_mix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Uniform in [-1, 1) from the counter (seed, block, var, point).
DGB_HD double dgb_noise_unit(uint64_t key_bv, uint64_t point)
{
    const uint64_t r = dgb_mix64(key_bv ^ dgb_mix64(point));
    const double u = (double)(r >> 11) * (1.0 / 9007199254740992.0);  // [0,1)
    return SY_SUB(SY_MUL(2.0, u), 1.0);
}

DGB_HD uint64_t dgb_noise_key(uint64_t seed, uint64_t block, uint32_t var)
{
    return dgb_mix64(dgb_mix64(seed ^ 0xD1B54A32D192ED03ull) ^ (block * 64u + var));
}

// Noise-free Brill-Lindquist value of variable v at (x,y,z).
DGB_HD double dgb_bl_value(int v, double x, double y, double z)
{
    if (v == 0 || v == 1) {  // alpha, chi
        const double zz = SY_SUB(z, DGB_SYNTH_PUNCTURE_Z);
        const double dx1 = SY_SUB(x, 1.0), dx2 = SY_ADD(x, 1.0);
        const double yz = SY_ADD(SY_MUL(y, y), SY_MUL(zz, zz));
        const double r1 = SY_SQRT(SY_ADD(SY_MUL(dx1, dx1), yz));
        const double r2 = SY_SQRT(SY_ADD(SY_MUL(dx2, dx2), yz));
        const double psi = SY_ADD(SY_ADD(1.0, SY_DIV(0.5, SY_MUL(2.0, r1))),
                                  SY_DIV(0.5, SY_MUL(2.0, r2)));
        const double psi2 = SY_MUL(psi, psi);
        double f = (v == 0) ? SY_DIV(1.0, psi2) : SY_DIV(1.0, SY_MUL(psi2, psi2));
        return f < DGB_SYNTH_CHI_FLOOR ? DGB_SYNTH_CHI_FLOOR : f;
    }
    // gt00, gt11, gt22 = 1
    if (v == 12 || v == 15 || v == 17) return 1.0;
    return 0.0;
}

// Field value at padded point (i,j,k) of a block with corner pmin and
// spacing h (x = pmin + i*h, the coordinate convention of
// BSSN_GR/src/rhs.cpp:210-216).
DGB_HD double dgb_synth_value(int v, uint64_t key_bv, uint64_t point, int i, int j, int k,
                              const double *pmin, const double *h, double noise)
{
    const double x = SY_ADD(pmin[0], SY_MUL((double)i, h[0]));
    const double y = SY_ADD(pmin[1], SY_MUL((double)j, h[1]));
    const double z = SY_ADD(pmin[2], SY_MUL((double)k, h[2]));
    const double base = dgb_bl_value(v, x, y, z);
    return SY_ADD(base, SY_MUL(noise, dgb_noise_unit(key_bv, point)));
}
