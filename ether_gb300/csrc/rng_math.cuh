// rng_math.cuh -- counter-based random numbers and the FP32 math of the sweep kernels.
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) replaces libgfortran's random_number
// (src/get_random_num.f90:29).  Every draw is addressed by
//     key     = (seed, stream)                    stream = per replica
//     counter = (c0, t, c2, purpose | colour << 8)
// so a draw depends only on (replica, sweep, site), never on thread scheduling.
//
// The kernels are compiled with --fmad=false: every + and * rounds on its own, and the
// only fused multiply-adds are the explicit fmaf() calls below.  The FP32 results are
// therefore reproducible operation by operation on any IEEE machine.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define ETHER_HD __host__ __device__ __forceinline__
#else
#define ETHER_HD inline
#endif

namespace ether {

enum Purpose : uint32_t { kMetro = 0, kOvrr = 1, kFresh = 2, kPT = 3 };

struct U4 { uint32_t x, y, z, w; };

ETHER_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

ETHER_HD U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                   uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = mulhi32(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = mulhi32(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    return U4{c0, c1, c2, c3};
}

// Philox with the ten round keys precomputed once (the key is fixed per replica), so a
// block costs two 32x32->64 multiplies and two three-input XORs per round.
struct Keys {
    uint32_t a[10], b[10];
};
ETHER_HD Keys key_schedule(uint32_t k0, uint32_t k1) {
    Keys K;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        K.a[r] = k0;
        K.b[r] = k1;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return K;
}
ETHER_HD U4 philox_k(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, const Keys &K) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = mulhi32(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = mulhi32(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ K.a[r], n2 = hi0 ^ c3 ^ K.b[r];
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    return U4{c0, c1, c2, c3};
}

// u32 -> [0,1) with 24 bits, and u32 -> [-1,1) with 24 bits (both exact in FP32).
ETHER_HD float u01(uint32_t u) { return (float)(u >> 8) * 0x1p-24f; }
ETHER_HD float upm1(uint32_t u) { return (float)(u >> 8) * 0x1p-23f - 1.0f; }

ETHER_HD float bits_f(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float f;
    __builtin_memcpy(&f, &b, 4);
    return f;
#endif
}

// e^x for x <= 0.  Cody-Waite reduction x = n ln2 + r with a two-part ln2, degree-7
// Taylor polynomial of e^r (|r| <= ln2/2) in Horner form, times 2^n built from exponent
// bits.  Below -87 the result is the smallest normal float: a uniform eta = 0 (log eta =
// -inf in the reference's test) is still accepted, any larger eta is rejected.
ETHER_HD float expf_neg(float x) {
    if (x < -87.0f) return 0x1p-126f;
    float n = rintf(x * 1.44269502f);
    float r = x - n * 0.693359375f;
    r = r - n * -2.12194440e-4f;
    float p = 1.98412698e-4f;
    p = fmaf(p, r, 1.38888889e-3f);
    p = fmaf(p, r, 8.33333333e-3f);
    p = fmaf(p, r, 4.16666667e-2f);
    p = fmaf(p, r, 1.66666667e-1f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    return p * bits_f((uint32_t)((int)n + 127) << 23);
}

// sin and cos for |x| <= 4: reduction by pi/2 (two-part constant), Taylor polynomials on
// |r| <= pi/4 (sine through r^9, cosine through r^8), quadrant swap.
ETHER_HD void sincos_own(float x, float *s, float *c) {
    float q = rintf(x * 0.636619772f);
    float r = x - q * 1.5703125f;
    r = r - q * 4.83826792e-4f;
    float r2 = r * r;
    float sp = 2.75573192e-6f;
    sp = fmaf(sp, r2, -1.98412698e-4f);
    sp = fmaf(sp, r2, 8.33333333e-3f);
    sp = fmaf(sp, r2, -1.66666667e-1f);
    float r3 = r * r2;
    float sn = fmaf(r3, sp, r);
    float cp = 2.48015873e-5f;
    cp = fmaf(cp, r2, -1.38888889e-3f);
    cp = fmaf(cp, r2, 4.16666667e-2f);
    cp = fmaf(cp, r2, -0.5f);
    float cs = fmaf(cp, r2, 1.0f);
    int iq = ((int)q) & 3;
    if (iq == 0) { *s = sn; *c = cs; }
    else if (iq == 1) { *s = cs; *c = -sn; }
    else if (iq == 2) { *s = -sn; *c = -cs; }
    else { *s = -cs; *c = sn; }
}

constexpr float kPiF = 3.14159274f;
constexpr float kTwoPiF = 6.28318548f;
constexpr int kMarsagliaMaxPairs = 64;

// Pair p of a Metropolis proposal: p = 0 uses words 1,2 of block 0 (word 0 is eta);
// p >= 1 uses block (p+1)/2, words 0,1 for odd p and 2,3 for even p.
ETHER_HD void metro_pair(uint32_t c0, uint32_t t, uint32_t c3, uint32_t k0, uint32_t k1,
                         const U4 &b0, int p, uint32_t *a, uint32_t *b) {
    if (p == 0) { *a = b0.y; *b = b0.z; return; }
    U4 o = philox(c0, t, (uint32_t)((p + 1) / 2), c3, k0, k1);
    if (p & 1) { *a = o.x; *b = o.y; } else { *a = o.z; *b = o.w; }
}

// Proposal of update_spin_details (src/update_spin_details.f90:30-51) in FP32.
// Marsaglia (George_Marsaglia.f90:29-39) or ANGLE, then normalisation.  Returns false if
// 64 Marsaglia pairs were all rejected (probability ~1e-43): the site keeps its spin.
struct Spin4 { float x, y, z, w; };

ETHER_HD bool propose(bool angle, float dphi, const Spin4 &S, uint32_t c0, uint32_t t,
                      uint32_t c3, uint32_t k0, uint32_t k1, const U4 &b0, Spin4 *out) {
    float nx, ny, nz, nphi;
    if (!angle) {
        float v1 = 0.f, v2 = 0.f, s = 0.f;
        bool ok = false;
        for (int p = 0; p < kMarsagliaMaxPairs; ++p) {
            uint32_t a, b;
            metro_pair(c0, t, c3, k0, k1, b0, p, &a, &b);
            v1 = upm1(a);
            v2 = upm1(b);
            s = v1 * v1 + v2 * v2;
            if (s < 1.0f) { ok = true; break; }
        }
        if (!ok) return false;
        float tq = sqrtf(1.0f - s);
        nx = (2.0f * v1) * tq;
        ny = (2.0f * v2) * tq;
        nz = 1.0f - 2.0f * s;
        nphi = 0.0f;
    } else {
        nz = upm1(b0.y);
        nphi = S.w + dphi * upm1(b0.z);
        if (nphi >= kPiF) nphi = nphi - kTwoPiF;
        else if (nphi < -kPiF) nphi = nphi + kTwoPiF;
        float r = sqrtf(1.0f - nz * nz);
        float sn, cs;
        sincos_own(nphi, &sn, &cs);
        nx = r * cs;
        ny = r * sn;
    }
    float inv = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
    out->x = nx * inv;
    out->y = ny * inv;
    out->z = nz * inv;
    out->w = nphi;
    return true;
}

}  // namespace ether
