// rng_math.cuh -- counter-based random numbers and the FP32 math of the sweep kernels.
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) replaces libgfortran's random_number
// (src/get_random_num.f90:29).  Every draw is addressed by
//     key     = (seed, 0x45544852)                            the same for a whole launch
//     counter = (c0, t, stream, purpose | colour << 8 | block << 16)
// where stream identifies the replica.  A draw depends only on (replica, sweep, site),
// never on thread scheduling, and because the key is launch-uniform its round schedule is
// computed once per warp in the uniform datapath instead of in every thread's registers.
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
constexpr uint32_t kKey1 = 0x45544852u;

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
        // one 32x32->64 multiply each (a single wide multiply on the GPU)
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0; c1 = (uint32_t)p1; c2 = n2; c3 = (uint32_t)p0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    return U4{c0, c1, c2, c3};
}

ETHER_HD U4 draw(uint32_t c0, uint32_t t, uint32_t stream, uint32_t tag, uint32_t seed) {
    return philox(c0, t, stream, tag, seed, kKey1);
}

// The ten round keys of the first key word, (seed + r * 0x9E3779B9).  Passed to the hottest
// kernel as a by-value parameter, so each round XORs with a constant-bank operand instead of
// recomputing the schedule per thread; the second key word's schedule is a compile-time
// constant.  Same numbers as draw().
struct RoundKeys {
    uint32_t k[10];
};
ETHER_HD RoundKeys round_keys(uint32_t seed) {
    RoundKeys K;
    for (int r = 0; r < 10; ++r) K.k[r] = seed + (uint32_t)r * 0x9E3779B9u;
    return K;
}
ETHER_HD U4 draw_rk(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, const RoundKeys &K) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ K.k[r];
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ (kKey1 + (uint32_t)r * 0xBB67AE85u);
        c0 = n0; c1 = (uint32_t)p1; c2 = n2; c3 = (uint32_t)p0;
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
    const bool tiny = x < -87.0f;  // a select, not an early return: no divergent exit
    x = tiny ? 0.0f : x;
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
    return tiny ? 0x1p-126f : p * bits_f((uint32_t)((int)n + 127) << 23);
}

// log x for a positive normal x: x = m 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s),
// s = (m - 1)/(m + 1), series through s^9 (|s| < 0.172: truncation < 1e-9).
ETHER_HD float logf_own(float x) {
#if defined(__CUDA_ARCH__)
    uint32_t u = __float_as_uint(x);
#else
    uint32_t u;
    __builtin_memcpy(&u, &x, 4);
#endif
    int e = (int)((u >> 23) & 0xFFu) - 127;
    float m = bits_f((u & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = 0.111111111f;
    p = fmaf(p, s2, 0.142857143f);
    p = fmaf(p, s2, 0.2f);
    p = fmaf(p, s2, 0.333333333f);
    p = fmaf(p, s2, 1.0f);
    const float lm = 2.0f * (s * p);
    return fmaf((float)e, 0.693147182f, lm);
}

// log(1 - y) for y in [0, 1) without cancellation: for y < 1/2, 2 atanh(s) with
// s = -y / (2 - y) (|s| <= 1/3, series through s^15: truncation < 1e-9); else the log of
// 1 - y, which is exact there.
ETHER_HD float log1m_own(float y) {
    if (y >= 0.5f) return logf_own(1.0f - y);
    const float s = -y / (2.0f - y);
    const float s2 = s * s;
    float p = 0.0666666667f;
    p = fmaf(p, s2, 0.0769230769f);
    p = fmaf(p, s2, 0.0909090909f);
    p = fmaf(p, s2, 0.111111111f);
    p = fmaf(p, s2, 0.142857143f);
    p = fmaf(p, s2, 0.2f);
    p = fmaf(p, s2, 0.333333333f);
    p = fmaf(p, s2, 1.0f);
    return 2.0f * (s * p);
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

// Proposal of update_spin_details (src/update_spin_details.f90:30-51) in FP32: Marsaglia
// (George_Marsaglia.f90:29-39) or ANGLE.  The reference then divides by the norm
// (update_spin_details.f90:50-51).  Both proposals are unit vectors by construction
// (4s(1-s) + (1-2s)^2 = 1; (1-z^2)(cos^2 + sin^2) + z^2 = 1), so in FP32 that division only
// moves the components by a few units in the last place; it is left out here and in the
// FP32 mirror (the FP64 replay keeps it).  A proposal replaces the spin whole, so the length
// error does not accumulate.  The Marsaglia pairs come in
// order p = 0, 1, 2, ...: pair 0 is words 1,2 of block 0 (word 0 is eta); pair p >= 1 is
// block (p+1)/2, words 0,1 for odd p and 2,3 for even p.  The first accepted pair wins.
// Blocks 0 and 1 (pairs 0-2, 99% of sites) are drawn by the caller and chosen among with
// selects, so every lane runs the same instructions; later pairs come from one loop taken
// by ~1% of sites, after which the lanes reconverge.  Returns false if 64 pairs were all
// rejected (probability ~1e-43): no proposal.
struct Spin4 { float x, y, z, w; };

ETHER_HD bool marsaglia(uint32_t c0, uint32_t t, uint32_t stream, uint32_t tag, const RoundKeys &K,
                        const U4 &b0, const U4 &b1, float *v1o, float *v2o, float *so) {
    const float a0 = upm1(b0.y), a1 = upm1(b0.z);
    const float c0a = upm1(b1.x), c1a = upm1(b1.y);
    const float d0 = upm1(b1.z), d1 = upm1(b1.w);
    const float s0 = a0 * a0 + a1 * a1, s1 = c0a * c0a + c1a * c1a, s2 = d0 * d0 + d1 * d1;
    const bool k0 = s0 < 1.0f, k1 = s1 < 1.0f, k2 = s2 < 1.0f;
    float v1 = k0 ? a0 : (k1 ? c0a : d0);
    float v2 = k0 ? a1 : (k1 ? c1a : d1);
    float s = k0 ? s0 : (k1 ? s1 : s2);
    bool ok = k0 || k1 || k2;
    if (!ok) {
        for (int blk = 2; blk <= kMarsagliaMaxPairs / 2 && !ok; ++blk) {
            const U4 o = draw_rk(c0, t, stream, tag | ((uint32_t)blk << 16), K);
            float w1 = upm1(o.x), w2 = upm1(o.y), q = w1 * w1 + w2 * w2;
            if (q < 1.0f) {
                v1 = w1; v2 = w2; s = q; ok = true;
            } else if (2 * blk != kMarsagliaMaxPairs) {
                w1 = upm1(o.z); w2 = upm1(o.w); q = w1 * w1 + w2 * w2;
                if (q < 1.0f) { v1 = w1; v2 = w2; s = q; ok = true; }
            }
        }
    }
    *v1o = v1; *v2o = v2; *so = s;
    return ok;
}

// b0, b1: blocks 0 and 1 of the site's draw (block 1 is used by Marsaglia only).
ETHER_HD bool propose(bool angle, float dphi, const Spin4 &S, uint32_t c0, uint32_t t,
                      uint32_t stream, uint32_t tag, const RoundKeys &K, const U4 &b0, const U4 &b1,
                      Spin4 *out) {
    float nx, ny, nz, nphi;
    if (!angle) {
        float v1, v2, s;
        if (!marsaglia(c0, t, stream, tag, K, b0, b1, &v1, &v2, &s)) return false;
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
    out->x = nx;
    out->y = ny;
    out->z = nz;
    out->w = nphi;
    return true;
}

}  // namespace ether
