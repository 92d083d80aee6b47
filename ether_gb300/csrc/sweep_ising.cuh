// sweep_ising.cuh -- device bodies of the Ising Metropolis colour phase
// (src/Metropolis.f90:39-62 with the Ising branch of update_spin_details.f90:34-35 and
// Hamiltonian.f90:34-52), shared by the per-context kernels (k_ising.cu) and the persistent
// batch kernel (k_batch.cu).
//
// Decision: a site flips iff its uniform u32 u <= T, T = max(ceil(2^32 p), 1) - 1 with
// p = exp(-β ΔE) -- the reference's -βΔE > log(η) for η = u 2^-32, η = 0 included.  T comes
// from a per-temperature table indexed by (site type, own spin, up-neighbour counts per
// (shell, neighbour species) group), built in FP64 on the host.
//
// Random numbers: the sites of a colour class are taken in groups of eight (rank >> 3).
// Site k of a group owns halfword k of two Philox blocks: block 0 gives the high 16 bits
// of its u, block 1 the low 16 bits.  Since u <= T  <=>  uh < Th  or  (uh == Th and
// ul <= Tl), block 1 is only evaluated when a high half ties (probability 2^-16): one
// Philox call serves eight site updates, and the decision is still the exact 32-bit one.
#pragma once
#include "internal.h"
#include "rng_math.cuh"

namespace ether {

__device__ __forceinline__ void warp_add_count(unsigned long long *dst, unsigned v) {
    unsigned s = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(dst, (unsigned long long)s);
}

__device__ __forceinline__ uint32_t half_of(const U4 &b, int k) {  // halfword k = 0..7
    const uint32_t w = (k >> 1) == 0 ? b.x : (k >> 1) == 1 ? b.y : (k >> 1) == 2 ? b.z : b.w;
    return (k & 1) ? (w >> 16) : (w & 0xFFFFu);
}

// ------------------------------------------------------------------ general lattice ----
// Neighbours of a colour class in ELL form: entry k of rank rho at k * n_c + rho (coalesced
// across a warp), in the CSR's order, padded to the class's widest site with entries that
// point at the site itself, so the loads are unconditional and only the sum is predicated.
struct IsingEll {
    uint8_t *sp;  // this replica's spins
    int col_off, n_c, width;
    const int32_t *ell, *ews;  // this class's block: neighbour storage index, table stride
    const uint16_t *deg;       // neighbours per storage index
    const uint16_t *itype;
    const int32_t *type_base, *type_half;
    const uint32_t *tb;  // this replica's temperature slot's thresholds
};

// One site: rank rho.  Threshold-table index = sum of stride * up-spin over the neighbours;
// the draw is halfword rho & 7 of the Philox block of group rho >> 3, and on a tie the
// same halfword of the group's second block.  W > 0: the class's ELL width, known at compile
// time (every load of the site issued at once); W = 0: A.width at run time.
template <int W = 0>
__device__ __forceinline__ bool ising_ell_site(const IsingEll &A, int rho, uint32_t t, uint32_t stream,
                                               uint32_t c3, uint32_t seed) {
    const int s = A.col_off + rho;
    const int dg = A.deg[s];
    int idx = 0;
    if constexpr (W > 0) {
        // the neighbours' storage indices, then all their spins, then the index sum
        int nb[W];
#pragma unroll
        for (int k = 0; k < W; ++k) nb[k] = A.ell[k * A.n_c + rho];  // ELL blocks hold < 2^31 entries
        int up[W];
#pragma unroll
        for (int k = 0; k < W; ++k) up[k] = A.sp[nb[k]];
#pragma unroll
        for (int k = 0; k < W; ++k) {
            const int w = A.ews[k * A.n_c + rho];
            if (k < dg) idx += w * up[k];
        }
    } else {
#pragma unroll 6
        for (int k = 0; k < A.width; ++k) {
            const int e = k * A.n_c + rho;
            const int up = A.sp[A.ell[e]];
            const int w = A.ews[e];
            if (k < dg) idx += w * up;
        }
    }
    const int own = A.sp[s];
    const int ty = A.itype[s];
    const uint32_t T = A.tb[A.type_base[ty] + own * A.type_half[ty] + idx];
    const uint32_t g = (uint32_t)rho >> 3;
    const int j = rho & 7;
    const U4 hi = draw(g, t, stream, c3, seed);
    const uint32_t uh = half_of(hi, j), th = T >> 16;
    bool flip = uh < th;
    if (uh == th) {
        const U4 lo = draw(g, t, stream, c3 | (1u << 16), seed);
        flip = half_of(lo, j) <= (T & 0xFFFFu);
    }
    if (flip) A.sp[s] = (uint8_t)(own ^ 1);
    return flip;
}

// ------------------------------------------------------- simple cubic, colour-split ----
// Colour c array: rho = (z*L2 + y)*H + xh, H = L1/2, site x = 2*xh + ((y+z+c)&1).
// All six neighbours live in the other colour's array: same xh in rows (y±1,z), (y,z±1),
// and xh, xh∓1 in row (y,z).  A thread takes W (4, 8 or 16) consecutive bytes of one row
// (W | H): half of a random-number group, one or two.  Byte sums of 0/1 spins never carry
// (max 6); e = n + 7 s (<= 13) is formed for four sites at once; flips are one predicated
// XOR per site and are counted with popc.
template <int W>
struct Vec {
    uint32_t w[W / 4];
};

template <int W>
__device__ __forceinline__ Vec<W> ldv(const uint8_t *p) {
    Vec<W> v;
    if constexpr (W == 4) {
        v.w[0] = *reinterpret_cast<const uint32_t *>(p);
    } else if constexpr (W == 8) {
        uint2 q = *reinterpret_cast<const uint2 *>(p);
        v.w[0] = q.x; v.w[1] = q.y;
    } else {
        uint4 q = *reinterpret_cast<const uint4 *>(p);
        v.w[0] = q.x; v.w[1] = q.y; v.w[2] = q.z; v.w[3] = q.w;
    }
    return v;
}
template <int W>
__device__ __forceinline__ void stv(uint8_t *p, const Vec<W> &v) {
    if constexpr (W == 4) {
        *reinterpret_cast<uint32_t *>(p) = v.w[0];
    } else if constexpr (W == 8) {
        *reinterpret_cast<uint2 *>(p) = make_uint2(v.w[0], v.w[1]);
    } else {
        *reinterpret_cast<uint4 *>(p) = make_uint4(v.w[0], v.w[1], v.w[2], v.w[3]);
    }
}

// Sites of word q (odd: words 1, 3 of the group's blocks) whose high random halves tie with
// their threshold's high half: decided by the low halves (block 1 of the group).  Returns
// the XOR mask of the extra flips.  Kept out of line: it runs for about one vector in 4000
// and must not cost the hot loop registers.
__device__ __noinline__ inline uint32_t resolve_ties(uint32_t grp, uint32_t t, uint32_t stream,
                                                     uint32_t c3, uint32_t seed, int odd,
                                                     uint32_t e4s, const uint32_t *s_th,
                                                     const uint32_t *s_tl) {
    const U4 rh = draw(grp, t, stream, c3, seed);
    const uint32_t ha = odd ? rh.z : rh.x, hb = odd ? rh.w : rh.y;
    const uint32_t h[4] = {ha & 0xFFFFu, ha >> 16, hb & 0xFFFFu, hb >> 16};
    uint32_t tie = 0;
    for (int k = 0; k < 4; ++k)
        if (h[k] == s_th[((e4s >> (8 * k)) & 0xFFu) >> 2]) tie |= 1u << k;
    if (!tie) return 0;
    const U4 rl = draw(grp, t, stream, c3 | (1u << 16), seed);
    const uint32_t la = odd ? rl.z : rl.x, lb = odd ? rl.w : rl.y;
    const uint32_t l[4] = {la & 0xFFFFu, la >> 16, lb & 0xFFFFu, lb >> 16};
    uint32_t m = 0;
    for (int k = 0; k < 4; ++k)
        if (((tie >> k) & 1u) && l[k] <= s_tl[((e4s >> (8 * k)) & 0xFFu) >> 2]) m |= 1u << (8 * k);
    return m;
}

struct IsingSc {
    uint8_t *own_a;       // this replica's array of the updated colour
    const uint8_t *opp;   // ... and of the other colour
    int L1, L2, L3, H;
    FastDiv fH, fL2;
    uint32_t colour;
};

// Word q of a vector: the four sites' threshold byte offsets (4 (n + 7 s)), given the own
// spins s0 and the six neighbour words.
template <int W>
__device__ __forceinline__ uint32_t sc_e4s(const Vec<W> &o0, uint32_t edge, int par, const Vec<W> &a,
                                           const Vec<W> &b, const Vec<W> &c, const Vec<W> &d, int q,
                                           uint32_t s0) {
    constexpr int NW = W / 4;
    uint32_t sh;
    if (par == 0) {  // neighbour x-1 -> xh-1: window shifted up by one byte
        const uint32_t lo = (q == 0) ? (edge << 24) : o0.w[q > 0 ? q - 1 : 0];
        sh = __funnelshift_l(lo, o0.w[q], 8);
    } else {         // neighbour x+1 -> xh+1: window shifted down by one byte
        const uint32_t hi = (q == NW - 1) ? edge : o0.w[q < NW - 1 ? q + 1 : q];
        sh = __funnelshift_r(o0.w[q], hi, 8);
    }
    const uint32_t n = o0.w[q] + sh + a.w[q] + b.w[q] + c.w[q] + d.w[q];
    // bytewise 4*(n + 7 s) <= 52: the byte offsets of the thresholds in s_th
    return (n + (s0 << 3) - s0) << 2;
}

// The update of one W-byte vector (sites rho0 .. rho0+W-1 of the updated colour) from its own
// spins `me` and the six neighbour words of the other colour; returns the new spins and adds
// the flips to the bytewise counts.  A site whose high random half ties with its threshold's
// high half (probability 2^-16) is decided by the low halves: whether any site of the vector
// ties is checked once, and the rare vector with a tie is finished by resolve_ties.
template <int W>
__device__ __forceinline__ Vec<W> ising_sc_update(const Vec<W> &me, const Vec<W> &o0, const Vec<W> &a,
                                                  const Vec<W> &b, const Vec<W> &c, const Vec<W> &d,
                                                  uint32_t edge, int par, int rho0, const uint32_t *s_th,
                                                  const uint32_t *s_tl, uint32_t t, uint32_t stream,
                                                  uint32_t c3, uint32_t seed, const RoundKeys &K,
                                                  uint32_t &cnt) {
    constexpr int NW = W / 4;
    const char *th_bytes = reinterpret_cast<const char *>(s_th);
    Vec<W> out;
    uint32_t e4[NW];
    bool tie = false;
    U4 rh{0, 0, 0, 0};
#pragma unroll
    for (int q = 0; q < NW; ++q) {
        // word q's half of its group's block: q & 1, or for W = 4 the vector's own half
        const int odd = W == 4 ? (rho0 >> 2) & 1 : q & 1;
        if (W == 4 || (q & 1) == 0) rh = draw_rk((uint32_t)((rho0 >> 3) + (q >> 1)), t, stream, c3, K);
        const uint32_t s0 = me.w[q];
        const uint32_t e4s = sc_e4s<W>(o0, edge, par, a, b, c, d, q, s0);
        e4[q] = e4s;
        const uint32_t t0 = *reinterpret_cast<const uint32_t *>(th_bytes + (e4s & 0xFFu));
        const uint32_t t1 = *reinterpret_cast<const uint32_t *>(th_bytes + __byte_perm(e4s, 0, 0x4441));
        const uint32_t t2 = *reinterpret_cast<const uint32_t *>(th_bytes + __byte_perm(e4s, 0, 0x4442));
        const uint32_t t3 = *reinterpret_cast<const uint32_t *>(th_bytes + (e4s >> 24));
        const uint32_t wa = odd ? rh.z : rh.x, wb = odd ? rh.w : rh.y;
        const uint32_t u0 = wa & 0xFFFFu, u1 = wa >> 16, u2 = wb & 0xFFFFu, u3 = wb >> 16;
        uint32_t m = 0;
        if (u0 < t0) m |= 0x00000001u;
        if (u1 < t1) m |= 0x00000100u;
        if (u2 < t2) m |= 0x00010000u;
        if (u3 < t3) m |= 0x01000000u;
        tie |= (u0 == t0) | (u1 == t1) | (u2 == t2) | (u3 == t3);
        out.w[q] = s0 ^ m;
        cnt += m;
    }
    if (tie) {
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            const uint32_t m = resolve_ties((uint32_t)((rho0 >> 3) + (q >> 1)), t, stream, c3, seed,
                                            W == 4 ? (rho0 >> 2) & 1 : q & 1, e4[q], s_th, s_tl);
            out.w[q] ^= m;
            cnt += m;
        }
    }
    return out;
}

// VPT vectors of W bytes per thread, vector indices vfirst + j*vstride (j < VPT, < nvec),
// one after another, loaded from global memory.  s_th / s_tl: the 14 thresholds' high / low
// halves in shared memory.  Returns the flips as bytewise counts (each byte <= NW VPT).
template <int W, int VPT>
__device__ __forceinline__ uint32_t ising_sc_vectors(const IsingSc &A, int vfirst, int vstride,
                                                     int nvec, const uint32_t *s_th,
                                                     const uint32_t *s_tl, uint32_t t,
                                                     uint32_t stream, uint32_t c3, uint32_t seed,
                                                     const RoundKeys &K) {
    static_assert(W == 4 || W == 8 || W == 16, "vector of half, one or two random-number groups");
    const int H = A.H, L2 = A.L2, L3 = A.L3;
    uint32_t cnt = 0;
#pragma unroll
    for (int j = 0; j < VPT; ++j) {
        const int v = vfirst + j * vstride;
        if (v >= nvec) break;
        const int rho0 = v * W;
        const int row = (int)fdiv((uint32_t)rho0, A.fH);
        const int xh0 = rho0 - row * H;
        const int z = (int)fdiv((uint32_t)row, A.fL2);
        const int y = row - z * L2;
        const int par = (y + z + (int)A.colour) & 1;
        const int ym = (y == 0 ? L2 - 1 : y - 1), yp = (y == L2 - 1 ? 0 : y + 1);
        const int zm = (z == 0 ? L3 - 1 : z - 1), zp = (z == L3 - 1 ? 0 : z + 1);
        const Vec<W> me = ldv<W>(A.own_a + rho0);
        const Vec<W> o0 = ldv<W>(A.opp + rho0);
        const Vec<W> a = ldv<W>(A.opp + (z * L2 + ym) * H + xh0);
        const Vec<W> b = ldv<W>(A.opp + (z * L2 + yp) * H + xh0);
        const Vec<W> c = ldv<W>(A.opp + (zm * L2 + y) * H + xh0);
        const Vec<W> d = ldv<W>(A.opp + (zp * L2 + y) * H + xh0);
        const uint32_t edge = par == 0 ? A.opp[row * H + (xh0 == 0 ? H - 1 : xh0 - 1)]
                                       : A.opp[row * H + (xh0 + W == H ? 0 : xh0 + W)];
        const Vec<W> out = ising_sc_update<W>(me, o0, a, b, c, d, edge, par, rho0, s_th, s_tl, t, stream,
                                              c3, seed, K, cnt);
        stv<W>(A.own_a + rho0, out);
    }
    return cnt;
}

// Sum of the four byte lanes (each <= 255).
__device__ __forceinline__ unsigned byte_sum(uint32_t cnt) {
    const uint32_t x = (cnt & 0x00FF00FFu) + ((cnt >> 8) & 0x00FF00FFu);
    return (x & 0xFFFFu) + (x >> 16);
}

// Loads a replica's 14 simple-cubic thresholds into shared memory (all threads call it).
__device__ __forceinline__ void load_sc_thresholds(const uint32_t *thr, uint32_t *s_th,
                                                   uint32_t *s_tl) {
    if (threadIdx.x < 14) {
        const uint32_t T = thr[threadIdx.x];
        s_th[threadIdx.x] = T >> 16;
        s_tl[threadIdx.x] = T & 0xFFFFu;
    }
}

}  // namespace ether
