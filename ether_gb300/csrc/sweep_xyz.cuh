// sweep_xyz.cuh -- device bodies of the Heisenberg (XYZ) Metropolis colour phase
// (src/Metropolis.f90:39-62 with update_spin_details.f90:30-51 and Hamiltonian.f90:34-143),
// shared by the per-context kernels (k_xyz.cu) and the persistent batch kernel (k_batch.cu).
//
// FP32 throughout, compiled with --fmad=false; the local exchange field is one fmaf chain
// per component over the neighbours in the reference's nn order (shells in order,
// neighbours by increasing site number), so every kernel variant and the oracle's FP32
// mirror round identically.
#pragma once
#include "internal.h"
#include "rng_math.cuh"

namespace ether {

__device__ __forceinline__ void warp_add_count_x(unsigned long long *dst, unsigned v) {
    unsigned s = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(dst, (unsigned long long)s);
}

struct XyzParams {
    int zeeman, sia, angle;
    float dphi;
    const uint8_t *species;
    const float *zee;
    const float *D;
    int nsp;  // species count: with one, the per-site species is not read
    int sia_local;            // per-site local-axis anisotropy D (a . S)^2
    const uint8_t *sia_cls;   // site -> class, indexed like the spin array the kernel updates:
                              // by storage index (general lattices) or, for the simple-cubic
                              // colour arrays, by rank (the table offset to the colour at launch)
    const float4 *sia_ax;     // class -> (a_x, a_y, a_z, D)
};

// Option sets of the XYZ kernels: kXyzExchange folds the Zeeman, SIA and ANGLE branches away
// at compile time (exchange only, Marsaglia proposals); kXyzGeneral reads them from P.
enum : int { kXyzExchange = 0, kXyzGeneral = 1 };

// ΔE of src/Hamiltonian.f90 for S -> n given the exchange field h.
template <int OPT>
__device__ __forceinline__ float delta_e(const XyzParams &P, int s, const float4 &S,
                                         const Spin4 &n, float hx, float hy, float hz) {
    float dx = n.x - S.x, dy = n.y - S.y, dz = n.z - S.z;
    float e = dx * hx;
    e = fmaf(dy, hy, e);
    e = fmaf(dz, hz, e);
    if (OPT != kXyzExchange && (P.zeeman || P.sia || P.sia_local)) {
        const int si = P.nsp == 1 ? 0 : P.species[s] - 1;
        if (P.zeeman) {
            const float *z = P.zee + 3 * si;
            e = fmaf(dx, z[0], e);
            e = fmaf(dy, z[1], e);
            e = fmaf(dz, z[2], e);
        }
        if (P.sia) {
            const float *D = P.D + 3 * si;
            float qx = n.x * n.x - S.x * S.x;
            float qy = n.y * n.y - S.y * S.y;
            float qz = n.z * n.z - S.z * S.z;
            e = fmaf(D[0], qx, e);
            e = fmaf(D[1], qy, e);
            e = fmaf(D[2], qz, e);
        }
        if (P.sia_local) {
            const float4 a = P.sia_ax[P.sia_cls[s]];
            float pn = a.x * n.x;
            pn = fmaf(a.y, n.y, pn);
            pn = fmaf(a.z, n.z, pn);
            float ps = a.x * S.x;
            ps = fmaf(a.y, S.y, ps);
            ps = fmaf(a.z, S.z, ps);
            e = fmaf(a.w, pn * pn - ps * ps, e);
        }
    }
    return e;
}

// The Metropolis decision of one site from its state S, the exchange field h and blocks 0
// and 1 of its draw (block 1 only for Marsaglia proposals): returns whether the proposal is
// accepted and, if so, the new state in out.
template <int OPT>
__device__ __forceinline__ bool metro_decide(const XyzParams &P, int s, const float4 &S, const U4 &b0,
                                             const U4 &b1, float hx, float hy, float hz, float beta_f,
                                             uint32_t rho, uint32_t t, uint32_t c3, const RoundKeys &K,
                                             uint32_t stream, float4 &out) {
    const bool angle = OPT != kXyzExchange && P.angle != 0;
    const float eta = u01(b0.x);
    Spin4 n;
    const Spin4 So{S.x, S.y, S.z, S.w};
    if (!propose(angle, P.dphi, So, rho, t, stream, c3, K, b0, b1, &n)) return false;
    const float e = delta_e<OPT>(P, s, S, n, hx, hy, hz);
    // exp evaluated on every lane (no divergent short-circuit); e <= 0 accepts regardless
    const float p = expf_neg(-(beta_f * fmaxf(e, 0.0f)));
    out = make_float4(n.x, n.y, n.z, n.w);
    return (e <= 0.0f) || (eta < p);
}

template <int OPT>
__device__ __forceinline__ void site_draws(const XyzParams &P, uint32_t rho, uint32_t t, uint32_t c3,
                                           const RoundKeys &K, uint32_t stream, U4 &b0, U4 &b1) {
    b0 = draw_rk(rho, t, stream, c3, K);
    b1 = U4{0u, 0u, 0u, 0u};
    if (!(OPT != kXyzExchange && P.angle != 0)) b1 = draw_rk(rho, t, stream, c3 | (1u << 16), K);
}

template <int OPT>
__device__ __forceinline__ bool metro_site(const XyzParams &P, float4 *sp, int s, uint32_t rho,
                                           float hx, float hy, float hz, float beta_f,
                                           uint32_t t, uint32_t c3, const RoundKeys &K, uint32_t stream) {
    const float4 S = sp[s];
    U4 b0, b1;
    site_draws<OPT>(P, rho, t, c3, K, stream, b0, b1);
    float4 n;
    const bool acc = metro_decide<OPT>(P, s, S, b0, b1, hx, hy, hz, beta_f, rho, t, c3, K, stream, n);
    if (acc) sp[s] = n;
    return acc;
}

// ------------------------------------------------------- simple cubic, colour-split ----
// Neighbours are summed in increasing site-number order, which is the reference's nn
// order: below-plane z neighbours, below-row y neighbours, the x pair, above-row y,
// above-plane z.  At a periodic boundary a pair changes side (u=0: both above, in
// order u+1, u-1; u=L-1: both below, in order u+1, u-1).
struct Acc3 {
    float x, y, z;
};
__device__ __forceinline__ void fma3(Acc3 &h, float jx, float jy, float jz, const float4 &S) {
    h.x = fmaf(jx, S.x, h.x);
    h.y = fmaf(jy, S.y, h.y);
    h.z = fmaf(jz, S.z, h.z);
}

__device__ __forceinline__ Acc3 sc_field(const float4 *__restrict__ opp, int L1, int L2, int L3,
                                         int H, int xh, int y, int z, int p, float jx, float jy,
                                         float jz) {
    const int row = z * L2 + y;
    const int x = 2 * xh + p;
    const int ym = (y == 0 ? L2 - 1 : y - 1), yp = (y == L2 - 1 ? 0 : y + 1);
    const int zm = (z == 0 ? L3 - 1 : z - 1), zp = (z == L3 - 1 ? 0 : z + 1);
    int xh_m, xh_p;
    if (p == 0) { xh_m = (xh == 0 ? H - 1 : xh - 1); xh_p = xh; }
    else { xh_m = xh; xh_p = (xh == H - 1 ? 0 : xh + 1); }
    const float4 Sxm = opp[row * H + xh_m];
    const float4 Sxp = opp[row * H + xh_p];
    const float4 Sym = opp[(z * L2 + ym) * H + xh];
    const float4 Syp = opp[(z * L2 + yp) * H + xh];
    const float4 Szm = opp[(zm * L2 + y) * H + xh];
    const float4 Szp = opp[(zp * L2 + y) * H + xh];
    Acc3 h{0.f, 0.f, 0.f};
    // below
    if (z == L3 - 1) { fma3(h, jx, jy, jz, Szp); fma3(h, jx, jy, jz, Szm); }
    else if (z != 0) fma3(h, jx, jy, jz, Szm);
    if (y == L2 - 1) { fma3(h, jx, jy, jz, Syp); fma3(h, jx, jy, jz, Sym); }
    else if (y != 0) fma3(h, jx, jy, jz, Sym);
    // x pair in index order
    const bool interior = (x != 0) && (x != L1 - 1);
    const float4 xa = interior ? Sxm : Sxp;
    const float4 xb = interior ? Sxp : Sxm;
    fma3(h, jx, jy, jz, xa);
    fma3(h, jx, jy, jz, xb);
    // above
    if (y == 0) { fma3(h, jx, jy, jz, Syp); fma3(h, jx, jy, jz, Sym); }
    else if (y != L2 - 1) fma3(h, jx, jy, jz, Syp);
    if (z == 0) { fma3(h, jx, jy, jz, Szp); fma3(h, jx, jy, jz, Szm); }
    else if (z != L3 - 1) fma3(h, jx, jy, jz, Szp);
    return h;
}

// Exchange field of rank rho of a colour class from its ELL block (ell: entries k * n_c + rho,
// coalesced across a warp), in the CSR's order -- the reference's nn order -- so the fmaf
// chain rounds as the oracle's.
// W > 0: the class's ELL width, known at compile time (every load of the site issued at
// once); W = 0: width at run time.
template <int W = 0>
__device__ __forceinline__ Acc3 ell_field(const float4 *__restrict__ sp, const int32_t *__restrict__ ell,
                                          const uint16_t *__restrict__ ej, const float4 *__restrict__ J4,
                                          int n_c, int width, int rho, int deg) {
    // The padding entries point at valid memory (the site itself, coupling 0), so the loads
    // are unconditional and can all be in flight at once; only the fmaf is predicated.
    Acc3 h{0.f, 0.f, 0.f};
    if constexpr (W > 0) {
        // the neighbours' storage indices, then all their spins, then the field
        int nb[W];
#pragma unroll
        for (int k = 0; k < W; ++k) nb[k] = ell[k * n_c + rho];  // ELL blocks hold < 2^31 entries
        float4 Sj[W];
#pragma unroll
        for (int k = 0; k < W; ++k) Sj[k] = sp[nb[k]];
#pragma unroll
        for (int k = 0; k < W; ++k) {
            const float4 Jv = J4[ej[k * n_c + rho]];
            if (k < deg) {
                h.x = fmaf(Jv.x, Sj[k].x, h.x);
                h.y = fmaf(Jv.y, Sj[k].y, h.y);
                h.z = fmaf(Jv.z, Sj[k].z, h.z);
            }
        }
    } else {
#pragma unroll 6
        for (int k = 0; k < width; ++k) {
            const int e = k * n_c + rho;
            const float4 Jv = J4[ej[e]];
            const float4 Sj = sp[ell[e]];
            if (k < deg) {
                h.x = fmaf(Jv.x, Sj.x, h.x);
                h.y = fmaf(Jv.y, Sj.y, h.y);
                h.z = fmaf(Jv.z, Sj.z, h.z);
            }
        }
    }
    return h;
}

// One Metropolis update of rank rho of a colour class of a general lattice (ELL block of the
// class: ell, ej; deg per storage index; W as ell_field's).
template <int OPT, int W = 0>
__device__ __forceinline__ bool xyz_ell_site(const XyzParams &P, float4 *sp, int col_off, int n_c, int rho,
                                             const int32_t *__restrict__ ell, const uint16_t *__restrict__ ej,
                                             const uint16_t *__restrict__ deg, int width,
                                             const float4 *__restrict__ J4, float beta_f, uint32_t t,
                                             uint32_t c3, const RoundKeys &K, uint32_t stream) {
    const int s = col_off + rho;
    const Acc3 h = ell_field<W>(sp, ell, ej, J4, n_c, width, rho, deg[s]);
    return metro_site<OPT>(P, sp, s, (uint32_t)rho, h.x, h.y, h.z, beta_f, t, c3, K, stream);
}

// One Metropolis update of rank rho of the simple-cubic colour array `own` (the other
// colour's array is `opp`).
struct XyzSc {
    float4 *own;
    const float4 *opp;
    int L1, L2, L3, H;
    FastDiv fH, fL2;
    uint32_t colour;
    float jx, jy, jz;
};
template <int OPT>
__device__ __forceinline__ bool xyz_sc_site(const XyzSc &A, const XyzParams &P, int rho,
                                            float beta_f, uint32_t t, uint32_t c3, const RoundKeys &K,
                                            uint32_t stream) {
    const int row = (int)fdiv((uint32_t)rho, A.fH);
    const int xh = rho - row * A.H;
    const int z = (int)fdiv((uint32_t)row, A.fL2), y = row - z * A.L2;
    const int p = (y + z + (int)A.colour) & 1;
    Acc3 h = sc_field(A.opp, A.L1, A.L2, A.L3, A.H, xh, y, z, p, A.jx, A.jy, A.jz);
    return metro_site<OPT>(P, A.own, rho, (uint32_t)rho, h.x, h.y, h.z, beta_f, t, c3, K, stream);
}

// VPT sites rho0 + j * step (j < VPT, all < n) in three passes -- loads and exchange fields,
// the Philox blocks, then decisions and stores -- so that the independent chains of the
// sites interleave.  Returns the number of accepted updates.
template <int OPT, int VPT>
__device__ __forceinline__ unsigned xyz_sc_sites(const XyzSc &A, const XyzParams &P, int rho0, int step,
                                                 int n, float beta_f, uint32_t t, uint32_t c3,
                                                 const RoundKeys &K, uint32_t stream) {
    float4 S[VPT];
    Acc3 h[VPT];
#pragma unroll
    for (int j = 0; j < VPT; ++j) {
        const int rho = min(rho0 + j * step, n - 1);  // a clamped duplicate is never stored
        const int row = (int)fdiv((uint32_t)rho, A.fH);
        const int xh = rho - row * A.H;
        const int z = (int)fdiv((uint32_t)row, A.fL2), y = row - z * A.L2;
        const int p = (y + z + (int)A.colour) & 1;
        h[j] = sc_field(A.opp, A.L1, A.L2, A.L3, A.H, xh, y, z, p, A.jx, A.jy, A.jz);
        S[j] = A.own[rho];
    }
    U4 b0[VPT], b1[VPT];
#pragma unroll
    for (int j = 0; j < VPT; ++j) site_draws<OPT>(P, (uint32_t)(rho0 + j * step), t, c3, K, stream, b0[j], b1[j]);
    unsigned acc = 0;
#pragma unroll
    for (int j = 0; j < VPT; ++j) {
        const int rho = rho0 + j * step;
        float4 nv;
        const bool a = metro_decide<OPT>(P, min(rho, n - 1), S[j], b0[j], b1[j], h[j].x, h[j].y, h[j].z,
                                         beta_f, (uint32_t)rho, t, c3, K, stream, nv);
        if (a && rho < n) {
            A.own[rho] = nv;
            ++acc;
        }
    }
    return acc;
}

}  // namespace ether
