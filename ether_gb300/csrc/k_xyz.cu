// k_xyz.cu -- Heisenberg (XYZ) colour phases: Metropolis (src/Metropolis.f90:39-62) with
// update_spin_details (src/update_spin_details.f90:30-51) and Hamiltonian
// (src/Hamiltonian.f90:34-143); overrelaxation (src/overrelaxation.f90:30-61 with
// get_ovrr_vec.f90:41-85); fresh_spins (src/fresh_spins.f90:31-38).
//
// FP32 throughout, compiled with --fmad=false; the local exchange field is one fmaf chain
// per component over the neighbours in the reference's nn order (shells in order,
// neighbours by increasing site number), so every kernel variant and the oracle's FP32
// mirror round identically.
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
};

// ΔE of src/Hamiltonian.f90 for S -> n given the exchange field h.
__device__ __forceinline__ float delta_e(const XyzParams &P, int s, const float4 &S,
                                         const Spin4 &n, float hx, float hy, float hz) {
    float dx = n.x - S.x, dy = n.y - S.y, dz = n.z - S.z;
    float e = dx * hx;
    e = fmaf(dy, hy, e);
    e = fmaf(dz, hz, e);
    if (P.zeeman || P.sia) {
        int si = P.species[s] - 1;
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
    }
    return e;
}

__device__ __forceinline__ bool metro_site(const XyzParams &P, float4 *sp, int s, uint32_t rho,
                                           float hx, float hy, float hz, float beta_f,
                                           uint32_t t, uint32_t c3, uint32_t seed, uint32_t stream) {
    const float4 S = sp[s];
    U4 b0 = draw(rho, t, stream, c3, seed);
    float eta = u01(b0.x);
    Spin4 n;
    Spin4 So{S.x, S.y, S.z, S.w};
    if (!propose(P.angle != 0, P.dphi, So, rho, t, stream, c3, seed, b0, &n)) return false;
    float e = delta_e(P, s, S, n, hx, hy, hz);
    // exp evaluated on every lane (no divergent short-circuit); e <= 0 accepts regardless
    const float p = expf_neg(-(beta_f * fmaxf(e, 0.0f)));
    bool acc = (e <= 0.0f) || (eta < p);
    if (acc) sp[s] = make_float4(n.x, n.y, n.z, n.w);
    return acc;
}

// ------------------------------------------------------------------ general lattice ----
__global__ void __launch_bounds__(256)
xyz_csr_kernel(float4 *__restrict__ spins4, int N, int col_off, int n_c, uint32_t colour,
               const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ nbr,
               const uint16_t *__restrict__ jidx, const float *__restrict__ J, XyzParams P,
               const float *__restrict__ beta_slot_f, const int32_t *__restrict__ slot_of_rep,
               const uint32_t *__restrict__ stream_id, const uint32_t *__restrict__ step,
               uint32_t seed, unsigned long long *__restrict__ acc_count) {
    const int r = blockIdx.y;
    float4 *sp = spins4 + (size_t)r * N;
    const float beta_f = beta_slot_f[slot_of_rep[r]];
    const uint32_t k1 = stream_id[r], t = step[r];
    const uint32_t c3 = kMetro | (colour << 8);
    unsigned acc = 0;
    for (int rho = blockIdx.x * blockDim.x + threadIdx.x; rho < n_c; rho += gridDim.x * blockDim.x) {
        const int s = col_off + rho;
        float hx = 0.f, hy = 0.f, hz = 0.f;
        for (int k = row_ptr[s]; k < row_ptr[s + 1]; ++k) {
            float4 Sj = sp[nbr[k]];
            const float *Jp = J + 3 * jidx[k];
            hx = fmaf(Jp[0], Sj.x, hx);
            hy = fmaf(Jp[1], Sj.y, hy);
            hz = fmaf(Jp[2], Sj.z, hz);
        }
        acc += metro_site(P, sp, s, (uint32_t)rho, hx, hy, hz, beta_f, t, c3, seed, k1) ? 1u : 0u;
    }
    warp_add_count_x(acc_count + r, acc);
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

__global__ void __launch_bounds__(256)
xyz_sc_kernel(float4 *__restrict__ spins4, int L1, int L2, int L3, FastDiv fH, FastDiv fL2, uint32_t colour, float jx,
              float jy, float jz, XyzParams P, const float *__restrict__ beta_slot_f,
              const int32_t *__restrict__ slot_of_rep, const uint32_t *__restrict__ stream_id,
              const uint32_t *__restrict__ step, uint32_t seed,
              unsigned long long *__restrict__ acc_count) {
    const int r = blockIdx.y;
    const int H = L1 >> 1;
    const int half = H * L2 * L3;
    float4 *base = spins4 + (size_t)r * 2 * half;
    float4 *own = base + (size_t)colour * half;
    const float4 *opp = base + (size_t)(colour ^ 1u) * half;
    const float beta_f = beta_slot_f[slot_of_rep[r]];
    const uint32_t k1 = stream_id[r], t = step[r];
    const uint32_t c3 = kMetro | (colour << 8);
    unsigned acc = 0;
    for (int rho = blockIdx.x * blockDim.x + threadIdx.x; rho < half; rho += gridDim.x * blockDim.x) {
        const int row = (int)fdiv((uint32_t)rho, fH);
        const int xh = rho - row * H;
        const int z = (int)fdiv((uint32_t)row, fL2), y = row - z * L2;
        const int p = (y + z + (int)colour) & 1;
        Acc3 h = sc_field(opp, L1, L2, L3, H, xh, y, z, p, jx, jy, jz);
        acc += metro_site(P, own, rho, (uint32_t)rho, h.x, h.y, h.z, beta_f, t, c3, seed, k1) ? 1u : 0u;
    }
    warp_add_count_x(acc_count + r, acc);
}

// ------------------------------------------------------------------ overrelaxation ----
// Reflection of overrelaxation.f90:44-47 about the exchange field A (get_ovrr_vec),
// then normalisation.  A site with A = 0 is left unchanged (the reference would divide
// by zero).  Pass `pass` < floor(ovrr_para) reflects every site; the last pass reflects a
// site iff its uniform < part.
__global__ void __launch_bounds__(256)
ovrr_csr_kernel(float4 *__restrict__ spins4, int N, int col_off, int n_c, uint32_t colour,
                int pass, float part, const int32_t *__restrict__ row_ptr,
                const int32_t *__restrict__ nbr, const uint16_t *__restrict__ jidx,
                const float *__restrict__ J, const uint32_t *__restrict__ stream_id,
                const uint32_t *__restrict__ ovrr_step, uint32_t seed) {
    const int r = blockIdx.y;
    float4 *sp = spins4 + (size_t)r * N;
    const uint32_t k1 = stream_id[r], t = ovrr_step[r];
    const uint32_t c3 = kOvrr | (colour << 8);
    for (int rho = blockIdx.x * blockDim.x + threadIdx.x; rho < n_c; rho += gridDim.x * blockDim.x) {
        const int s = col_off + rho;
        if (part < 1.0f) {
            U4 o = draw((uint32_t)rho, t, k1, c3 | ((uint32_t)pass << 16), seed);
            if (!(u01(o.x) < part)) continue;
        }
        float hx = 0.f, hy = 0.f, hz = 0.f;
        for (int k = row_ptr[s]; k < row_ptr[s + 1]; ++k) {
            float4 Sj = sp[nbr[k]];
            const float *Jp = J + 3 * jidx[k];
            hx = fmaf(Jp[0], Sj.x, hx);
            hy = fmaf(Jp[1], Sj.y, hy);
            hz = fmaf(Jp[2], Sj.z, hz);
        }
        float4 S = sp[s];
        float d = hx * S.x;
        d = fmaf(hy, S.y, d);
        d = fmaf(hz, S.z, d);
        float a2 = hx * hx;
        a2 = fmaf(hy, hy, a2);
        a2 = fmaf(hz, hz, a2);
        if (!(a2 > 0.0f)) continue;
        float f = 2.0f * (d / a2);
        float nx = f * hx - S.x, ny = f * hy - S.y, nz = f * hz - S.z;
        float inv = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
        sp[s] = make_float4(nx * inv, ny * inv, nz * inv, S.w);
    }
}

// ------------------------------------------------------------------ fresh spins -------
// key (seed, stream), counter (site number, call, block, kFresh).  Marsaglia pairs:
// p -> block p/2, words 2(p&1), 2(p&1)+1.  ANGLE: z from word 0, phi step from word 1.
__global__ void fresh_kernel(uint8_t *__restrict__ spins, float4 *__restrict__ spins4, int N,
                             int model, int angle, float dphi,
                             const int32_t *__restrict__ site_of_storage,
                             const uint32_t *__restrict__ stream_id,
                             const uint32_t *__restrict__ fresh_call, uint32_t seed) {
    const int r = blockIdx.y;
    const uint32_t k1 = stream_id[r], call = fresh_call[r];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += gridDim.x * blockDim.x) {
        if (model == 0) {
            spins[(size_t)r * N + s] ^= 1u;
            continue;
        }
        const uint32_t i = (uint32_t)site_of_storage[s];
        float4 S = spins4[(size_t)r * N + s];
        U4 o = draw(i, call, k1, kFresh, seed);
        float nx, ny, nz, nphi;
        if (!angle) {
            float v1 = 0.f, v2 = 0.f, q = 0.f;
            bool ok = false;
            U4 w = o;
            for (int p = 0; p < kMarsagliaMaxPairs; ++p) {
                if (p >= 2 && (p & 1) == 0) w = draw(i, call, k1, kFresh | ((uint32_t)(p / 2) << 16), seed);
                uint32_t a = (p & 1) ? w.z : w.x;
                uint32_t b = (p & 1) ? w.w : w.y;
                v1 = upm1(a);
                v2 = upm1(b);
                q = v1 * v1 + v2 * v2;
                if (q < 1.0f) { ok = true; break; }
            }
            if (!ok) continue;
            float tq = sqrtf(1.0f - q);
            nx = (2.0f * v1) * tq;
            ny = (2.0f * v2) * tq;
            nz = 1.0f - 2.0f * q;
            nphi = 0.0f;
        } else {
            nz = upm1(o.x);
            nphi = S.w + dphi * upm1(o.y);
            if (nphi >= kPiF) nphi = nphi - kTwoPiF;
            else if (nphi < -kPiF) nphi = nphi + kTwoPiF;
            float rr = sqrtf(1.0f - nz * nz);
            float sn, cs;
            sincos_own(nphi, &sn, &cs);
            nx = rr * cs;
            ny = rr * sn;
        }
        float inv = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
        spins4[(size_t)r * N + s] = make_float4(nx * inv, ny * inv, nz * inv, nphi);
    }
}

__global__ void advance_kernel(uint32_t *__restrict__ counter, int R) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < R) counter[r] += 1u;
}

static int blocks_for_x(const Ctx &c, long work, int bs) {
    long need = (work + bs - 1) / bs;
    long cap = (long)c.sm_count * 8 / (c.R > 0 ? c.R : 1);
    if (cap < 1) cap = 1;
    if (need > cap) need = cap;
    if (need < 1) need = 1;
    return (int)need;
}

static XyzParams xyz_params(const Ctx &c) {
    XyzParams P;
    P.zeeman = c.zeeman;
    P.sia = c.sia;
    P.angle = c.angle;
    P.dphi = (float)c.dphi;
    P.species = c.t.species;
    P.zee = c.t.zee;
    P.D = c.t.D;
    return P;
}

cudaError_t launch_xyz_sweep(Ctx &c, int colour) {
    const int bs = 256;
    XyzParams P = xyz_params(c);
    if (c.fast) {
        const int half = c.N / 2;
        dim3 grid(blocks_for_x(c, half, bs), c.R);
        // single shell, single species: J(1,1,1,:)
        float jx = c.h_Jf[0], jy = c.h_Jf[1], jz = c.h_Jf[2];
        xyz_sc_kernel<<<grid, bs, 0, c.stream>>>(c.spins4, c.L[0], c.L[1], c.L[2], make_fastdiv((uint32_t)(c.L[0] / 2)), make_fastdiv((uint32_t)c.L[1]),
                                                 (uint32_t)colour, jx, jy, jz, P, c.beta_slot_f,
                                                 c.slot_of_rep, c.stream_id, c.step, c.seed,
                                                 c.acc_count);
    } else {
        const int n_c = c.col_off[colour + 1] - c.col_off[colour];
        if (n_c == 0) return cudaSuccess;
        dim3 grid(blocks_for_x(c, n_c, bs), c.R);
        xyz_csr_kernel<<<grid, bs, 0, c.stream>>>(c.spins4, c.N, c.col_off[colour], n_c,
                                                  (uint32_t)colour, c.t.row_ptr, c.t.nbr,
                                                  c.t.jidx, c.t.J, P, c.beta_slot_f,
                                                  c.slot_of_rep, c.stream_id, c.step, c.seed,
                                                  c.acc_count);
    }
    c.launches++;
    return cudaGetLastError();
}

cudaError_t launch_overrelax(Ctx &c, int colour, int pass, float part) {
    const int bs = 256;
    const int n_c = c.col_off[colour + 1] - c.col_off[colour];
    if (n_c == 0) return cudaSuccess;
    dim3 grid(blocks_for_x(c, n_c, bs), c.R);
    ovrr_csr_kernel<<<grid, bs, 0, c.stream>>>(c.spins4, c.N, c.col_off[colour], n_c,
                                               (uint32_t)colour, pass, part, c.t.row_ptr,
                                               c.t.nbr, c.t.jidx, c.t.J, c.stream_id,
                                               c.ovrr_step, c.seed);
    c.launches++;
    return cudaGetLastError();
}

cudaError_t launch_fresh(Ctx &c) {
    const int bs = 256;
    dim3 grid(blocks_for_x(c, c.N, bs), c.R);
    fresh_kernel<<<grid, bs, 0, c.stream>>>(c.spins, c.spins4, c.N, c.model, c.angle,
                                            (float)c.dphi, c.t.site_of_storage, c.stream_id,
                                            c.fresh_call, c.seed);
    c.launches++;
    return cudaGetLastError();
}

cudaError_t launch_advance(Ctx &c, uint32_t *counter) {
    advance_kernel<<<(c.R + 255) / 256, 256, 0, c.stream>>>(counter, c.R);
    c.launches++;
    return cudaGetLastError();
}

}  // namespace ether
