// k_xyz.cu -- per-context launches of the Heisenberg (XYZ) colour phases (Metropolis bodies
// in sweep_xyz.cuh); overrelaxation (src/overrelaxation.f90:30-61 with
// get_ovrr_vec.f90:41-85); fresh_spins (src/fresh_spins.f90:31-38).
#include <algorithm>

#include "sweep_xyz.cuh"

namespace ether {

// ------------------------------------------------------------------ general lattice ----
// One thread per rank of the colour class (xyz_ell_site); W: the class's ELL width at compile
// time (0: at run time).
template <int OPT, int W>
__global__ void __launch_bounds__(256)
xyz_ell_kernel(float4 *__restrict__ spins4, int N, int col_off, int n_c, uint32_t colour,
               const int32_t *__restrict__ ell, const uint16_t *__restrict__ ej,
               const uint16_t *__restrict__ deg, int width, const float4 *__restrict__ J4, XyzParams P,
               const float *__restrict__ beta_slot_f, const int32_t *__restrict__ slot_of_rep,
               const uint32_t *__restrict__ stream_id, const uint32_t *__restrict__ step,
               const RoundKeys K, unsigned long long *__restrict__ acc_count) {
    const int r = blockIdx.y;
    float4 *sp = spins4 + (size_t)r * N;
    const float beta_f = beta_slot_f[slot_of_rep[r]];
    const uint32_t k1 = stream_id[r], t = step[r];
    const uint32_t c3 = kMetro | (colour << 8);
    unsigned acc = 0;
    for (int rho = blockIdx.x * blockDim.x + threadIdx.x; rho < n_c; rho += gridDim.x * blockDim.x) {
        acc += xyz_ell_site<OPT, W>(P, sp, col_off, n_c, rho, ell, ej, deg, width, J4, beta_f, t, c3, K, k1) ? 1u : 0u;
    }
    warp_add_count_x(acc_count + r, acc);
}

// Simple cubic, colour-split arrays.  A block takes VPT * 256 consecutive ranks per step,
// thread i the ranks i, i + 256, ... (coalesced), processed side by side (xyz_sc_sites);
// MINB is the register cap (blocks per SM).
template <int OPT, int VPT, int MINB>
__global__ void __launch_bounds__(256, MINB)
xyz_sc_kernel(float4 *__restrict__ spins4, int L1, int L2, int L3, FastDiv fH, FastDiv fL2, uint32_t colour, float jx,
              float jy, float jz, XyzParams P, const float *__restrict__ beta_slot_f,
              const int32_t *__restrict__ slot_of_rep, const uint32_t *__restrict__ stream_id,
              const uint32_t *__restrict__ step, const RoundKeys K,
              unsigned long long *__restrict__ acc_count) {
    const int r = blockIdx.y;
    const int H = L1 >> 1;
    const int half = H * L2 * L3;
    float4 *base = spins4 + (size_t)r * 2 * half;
    const XyzSc A{base + (size_t)colour * half, base + (size_t)(colour ^ 1u) * half, L1, L2, L3, H,
                  fH, fL2, colour, jx, jy, jz};
    const float beta_f = beta_slot_f[slot_of_rep[r]];
    const uint32_t k1 = stream_id[r], t = step[r];
    const uint32_t c3 = kMetro | (colour << 8);
    unsigned acc = 0;
    const int tile = VPT * (int)blockDim.x;
    for (int rho0 = blockIdx.x * tile + threadIdx.x; rho0 < half; rho0 += gridDim.x * tile)
        acc += xyz_sc_sites<OPT, VPT>(A, P, rho0, (int)blockDim.x, half, beta_f, t, c3, K, k1);
    warp_add_count_x(acc_count + r, acc);
}

// ------------------------------------------------------------------ overrelaxation ----
// Reflection of overrelaxation.f90:44-47 about the exchange field A (get_ovrr_vec),
// then normalisation.  A site with A = 0 is left unchanged (the reference would divide
// by zero).  Pass `pass` < floor(ovrr_para) reflects every site; the last pass reflects a
// site iff its uniform < part.  Neighbours from the colour class's ELL block.
__device__ __forceinline__ void ovrr_reflect(float4 *site, float hx, float hy, float hz) {
    const float4 S = *site;
    float d = hx * S.x;
    d = fmaf(hy, S.y, d);
    d = fmaf(hz, S.z, d);
    float a2 = hx * hx;
    a2 = fmaf(hy, hy, a2);
    a2 = fmaf(hz, hz, a2);
    if (!(a2 > 0.0f)) return;
    const float f = 2.0f * (d / a2);
    const float nx = f * hx - S.x, ny = f * hy - S.y, nz = f * hz - S.z;
    const float inv = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
    *site = make_float4(nx * inv, ny * inv, nz * inv, S.w);
}

__global__ void __launch_bounds__(256)
ovrr_ell_kernel(float4 *__restrict__ spins4, int N, int col_off, int n_c, uint32_t colour,
                int pass, float part, const int32_t *__restrict__ ell, const uint16_t *__restrict__ ej,
                const uint16_t *__restrict__ deg, int width, const float4 *__restrict__ J4,
                const uint32_t *__restrict__ stream_id, const uint32_t *__restrict__ ovrr_step,
                uint32_t seed) {
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
        const Acc3 h = ell_field(sp, ell, ej, J4, n_c, width, rho, deg[s]);
        ovrr_reflect(sp + s, h.x, h.y, h.z);
    }
}

// The same on a simple-cubic lattice: neighbours from the other colour's array in closed
// form (sc_field sums them in the order of the ELL block, so the results are the same).
__global__ void __launch_bounds__(256)
ovrr_sc_kernel(float4 *__restrict__ spins4, int L1, int L2, int L3, FastDiv fH, FastDiv fL2, uint32_t colour,
               int pass, float part, float jx, float jy, float jz, const uint32_t *__restrict__ stream_id,
               const uint32_t *__restrict__ ovrr_step, uint32_t seed) {
    const int r = blockIdx.y;
    const int H = L1 >> 1;
    const int half = H * L2 * L3;
    float4 *base = spins4 + (size_t)r * 2 * half;
    float4 *own = base + (size_t)colour * half;
    const float4 *opp = base + (size_t)(colour ^ 1u) * half;
    const uint32_t k1 = stream_id[r], t = ovrr_step[r];
    const uint32_t c3 = kOvrr | (colour << 8);
    for (int rho = blockIdx.x * blockDim.x + threadIdx.x; rho < half; rho += gridDim.x * blockDim.x) {
        if (part < 1.0f) {
            U4 o = draw((uint32_t)rho, t, k1, c3 | ((uint32_t)pass << 16), seed);
            if (!(u01(o.x) < part)) continue;
        }
        const int row = (int)fdiv((uint32_t)rho, fH);
        const int xh = rho - row * H;
        const int z = (int)fdiv((uint32_t)row, fL2), y = row - z * L2;
        const int p = (y + z + (int)colour) & 1;
        const Acc3 h = sc_field(opp, L1, L2, L3, H, xh, y, z, p, jx, jy, jz);
        ovrr_reflect(own + rho, h.x, h.y, h.z);
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
    P.nsp = c.nsp;
    P.sia_local = c.sia_local;
    P.sia_cls = c.t.sia_cls;
    P.sia_ax = c.t.sia_ax;
    return P;
}

template <int OPT, int VPT, int MINB>
static void launch_xyz_sc(Ctx &c, int colour, const XyzParams &P, const RoundKeys &K) {
    const int bs = 256;
    const int half = c.N / 2;
    dim3 grid(blocks_for_x(c, (half + VPT - 1) / VPT, bs), c.R);
    // single shell, single species: J(1,1,1,:)
    const float jx = c.h_Jf[0], jy = c.h_Jf[1], jz = c.h_Jf[2];
    XyzParams Pc = P;  // the kernel indexes sites by rank in the colour array
    if (Pc.sia_cls) Pc.sia_cls += (size_t)colour * half;
    xyz_sc_kernel<OPT, VPT, MINB><<<grid, bs, 0, c.stream>>>(
        c.spins4, c.L[0], c.L[1], c.L[2], make_fastdiv((uint32_t)(c.L[0] / 2)), make_fastdiv((uint32_t)c.L[1]),
        (uint32_t)colour, jx, jy, jz, Pc, c.beta_slot_f, c.slot_of_rep, c.stream_id, c.step, K, c.acc_count);
}

// xyz_variant = 10 * VPT + MINB (11 = one site per thread, no register cap)
template <int OPT>
static void launch_xyz_sc_opt(Ctx &c, int colour, const XyzParams &P, const RoundKeys &K) {
    switch (c.xyz_variant) {
        case 12: launch_xyz_sc<OPT, 1, 2>(c, colour, P, K); break;
        case 13: launch_xyz_sc<OPT, 1, 3>(c, colour, P, K); break;
        case 14: launch_xyz_sc<OPT, 1, 4>(c, colour, P, K); break;
        case 15: launch_xyz_sc<OPT, 1, 5>(c, colour, P, K); break;
        case 21: launch_xyz_sc<OPT, 2, 1>(c, colour, P, K); break;
        case 22: launch_xyz_sc<OPT, 2, 2>(c, colour, P, K); break;
        default: launch_xyz_sc<OPT, 1, 1>(c, colour, P, K); break;
    }
}

// The general-lattice kernel for a class's ELL width: common widths at compile time.
template <int OPT>
static auto ell_kernel_for(int width) {
    switch (width) {
        case 4: return xyz_ell_kernel<OPT, 4>;
        case 6: return xyz_ell_kernel<OPT, 6>;
        case 8: return xyz_ell_kernel<OPT, 8>;
        case 12: return xyz_ell_kernel<OPT, 12>;
        case 14: return xyz_ell_kernel<OPT, 14>;
        case 18: return xyz_ell_kernel<OPT, 18>;
        case 24: return xyz_ell_kernel<OPT, 24>;
        default: return xyz_ell_kernel<OPT, 0>;
    }
}

bool xyz_variant_valid(int v) { return (v >= 11 && v <= 15) || v == 21 || v == 22; }

cudaError_t launch_xyz_sweep(Ctx &c, int colour) {
    const int bs = 256;
    XyzParams P = xyz_params(c);
    const RoundKeys K = round_keys(c.seed);
    const bool exchange_only = !P.zeeman && !P.sia && !P.angle && !P.sia_local;
    if (c.fast) {
        if (exchange_only) launch_xyz_sc_opt<kXyzExchange>(c, colour, P, K);
        else launch_xyz_sc_opt<kXyzGeneral>(c, colour, P, K);
    } else {
        const int n_c = c.col_off[colour + 1] - c.col_off[colour];
        if (n_c == 0) return cudaSuccess;
        const int r0 = c.rw0, nr = c.rwn ? c.rwn : c.R;  // replica window (the grid keeps the full R's width)
        dim3 grid(blocks_for_x(c, n_c, bs), nr);
        const int32_t *ell = c.t.ell_nbr + c.ell_off[colour];
        const uint16_t *ej = c.t.ell_j + c.ell_off[colour];
        auto k = exchange_only ? ell_kernel_for<kXyzExchange>(c.ell_width[colour])
                               : ell_kernel_for<kXyzGeneral>(c.ell_width[colour]);
        k<<<grid, bs, 0, c.stream>>>(c.spins4 + (size_t)r0 * c.N, c.N, c.col_off[colour], n_c, (uint32_t)colour, ell,
                                     ej, c.t.ell_deg, c.ell_width[colour], c.t.J4, P, c.beta_slot_f,
                                     c.slot_of_rep + r0, c.stream_id + r0, c.step + r0, K, c.acc_count + r0);
    }
    c.launches++;
    return cudaGetLastError();
}

cudaError_t launch_overrelax(Ctx &c, int colour, int pass, float part) {
    const int bs = 256;
    const int n_c = c.col_off[colour + 1] - c.col_off[colour];
    if (n_c == 0) return cudaSuccess;
    dim3 grid(blocks_for_x(c, n_c, bs), c.R);
    if (c.fast) {
        ovrr_sc_kernel<<<grid, bs, 0, c.stream>>>(c.spins4, c.L[0], c.L[1], c.L[2], make_fastdiv((uint32_t)(c.L[0] / 2)),
                                                  make_fastdiv((uint32_t)c.L[1]), (uint32_t)colour, pass, part,
                                                  c.h_Jf[0], c.h_Jf[1], c.h_Jf[2], c.stream_id, c.ovrr_step, c.seed);
        c.launches++;
        return cudaGetLastError();
    }
    ovrr_ell_kernel<<<grid, bs, 0, c.stream>>>(c.spins4, c.N, c.col_off[colour], n_c, (uint32_t)colour, pass,
                                               part, c.t.ell_nbr + c.ell_off[colour],
                                               c.t.ell_j + c.ell_off[colour], c.t.ell_deg,
                                               c.ell_width[colour], c.t.J4, c.stream_id, c.ovrr_step,
                                               c.seed);
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

// Replica 0's bytes copied into replicas 1 .. R-1 (16-byte words when the size allows).
__global__ void broadcast_kernel(uint8_t *__restrict__ base, long long bytes, int R) {
    const long long total = bytes * (R - 1);
    const long long stride = (long long)gridDim.x * blockDim.x;
    if ((bytes & 15) == 0) {
        const uint4 *src = reinterpret_cast<const uint4 *>(base);
        uint4 *dst = reinterpret_cast<uint4 *>(base + bytes);
        const long long w = bytes >> 4;
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (total >> 4); i += stride)
            dst[i] = src[i % w];
    } else {
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += stride)
            base[bytes + i] = base[i % bytes];
    }
}

cudaError_t launch_broadcast(Ctx &c, void *base, size_t bytes_per_replica) {
    if (c.R < 2) return cudaSuccess;
    const long long work = (long long)bytes_per_replica * (c.R - 1) / 16 + 1;
    const int grid = (int)std::min<long long>((work + 255) / 256, (long long)c.sm_count * 8);
    broadcast_kernel<<<grid, 256, 0, c.stream>>>(reinterpret_cast<uint8_t *>(base), (long long)bytes_per_replica, c.R);
    c.launches++;
    return cudaGetLastError();
}

// Acceptance ratios of the sweeps since the snapshot: out[r] = (acc[r] - before[r]) / N.
__global__ void accept_ratio_kernel(const unsigned long long *__restrict__ acc,
                                    const unsigned long long *__restrict__ before, int R, double invN,
                                    double *__restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < R) out[r] = (double)(acc[r] - before[r]) * invN;
}

cudaError_t launch_accept_ratio(Ctx &c, double *out) {
    accept_ratio_kernel<<<(c.R + 255) / 256, 256, 0, c.stream>>>(c.acc_count, c.acc_before, c.R,
                                                                  1.0 / (double)c.N, out);
    c.launches++;
    return cudaGetLastError();
}

cudaError_t launch_advance(Ctx &c, uint32_t *counter) {
    const int r0 = c.rw0, nr = c.rwn ? c.rwn : c.R;
    advance_kernel<<<(nr + 255) / 256, 256, 0, c.stream>>>(counter + r0, nr);
    c.launches++;
    return cudaGetLastError();
}

}  // namespace ether
