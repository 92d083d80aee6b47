// k_learn.cu -- learned patch proposal for the simple-cubic Ising model (ether_learn_* in the
// C-ABI).  The reference has no learned move; what it fixes is the target distribution,
// exp(-beta E) with E = sum over bonds of J s_i s_j (src/Hamiltonian.f90:57-105,
// src/Metropolis.f90:50-56), and every learned move below is accepted or rejected by exact
// Metropolis-Hastings against that energy, so the stationary distribution is unchanged.
//
// Move (one "learned sweep" = patch class 0, then class 1; patches of a class share no bond):
//   * per replica and sweep a Philox offset (ox, oy, oz) in [0,4)^3 tiles the lattice with 4^3
//     patches; canonical frame reflected in x when ox+oy+oz is odd, so the 32 network-proposed
//     A-sites are always colour 0 and the 32 B-sites colour 1;
//   * network: input = the 96 boundary spins and 4 beta J; 128 -> 128 -> 128 -> 32 MLP, BF16
//     weights and activations, FP32 accumulation, on the tensor cores (tcgen05, accumulators in
//     TMEM): one CTA takes 128 patches, thread p owns patch p = TMEM lane p through all three
//     layers and then performs the patch's Metropolis-Hastings step;
//   * proposal: A-site k up with probability T_k / 2^32 from the logit; every B-site then from
//     its exact heat-bath conditional given the new A-sites and the boundary;
//   * acceptance: log alpha = log q(old) - log q(new) - beta J (bond change), FP32 in a fixed
//     order with an own exp (the same operations as oracle/learn_oracle.c, which replays a
//     sweep bit for bit given the logits).
// Training: maximum likelihood of the A-sites given the boundary on configurations the plain
// sweep produced (any temperature of the context's ladder), Adam, straight-through BF16
// rounding; hand-written FP32 GEMM, activation and optimiser kernels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "internal.h"
#include "learn_common.cuh"
#include "rng_math.cuh"
#include "tc_util.cuh"

namespace ether {
namespace learn {

constexpr int NI = 128, NO = 32;  // network input and output widths (hidden: NH)
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NI, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NO * NH, NPARAM = OFF_B3 + NO;

// Packed inference image (global memory, copied to shared memory by every CTA):
// W1 (2 tiles x 128 rows x 128 B), W2 (same), W3 (2 tiles x 32 rows x 128 B), b1, b2, b3 (FP32).
constexpr int IMG_W1 = 0, IMG_W2 = 32768, IMG_W3 = 65536, IMG_B1 = 73728, IMG_B2 = IMG_B1 + 512,
              IMG_B3 = IMG_B2 + 512, IMG_BYTES = IMG_B3 + 128;
// Shared memory of the patch kernel (from a 1024-byte aligned base).
constexpr int SM_A = 73728, SM_BIAS = SM_A + 32768, SM_PATCH = SM_BIAS + 1152,
              SM_BAR = SM_PATCH + 128 * 28, SM_BYTES = SM_BAR + 16;
constexpr int kThreads = 128;

// ------------------------------------------------------------------ patch geometry ----
// Local sites 0..31 = A-sites, 32..63 = B-sites, packed (a | b << 2 | c << 4); boundary
// sites packed ((a+1) | (b+1) << 4 | (c+1) << 8).  The neighbour tables below (B-site
// neighbours: >= 0 A-site index, < 0 boundary -(1 + index); A-site boundary neighbours) are
// built once on the host and must agree with the closed forms the kernels use.
__constant__ uint8_t c_site[64];
__constant__ uint16_t c_bnd[96];

struct Geometry {
    uint8_t site[64];
    uint16_t bnd[96];
    int8_t Bn[32][6];
    int8_t Ab[32][3];
};

static int face_index(int a, int b, int c) {
    if (a == -1) return b + 4 * c;
    if (a == 4) return 16 + b + 4 * c;
    if (b == -1) return 32 + a + 4 * c;
    if (b == 4) return 48 + a + 4 * c;
    if (c == -1) return 64 + a + 4 * b;
    return 80 + a + 4 * b;
}

static bool closed_forms_agree(const Geometry &g);

static Geometry make_geometry() {
    Geometry g;
    int A[32][3], B[32][3], na = 0, nb = 0, idx_of[64];
    for (int lin = 0; lin < 64; ++lin) {
        const int a = lin & 3, b = (lin >> 2) & 3, c = lin >> 4;
        if (((a + b + c) & 1) == 0) {
            A[na][0] = a; A[na][1] = b; A[na][2] = c;
            idx_of[lin] = na++;
        } else {
            B[nb][0] = a; B[nb][1] = b; B[nb][2] = c;
            idx_of[lin] = nb++;
        }
    }
    for (int k = 0; k < 32; ++k) {
        g.site[k] = (uint8_t)(A[k][0] | (A[k][1] << 2) | (A[k][2] << 4));
        g.site[32 + k] = (uint8_t)(B[k][0] | (B[k][1] << 2) | (B[k][2] << 4));
    }
    for (int f = 0; f < 6; ++f)
        for (int u = 0; u < 4; ++u)
            for (int v = 0; v < 4; ++v) {
                const int e = (f & 1) ? 4 : -1;
                int a, b, c;
                if (f < 2) { a = e; b = u; c = v; }
                else if (f < 4) { a = u; b = e; c = v; }
                else { a = u; b = v; c = e; }
                g.bnd[face_index(a, b, c)] = (uint16_t)((a + 1) | ((b + 1) << 4) | ((c + 1) << 8));
            }
    static const int d[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
    for (int m = 0; m < 32; ++m)
        for (int q = 0; q < 6; ++q) {
            const int a = B[m][0] + d[q][0], b = B[m][1] + d[q][1], c = B[m][2] + d[q][2];
            if (a < 0 || a > 3 || b < 0 || b > 3 || c < 0 || c > 3) g.Bn[m][q] = (int8_t)(-(1 + face_index(a, b, c)));
            else g.Bn[m][q] = (int8_t)idx_of[a + 4 * b + 16 * c];
        }
    for (int k = 0; k < 32; ++k) {
        int n = 0;
        for (int q = 0; q < 3; ++q) g.Ab[k][q] = -1;
        for (int q = 0; q < 6; ++q) {
            const int a = A[k][0] + d[q][0], b = A[k][1] + d[q][1], c = A[k][2] + d[q][2];
            if (a < 0 || a > 3 || b < 0 || b > 3 || c < 0 || c > 3) g.Ab[k][n++] = (int8_t)face_index(a, b, c);
        }
    }
    return g;
}

// Closed forms of the same geometry (geo_*) are in learn_common.cuh.

// ------------------------------------------------------------- own FP32 functions ----
// Same operation sequence as oracle/learn_oracle.c (compiled with --fmad=false: explicit
// fmaf only).
// sigmoid(z) = r or e r with e = exp(-|z|), r = 1 / (1 + e) correctly rounded.
__device__ __forceinline__ float sigmoid_own(float z) {
    const float e = expf_neg(-fabsf(z));
    const float r = __frcp_rn(1.0f + e);
    return z >= 0.0f ? r : e * r;
}
__device__ __forceinline__ uint32_t thr_of_logit(float z) {
    float t = sigmoid_own(z) * 4294967296.0f;
    t = fmaxf(t, 1.0f);
    t = fminf(t, 4294967040.0f);
    return (uint32_t)t;
}

// ------------------------------------------------------------------- the patch kernel ----
struct PatchParams {
    const uint8_t *img;           // packed weights + biases (IMG_BYTES)
    int *err;
    // lattice mode
    uint8_t *spins;
    int L1, L2, L3, H;
    long long half;               // sites per colour per replica
    int P1, P2, P3, cls;
    long long Pc;                 // patches of one class per replica
    int R;
    const uint32_t *stream_id, *lstep;
    const int32_t *slot_of_rep;
    const float *k4, *betaJf;     // per slot
    const uint32_t *TB;           // per slot x 7
    const float *LBup, *LBdn;     // per slot x 7
    uint32_t seed;
    unsigned long long *acc;      // per replica: accepted patches
    float *dump;                  // optional [R][Pc][32] logits of this class
    // forward mode
    const __nv_bfloat16 *X;       // [B][128]
    int B;
    float *Z;                     // [B][32]
};

__device__ __forceinline__ int wrap(int x, int L) { return x >= L ? x - L : (x < 0 ? x + L : x); }

// storage byte of canonical (a, b, c) in [-1, 4] of the patch at origin o with reflection par
__device__ __forceinline__ long long site_addr(const PatchParams &P, int o0, int o1, int o2, int par,
                                               int a, int b, int c) {
    const int x = wrap(o0 + (par ? 3 - a : a), P.L1);
    const int y = wrap(o1 + b, P.L2);
    const int z = wrap(o2 + c, P.L3);
    return (long long)((x + y + z) & 1) * P.half + ((long long)z * P.L2 + y) * P.H + (x >> 1);
}

// Per tile of 128 patches:
//   1. thread p decodes patch p (replica, origin, reflection) into shared memory;
//   2. each warp gathers its 32 patches cooperatively: lane l loads sites l, l+32, .., l+128
//      of the list [96 boundary | 32 A | 32 B] and five ballots give the patch's bit masks;
//   3. thread p writes its network input row (boundary spins, 4 beta J) into the A tile;
//   4. three tcgen05 layers, TMEM lane p = patch p;
//   5. thread p's Metropolis-Hastings step from the masks and its 32 logits.
template <int MODE>  // 0: lattice patches + Metropolis-Hastings, 1: network forward on X
__global__ void __launch_bounds__(kThreads, 2) patch_kernel(PatchParams P) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    float *bias = reinterpret_cast<float *>(base + SM_BIAS);  // b1[128], b2[128], b3[32]
    uint32_t *s_org = reinterpret_cast<uint32_t *>(base + SM_PATCH);  // origin | par << 30
    int32_t *s_rep = reinterpret_cast<int32_t *>(s_org + 128);       // replica, -1 = none
    uint32_t *s_bits = reinterpret_cast<uint32_t *>(s_rep + 128);    // [128][5]
    uint64_t *bar = reinterpret_cast<uint64_t *>(base + SM_BAR);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(base + SM_BAR + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // weights and biases into shared memory (plain 16-byte copies; the image is pre-swizzled)
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(P.img);
        uint4 *dw = reinterpret_cast<uint4 *>(base);
        constexpr int nw = IMG_B1 / 16;  // 4608 = 36 x 128
        for (int i0 = 0; i0 < nw; i0 += 8 * kThreads) {
            uint4 v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int i = i0 + u * kThreads + tid;
                if (i < nw) v[u] = __ldg(src + i);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int i = i0 + u * kThreads + tid;
                if (i < nw) dw[i] = v[u];
            }
        }
        uint4 *db = reinterpret_cast<uint4 *>(base + SM_BIAS);
        for (int i = tid; i < (IMG_BYTES - IMG_B1) / 16; i += kThreads) db[i] = src[nw + i];
    }
    if (tid == 0) {
        tc::mbar_init(tc::smem_u32(bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(tc::smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t sA = tc::smem_u32(base + SM_A);
    const uint32_t sW1 = tc::smem_u32(base + IMG_W1), sW2 = tc::smem_u32(base + IMG_W2),
                   sW3 = tc::smem_u32(base + IMG_W3);
    uint8_t *arow = base + SM_A;
    uint32_t phase = 0;
    bool ok = true;

    // this lane's five sites of every patch: canonical (a, b, c) + 1, packed 4 bits each
    uint32_t my_site[5];
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        const int i = lane + 32 * c;
        if (i < 96) {
            my_site[c] = c_bnd[i];
        } else {
            const uint8_t e = c_site[i - 96];
            my_site[c] = (uint32_t)(((e & 3) + 1) | ((((e >> 2) & 3) + 1) << 4) | (((e >> 4) + 1) << 8));
        }
    }

    const long long total = MODE == 0 ? (long long)P.R * P.Pc : (long long)P.B;
    const long long ntiles = (total + kThreads - 1) / kThreads;
    for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const long long w = tile * kThreads + tid;
        const bool valid = w < total;
        int r = 0;
        long long q = 0;
        uint32_t pidx = 0, t = 0, stream = 0;
        uint32_t bnd0 = 0, bnd1 = 0, bnd2 = 0, ao = 0, bo = 0;
        float k4 = 0.f;
        int o0 = 0, o1 = 0, o2 = 0, par = 0;
        if (MODE == 0) {
            // ------------------------------------------------------- 1. decode --------
            if (valid) {
                r = (int)(w / P.Pc);
                q = w - (long long)r * P.Pc;
                const int half1 = P.P1 >> 1;
                const int tt = (int)(q % half1);
                const long long row = q / half1;
                const int pj = (int)(row % P.P2), pk = (int)(row / P.P2);
                const int pi = 2 * tt + ((P.cls + pj + pk) & 1);
                pidx = (uint32_t)(pi + P.P1 * (pj + P.P2 * pk));
                t = P.lstep[r];
                stream = P.stream_id[r];
                const U4 ow = draw(0xFFFFFFFFu, t, stream, kLearn | (0xFFu << 8), P.seed);
                const int ox = (int)(ow.x & 3u), oy = (int)((ow.x >> 2) & 3u), oz = (int)((ow.x >> 4) & 3u);
                par = (ox + oy + oz) & 1;
                o0 = 4 * pi + ox;
                o1 = 4 * pj + oy;
                o2 = 4 * pk + oz;
                k4 = P.k4[P.slot_of_rep[r]];
            }
            s_org[tid] = (uint32_t)o0 | ((uint32_t)o1 << 10) | ((uint32_t)o2 << 20) | ((uint32_t)par << 30);
            s_rep[tid] = valid ? r : -1;
            __syncthreads();
            // ------------------------------------------------------- 2. gather --------
#pragma unroll 4
            for (int j = 0; j < 32; ++j) {
                const int pp = warp * 32 + j;
                const int rr = s_rep[pp];
                if (rr < 0) continue;  // warp-uniform
                const uint32_t og = s_org[pp];
                const int g0 = (int)(og & 1023u), g1 = (int)((og >> 10) & 1023u), g2 = (int)((og >> 20) & 1023u);
                const int gp = (int)(og >> 30);
                const uint8_t *sp = P.spins + (long long)rr * 2 * P.half;
                uint32_t v[5];
#pragma unroll
                for (int c = 0; c < 5; ++c) {
                    const uint32_t e = my_site[c];
                    v[c] = sp[site_addr(P, g0, g1, g2, gp, (int)(e & 15u) - 1, (int)((e >> 4) & 15u) - 1,
                                        (int)(e >> 8) - 1)];
                }
#pragma unroll
                for (int c = 0; c < 5; ++c) {
                    const uint32_t m = __ballot_sync(0xffffffffu, v[c] != 0);
                    if (lane == c) s_bits[pp * 5 + c] = m;
                }
            }
            __syncthreads();
            if (valid) {
                bnd0 = s_bits[tid * 5 + 0];
                bnd1 = s_bits[tid * 5 + 1];
                bnd2 = s_bits[tid * 5 + 2];
                ao = s_bits[tid * 5 + 3];
                bo = s_bits[tid * 5 + 4];
            }
        }
        // ------------------------------------------------------------- 3. input row ------
#pragma unroll 1
        for (int ch = 0; ch < 16; ++ch) {
            uint32_t pk4[4];
            if (MODE == 1) {
                if (valid) {
                    const uint4 v = reinterpret_cast<const uint4 *>(P.X + (size_t)w * NI)[ch];
                    pk4[0] = v.x; pk4[1] = v.y; pk4[2] = v.z; pk4[3] = v.w;
                } else {
                    pk4[0] = pk4[1] = pk4[2] = pk4[3] = 0u;
                }
            } else {
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    float v0 = 0.f, v1 = 0.f;
                    const int i0 = ch * 8 + 2 * h, i1 = i0 + 1;
                    if (valid) {
                        if (i0 < 96) {
                            const uint32_t wd = i0 < 32 ? bnd0 : (i0 < 64 ? bnd1 : bnd2);
                            v0 = ((wd >> (i0 & 31)) & 1u) ? 1.0f : -1.0f;
                            v1 = ((wd >> (i1 & 31)) & 1u) ? 1.0f : -1.0f;
                        } else if (i0 == 96) {
                            v0 = k4;
                        }
                    }
                    const __nv_bfloat162 bv = __floats2bfloat162_rn(v0, v1);
                    pk4[h] = *reinterpret_cast<const uint32_t *>(&bv);
                }
            }
            const int k = ch * 8;
            uint8_t *dst = arow + (k >> 6) * 16384 + tc::swz(tid, k & 63);
            *reinterpret_cast<uint4 *>(dst) = make_uint4(pk4[0], pk4[1], pk4[2], pk4[3]);
        }
        // --------------------------------------------------------------- 4. layers -------
        float z[32];
#pragma unroll 1
        for (int layer = 0; layer < 3 && ok; ++layer) {
            tc::fence_proxy_async();
            tc::fence_before();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after();
                const int n = layer == 2 ? NO : NH;
                const uint32_t idesc = tc::make_idesc(128, n);
                const uint32_t sw = layer == 0 ? sW1 : (layer == 1 ? sW2 : sW3);
                const uint32_t wtile = (uint32_t)n * 128u;  // bytes of one 64-column tile of W
                const uint32_t dcol = layer == 1 ? 128u : 0u;
#pragma unroll
                for (int kk = 0; kk < 8; ++kk) {
                    const uint32_t ao_ = (uint32_t)(kk >> 2) * 16384u + (uint32_t)(kk & 3) * 32u;
                    const uint32_t bo_ = (uint32_t)(kk >> 2) * wtile + (uint32_t)(kk & 3) * 32u;
                    tc::umma(tmem + dcol, tc::make_desc(sA + ao_), tc::make_desc(sw + bo_), idesc, kk > 0 ? 1u : 0u);
                }
                tc::umma_commit(tc::smem_u32(bar));
            }
            const bool got = tc::mbar_wait(tc::smem_u32(bar), phase, P.err, 1);
            phase ^= 1u;
            ok = __syncthreads_and(got ? 1 : 0) != 0;
            if (!ok) break;
            tc::fence_after();
            if (layer < 2) {
                // bias, ReLU, BF16, back into the A tile as the next layer's input
                const uint32_t dcol = layer == 1 ? 128u : 0u;
                const float *bl = bias + layer * 128;
#pragma unroll 1
                for (int cc = 0; cc < 4; ++cc) {
                    uint32_t v[32];
                    tc::tmem_ld32(lane_base + dcol + 32u * cc, v);
                    tc::tmem_wait_ld();
#pragma unroll
                    for (int g = 0; g < 4; ++g) {
                        uint32_t pk4[4];
#pragma unroll
                        for (int h = 0; h < 4; ++h) {
                            const int c0 = 8 * g + 2 * h;
                            const float a0 = fmaxf(__uint_as_float(v[c0]) + bl[32 * cc + c0], 0.0f);
                            const float a1 = fmaxf(__uint_as_float(v[c0 + 1]) + bl[32 * cc + c0 + 1], 0.0f);
                            const __nv_bfloat162 bv = __floats2bfloat162_rn(a0, a1);
                            pk4[h] = *reinterpret_cast<const uint32_t *>(&bv);
                        }
                        const int k = 32 * cc + 8 * g;
                        uint8_t *dst = arow + (k >> 6) * 16384 + tc::swz(tid, k & 63);
                        *reinterpret_cast<uint4 *>(dst) = make_uint4(pk4[0], pk4[1], pk4[2], pk4[3]);
                    }
                }
            } else {
                uint32_t v[32];
                tc::tmem_ld32(lane_base, v);
                tc::tmem_wait_ld();
#pragma unroll
                for (int k = 0; k < 32; ++k) z[k] = __uint_as_float(v[k]) + bias[256 + k];
            }
        }
        if (!ok) break;
        tc::fence_before();  // TMEM reads done before the next tile's MMAs (barrier at its layer 0)
        if (!valid) continue;
        if (MODE == 1) {
            float *zo = P.Z + (size_t)w * NO;
#pragma unroll
            for (int k = 0; k < 32; ++k) zo[k] = z[k];
            continue;
        }
        if (P.dump) {
            float *zo = P.dump + ((size_t)r * P.Pc + q) * NO;
#pragma unroll
            for (int k = 0; k < 32; ++k) zo[k] = z[k];
        }
        // ---------------------------------------------- 5. Metropolis-Hastings step ----
        // d = log q(new) - log q(old): A-sites that changed add +-z_k (log-odds), then the
        // B-sites' heat-bath log probabilities (tables); log alpha = (0 - d) - beta J dB.
        const int slot = P.slot_of_rep[r];
        const uint32_t *TB = P.TB + 7 * slot;
        const float *LBup = P.LBup + 7 * slot, *LBdn = P.LBdn + 7 * slot;
        uint32_t an = 0, bn = 0;
        float d = 0.0f;
        U4 rw{0, 0, 0, 0};
#pragma unroll
        for (int k = 0; k < 32; ++k) {
            if ((k & 3) == 0) rw = draw(pidx, t, stream, kLearn | ((uint32_t)(k >> 2) << 16), P.seed);
            const uint32_t u = (k & 3) == 0 ? rw.x : (k & 3) == 1 ? rw.y : (k & 3) == 2 ? rw.z : rw.w;
            const bool up = u < thr_of_logit(z[k]);
            an |= (up ? 1u : 0u) << k;
            if (up != (((ao >> k) & 1u) != 0)) d += up ? z[k] : -z[k];
        }
        int bond_n = 0, bond_o = 0;
#pragma unroll
        for (int m = 0; m < 32; ++m) {
            if ((m & 3) == 0) rw = draw(pidx, t, stream, kLearn | ((uint32_t)(8 + (m >> 2)) << 16), P.seed);
            const uint32_t u = (m & 3) == 0 ? rw.x : (m & 3) == 1 ? rw.y : (m & 3) == 2 ? rw.z : rw.w;
            // up-neighbour counts (the heat-bath table index (n + 6) / 2)
            int qn = 0, qo = 0;
#pragma unroll
            for (int qq = 0; qq < 6; ++qq) {
                const int cd = geo_bn(m, qq);
                if (cd >= 0) {
                    qn += (int)((an >> cd) & 1u);
                    qo += (int)((ao >> cd) & 1u);
                } else {
                    const int bi = -cd - 1;
                    const uint32_t wd = bi < 32 ? bnd0 : (bi < 64 ? bnd1 : bnd2);
                    const int sb = (int)((wd >> (bi & 31)) & 1u);
                    qn += sb;
                    qo += sb;
                }
            }
            const int nn = 2 * qn - 6, no = 2 * qo - 6;
            const bool up = u < TB[qn];
            bn |= (up ? 1u : 0u) << m;
            const bool upo = ((bo >> m) & 1u) != 0;
            const float lbn = up ? LBup[qn] : LBdn[qn];
            const float lbo = upo ? LBup[qo] : LBdn[qo];
            d += lbn - lbo;
            bond_n += (up ? 1 : -1) * nn;
            bond_o += (upo ? 1 : -1) * no;
        }
#pragma unroll
        for (int k = 0; k < 32; ++k) {
            int sb = 0;
#pragma unroll
            for (int qq = 0; qq < 6; ++qq) {
                const int bi = geo_ab(k, qq);
                if (bi < 0) continue;
                const uint32_t wd = bi < 32 ? bnd0 : (bi < 64 ? bnd1 : bnd2);
                sb += ((wd >> (bi & 31)) & 1u) ? 1 : -1;
            }
            bond_n += (((an >> k) & 1u) ? 1 : -1) * sb;
            bond_o += (((ao >> k) & 1u) ? 1 : -1) * sb;
        }
        rw = draw(pidx, t, stream, kLearn | (16u << 16), P.seed);
        const float la = (0.0f - d) - P.betaJf[slot] * (float)(bond_n - bond_o);
        bool acc = la >= 0.0f;
        if (!acc) acc = u01(rw.x) < expf_neg(la);
        if (acc) {
            uint8_t *sp = P.spins + (long long)r * 2 * P.half;
            for (int k = 0; k < 32; ++k) {
                const uint8_t e = c_site[k], f = c_site[32 + k];
                sp[site_addr(P, o0, o1, o2, par, e & 3, (e >> 2) & 3, e >> 4)] = (uint8_t)((an >> k) & 1u);
                sp[site_addr(P, o0, o1, o2, par, f & 3, (f >> 2) & 3, f >> 4)] = (uint8_t)((bn >> k) & 1u);
            }
            atomicAdd(P.acc + r, 1ull);
        }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
    }
}

// ------------------------------------------------------------------ training data ----
// n samples per replica: a random offset and patch, its network input (BF16) and A-site bits.
__global__ void collect_kernel(const uint8_t *__restrict__ spins, int L1, int L2, int L3, int H,
                               long long half, int R, int per_rep, const uint32_t *__restrict__ stream_id,
                               const int32_t *__restrict__ slot_of_rep, const float *__restrict__ k4,
                               uint32_t seed, uint32_t call, __nv_bfloat16 *__restrict__ X,
                               uint32_t *__restrict__ Y, long long write0, long long cap) {
    const long long total = (long long)R * per_rep;
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < total;
         w += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(w / per_rep), s = (int)(w - (long long)r * per_rep);
        const U4 d = draw((uint32_t)s, call, stream_id[r], kLearn | (0xFEu << 8), seed);
        const int ox = (int)(d.x & 3u), oy = (int)((d.x >> 2) & 3u), oz = (int)((d.x >> 4) & 3u);
        const int par = (ox + oy + oz) & 1;
        const int o0 = 4 * (int)(d.y % (uint32_t)(L1 / 4)) + ox;
        const int o1 = 4 * (int)(d.z % (uint32_t)(L2 / 4)) + oy;
        const int o2 = 4 * (int)(d.w % (uint32_t)(L3 / 4)) + oz;
        const uint8_t *sp = spins + (long long)r * 2 * half;
        PatchParams P;
        P.L1 = L1; P.L2 = L2; P.L3 = L3; P.H = H; P.half = half;
        const long long row = (write0 + w) % cap;
        __nv_bfloat16 *xr = X + (size_t)row * NI;
        for (int i = 0; i < 96; ++i) {
            const uint16_t e = c_bnd[i];
            const int a = (int)(e & 15u) - 1, b = (int)((e >> 4) & 15u) - 1, c = (int)(e >> 8) - 1;
            xr[i] = __float2bfloat16_rn(sp[site_addr(P, o0, o1, o2, par, a, b, c)] ? 1.0f : -1.0f);
        }
        xr[96] = __float2bfloat16_rn(k4[slot_of_rep[r]]);
        for (int i = 97; i < NI; ++i) xr[i] = __float2bfloat16_rn(0.0f);
        uint32_t ab = 0;
        for (int k = 0; k < 32; ++k) {
            const uint8_t e = c_site[k];
            ab |= (uint32_t)sp[site_addr(P, o0, o1, o2, par, e & 3, (e >> 2) & 3, e >> 4)] << k;
        }
        Y[row] = ab;
    }
}

// --------------------------------------------------------------- training kernels ----
// C (M x N, ldc) = beta C + sum_k A(m, k) B(k, n), A(m, k) = ta ? A[k lda + m] : A[m lda + k],
// B(k, n) = tb ? B[n ldb + k] : B[k ldb + n].  64 x 64 tiles, 16 x 16 threads of 4 x 4, K in
// steps of 16; fixed summation order.
__global__ void __launch_bounds__(256)
gemm_kernel(int M, int N, int K, const float *__restrict__ A, int lda, int ta, const float *__restrict__ B,
            int ldb, int tb, float *__restrict__ C, int ldc, float beta) {
    __shared__ float As[16][68], Bs[16][68];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int e = threadIdx.x; e < 16 * 64; e += 256) {
            const int kk = e >> 6, mm = e & 63;
            const int m = m0 + mm, k = k0 + kk;
            float va = 0.f;
            if (m < M && k < K) va = ta ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
            As[kk][mm] = va;
            const int n = n0 + mm;
            float vb = 0.f;
            if (n < N && k < K) vb = tb ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n];
            Bs[kk][mm] = vb;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
            if (m < M && n < N) {
                float *c = C + (size_t)m * ldc + n;
                *c = beta == 0.f ? acc[i][j] : fmaf(beta, *c, acc[i][j]);
            }
        }
}

__device__ __forceinline__ float bf16r(float f) { return __bfloat162float(__float2bfloat16_rn(f)); }

// minibatch: rows of the data set chosen by Philox, BF16 -> FP32, targets as 0/1
__global__ void batch_kernel(const __nv_bfloat16 *__restrict__ X, const uint32_t *__restrict__ Y,
                             long long n, int B, uint32_t seed, uint32_t step, float *__restrict__ Xb,
                             float *__restrict__ Yb) {
    const int b = blockIdx.x;
    if (b >= B) return;
    __shared__ long long row;
    if (threadIdx.x == 0) {
        const U4 d = draw((uint32_t)b, step, 0x4C524E00u, kLearn | (0xFDu << 8), seed);
        row = (long long)((((unsigned long long)d.y << 32) | d.x) % (unsigned long long)n);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NI; i += blockDim.x) Xb[(size_t)b * NI + i] = __bfloat162float(X[(size_t)row * NI + i]);
    for (int i = threadIdx.x; i < NO; i += blockDim.x) Yb[(size_t)b * NO + i] = (float)((Y[row] >> i) & 1u);
}

__global__ void quantise_kernel(const float *__restrict__ p, float *__restrict__ q, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const bool is_bias = (i >= OFF_B1 && i < OFF_W2) || (i >= OFF_B2 && i < OFF_W3) || i >= OFF_B3;
        q[i] = is_bias ? p[i] : bf16r(p[i]);
    }
}

__global__ void bias_relu_kernel(float *__restrict__ Hm, const float *__restrict__ b, int rows, int cols) {
    const long long n = (long long)rows * cols;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        Hm[i] = bf16r(fmaxf(Hm[i] + b[i % cols], 0.0f));
}

// logits += b3; dZ = (sigmoid - y) / B; loss += softplus(z) - y z (block sums, one atomic each)
__global__ void bce_kernel(float *__restrict__ Zm, const float *__restrict__ b3, const float *__restrict__ Yb,
                           float *__restrict__ dZ, int B, double *__restrict__ loss) {
    __shared__ double red[256];
    double s = 0.0;
    const int n = B * NO;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float zz = Zm[i] + b3[i % NO];
        const float y = Yb[i];
        const float p = 1.0f / (1.0f + expf(-zz));
        dZ[i] = (p - y) / (float)B;
        const float sp = zz > 0.0f ? zz + log1pf(expf(-zz)) : log1pf(expf(zz));
        s += (double)(sp - y * zz);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0] / B);
}

__global__ void colsum_kernel(const float *__restrict__ D, int rows, int cols, float *__restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.f;
    for (int r = 0; r < rows; ++r) s += D[(size_t)r * cols + c];
    out[c] = s;
}

__global__ void relu_mask_kernel(float *__restrict__ dH, const float *__restrict__ Hm, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (!(Hm[i] > 0.0f)) dH[i] = 0.0f;
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, int n, float lr, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = 0.9f * m[i] + 0.1f * gi;
        const float vi = 0.999f * v[i] + 0.001f * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
    }
}

// inference image: quantised weights as BF16 in the swizzled K-major tiles, biases FP32
__global__ void pack_kernel(const float *__restrict__ q, uint8_t *__restrict__ img) {
    const int total = NH * NI + NH * NH + NO * NH;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        int base, rows, off, idx = e;
        if (idx < NH * NI) { base = IMG_W1; rows = NH; off = OFF_W1; }
        else if ((idx -= NH * NI) < NH * NH) { base = IMG_W2; rows = NH; off = OFF_W2; }
        else { idx -= NH * NH; base = IMG_W3; rows = NO; off = OFF_W3; }
        const int n = idx / NI, k = idx % NI;
        const uint32_t o = (uint32_t)base + (uint32_t)(k >> 6) * (uint32_t)(rows * 128) + tc::swz(n, k & 63);
        *reinterpret_cast<__nv_bfloat16 *>(img + o) = __float2bfloat16_rn(q[off + idx]);
    }
    float *bf = reinterpret_cast<float *>(img + IMG_B1);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NH + NH + NO; i += gridDim.x * blockDim.x)
        bf[i] = i < NH ? q[OFF_B1 + i] : (i < 2 * NH ? q[OFF_B2 + i - NH] : q[OFF_B3 + i - 2 * NH]);
}

__global__ void advance_lstep_kernel(uint32_t *c, int R) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < R) c[r] += 1u;
}

static bool closed_forms_agree(const Geometry &g) {
    for (int m = 0; m < 32; ++m) {
        for (int q = 0; q < 6; ++q)
            if (geo_bn(m, q) != g.Bn[m][q]) return false;
        int n = 0;
        for (int q = 0; q < 6; ++q) {
            const int bi = geo_ab(m, q);
            if (bi >= 0 && (n >= 3 || g.Ab[m][n++] != bi)) return false;
        }
        if (n < 3 && g.Ab[m][n] != -1) return false;
        if ((g.site[m] & 3) != geo_a_a(m) || (g.site[32 + m] & 3) != geo_b_a(m)) return false;
    }
    return true;
}

}  // namespace learn
}  // namespace ether

using namespace ether;
using namespace ether::learn;

struct ether_learn {
    ether_ctx *ctx = nullptr;
    learn::XyzLearn *xyz = nullptr;  // an XYZ context's learner (k_learn_xyz.cu); the rest unused
    uint32_t seed = 0;
    int R = 0, L[3] = {0, 0, 0}, P[3] = {0, 0, 0};
    long long Pc = 0, half = 0;
    double J = 0.0;
    // parameters (device): master, quantised, gradient, Adam moments; inference image
    float *p = nullptr, *pq = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    uint8_t *img = nullptr;
    int adam_t = 0;
    // data set
    __nv_bfloat16 *X = nullptr;
    uint32_t *Y = nullptr;
    long long cap = 0, n = 0, write = 0;
    uint32_t collect_calls = 0;
    // training scratch (max batch)
    int maxB = 0;
    float *Xb = nullptr, *Yb = nullptr, *H1 = nullptr, *H2 = nullptr, *Z = nullptr, *dZ = nullptr,
          *dH1 = nullptr, *dH2 = nullptr;
    double *loss = nullptr;
    // sweeps
    uint32_t *lstep = nullptr;
    float *k4 = nullptr, *betaJf = nullptr, *LBup = nullptr, *LBdn = nullptr;
    uint32_t *TB = nullptr;
    unsigned long long *acc = nullptr;
    float *dump = nullptr;
    bool dump_on = false;
    std::vector<double> tables_for;  // beta slots the tables were built for
    int *err = nullptr;
    int sm_count = 0;
    uint64_t launches = 0, proposed = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float sweep_ms = 0.f, train_ms = 0.f;
    int timed = 0;  // 1: sweep, 2: train pending in e0/e1
    int timed_n = 0;
};

namespace {

int lfail(int code, const std::string &msg) {
    set_error(msg);
    return code;
}

#define LCUDA(expr)                                                                          \
    do {                                                                                     \
        cudaError_t _e = (expr);                                                             \
        if (_e != cudaSuccess)                                                               \
            return lfail(_e == cudaErrorMemoryAllocation ? ETHER_ERR_NOMEM : ETHER_ERR_CUDA,  \
                         std::string(#expr) + ": " + cudaGetErrorString(_e));                \
    } while (0)

bool g_geometry_uploaded = false;

int upload_geometry() {
    if (g_geometry_uploaded) return ETHER_OK;
    const Geometry g = make_geometry();
    if (!closed_forms_agree(g)) return lfail(ETHER_ERR_CUDA, "learned proposal: inconsistent patch geometry");
    LCUDA(cudaMemcpyToSymbol(c_site, g.site, sizeof g.site));
    LCUDA(cudaMemcpyToSymbol(c_bnd, g.bnd, sizeof g.bnd));
    g_geometry_uploaded = true;
    return ETHER_OK;
}

float bf16_host(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    std::memcpy(&f, &u, 4);
    return f;
}

// Per temperature slot: 4 beta J (BF16-exact), beta J (FP32), heat-bath thresholds and logs.
int refresh_tables(ether_learn &l) {
    const Ctx &c = l.ctx->c;
    if (l.tables_for == c.beta_slots) return ETHER_OK;
    const int S = c.n_slots;
    std::vector<float> k4(S), bj(S), lu(7 * S), ld(7 * S);
    std::vector<uint32_t> tb(7 * S);
    for (int s = 0; s < S; ++s) {
        const double betaJ = c.beta_slots[s] * l.J;
        k4[s] = bf16_host((float)(4.0 * betaJ));
        bj[s] = (float)betaJ;
        for (int qi = 0; qi < 7; ++qi) {
            const int nsum = 2 * qi - 6;
            const double pu = 1.0 / (1.0 + std::exp(2.0 * betaJ * nsum));
            double t = std::floor(pu * 4294967296.0 + 0.5);
            t = std::min(std::max(t, 1.0), 4294967295.0);
            tb[7 * s + qi] = (uint32_t)t;
            lu[7 * s + qi] = (float)std::log(t / 4294967296.0);
            ld[7 * s + qi] = (float)std::log((4294967296.0 - t) / 4294967296.0);
        }
    }
    cudaFree(l.k4); cudaFree(l.betaJf); cudaFree(l.TB); cudaFree(l.LBup); cudaFree(l.LBdn);
    l.k4 = l.betaJf = l.LBup = l.LBdn = nullptr;
    l.TB = nullptr;
    LCUDA(cudaMalloc((void **)&l.k4, S * sizeof(float)));
    LCUDA(cudaMalloc((void **)&l.betaJf, S * sizeof(float)));
    LCUDA(cudaMalloc((void **)&l.TB, 7 * S * sizeof(uint32_t)));
    LCUDA(cudaMalloc((void **)&l.LBup, 7 * S * sizeof(float)));
    LCUDA(cudaMalloc((void **)&l.LBdn, 7 * S * sizeof(float)));
    LCUDA(cudaMemcpy(l.k4, k4.data(), S * sizeof(float), cudaMemcpyHostToDevice));
    LCUDA(cudaMemcpy(l.betaJf, bj.data(), S * sizeof(float), cudaMemcpyHostToDevice));
    LCUDA(cudaMemcpy(l.TB, tb.data(), 7 * S * sizeof(uint32_t), cudaMemcpyHostToDevice));
    LCUDA(cudaMemcpy(l.LBup, lu.data(), 7 * S * sizeof(float), cudaMemcpyHostToDevice));
    LCUDA(cudaMemcpy(l.LBdn, ld.data(), 7 * S * sizeof(float), cudaMemcpyHostToDevice));
    l.tables_for = c.beta_slots;
    return ETHER_OK;
}

int quantise_and_pack(ether_learn &l, cudaStream_t st) {
    quantise_kernel<<<64, 256, 0, st>>>(l.p, l.pq, NPARAM);
    pack_kernel<<<64, 256, 0, st>>>(l.pq, l.img);
    l.launches += 2;
    LCUDA(cudaGetLastError());
    return ETHER_OK;
}

int ensure_batch(ether_learn &l, int B) {
    if (B <= l.maxB) return ETHER_OK;
    float **bufs[] = {&l.Xb, &l.Yb, &l.H1, &l.H2, &l.Z, &l.dZ, &l.dH1, &l.dH2};
    const size_t cols[] = {NI, NO, NH, NH, NO, NO, NH, NH};
    for (int i = 0; i < 8; ++i) {
        cudaFree(*bufs[i]);
        *bufs[i] = nullptr;
        LCUDA(cudaMalloc((void **)bufs[i], (size_t)B * cols[i] * sizeof(float)));
    }
    l.maxB = B;
    return ETHER_OK;
}

void gemm(cudaStream_t st, int M, int N, int K, const float *A, int lda, int ta, const float *B, int ldb,
          int tb, float *C, int ldc) {
    dim3 grid((N + 63) / 64, (M + 63) / 64);
    gemm_kernel<<<grid, 256, 0, st>>>(M, N, K, A, lda, ta, B, ldb, tb, C, ldc, 0.f);
}

// Forward and backward of a batch already in Xb / Yb; gradients into l.g, mean loss added to *l.loss.
int forward_backward(ether_learn &l, int B, cudaStream_t st) {
    const float *W1 = l.pq + OFF_W1, *W2 = l.pq + OFF_W2, *W3 = l.pq + OFF_W3;
    gemm(st, B, NH, NI, l.Xb, NI, 0, W1, NI, 1, l.H1, NH);
    bias_relu_kernel<<<256, 256, 0, st>>>(l.H1, l.pq + OFF_B1, B, NH);
    gemm(st, B, NH, NH, l.H1, NH, 0, W2, NH, 1, l.H2, NH);
    bias_relu_kernel<<<256, 256, 0, st>>>(l.H2, l.pq + OFF_B2, B, NH);
    gemm(st, B, NO, NH, l.H2, NH, 0, W3, NH, 1, l.Z, NO);
    bce_kernel<<<64, 256, 0, st>>>(l.Z, l.pq + OFF_B3, l.Yb, l.dZ, B, l.loss);
    gemm(st, NO, NH, B, l.dZ, NO, 1, l.H2, NH, 0, l.g + OFF_W3, NH);
    colsum_kernel<<<1, 128, 0, st>>>(l.dZ, B, NO, l.g + OFF_B3);
    gemm(st, B, NH, NO, l.dZ, NO, 0, W3, NH, 0, l.dH2, NH);
    relu_mask_kernel<<<256, 256, 0, st>>>(l.dH2, l.H2, (long long)B * NH);
    gemm(st, NH, NH, B, l.dH2, NH, 1, l.H1, NH, 0, l.g + OFF_W2, NH);
    colsum_kernel<<<1, 128, 0, st>>>(l.dH2, B, NH, l.g + OFF_B2);
    gemm(st, B, NH, NH, l.dH2, NH, 0, W2, NH, 0, l.dH1, NH);
    relu_mask_kernel<<<256, 256, 0, st>>>(l.dH1, l.H1, (long long)B * NH);
    gemm(st, NH, NI, B, l.dH1, NH, 1, l.Xb, NI, 0, l.g + OFF_W1, NI);
    colsum_kernel<<<1, 128, 0, st>>>(l.dH1, B, NH, l.g + OFF_B1);
    l.launches += 17;
    LCUDA(cudaGetLastError());
    return ETHER_OK;
}

int read_err(ether_learn &l) {
    int e = 0;
    LCUDA(cudaMemcpy(&e, l.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        cudaMemset(l.err, 0, sizeof(int));
        return lfail(ETHER_ERR_TIMEOUT, "learned-proposal kernel: a bounded tensor-core wait ran out (code " +
                                            std::to_string(e) + ")");
    }
    return ETHER_OK;
}

int launch_patches(ether_learn &l, int cls, float *dump) {
    Ctx &c = l.ctx->c;
    PatchParams P;
    std::memset(&P, 0, sizeof(P));
    P.img = l.img;
    P.err = l.err;
    P.spins = c.spins;
    P.L1 = l.L[0]; P.L2 = l.L[1]; P.L3 = l.L[2]; P.H = l.L[0] / 2;
    P.half = l.half;
    P.P1 = l.P[0]; P.P2 = l.P[1]; P.P3 = l.P[2];
    P.cls = cls;
    P.Pc = l.Pc;
    P.R = l.R;
    P.stream_id = c.stream_id;
    P.lstep = l.lstep;
    P.slot_of_rep = c.slot_of_rep;
    P.k4 = l.k4; P.betaJf = l.betaJf; P.TB = l.TB; P.LBup = l.LBup; P.LBdn = l.LBdn;
    P.seed = c.seed;
    P.acc = l.acc;
    P.dump = dump;
    const long long tiles = ((long long)l.R * l.Pc + kThreads - 1) / kThreads;
    const int grid = (int)std::max<long long>(1, std::min<long long>(tiles, 2LL * l.sm_count));
    patch_kernel<0><<<grid, kThreads, SM_BYTES + 1024, c.stream>>>(P);
    l.launches++;
    LCUDA(cudaGetLastError());
    return ETHER_OK;
}

}  // namespace

extern "C" int ether_learn_create(ether_ctx *h, const ether_learn_desc *d, ether_learn **out) {
    if (!out) return lfail(ETHER_ERR_ARG, "null output handle");
    *out = nullptr;
    if (!h || !d) return lfail(ETHER_ERR_ARG, "null context or descriptor");
    Ctx &c = h->c;
    if (d->patch != 4 || d->hidden != 128)
        return lfail(ETHER_ERR_UNSUPPORTED, "learned proposal: patch 4 and hidden width 128 only");
    if (c.model == ETHER_MODEL_XYZ) {
        learn::XyzLearn *x = nullptr;
        const int rc = learn::xyz_create(h, d, &x);
        if (rc) return rc;
        ether_learn *l = new ether_learn();
        l->ctx = h;
        l->xyz = x;
        *out = l;
        return ETHER_OK;
    }
    // c.L is set once the lattice is verified to be the periodic simple-cubic one (whose
    // storage is the checkerboard split the kernels address arithmetically)
    if (c.model != ETHER_MODEL_ISING || c.L[0] <= 0 || c.nsp != 1 || c.nsh != 1 || c.zeeman)
        return lfail(ETHER_ERR_UNSUPPORTED, "learned proposal: simple-cubic Ising, one species, one shell, no Zeeman term");
    if (c.L[0] % 8 || c.L[1] % 8 || c.L[2] % 8 || c.L[0] > 1016 || c.L[1] > 1016 || c.L[2] > 1016)
        return lfail(ETHER_ERR_UNSUPPORTED, "learned proposal: every extent a multiple of 8, at most 1016");
    if (d->capacity < 1024) return lfail(ETHER_ERR_ARG, "training capacity below 1024 samples");
    int rc = upload_geometry();
    if (rc) return rc;
    ether_learn *l = new ether_learn();
    l->ctx = h;
    l->seed = d->seed;
    l->R = c.R;
    for (int a = 0; a < 3; ++a) {
        l->L[a] = c.L[a];
        l->P[a] = c.L[a] / 4;
    }
    l->Pc = (long long)l->P[0] * l->P[1] * l->P[2] / 2;
    l->half = (long long)(c.L[0] / 2) * c.L[1] * c.L[2];
    l->J = c.h_Jd[2];
    l->cap = d->capacity;
    auto fail_free = [&](cudaError_t e) {
        ether_learn_destroy(l);
        return lfail(e == cudaErrorMemoryAllocation ? ETHER_ERR_NOMEM : ETHER_ERR_CUDA,
                     std::string("learned proposal set-up: ") + cudaGetErrorString(e));
    };
    cudaError_t e = cudaSuccess;
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&l->sm_count, cudaDevAttrMultiProcessorCount, dev);
    float **pb[] = {&l->p, &l->pq, &l->g, &l->m, &l->v};
    for (float **b : pb)
        if (e == cudaSuccess) e = cudaMalloc((void **)b, NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&l->img, IMG_BYTES);
    if (e == cudaSuccess) e = cudaMalloc((void **)&l->X, (size_t)l->cap * NI * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc((void **)&l->Y, (size_t)l->cap * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc((void **)&l->loss, sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void **)&l->lstep, l->R * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc((void **)&l->acc, l->R * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc((void **)&l->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(l->lstep, 0, l->R * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(l->acc, 0, l->R * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(l->err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(l->m, 0, NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(l->v, 0, NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaEventCreate(&l->e0);
    if (e == cudaSuccess) e = cudaEventCreate(&l->e1);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(patch_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_BYTES + 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(patch_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_BYTES + 1024);
    if (e != cudaSuccess) return fail_free(e);
    // He initialisation (last layer small): the untrained network proposes nearly uniform spins
    std::vector<float> p(NPARAM, 0.f);
    std::mt19937 gen(d->seed ^ 0x9E3779B9u);
    std::normal_distribution<float> nd(0.f, 1.f);
    for (int i = 0; i < NH * NI; ++i) p[OFF_W1 + i] = nd(gen) * std::sqrt(2.0f / NI);
    for (int i = 0; i < NH * NH; ++i) p[OFF_W2 + i] = nd(gen) * std::sqrt(2.0f / NH);
    for (int i = 0; i < NO * NH; ++i) p[OFF_W3 + i] = nd(gen) * 0.01f;
    e = cudaMemcpy(l->p, p.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail_free(e);
    rc = quantise_and_pack(*l, c.stream);
    if (rc) {
        ether_learn_destroy(l);
        return rc;
    }
    *out = l;
    return ETHER_OK;
}

extern "C" int ether_learn_destroy(ether_learn *l) {
    if (!l) return ETHER_OK;
    if (l->xyz) {
        learn::xyz_destroy(l->xyz);
        delete l;
        return ETHER_OK;
    }
    if (l->ctx) cudaStreamSynchronize(l->ctx->c.stream);
    void *ptrs[] = {l->p, l->pq, l->g, l->m, l->v, l->img, l->X, l->Y, l->Xb, l->Yb, l->H1, l->H2,
                    l->Z, l->dZ, l->dH1, l->dH2, l->loss, l->lstep, l->k4, l->betaJf, l->TB,
                    l->LBup, l->LBdn, l->acc, l->dump, l->err};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (l->e0) cudaEventDestroy(l->e0);
    if (l->e1) cudaEventDestroy(l->e1);
    delete l;
    return ETHER_OK;
}

extern "C" int ether_learn_collect(ether_learn *l, int32_t per_replica) {
    if (!l) return lfail(ETHER_ERR_ARG, "null handle");
    if (per_replica < 1) return lfail(ETHER_ERR_ARG, "samples per replica must be positive");
    Ctx &c = l->ctx->c;
    if (!c.beta_set) return lfail(ETHER_ERR_STATE, "beta not set");
    if (l->xyz) return learn::xyz_collect(l->xyz, per_replica);
    int rc = refresh_tables(*l);
    if (rc) return rc;
    const long long total = (long long)l->R * per_replica;
    const int grid = (int)std::min<long long>((total + 255) / 256, 4LL * l->sm_count);
    collect_kernel<<<grid, 256, 0, c.stream>>>(c.spins, l->L[0], l->L[1], l->L[2], l->L[0] / 2, l->half,
                                               l->R, per_replica, c.stream_id, c.slot_of_rep, l->k4,
                                               c.seed, l->collect_calls, l->X, l->Y, l->write, l->cap);
    LCUDA(cudaGetLastError());
    l->launches++;
    l->collect_calls++;
    l->write = (l->write + total) % l->cap;
    l->n = std::min(l->cap, l->n + total);
    return ETHER_OK;
}

extern "C" int ether_learn_train(ether_learn *l, int32_t steps, int32_t batch, float lr, double *loss_out) {
    if (!l) return lfail(ETHER_ERR_ARG, "null handle");
    if (steps < 0 || batch < 1 || batch > 65536 || !(lr > 0.f)) return lfail(ETHER_ERR_ARG, "bad training arguments");
    if (l->xyz) return learn::xyz_train(l->xyz, steps, batch, lr, loss_out);
    if (l->n == 0) return lfail(ETHER_ERR_STATE, "no training samples (ether_learn_collect)");
    int rc = ensure_batch(*l, batch);
    if (rc) return rc;
    cudaStream_t st = l->ctx->c.stream;
    LCUDA(cudaEventRecord(l->e0, st));
    for (int s = 0; s < steps; ++s) {
        LCUDA(cudaMemsetAsync(l->loss, 0, sizeof(double), st));
        batch_kernel<<<batch, 128, 0, st>>>(l->X, l->Y, l->n, batch, l->seed, (uint32_t)(l->adam_t + 1), l->Xb, l->Yb);
        l->launches++;
        rc = forward_backward(*l, batch, st);
        if (rc) return rc;
        ++l->adam_t;
        const float c1 = 1.0f - std::pow(0.9f, (float)l->adam_t), c2 = 1.0f - std::pow(0.999f, (float)l->adam_t);
        adam_kernel<<<64, 256, 0, st>>>(l->p, l->g, l->m, l->v, NPARAM, lr, c1, c2);
        quantise_kernel<<<64, 256, 0, st>>>(l->p, l->pq, NPARAM);
        l->launches += 2;
    }
    rc = quantise_and_pack(*l, st);
    if (rc) return rc;
    LCUDA(cudaEventRecord(l->e1, st));
    if (loss_out) {
        LCUDA(cudaMemcpyAsync(loss_out, l->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
        LCUDA(cudaStreamSynchronize(st));
    }
    l->timed = 2;
    return ETHER_OK;
}

extern "C" int ether_learn_sweep(ether_learn *l, int32_t nsweeps) {
    if (!l) return lfail(ETHER_ERR_ARG, "null handle");
    if (nsweeps < 0) return lfail(ETHER_ERR_ARG, "negative sweep count");
    Ctx &c = l->ctx->c;
    if (!c.beta_set) return lfail(ETHER_ERR_STATE, "beta not set");
    if (l->xyz) return learn::xyz_sweep(l->xyz, nsweeps);
    int rc = refresh_tables(*l);
    if (rc) return rc;
    if (l->dump_on && !l->dump)
        LCUDA(cudaMalloc((void **)&l->dump, 2 * (size_t)l->R * l->Pc * NO * sizeof(float)));
    LCUDA(cudaEventRecord(l->e0, c.stream));
    for (int s = 0; s < nsweeps; ++s) {
        for (int cls = 0; cls < 2; ++cls) {
            float *dump = (l->dump_on && s == nsweeps - 1) ? l->dump + (size_t)cls * l->R * l->Pc * NO : nullptr;
            rc = launch_patches(*l, cls, dump);
            if (rc) return rc;
        }
        advance_lstep_kernel<<<(l->R + 255) / 256, 256, 0, c.stream>>>(l->lstep, l->R);
        l->launches++;
        l->proposed += 2ull * (uint64_t)l->R * (uint64_t)l->Pc;
    }
    LCUDA(cudaEventRecord(l->e1, c.stream));
    LCUDA(cudaGetLastError());
    l->timed = 1;
    l->timed_n = nsweeps;
    return ETHER_OK;
}

extern "C" int ether_learn_batch_sweep(ether_learn *const *learns, int32_t n, int32_t nsweeps,
                                       int32_t plain_per_sweep) {
    if (!learns || n <= 0 || nsweeps < 0 || plain_per_sweep < 0) return lfail(ETHER_ERR_ARG, "invalid argument");
    for (int k = 0; k < n; ++k) {
        if (!learns[k]) return lfail(ETHER_ERR_ARG, "null learner");
        if (!learns[k]->ctx->c.beta_set) return lfail(ETHER_ERR_STATE, "beta not set");
        for (int j = 0; j < k; ++j)
            if (learns[j]->ctx == learns[k]->ctx) return lfail(ETHER_ERR_ARG, "two learners of one context");
    }
    // step s of every context before step s + 1 of any: each context's stream gets its own
    // work in order, the contexts run side by side
    for (int s = 0; s < nsweeps; ++s)
        for (int k = 0; k < n; ++k) {
            for (int p = 0; p < plain_per_sweep; ++p) {
                const int rc = plain_sweep(learns[k]->ctx->c);
                if (rc) return rc;
            }
            const int rc = ether_learn_sweep(learns[k], 1);
            if (rc) return rc;
        }
    return ETHER_OK;
}

extern "C" int ether_learn_record_series(ether_learn *l, int32_t nsteps, int32_t plain_per_step,
                                         int32_t learned_per_step, int32_t stride, double *absM) {
    if (!l || !absM) return lfail(ETHER_ERR_ARG, "null argument");
    if (nsteps < 1 || plain_per_step < 0 || learned_per_step < 0 || plain_per_step + learned_per_step < 1 ||
        stride < 1 || nsteps / stride < 1)
        return lfail(ETHER_ERR_ARG, "need nsteps >= stride >= 1 and at least one sweep per step");
    Ctx &c = l->ctx->c;
    if (!c.beta_set) return lfail(ETHER_ERR_STATE, "beta not set");
    if (l->xyz) return learn::xyz_record_series(l->xyz, nsteps, plain_per_step, learned_per_step, stride, absM);
    int rc = refresh_tables(*l);
    if (rc) return rc;
    const int nrec = nsteps / stride;
    const size_t bytes = sizeof(double) * (size_t)nrec * l->R;
    double *mser = nullptr;
    LCUDA(cudaMalloc((void **)&mser, bytes));
    for (int t = 0; t < nsteps && rc == ETHER_OK; ++t) {
        for (int k = 0; k < plain_per_step && rc == ETHER_OK; ++k) rc = plain_sweep(c);
        for (int k = 0; k < learned_per_step && rc == ETHER_OK; ++k) {
            for (int cls = 0; cls < 2 && rc == ETHER_OK; ++cls) rc = launch_patches(*l, cls, nullptr);
            if (rc == ETHER_OK) {
                advance_lstep_kernel<<<(l->R + 255) / 256, 256, 0, c.stream>>>(l->lstep, l->R);
                l->launches++;
                l->proposed += 2ull * (uint64_t)l->R * (uint64_t)l->Pc;
            }
        }
        if (rc == ETHER_OK && (t + 1) % stride == 0 && (t + 1) / stride <= nrec) {
            const cudaError_t e = launch_record(c, (t + 1) / stride - 1, false, mser, nullptr);
            if (e != cudaSuccess) rc = lfail(ETHER_ERR_CUDA, std::string("record: ") + cudaGetErrorString(e));
        }
    }
    if (rc == ETHER_OK) {
        cudaError_t e = cudaMemcpyAsync(absM, mser, bytes, cudaMemcpyDeviceToHost, c.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) rc = lfail(ETHER_ERR_CUDA, std::string("series copy: ") + cudaGetErrorString(e));
    }
    cudaFree(mser);
    if (rc) return rc;
    return read_err(*l);
}

extern "C" int ether_learn_get_accepts(ether_learn *l, uint64_t *accepted) {
    if (!l || !accepted) return lfail(ETHER_ERR_ARG, "null argument");
    if (l->xyz) return learn::xyz_get_accepts(l->xyz, accepted);
    LCUDA(cudaMemcpyAsync(accepted, l->acc, l->R * sizeof(uint64_t), cudaMemcpyDeviceToHost, l->ctx->c.stream));
    LCUDA(cudaStreamSynchronize(l->ctx->c.stream));
    return read_err(*l);
}

extern "C" int ether_learn_set_dump(ether_learn *l, int32_t on) {
    if (!l) return lfail(ETHER_ERR_ARG, "null handle");
    if (l->xyz) learn::xyz_set_dump(l->xyz, on != 0);
    l->dump_on = on != 0;
    return ETHER_OK;
}

extern "C" int ether_learn_get_dump(ether_learn *l, float *logits) {
    if (!l || !logits) return lfail(ETHER_ERR_ARG, "null argument");
    if (l->xyz) return learn::xyz_get_dump(l->xyz, logits);
    if (!l->dump) return lfail(ETHER_ERR_STATE, "no logits recorded (ether_learn_set_dump, then a sweep)");
    LCUDA(cudaMemcpyAsync(logits, l->dump, 2 * (size_t)l->R * l->Pc * NO * sizeof(float),
                          cudaMemcpyDeviceToHost, l->ctx->c.stream));
    LCUDA(cudaStreamSynchronize(l->ctx->c.stream));
    return read_err(*l);
}

extern "C" int ether_learn_get_params(ether_learn *l, float *params) {
    if (!l || !params) return lfail(ETHER_ERR_ARG, "null argument");
    if (l->xyz) return learn::xyz_get_params(l->xyz, params);
    LCUDA(cudaMemcpyAsync(params, l->p, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, l->ctx->c.stream));
    LCUDA(cudaStreamSynchronize(l->ctx->c.stream));
    return ETHER_OK;
}

extern "C" int ether_learn_set_params(ether_learn *l, const float *params) {
    if (!l || !params) return lfail(ETHER_ERR_ARG, "null argument");
    if (l->xyz) return learn::xyz_set_params(l->xyz, params);
    for (int i = 0; i < NPARAM; ++i)
        if (!std::isfinite(params[i])) return lfail(ETHER_ERR_ARG, "non-finite parameter " + std::to_string(i));
    cudaStream_t st = l->ctx->c.stream;
    LCUDA(cudaMemcpyAsync(l->p, params, NPARAM * sizeof(float), cudaMemcpyHostToDevice, st));
    LCUDA(cudaMemsetAsync(l->m, 0, NPARAM * sizeof(float), st));
    LCUDA(cudaMemsetAsync(l->v, 0, NPARAM * sizeof(float), st));
    l->adam_t = 0;
    int rc = quantise_and_pack(*l, st);
    if (rc) return rc;
    LCUDA(cudaStreamSynchronize(st));
    return ETHER_OK;
}

extern "C" int ether_learn_loss_grad(ether_learn *l, const float *x, const uint32_t *y, int32_t B,
                                     double *loss, float *grad) {
    if (!l || !x || !y || !grad) return lfail(ETHER_ERR_ARG, "null argument");
    if (B < 1 || B > 65536) return lfail(ETHER_ERR_ARG, "batch out of range");
    if (l->xyz) return lfail(ETHER_ERR_UNSUPPORTED, "XYZ learner: targets are spin components (ether_learn_loss_grad_f)");
    int rc = ensure_batch(*l, B);
    if (rc) return rc;
    cudaStream_t st = l->ctx->c.stream;
    std::vector<float> yf((size_t)B * NO);
    for (int b = 0; b < B; ++b)
        for (int o = 0; o < NO; ++o) yf[(size_t)b * NO + o] = (float)((y[b] >> o) & 1u);
    LCUDA(cudaMemcpyAsync(l->Xb, x, (size_t)B * NI * sizeof(float), cudaMemcpyHostToDevice, st));
    LCUDA(cudaMemcpyAsync(l->Yb, yf.data(), (size_t)B * NO * sizeof(float), cudaMemcpyHostToDevice, st));
    LCUDA(cudaMemsetAsync(l->loss, 0, sizeof(double), st));
    rc = forward_backward(*l, B, st);
    if (rc) return rc;
    double lv = 0.0;
    LCUDA(cudaMemcpyAsync(&lv, l->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
    LCUDA(cudaMemcpyAsync(grad, l->g, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, st));
    LCUDA(cudaStreamSynchronize(st));
    if (loss) *loss = lv;
    return ETHER_OK;
}

extern "C" int ether_learn_forward(ether_learn *l, const float *x, int32_t B, float *logits) {
    if (!l || !x || !logits) return lfail(ETHER_ERR_ARG, "null argument");
    if (B < 1 || B > (1 << 22)) return lfail(ETHER_ERR_ARG, "batch out of range");
    if (l->xyz) return learn::xyz_forward(l->xyz, x, B, logits);
    cudaStream_t st = l->ctx->c.stream;
    std::vector<__nv_bfloat16> xb((size_t)B * NI);
    for (size_t i = 0; i < xb.size(); ++i) xb[i] = __float2bfloat16_rn(x[i]);
    __nv_bfloat16 *dX = nullptr;
    float *dZ = nullptr;
    LCUDA(cudaMalloc((void **)&dX, xb.size() * sizeof(__nv_bfloat16)));
    cudaError_t e = cudaMalloc((void **)&dZ, (size_t)B * NO * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dX, xb.data(), xb.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        PatchParams P;
        std::memset(&P, 0, sizeof(P));
        P.img = l->img;
        P.err = l->err;
        P.X = dX;
        P.B = B;
        P.Z = dZ;
        const int tiles = (B + kThreads - 1) / kThreads;
        patch_kernel<1><<<std::min(tiles, 2 * l->sm_count), kThreads, SM_BYTES + 1024, st>>>(P);
        l->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(logits, dZ, (size_t)B * NO * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dX);
    cudaFree(dZ);
    if (e != cudaSuccess) return lfail(ETHER_ERR_CUDA, std::string("learned forward: ") + cudaGetErrorString(e));
    return read_err(*l);
}

extern "C" int ether_learn_get_info(ether_learn *l, ether_learn_info *info) {
    if (!l || !info) return lfail(ETHER_ERR_ARG, "null argument");
    if (l->xyz) return learn::xyz_info(l->xyz, info);
    if (l->timed) {
        float ms = 0.f;
        LCUDA(cudaEventSynchronize(l->e1));
        LCUDA(cudaEventElapsedTime(&ms, l->e0, l->e1));
        if (l->timed == 1) l->sweep_ms = l->timed_n > 0 ? ms / l->timed_n : 0.f;
        else l->train_ms = ms;
        l->timed = 0;
    }
    int rc = read_err(*l);
    if (rc) return rc;
    info->n_params = NPARAM;
    info->patches_per_class = l->Pc;
    info->n_samples = l->n;
    info->capacity = l->cap;
    info->train_steps = l->adam_t;
    info->proposed = l->proposed;
    info->kernel_launches = l->launches;
    info->last_sweep_ms = l->sweep_ms;
    info->last_train_ms = l->train_ms;
    return ETHER_OK;
}

extern "C" int ether_learn_loss_grad_f(ether_learn *l, const float *x, const float *y, int32_t B, double *loss,
                                       float *grad) {
    if (!l || !x || !y || !grad) return lfail(ETHER_ERR_ARG, "null argument");
    if (B < 1 || B > 65536) return lfail(ETHER_ERR_ARG, "batch out of range");
    if (l->xyz) return learn::xyz_loss_grad(l->xyz, x, y, B, loss, grad);
    // Ising: targets 0 / 1 per output, packed as the A-site bits
    std::vector<uint32_t> bits((size_t)B, 0u);
    for (int b = 0; b < B; ++b)
        for (int o = 0; o < NO; ++o)
            if (y[(size_t)b * NO + o] > 0.5f) bits[b] |= 1u << o;
    return ether_learn_loss_grad(l, x, bits.data(), B, loss, grad);
}

extern "C" int ether_learn_get_shape(ether_learn *l, int32_t *n_inputs, int32_t *n_outputs, int32_t *n_params) {
    if (!l || !n_inputs || !n_outputs || !n_params) return lfail(ETHER_ERR_ARG, "null argument");
    int ni = NI, no = NO, np = NPARAM;
    if (l->xyz) learn::xyz_shape(&ni, &no, &np);
    *n_inputs = ni;
    *n_outputs = no;
    *n_params = np;
    return ETHER_OK;
}
