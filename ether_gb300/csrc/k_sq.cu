// k_sq.cu -- structure factor S(q) (utility/Structure_Factor/structure_factor.f90:99-183) on
// a 3-D grid of q, as a dense (q x sites) x (sites x spin components) contraction on the
// fifth-generation tensor cores.
//
//   D[2q + c, 3r + a] = sum_i A[2q + c, i] B[i, 3r + a],  A = cos / sin (q.r_i),  B = S_{r,i,a}
//
// Both operands are split into BF16 high and low parts (x = hi + lo, lo = bf16(x - hi)) and
// D = A_hi B_hi + A_hi B_lo + A_lo B_hi is accumulated in FP32 in tensor memory: about 16
// significant bits per product instead of BF16's 8.
//
// Ising spins are +-1 along z: B_lo is identically zero and the x, y components vanish, so
// the Ising form (ISING = true) keeps one column per replica (S_z; up to 256 replicas per
// pass instead of 85), loads no B_lo tile and issues two products per K-step
// (A_hi B_hi + A_lo B_hi) instead of three.
//
// One CTA owns a 128-row tile of D (64 q-points: consecutive h1 at fixed h2, h3) and all
// 3R columns (<= 256).  Per 64-site k-block:
//   * warps 0-7 generate the A tile in shared memory.  Warp w takes sites 8w .. 8w+7 (one
//     16-byte chunk of every row), lane l the site 8w + l/4 and the q-points h1_0 + 4a + l%4
//     (a = 0..15): phase factors
//       exp(i q.r) = E1[h1_0 + l%4][i] * E2[h2][i] * E3[h3][i] * b4_i^a,  b4_i = exp(2 pi i 4 dq_1 u_i)
//     (complex FP32 from FP64-built tables, 15 steps of the recurrence), split into hi/lo
//     BF16 pairs (cos, sin) and written four 8x8 blocks at a time with stmatrix.trans into the
//     K-major 128-byte-swizzled layout the MMA descriptors describe;
//   * one thread of warp 8 loads the B_hi / B_lo tiles with TMA (same swizzle) and issues the
//     12 tcgen05.mma (3 products x 4 K-steps of 16), then tcgen05.commit to the stage's
//     "empty" barrier;
//   * two stages: A generation and TMA of block k+1 overlap the MMAs of block k.
// Epilogue: warps 0-7 read the accumulator with tcgen05.ld (warp w owns TMEM lanes 32(w%4)..),
// pair cos/sin rows with a lane shuffle and write |S(q)|^2 / N^2 and |S_a(q)| / N.
//
// Every mbarrier wait is bounded (%globaltimer, 2 s): on expiry the kernel records an error
// code and stops issuing work; the issuing thread waits (bounded) for the TMA copies it
// started, every thread waits for the MMAs issued so far (the `done` commit), and the TMEM is
// freed only once those have completed.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <string>
#include <vector>

#include "internal.h"
#include "tc_util.cuh"

namespace ether {
namespace sq {

constexpr int kBM = 128;        // rows per tile (64 q-points x cos/sin)
constexpr int kBK = 64;         // sites per k-block (128 bytes of BF16)
constexpr int kStages = 2;
constexpr int kProducers = 256; // warps 0-7
constexpr int kThreads = 288;   // + warp 8 (TMA + MMA issue)

struct Smem {
    // stage s: A_hi, A_lo (kBM x kBK bf16 each), B_hi, B_lo (BN x kBK bf16 each)
    // laid out from a 1024-byte aligned base; barriers at the end
    static constexpr int a_bytes = kBM * kBK * 2;  // 16 KB
};

using namespace tc;

// Instruction descriptor for this kernel's M = 128 tiles.
__host__ __device__ constexpr uint32_t make_idesc(int n) { return tc::make_idesc(kBM, n); }

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int c0, int c1, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(map), "r"(c0), "r"(c1), "r"(bar) : "memory");
}

struct Cplx {
    float re, im;
};
__device__ __forceinline__ Cplx cmul(Cplx a, Cplx b) {
    return Cplx{fmaf(a.re, b.re, -(a.im * b.im)), fmaf(a.re, b.im, a.im * b.re)};
}

struct SqParams {
    int nk;            // k-blocks
    int M1, M2, M3;    // q-grid extents (M1 % 64 == 0)
    int N;             // sites (true count)
    int Kpad;          // sites padded to kBK
    int R;             // replicas in this launch
    int BN;            // columns (3R, or R for Ising, padded to 16)
    const float2 *E1;  // [M1/64][4][Kpad]  exp(2 pi i (q0_1 + (64 t + p) dq_1) u_i)
    const float2 *E2;  // [M2][Kpad]
    const float2 *E3;  // [M3][Kpad]
    const float2 *bb;  // [Kpad]            exp(2 pi i 4 dq_1 u_i)
    float *sq;         // [R][Q]
    float *comp;       // [R][Q][3]
    int *err;
};

template <bool ISING>
__global__ void __launch_bounds__(kThreads, 1)
sq_kernel(const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo,
          SqParams P) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int b_bytes = P.BN * kBK * 2;
    constexpr int nb = ISING ? 1 : 2;                          // B tiles per stage: hi (, lo)
    const int stage_bytes = 2 * Smem::a_bytes + nb * b_bytes;  // multiple of 1024 (BN % 16 == 0 -> b_bytes % 2048 == 0)
    uint8_t *bar_area = base + kStages * stage_bytes;
    uint64_t *full = reinterpret_cast<uint64_t *>(bar_area);
    uint64_t *empty = full + kStages;
    uint64_t *done = empty + kStages;
    uint64_t *tmab = done + 1;  // per stage: the two B-tile copies have landed
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(tmab + kStages);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tile = blockIdx.x;
    const int tiles1 = P.M1 / 64;
    const int t1 = tile % tiles1, h2 = (tile / tiles1) % P.M2, h3 = tile / (tiles1 * P.M2);
    const int h1_0 = t1 * 64;

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(smem_u32(&full[s]), kProducers);
            mbar_init(smem_u32(&empty[s]), 1);
            mbar_init(smem_u32(&tmab[s]), 1);
        }
        mbar_init(smem_u32(done), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == kProducers / 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;
    bool ok = true;

    if (warp < kProducers / 32) {
        // ------------------------------------------------------------- producers ----------
        // lane = (site i = 8 warp + lane / 4 of the k-block, q-phase ph = lane % 4): q-points
        // h1_0 + 4a + ph, rows 8a + 2ph (cos) and 8a + 2ph + 1 (sin) = rows 2ph, 2ph + 1 of
        // atom a.  stmatrix.trans stores thread t's register (low, high) = (cos, sin) of site
        // t / 4 at rows 2(t % 4), 2(t % 4) + 1 of an 8x8 block, whose row r lane 8m + r
        // addresses (block m of the x4 = atom 4g + m); the rows are 16-byte chunks `warp` of
        // the swizzled rows.
        const int i = 8 * warp + (lane >> 2);
        const int ph = lane & 3;
        const int xr = lane & 7;
        const uint32_t rowoff = (uint32_t)((lane >> 3) * 1024 + xr * 128 + ((warp ^ xr) << 4));
        const size_t e1row = ((size_t)(h1_0 >> 6) * 4 + ph) * P.Kpad;
        const size_t e2row = (size_t)h2 * P.Kpad, e3row = (size_t)h3 * P.Kpad;
        // phase factors of the first k-block, then prefetched one block ahead
        float2 e1 = P.E1[e1row + i], e2 = P.E2[e2row + i], e3 = P.E3[e3row + i], bq = P.bb[i];
        for (int kb = 0; kb < P.nk && ok; ++kb) {
            const int s = kb & 1, f = kb >> 1;
            const Cplx p23 = cmul(Cplx{e2.x, e2.y}, Cplx{e3.x, e3.y});
            Cplx z = cmul(Cplx{e1.x, e1.y}, p23);
            const Cplx b{bq.x, bq.y};
            if (kb + 1 < P.nk) {
                const int nxt = (kb + 1) * kBK + i;
                e1 = P.E1[e1row + nxt];
                e2 = P.E2[e2row + nxt];
                e3 = P.E3[e3row + nxt];
                bq = P.bb[nxt];
            }
            // stmatrix is warp-collective: the warp goes on only if every lane's wait succeeded
            if (f >= 1 && !__all_sync(0xffffffffu, mbar_wait(smem_u32(&empty[s]), (f - 1) & 1, P.err, 1))) {
                ok = false;
                break;
            }
            const uint32_t a_hi = smem_u32(base + s * stage_bytes) + rowoff;
            const uint32_t a_lo = a_hi + Smem::a_bytes;
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                uint32_t hi[4], lo[4];
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    const __nv_bfloat162 h = __floats2bfloat162_rn(z.re, z.im);
                    const __nv_bfloat162 l = __floats2bfloat162_rn(z.re - __low2float(h), z.im - __high2float(h));
                    hi[m] = *reinterpret_cast<const uint32_t *>(&h);
                    lo[m] = *reinterpret_cast<const uint32_t *>(&l);
                    z = cmul(z, b);
                }
                const uint32_t o = (uint32_t)(g * 4 * 1024);
                asm volatile("stmatrix.sync.aligned.m8n8.x4.trans.shared.b16 [%0], {%1, %2, %3, %4};"
                             ::"r"(a_hi + o), "r"(hi[0]), "r"(hi[1]), "r"(hi[2]), "r"(hi[3]) : "memory");
                asm volatile("stmatrix.sync.aligned.m8n8.x4.trans.shared.b16 [%0], {%1, %2, %3, %4};"
                             ::"r"(a_lo + o), "r"(lo[0]), "r"(lo[1]), "r"(lo[2]), "r"(lo[3]) : "memory");
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(smem_u32(&full[s]));
        }
    } else if (lane == 0) {
        // ------------------------------------------------------- TMA + MMA issue --------
        const uint32_t idesc = make_idesc(P.BN);
        const uint32_t tx = (uint32_t)nb * (uint32_t)b_bytes;
        auto issue_tma = [&](int kb) -> bool {
            const int s = kb & 1, f = kb >> 1;
            if (f >= 1 && !mbar_wait(smem_u32(&empty[s]), (f - 1) & 1, P.err, 2)) return false;
            uint8_t *b_hi = base + s * stage_bytes + 2 * Smem::a_bytes;
            uint8_t *b_lo = b_hi + b_bytes;
            mbar_arrive_tx(smem_u32(&tmab[s]), tx);
            tma_load_2d(smem_u32(b_hi), &map_hi, kb * kBK, 0, smem_u32(&tmab[s]));
            if (!ISING) tma_load_2d(smem_u32(b_lo), &map_lo, kb * kBK, 0, smem_u32(&tmab[s]));
            return true;
        };
        int issued = 0;
        int tma_next = 0;    // k-blocks whose copies were started: 0 .. tma_next - 1
        int tma_waited = 0;  // k-blocks whose copies were seen complete: 0 .. tma_waited - 1
        if (P.nk > 0) {
            ok = issue_tma(0);
            tma_next = ok ? 1 : 0;
        }
        for (int kb = 0; kb < P.nk && ok; ++kb) {
            if (kb + 1 < P.nk) {
                if (!issue_tma(kb + 1)) { ok = false; break; }
                tma_next = kb + 2;
            }
            const int s = kb & 1, f = kb >> 1;
            if (!mbar_wait(smem_u32(&tmab[s]), f & 1, P.err, 3)) { ok = false; break; }
            tma_waited = kb + 1;
            if (!mbar_wait(smem_u32(&full[s]), f & 1, P.err, 3)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t a_hi = smem_u32(base + s * stage_bytes);
            const uint32_t a_lo = a_hi + Smem::a_bytes;
            const uint32_t b_hi = a_hi + 2 * Smem::a_bytes;
            const uint32_t b_lo = b_hi + b_bytes;
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {
                const uint32_t o = kk * 32;  // 16 BF16 along K
                umma(tmem, make_desc(a_hi + o), make_desc(b_hi + o), idesc, (kb | kk) ? 1u : 0u);
                if (!ISING) umma(tmem, make_desc(a_hi + o), make_desc(b_lo + o), idesc, 1u);
                umma(tmem, make_desc(a_lo + o), make_desc(b_hi + o), idesc, 1u);
            }
            umma_commit(smem_u32(&empty[s]));
            ++issued;
        }
        // after a failed wait: the copies already started still write into this block's
        // shared memory, so wait for them (bounded) before the block can exit
        for (int kb = tma_waited; kb < tma_next; ++kb)
            mbar_wait(smem_u32(&tmab[kb & 1]), (kb >> 1) & 1, P.err, 5);
        umma_commit(smem_u32(done));  // arrives once everything issued above has completed
    }

    // ------------------------------------------------------------------ epilogue ------
    __syncwarp();
    const bool fin = mbar_wait(smem_u32(done), 0, P.err, 4);
    asm volatile("tcgen05.fence::after_thread_sync;");
    // tcgen05.ld is warp-collective: the whole warp reads, or none of it does
    const bool go = __all_sync(0xffffffffu, fin && ok) && *(volatile int *)P.err == 0;
    if (warp < kProducers / 32 && __all_sync(0xffffffffu, go)) {
        // warp w reads TMEM lanes 32 (w % 4) ..; warps w and w + 4 share the rows and split
        // the replicas between them
        const int Q = P.M1 * P.M2 * P.M3;
        const int wl = warp & 3;
        const int row = wl * 32 + lane;    // TMEM lane = D row
        const int qloc = row >> 1;         // rows 2q, 2q+1 = cos, sin
        const int q = h1_0 + qloc + P.M1 * (h2 + P.M2 * h3);
        const float invN = 1.0f / (float)P.N;
        if (ISING) {
            // column r = S_z of replica r: four replicas per TMEM load
            for (int r0 = 4 * (warp >> 2); r0 < P.R; r0 += 4 * (kProducers / 128)) {
                uint32_t v[4];
                const uint32_t taddr = tmem + ((uint32_t)(wl * 32) << 16) + (uint32_t)r0;
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                             : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]) : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float mine = __uint_as_float(v[j]);
                    const float other = __shfl_xor_sync(0xffffffffu, mine, 1);
                    const float m2 = mine * mine + other * other;
                    if ((lane & 1) == 0 && r0 + j < P.R) {
                        P.sq[(size_t)(r0 + j) * Q + q] = m2 * invN * invN;
                        float *c = P.comp + ((size_t)(r0 + j) * Q + q) * 3;
                        c[0] = 0.f;
                        c[1] = 0.f;
                        c[2] = sqrtf(m2) * invN;
                    }
                }
            }
        }
        for (int r = warp >> 2; !ISING && r < P.R; r += kProducers / 128) {
            uint32_t v[4];
            const uint32_t taddr = tmem + ((uint32_t)(wl * 32) << 16) + (uint32_t)(3 * r);
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]) : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float tot = 0.f, mag[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float mine = __uint_as_float(v[a]);
                const float other = __shfl_xor_sync(0xffffffffu, mine, 1);
                const float m2 = mine * mine + other * other;  // Re^2 + Im^2
                tot += m2;
                mag[a] = sqrtf(m2) * invN;
            }
            if ((lane & 1) == 0) {
                P.sq[(size_t)r * Q + q] = tot * invN * invN;
                float *c = P.comp + ((size_t)r * Q + q) * 3;
                c[0] = mag[0];
                c[1] = mag[1];
                c[2] = mag[2];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == kProducers / 32) {
        // the MMAs write the TMEM until `done` arrives: free it only after that (one more
        // bounded wait if the first one ran out)
        const bool drained = __all_sync(0xffffffffu, fin || mbar_wait(smem_u32(done), 0, P.err, 6));
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (drained) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
    }
}

// B = spins in BF16 hi / lo, [BN rows = 3r + a][Kpad sites] (sites in storage order).
__global__ void sq_prep_b(const uint8_t *__restrict__ spins, const float4 *__restrict__ spins4,
                          int model, int N, int Kpad, int r0, int R, int BN,
                          __nv_bfloat16 *__restrict__ bhi, __nv_bfloat16 *__restrict__ blo) {
    const long total = (long)BN * Kpad;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
        const int n = (int)(e / Kpad), k = (int)(e - (long)n * Kpad);
        // Ising: one row per replica (S_z); XYZ: rows 3r + a
        const int r = model == 0 ? n : n / 3, a = model == 0 ? 2 : n - 3 * r;
        float x = 0.f;
        if (r < R && k < N) {
            if (model == 0) x = spins[(size_t)(r0 + r) * N + k] ? 1.f : -1.f;
            else {
                const float4 S = spins4[(size_t)(r0 + r) * N + k];
                x = a == 0 ? S.x : a == 1 ? S.y : S.z;
            }
        }
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        bhi[e] = h;
        blo[e] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
}

}  // namespace sq
}  // namespace ether

using namespace ether;
using namespace ether::sq;

namespace ether {
// The driver's cuTensorMapEncodeTiled, looked up once through the runtime (no -lcuda).
void *tma_encode_tiled_fn() {
    static void *fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = p;
    }
    return fn;
}
}  // namespace ether

namespace {
PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ether::tma_encode_tiled_fn());
}
}  // namespace

namespace ether {
// Host driver for ether_structure_factor (declared in the C-ABI, defined in ether_api.cu
// through this function).
int structure_factor_launch(Ctx &c, const double *frac /*3N, storage order*/, const int nq[3],
                            const double q0[3], const double dq[3], float *sq_host,
                            float *comp_host, std::string &msg) {
    const int N = c.N;
    const int Kpad = (N + kBK - 1) / kBK * kBK;
    const int M1 = nq[0], M2 = nq[1], M3 = nq[2];
    const long Q = (long)M1 * M2 * M3;
    if (M1 <= 0 || M2 <= 0 || M3 <= 0 || M1 % 64 != 0) { msg = "nq[0] must be a positive multiple of 64, nq[1], nq[2] positive"; return ETHER_ERR_ARG; }
    if (Q * 2 > 0x7FFFFFFFL) { msg = "q-grid too large"; return ETHER_ERR_ARG; }
    PFN_cuTensorMapEncodeTiled_v12000 encode = get_encode();
    if (!encode) { msg = "cuTensorMapEncodeTiled not available"; return ETHER_ERR_CUDA; }
    // phase tables in FP64 on the host
    const double tp = 2.0 * M_PI;
    // E1 row 4t + p: the phase at h1 = 64t + p (the first q-point of q-phase p of tile t)
    std::vector<float2> E1((size_t)(M1 / 16) * Kpad, make_float2(0.f, 0.f));
    std::vector<float2> E2((size_t)M2 * Kpad, make_float2(0.f, 0.f)), E3((size_t)M3 * Kpad, make_float2(0.f, 0.f));
    std::vector<float2> bb(Kpad, make_float2(1.f, 0.f));
    for (int i = 0; i < N; ++i) {
        const double u = frac[3 * i], v = frac[3 * i + 1], w = frac[3 * i + 2];
        for (int m = 0; m < M1 / 16; ++m) {
            const double ph = tp * (q0[0] + (64.0 * (m >> 2) + (m & 3)) * dq[0]) * u;
            E1[(size_t)m * Kpad + i] = make_float2((float)cos(ph), (float)sin(ph));
        }
        for (int h = 0; h < M2; ++h) {
            const double ph = tp * (q0[1] + h * dq[1]) * v;
            E2[(size_t)h * Kpad + i] = make_float2((float)cos(ph), (float)sin(ph));
        }
        for (int h = 0; h < M3; ++h) {
            const double ph = tp * (q0[2] + h * dq[2]) * w;
            E3[(size_t)h * Kpad + i] = make_float2((float)cos(ph), (float)sin(ph));
        }
        const double ph = tp * 4.0 * dq[0] * u;
        bb[i] = make_float2((float)cos(ph), (float)sin(ph));
    }
    const bool ising = c.model == ETHER_MODEL_ISING;
    const int cols = ising ? 1 : 3;            // TMEM columns per replica
    const int rmax = ising ? 256 : 85;         // 3 * 85 = 255 <= 256 columns of TMEM per pass
    float2 *dE1 = nullptr, *dE2 = nullptr, *dE3 = nullptr, *dbb = nullptr;
    __nv_bfloat16 *bhi = nullptr, *blo = nullptr;
    float *dsq = nullptr, *dcomp = nullptr;
    int *derr = nullptr;
    int rc = ETHER_OK;
    const int rpass = std::min(c.R, rmax);
    const int BNmax = (cols * rpass + 15) / 16 * 16;
    auto cleanup = [&]() {
        cudaFree(dE1); cudaFree(dE2); cudaFree(dE3); cudaFree(dbb); cudaFree(bhi); cudaFree(blo);
        cudaFree(dsq); cudaFree(dcomp); cudaFree(derr);
    };
#define SQ_TRY(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { msg = std::string(#x) + ": " + cudaGetErrorString(e_); cleanup(); return ETHER_ERR_CUDA; } } while (0)
    SQ_TRY(cudaMalloc(&dE1, E1.size() * sizeof(float2)));
    SQ_TRY(cudaMalloc(&dE2, E2.size() * sizeof(float2)));
    SQ_TRY(cudaMalloc(&dE3, E3.size() * sizeof(float2)));
    SQ_TRY(cudaMalloc(&dbb, bb.size() * sizeof(float2)));
    SQ_TRY(cudaMalloc(&bhi, (size_t)BNmax * Kpad * 2));
    SQ_TRY(cudaMalloc(&blo, (size_t)BNmax * Kpad * 2));
    SQ_TRY(cudaMalloc(&dsq, (size_t)rpass * Q * sizeof(float)));
    SQ_TRY(cudaMalloc(&dcomp, (size_t)rpass * Q * 3 * sizeof(float)));
    SQ_TRY(cudaMalloc(&derr, sizeof(int)));
    SQ_TRY(cudaMemcpyAsync(dE1, E1.data(), E1.size() * sizeof(float2), cudaMemcpyHostToDevice, c.stream));
    SQ_TRY(cudaMemcpyAsync(dE2, E2.data(), E2.size() * sizeof(float2), cudaMemcpyHostToDevice, c.stream));
    SQ_TRY(cudaMemcpyAsync(dE3, E3.data(), E3.size() * sizeof(float2), cudaMemcpyHostToDevice, c.stream));
    SQ_TRY(cudaMemcpyAsync(dbb, bb.data(), bb.size() * sizeof(float2), cudaMemcpyHostToDevice, c.stream));
    for (int r0 = 0; r0 < c.R && rc == ETHER_OK; r0 += rpass) {
        const int R = std::min(rpass, c.R - r0);
        const int BN = (cols * R + 15) / 16 * 16;
        SQ_TRY(cudaMemsetAsync(derr, 0, sizeof(int), c.stream));
        sq_prep_b<<<std::max(1, std::min(4096, (int)(((long)BN * Kpad + 255) / 256))), 256, 0, c.stream>>>(
            c.spins, c.spins4, c.model, N, Kpad, r0, R, BN, bhi, blo);
        c.launches++;
        CUtensorMap mh, ml;
        cuuint64_t gdim[2] = {(cuuint64_t)Kpad, (cuuint64_t)BN};
        cuuint64_t gstride[1] = {(cuuint64_t)Kpad * 2};
        cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)BN};
        cuuint32_t estride[2] = {1, 1};
        CUresult cr = encode(&mh, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, bhi, gdim, gstride, box, estride,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (cr == CUDA_SUCCESS)
            cr = encode(&ml, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, blo, gdim, gstride, box, estride,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (cr != CUDA_SUCCESS) { msg = "cuTensorMapEncodeTiled failed"; cleanup(); return ETHER_ERR_CUDA; }
        SqParams P;
        P.nk = Kpad / kBK;
        P.M1 = M1; P.M2 = M2; P.M3 = M3;
        P.N = N; P.Kpad = Kpad; P.R = R; P.BN = BN;
        P.E1 = dE1; P.E2 = dE2; P.E3 = dE3; P.bb = dbb;
        P.sq = dsq; P.comp = dcomp; P.err = derr;
        const int stage_bytes = 2 * Smem::a_bytes + (ising ? 1 : 2) * BN * kBK * 2;
        const int smem = 1024 + kStages * stage_bytes + 64;
        auto kern = ising ? sq_kernel<true> : sq_kernel<false>;
        SQ_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        const int tiles = (int)(Q / 64);
        cudaEvent_t ev0, ev1;
        SQ_TRY(cudaEventCreate(&ev0));
        SQ_TRY(cudaEventCreate(&ev1));
        SQ_TRY(cudaEventRecord(ev0, c.stream));
        kern<<<tiles, kThreads, smem, c.stream>>>(mh, ml, P);
        c.launches++;
        SQ_TRY(cudaGetLastError());
        SQ_TRY(cudaEventRecord(ev1, c.stream));
        SQ_TRY(cudaEventSynchronize(ev1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev0, ev1);
        if (r0 == 0) c.sq_ms = 0.f;
        c.sq_ms += ms;
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        int herr = 0;
        SQ_TRY(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        SQ_TRY(cudaMemcpyAsync(sq_host + (size_t)r0 * Q, dsq, (size_t)R * Q * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
        SQ_TRY(cudaMemcpyAsync(comp_host + (size_t)r0 * Q * 3, dcomp, (size_t)R * Q * 3 * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
        SQ_TRY(cudaStreamSynchronize(c.stream));
        if (herr) { msg = "structure-factor kernel: a pipeline wait timed out (stage " + std::to_string(herr) + ")"; rc = ETHER_ERR_TIMEOUT; }
    }
#undef SQ_TRY
    cleanup();
    return rc;
}
}  // namespace ether
