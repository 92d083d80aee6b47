// k_learn_xyz.cu -- learned patch proposal for the simple-cubic Heisenberg (XYZ) model, the
// ether_learn_* functions of an XYZ context.  The reference has no learned move; what it
// fixes is the target distribution exp(-beta E), E = sum over bonds of S_i . (J o S_j) with the
// diagonal exchange (Jxx, Jyy, Jzz) (src/Hamiltonian.f90:57-105, src/Metropolis.f90:50-56),
// and every learned move is accepted or rejected by exact Metropolis-Hastings against it.
//
// Move (patch tiling, classes, offsets and canonical frame as the Ising learner's):
//   * network: input = the 96 boundary spins (3 components each, BF16-rounded) and
//     beta (Jxx, Jyy, Jzz), zero-padded to 304; 128 -> 128 (ReLU, BF16 activations) -> 96;
//     outputs 3k .. 3k+2 (+ bias) are the von Mises-Fisher parameter m_k of A-site k;
//     inference: xmlp_kernel, the three layers on the tensor cores (tcgen05, TMA-loaded
//     inputs, weights resident in shared memory, FP32 accumulators in tensor memory; the
//     hidden layers' bias (BF16) + ReLU + BF16 rounding in the epilogue); training on the FP32
//     GEMM of k_learn.cu;
//   * proposal: A-site k ~ vMF(m_k) (Wood's exact sampler on the sphere, own log / exp /
//     sincos); then every B-site from its exact heat-bath conditional vMF(-beta g), g = J o
//     (sum of its six neighbours: new A-sites and the boundary); a vMF with |m| < 1e-3 is
//     taken as uniform, in the sampler and in the density alike;
//   * acceptance: log alpha = sum over the patch's 64 sites of (-beta E_site - log q_site),
//     new minus old, with E_site the site's bonds to the boundary (A) or to all six
//     neighbours (B); one warp per patch, lane k = A-site k and B-site k, the 32 lane terms
//     summed by a xor butterfly (the order oracle/learn_oracle.c replays bit for bit).
// Training: maximum likelihood of the A-sites given the boundary (vMF negative log density)
// on patches of configurations the plain sweep produced, Adam, straight-through BF16.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "internal.h"
#include "learn_common.cuh"
#include "rng_math.cuh"
#include "tc_util.cuh"

namespace ether {
namespace learn {

constexpr int XNI = 304, XNO = 96;  // 96 x 3 boundary components + beta (Jxx, Jyy, Jzz), padded
constexpr int XOFF_W1 = 0, XOFF_B1 = XOFF_W1 + NH * XNI, XOFF_W2 = XOFF_B1 + NH, XOFF_B2 = XOFF_W2 + NH * NH,
              XOFF_W3 = XOFF_B2 + NH, XOFF_B3 = XOFF_W3 + XNO * NH, XNPARAM = XOFF_B3 + XNO;
constexpr float kKappaMin = 1e-3f;        // below: the vMF is the uniform distribution
constexpr float kLog4Pi = 2.53102425f;    // log(4 pi)
constexpr float kLog2Pi = 1.83787707f;    // log(2 pi)
constexpr float kPi = 3.14159265f;
constexpr long long kChunkPatches = 1LL << 19;  // inference rows per pass

// ------------------------------------------------------------ von Mises-Fisher (own) ----
// The same FP32 operation sequences as oracle/learn_oracle.c (--fmad=false; fmaf explicit).
__host__ __device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    float d = ax * bx;
    d = fmaf(ay, by, d);
    return fmaf(az, bz, d);
}

// 1 - e^{-2 kappa}: Taylor series of 1 - e^{-y} for y = 2 kappa < 1/2 (through y^8:
// truncation < 1e-8 relative), else direct.
__host__ __device__ __forceinline__ float vmf_oneminus(float kappa) {
    const float y = 2.0f * kappa;
    if (y >= 0.5f) return 1.0f - expf_neg(-y);
    float p = 2.48015873e-5f;  // 1/40320
    p = fmaf(p, y, -1.98412698e-4f);
    p = fmaf(p, y, 1.38888889e-3f);
    p = fmaf(p, y, -8.33333333e-3f);
    p = fmaf(p, y, 4.16666667e-2f);
    p = fmaf(p, y, -1.66666667e-1f);
    p = fmaf(p, y, 0.5f);
    p = fmaf(p, y, -1.0f);
    return -(y * p);
}

__host__ __device__ __forceinline__ float rcp_f(float x) {
#if defined(__CUDA_ARCH__)
    return __frcp_rn(x);
#else
    return 1.0f / x;
#endif
}

// A von Mises-Fisher distribution on the unit sphere, vMF(m): kappa = |m|, rk = 1 / kappa,
// log density at x = c + (m . x - kappa) with c = log(kappa / (1 - e^{-2 kappa})) - log 2 pi;
// the uniform distribution (log density -log 4 pi) for kappa < kKappaMin.
struct Vmf {
    float mx, my, mz, kappa, rk, c;
    bool uni;
};
__host__ __device__ __forceinline__ Vmf vmf_prep(float mx, float my, float mz) {
    Vmf V;
    V.mx = mx;
    V.my = my;
    V.mz = mz;
    V.kappa = sqrtf(dot3(mx, my, mz, mx, my, mz));
    V.uni = V.kappa < kKappaMin;
    V.rk = V.uni ? 0.0f : rcp_f(V.kappa);
    V.c = V.uni ? -kLog4Pi : logf_own(V.kappa * rcp_f(vmf_oneminus(V.kappa))) - kLog2Pi;
    return V;
}
__host__ __device__ __forceinline__ float vmf_logpdf(const Vmf &V, float x, float y, float z) {
    return V.uni ? -kLog4Pi : V.c + (dot3(V.mx, V.my, V.mz, x, y, z) - V.kappa);
}

// A sample of vMF from the uniforms u in [0, 1) and v in [-1, 1): Wood's method on the
// sphere, 1 - w = -log(1 - (1 - u)(1 - e^{-2 kappa})) / kappa, azimuth pi v about the mean
// direction; the result is normalised.
__host__ __device__ __forceinline__ void vmf_sample(const Vmf &V, float u, float v, float *ox, float *oy, float *oz) {
    float ux = 0.0f, uy = 0.0f, uz = 1.0f, om;
    if (V.uni) {
        om = 2.0f * (1.0f - u);  // 1 - w: w = 2u - 1, uniform on [-1, 1)
    } else {
        ux = V.mx * V.rk;
        uy = V.my * V.rk;
        uz = V.mz * V.rk;
        om = -log1m_own((1.0f - u) * vmf_oneminus(V.kappa)) * V.rk;
    }
    om = fminf(fmaxf(om, 0.0f), 2.0f);
    const float w = 1.0f - om;
    const float r = sqrtf(om * (2.0f - om));
    // e1 perpendicular to the mean direction, e2 = mean x e1: (-uy, ux, 0) / |.| when
    // |uz| < 0.9, else (0, uz, -uy) / |.| -- one normalisation of the selected vector, so the
    // lanes of a warp do not diverge (the same operations as the two separate branches)
    const bool flat = fabsf(uz) < 0.9f;
    const float pa = flat ? uy : 0.0f, pb = flat ? ux : uz, pc = flat ? 0.0f : uy;
    const float rn = rcp_f(sqrtf(dot3(pa, pb, pc, pa, pb, pc)));
    const float e1x = flat ? -uy * rn : 0.0f;
    const float e1y = pb * rn;
    const float e1z = flat ? 0.0f : -uy * rn;
    const float e2x = uy * e1z - uz * e1y, e2y = uz * e1x - ux * e1z, e2z = ux * e1y - uy * e1x;
    float sn, cs;
    sincos_own(kPi * v, &sn, &cs);
    const float px = cs * e1x + sn * e2x, py = cs * e1y + sn * e2y, pz = cs * e1z + sn * e2z;
    const float x = w * ux + r * px, y = w * uy + r * py, z = w * uz + r * pz;
    const float rnn = rcp_f(sqrtf(dot3(x, y, z, x, y, z)));
    *ox = x * rnn;
    *oy = y * rnn;
    *oz = z * rnn;
}

// ------------------------------------------------------------------------ patches ----
struct XPatchParams {
    float4 *spins4;
    int L1, L2, L3, H;
    long long half;      // sites per colour per replica
    int P1, P2, P3, cls;
    long long Pc;        // patches of one class per replica
    int r0, nrep;        // replicas of this pass
    const uint32_t *stream_id, *lstep;
    const int32_t *slot_of_rep;
    const float *beta_slot_f;
    float jx, jy, jz;
    uint32_t seed;
    RoundKeys K;         // Philox round keys of seed
};

__device__ __forceinline__ int xwrap(int x, int L) { return x >= L ? x - L : (x < 0 ? x + L : x); }

// storage index of canonical (a, b, c) in [-1, 4] of the patch at origin o with reflection par
__device__ __forceinline__ long long xsite(const XPatchParams &P, int o0, int o1, int o2, int par, int a, int b,
                                           int c) {
    const int x = xwrap(o0 + (par ? 3 - a : a), P.L1);
    const int y = xwrap(o1 + b, P.L2);
    const int z = xwrap(o2 + c, P.L3);
    return (long long)((x + y + z) & 1) * P.half + ((long long)z * P.L2 + y) * P.H + (x >> 1);
}

// Patch w of this pass: replica, patch number pidx, sweep counter t, origin and reflection
// (the Ising learner's decoding: class cls of the offset tiling of replica r's sweep t).
// A pass holds fewer than 2^31 patches and a class fewer than 2^31 per replica (32-bit
// arithmetic).
struct XPatch {
    int r, o0, o1, o2, par, q;
    uint32_t pidx, t, stream;
};
__device__ __forceinline__ XPatch xdecode(const XPatchParams &P, int w) {
    XPatch D;
    const int Pc = (int)P.Pc;
    const int rr = w / Pc;
    D.r = P.r0 + rr;
    D.q = w - rr * Pc;
    const int half1 = P.P1 >> 1;
    const int row = D.q / half1;
    const int tt = D.q - row * half1;
    const int pk = row / P.P2, pj = row - pk * P.P2;
    const int pi = 2 * tt + ((P.cls + pj + pk) & 1);
    D.pidx = (uint32_t)(pi + P.P1 * (pj + P.P2 * pk));
    D.t = P.lstep[D.r];
    D.stream = P.stream_id[D.r];
    const U4 ow = draw_rk(0xFFFFFFFFu, D.t, D.stream, kLearn | (0xFFu << 8), P.K);
    const int ox = (int)(ow.x & 3u), oy = (int)((ow.x >> 2) & 3u), oz = (int)((ow.x >> 4) & 3u);
    D.par = (ox + oy + oz) & 1;
    D.o0 = 4 * pi + ox;
    D.o1 = 4 * pj + oy;
    D.o2 = 4 * pk + oz;
    return D;
}

__device__ __forceinline__ float xbf16r(float f) { return __bfloat162float(__float2bfloat16_rn(f)); }
__device__ __forceinline__ void xput(float *p, float v) { *p = v; }
__device__ __forceinline__ void xput(__nv_bfloat16 *p, float v) { *p = __float2bfloat16_rn(v); }

// Network input row of a patch, written by its warp: boundary site i (face order) at
// 3i .. 3i+2, then beta (Jxx, Jyy, Jzz), zeros to XNI; every value BF16-rounded.
template <typename T>
__device__ __forceinline__ void xinput_row(const XPatchParams &P, const float4 *sp, int o0, int o1, int o2, int par,
                                           float beta, T *row, int lane) {
    for (int i = lane; i < 96; i += 32) {
        int a, b, c;
        geo_bnd(i, a, b, c);
        const float4 S = sp[xsite(P, o0, o1, o2, par, a, b, c)];
        xput(row + 3 * i, xbf16r(S.x));
        xput(row + 3 * i + 1, xbf16r(S.y));
        xput(row + 3 * i + 2, xbf16r(S.z));
    }
    if (lane < XNI - 288) {
        const float v = lane == 0 ? beta * P.jx : lane == 1 ? beta * P.jy : lane == 2 ? beta * P.jz : 0.0f;
        xput(row + 288 + lane, xbf16r(v));
    }
}

// Network inputs of the patches of one pass (one warp per patch).
__global__ void __launch_bounds__(256) xinputs_kernel(XPatchParams P, __nv_bfloat16 *__restrict__ X) {
    const int lane = threadIdx.x & 31;
    const int nwarps = (int)gridDim.x * (int)(blockDim.x >> 5);
    const int total = P.nrep * (int)P.Pc;
    for (int w = (int)blockIdx.x * (int)(blockDim.x >> 5) + (int)(threadIdx.x >> 5); w < total; w += nwarps) {
        const XPatch D = xdecode(P, w);
        const float4 *sp = P.spins4 + (long long)D.r * 2 * P.half;
        const float beta = P.beta_slot_f[P.slot_of_rep[D.r]];
        xinput_row(P, sp, D.o0, D.o1, D.o2, D.par, beta, X + (size_t)w * XNI, lane);
    }
}

// Training samples (one warp each): per replica a random offset and patch, its input row
// (BF16) and the A-site spins (FP32, 3 per site).
__global__ void __launch_bounds__(256) xcollect_kernel(XPatchParams P, int per_rep, uint32_t call,
                                                       __nv_bfloat16 *__restrict__ X, float *__restrict__ Y,
                                                       long long write0, long long cap) {
    const int lane = threadIdx.x & 31;
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    const long long total = (long long)P.nrep * per_rep;
    for (long long w = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); w < total; w += nwarps) {
        const int r = (int)(w / per_rep), s = (int)(w - (long long)r * per_rep);
        const U4 d = draw((uint32_t)s, call, P.stream_id[r], kLearn | (0xFEu << 8), P.seed);
        const int ox = (int)(d.x & 3u), oy = (int)((d.x >> 2) & 3u), oz = (int)((d.x >> 4) & 3u);
        const int par = (ox + oy + oz) & 1;
        const int o0 = 4 * (int)(d.y % (uint32_t)(P.L1 / 4)) + ox;
        const int o1 = 4 * (int)(d.z % (uint32_t)(P.L2 / 4)) + oy;
        const int o2 = 4 * (int)(d.w % (uint32_t)(P.L3 / 4)) + oz;
        const float4 *sp = P.spins4 + (long long)r * 2 * P.half;
        const long long row = (write0 + w) % cap;
        const float beta = P.beta_slot_f[P.slot_of_rep[r]];
        xinput_row(P, sp, o0, o1, o2, par, beta, X + (size_t)row * XNI, lane);
        const int k = lane, rw = k >> 1;
        const float4 S = sp[xsite(P, o0, o1, o2, par, geo_a_a(k), rw & 3, rw >> 2)];
        float *y = Y + (size_t)row * XNO + 3 * k;
        y[0] = S.x;
        y[1] = S.y;
        y[2] = S.z;
    }
}

// minibatch: rows of the data set chosen by Philox, BF16 -> FP32
__global__ void xbatch_kernel(const __nv_bfloat16 *__restrict__ X, const float *__restrict__ Y, long long n, int B,
                              uint32_t seed, uint32_t step, float *__restrict__ Xb, float *__restrict__ Yb) {
    const int b = blockIdx.x;
    if (b >= B) return;
    __shared__ long long row;
    if (threadIdx.x == 0) {
        const U4 d = draw((uint32_t)b, step, 0x4C524E01u, kLearn | (0xFDu << 8), seed);
        row = (long long)((((unsigned long long)d.y << 32) | d.x) % (unsigned long long)n);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < XNI; i += blockDim.x) Xb[(size_t)b * XNI + i] = __bfloat162float(X[(size_t)row * XNI + i]);
    for (int i = threadIdx.x; i < XNO; i += blockDim.x) Yb[(size_t)b * XNO + i] = Y[(size_t)row * XNO + i];
}

__global__ void to_bf16_kernel(const float *__restrict__ q, __nv_bfloat16 *__restrict__ o, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) o[i] = __float2bfloat16_rn(q[i]);
}

// weights BF16-rounded, biases kept
__global__ void xquantise_kernel(const float *__restrict__ p, float *__restrict__ q, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const bool is_bias = (i >= XOFF_B1 && i < XOFF_W2) || (i >= XOFF_B2 && i < XOFF_W3) || i >= XOFF_B3;
        q[i] = is_bias ? p[i] : xbf16r(p[i]);
    }
}

// m = z + b3 per A-site; loss += -(log C(kappa) + m . y) / B, C(kappa) = kappa / (4 pi sinh kappa);
// dZ = -(y + A(kappa) m) / B with A = (1/kappa - coth kappa) / kappa (series below 1e-2).
__global__ void vmf_loss_kernel(float *__restrict__ Zm, const float *__restrict__ b3, const float *__restrict__ Yb,
                                float *__restrict__ dZ, int B, double *__restrict__ loss) {
    __shared__ double red[256];
    double s = 0.0;
    const int n = B * 32;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int b = i >> 5, k = i & 31;
        const float *z = Zm + (size_t)b * XNO + 3 * k;
        const float *y = Yb + (size_t)b * XNO + 3 * k;
        const float mx = z[0] + b3[3 * k], my = z[1] + b3[3 * k + 1], mz = z[2] + b3[3 * k + 2];
        const float kap = sqrtf(mx * mx + my * my + mz * mz);
        float logc, A;
        if (kap < 1e-2f) {
            const float k2 = kap * kap;
            logc = -kLog4Pi - k2 * (1.0f / 6.0f) + k2 * k2 * (1.0f / 180.0f);
            A = -1.0f / 3.0f + k2 * (1.0f / 45.0f);
        } else {
            logc = logf(kap) - kap - logf(-expm1f(-2.0f * kap)) - kLog2Pi;
            A = (1.0f / kap - 1.0f / tanhf(kap)) / kap;
        }
        const float my_dot = mx * y[0] + my * y[1] + mz * y[2];
        s += -(double)(logc + my_dot);
        float *g = dZ + (size_t)b * XNO + 3 * k;
        g[0] = -(y[0] + A * mx) / (float)B;
        g[1] = -(y[1] + A * my) / (float)B;
        g[2] = -(y[2] + A * mz) / (float)B;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0] / B);
}

// The Metropolis-Hastings step of the patches of one pass (one warp per patch; lane k owns
// A-site k and B-site k).  Z: the pass's network outputs (bias b3 added here); dump: optional
// [R][Pc][96] parameters m of this class.
__global__ void __launch_bounds__(256, 4) xpatch_kernel(XPatchParams P, const float *__restrict__ Z,
                                                     const float *__restrict__ b3, float *__restrict__ dump,
                                                     unsigned long long *__restrict__ acc) {
    const int k = threadIdx.x & 31;
    const int nwarps = (int)gridDim.x * (int)(blockDim.x >> 5);
    const int total = P.nrep * (int)P.Pc;
    for (int w = (int)blockIdx.x * (int)(blockDim.x >> 5) + (int)(threadIdx.x >> 5); w < total; w += nwarps) {
        const XPatch D = xdecode(P, w);
        float4 *sp = P.spins4 + (long long)D.r * 2 * P.half;
        const float beta = P.beta_slot_f[P.slot_of_rep[D.r]];
        const float nbeta = -beta;
        // ---- A-site k: vMF(m_k) proposal; its bonds to the boundary
        const int rowk = k >> 1;
        const long long ia = xsite(P, D.o0, D.o1, D.o2, D.par, geo_a_a(k), rowk & 3, rowk >> 2);
        const float4 xo = sp[ia];
        const float *zr = Z + (size_t)w * XNO + 3 * k;
        const float mx = zr[0] + b3[3 * k], my = zr[1] + b3[3 * k + 1], mz = zr[2] + b3[3 * k + 2];
        if (dump) {
            float *dr = dump + ((size_t)D.r * P.Pc + D.q) * XNO + 3 * k;
            dr[0] = mx;
            dr[1] = my;
            dr[2] = mz;
        }
        float bx = 0.0f, by = 0.0f, bz = 0.0f;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const int bi = geo_ab(k, q);
            if (bi < 0) continue;
            int a, b, c;
            geo_bnd(bi, a, b, c);
            const float4 S = sp[xsite(P, D.o0, D.o1, D.o2, D.par, a, b, c)];
            bx += S.x;
            by += S.y;
            bz += S.z;
        }
        const float hx = P.jx * bx, hy = P.jy * by, hz = P.jz * bz;
        const U4 rw = draw_rk(D.pidx, D.t, D.stream, kLearn | ((uint32_t)(32 + k) << 16), P.K);
        const Vmf VA = vmf_prep(mx, my, mz);
        float nx, ny, nz;
        vmf_sample(VA, u01(rw.x), upm1(rw.y), &nx, &ny, &nz);
        const float sa_new = nbeta * dot3(nx, ny, nz, hx, hy, hz) - vmf_logpdf(VA, nx, ny, nz);
        const float sa_old = nbeta * dot3(xo.x, xo.y, xo.z, hx, hy, hz) - vmf_logpdf(VA, xo.x, xo.y, xo.z);
        // ---- B-site k: heat bath vMF(-beta J o (sum of its six neighbours)), new and old
        const int rowm = k >> 1;
        const long long ib = xsite(P, D.o0, D.o1, D.o2, D.par, geo_b_a(k), rowm & 3, rowm >> 2);
        const float4 yo = sp[ib];
        float gnx = 0.0f, gny = 0.0f, gnz = 0.0f, gox = 0.0f, goy = 0.0f, goz = 0.0f;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const int cd = geo_bn(k, q);
            const int src = cd >= 0 ? cd : k;
            float snx = __shfl_sync(0xffffffffu, nx, src), sny = __shfl_sync(0xffffffffu, ny, src),
                  snz = __shfl_sync(0xffffffffu, nz, src);
            float sox = __shfl_sync(0xffffffffu, xo.x, src), soy = __shfl_sync(0xffffffffu, xo.y, src),
                  soz = __shfl_sync(0xffffffffu, xo.z, src);
            if (cd < 0) {
                int a, b, c;
                geo_bnd(-cd - 1, a, b, c);
                const float4 S = sp[xsite(P, D.o0, D.o1, D.o2, D.par, a, b, c)];
                snx = sox = S.x;
                sny = soy = S.y;
                snz = soz = S.z;
            }
            gnx += snx; gny += sny; gnz += snz;
            gox += sox; goy += soy; goz += soz;
        }
        const float mbnx = nbeta * (P.jx * gnx), mbny = nbeta * (P.jy * gny), mbnz = nbeta * (P.jz * gnz);
        const float mbox = nbeta * (P.jx * gox), mboy = nbeta * (P.jy * goy), mboz = nbeta * (P.jz * goz);
        const Vmf VBn = vmf_prep(mbnx, mbny, mbnz), VBo = vmf_prep(mbox, mboy, mboz);
        float ynx, yny, ynz;
        vmf_sample(VBn, u01(rw.z), upm1(rw.w), &ynx, &yny, &ynz);
        const float sb_new = dot3(mbnx, mbny, mbnz, ynx, yny, ynz) - vmf_logpdf(VBn, ynx, yny, ynz);
        const float sb_old = dot3(mbox, mboy, mboz, yo.x, yo.y, yo.z) - vmf_logpdf(VBo, yo.x, yo.y, yo.z);
        // ---- log alpha: the 32 lane terms by a xor butterfly (the same sum on every lane)
        float la = (sa_new + sb_new) - (sa_old + sb_old);
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) la += __shfl_xor_sync(0xffffffffu, la, o);
        const U4 ra = draw_rk(D.pidx, D.t, D.stream, kLearn | (16u << 16), P.K);
        const bool accept = la >= 0.0f || u01(ra.x) < expf_neg(la);
        if (accept) {
            sp[ia] = make_float4(nx, ny, nz, xo.w);
            sp[ib] = make_float4(ynx, yny, ynz, yo.w);
            if (k == 0) atomicAdd(acc + D.r, 1ull);
        }
    }
}

// ------------------------------------------------------------ inference network ----
// xmlp_kernel: Z = W3 . h2, h2 = bf16(relu(W2 . h1 + b2)), h1 = bf16(relu(W1 . x + b1)) for
// 128-row tiles of X (M x 304, BF16) on the fifth-generation tensor cores.  A persistent CTA of
// four warps keeps the three weight matrices in shared memory (the image packed by
// xpack_kernel: BF16, K-major, 128-byte swizzle, W1's K zero-padded to 320) and per tile:
//   * thread 0 loads the X tile with five TMA copies (64 columns each; the columns past 304
//     and the rows past M read as zeros), then issues each layer's tcgen05.mma chain (K = 16
//     per instruction, FP32 accumulators in tensor memory: layer 1 in columns 0-127, layer 2
//     in 128-255, layer 3 in 0-95) and commits it to an mbarrier;
//   * thread p owns row p = TMEM lane p: after layers 1 and 2 it reads its 128 accumulators
//     (tcgen05.ld), adds the BF16 bias, applies ReLU, rounds to BF16 and writes the next
//     layer's A operand over the X tile; after layer 3 it writes its 96 outputs to Z;
//   * once layer 3 has read its operand, the next tile's X copies start, under the last
//     epilogue.
// Every wait is bounded (2 s of %globaltimer): on expiry the kernel records an error code,
// stops, waits (bounded) for the copies and MMAs it started, and frees its tensor memory.
constexpr int XKT1 = 5;  // 64-column K-tiles of layer 1
constexpr int XIMG_W1 = 0, XIMG_W2 = XIMG_W1 + XKT1 * 16384, XIMG_W3 = XIMG_W2 + 2 * 16384,
              XIMG_B = XIMG_W3 + 2 * XNO * 128, XIMG_BYTES = XIMG_B + 2 * NH * 4;
constexpr int XSM_A = (XIMG_BYTES + 1023) / 1024 * 1024;  // X tile, then h1 / h2
constexpr int XSM_BAR = XSM_A + XKT1 * 16384;
constexpr int XSM_BYTES = XSM_BAR + 64 + 1024;            // + barriers, + alignment slack
constexpr uint32_t kXTileBytes = XKT1 * 16384;
static_assert(XSM_BYTES <= 232448, "xmlp_kernel shared memory above the 227 KB opt-in limit");

// the inference image from the BF16 parameters: W1, W2, W3 swizzled, b1, b2 as FP32
__global__ void xpack_kernel(const __nv_bfloat16 *__restrict__ W16, uint8_t *__restrict__ img) {
    const int total = NH * XNI + NH * NH + XNO * NH;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        int base, rows, off, K, idx = e;
        if (idx < NH * XNI) { base = XIMG_W1; rows = NH; off = XOFF_W1; K = XNI; }
        else if ((idx -= NH * XNI) < NH * NH) { base = XIMG_W2; rows = NH; off = XOFF_W2; K = NH; }
        else { idx -= NH * NH; base = XIMG_W3; rows = XNO; off = XOFF_W3; K = NH; }
        const int n = idx / K, k = idx % K;
        const uint32_t o = (uint32_t)base + (uint32_t)(k >> 6) * (uint32_t)(rows * 128) + tc::swz(n, k & 63);
        *reinterpret_cast<__nv_bfloat16 *>(img + o) = W16[off + idx];
    }
    float *bf = reinterpret_cast<float *>(img + XIMG_B);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * NH; i += gridDim.x * blockDim.x)
        bf[i] = __bfloat162float(W16[(i < NH ? XOFF_B1 : XOFF_B2 - NH) + i]);
}

__device__ __forceinline__ void xtma_load(uint32_t dst, const CUtensorMap *map, int c0, int c1, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(map), "r"(c0), "r"(c1), "r"(bar) : "memory");
}

__global__ void __launch_bounds__(128, 1)
xmlp_kernel(const __grid_constant__ CUtensorMap xmap, const uint8_t *__restrict__ img, float *__restrict__ Z, int M,
            int *__restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bar_x = reinterpret_cast<uint64_t *>(base + XSM_BAR);  // the X tile has landed
    uint64_t *bar_m = bar_x + 1;                                     // a layer's MMAs are done
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar_m + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int ntiles = (M + 127) / 128;

    {  // weights and biases into shared memory (plain 16-byte copies of the swizzled image)
        const uint4 *src = reinterpret_cast<const uint4 *>(img);
        uint4 *dst = reinterpret_cast<uint4 *>(base);
        for (int i = tid; i < XIMG_BYTES / 16; i += 128) dst[i] = __ldg(src + i);
    }
    if (tid == 0) {
        tc::mbar_init(tc::smem_u32(bar_x), 1);
        tc::mbar_init(tc::smem_u32(bar_m), 1);
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
    const uint32_t sA = tc::smem_u32(base + XSM_A);
    const uint32_t sW1 = tc::smem_u32(base + XIMG_W1), sW2 = tc::smem_u32(base + XIMG_W2),
                   sW3 = tc::smem_u32(base + XIMG_W3);
    const float *bias = reinterpret_cast<const float *>(base + XIMG_B);
    uint8_t *arow = base + XSM_A;

    auto load_x = [&](int tile) {  // thread 0
        tc::mbar_arrive_tx(tc::smem_u32(bar_x), kXTileBytes);
#pragma unroll
        for (int kt = 0; kt < XKT1; ++kt)
            xtma_load(sA + (uint32_t)kt * 16384u, &xmap, 64 * kt, 128 * tile, tc::smem_u32(bar_x));
    };
    // one layer: K-steps of 16 over nkt 64-column tiles of A and B (B tiles of n rows), into
    // TMEM column dcol, committed to bar_m
    auto layer = [&](uint32_t sB, int n, int ksteps, uint32_t dcol) {  // thread 0
        tc::fence_after();
        const uint32_t idesc = tc::make_idesc(128, n);
        for (int ks = 0; ks < ksteps; ++ks) {
            const uint32_t ao = (uint32_t)(ks >> 2) * 16384u + (uint32_t)(ks & 3) * 32u;
            const uint32_t bo = (uint32_t)(ks >> 2) * (uint32_t)(n * 128) + (uint32_t)(ks & 3) * 32u;
            tc::umma(tmem + dcol, tc::make_desc(sA + ao), tc::make_desc(sB + bo), idesc, ks > 0 ? 1u : 0u);
        }
        tc::umma_commit(tc::smem_u32(bar_m));
    };
    // this thread's 128 accumulators at dcol -> bf16(relu(acc + b)) -> A tiles 0, 1 of row tid
    auto hidden = [&](uint32_t dcol, const float *b) {
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
                    const float a0 = fmaxf(__uint_as_float(v[c0]) + b[32 * cc + c0], 0.0f);
                    const float a1 = fmaxf(__uint_as_float(v[c0 + 1]) + b[32 * cc + c0 + 1], 0.0f);
                    const __nv_bfloat162 bv = __floats2bfloat162_rn(a0, a1);
                    pk4[h] = *reinterpret_cast<const uint32_t *>(&bv);
                }
                const int k = 32 * cc + 8 * g;
                *reinterpret_cast<uint4 *>(arow + (k >> 6) * 16384 + tc::swz(tid, k & 63)) =
                    make_uint4(pk4[0], pk4[1], pk4[2], pk4[3]);
            }
        }
    };

    bool ok = true, x_pending = false, m_pending = false;
    uint32_t ph_x = 0, ph_m = 0;
    auto wait_m = [&](int code) -> bool {  // every thread: the committed MMAs are done
        const bool got = tc::mbar_wait(tc::smem_u32(bar_m), ph_m, err, code);
        if (got) {
            ph_m ^= 1u;
            m_pending = false;
        }
        const bool all = __syncthreads_and(got ? 1 : 0) != 0;
        tc::fence_after();
        return all;
    };
    if (tid == 0 && (int)blockIdx.x < ntiles) {
        load_x(blockIdx.x);
        x_pending = true;
    }
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        // ---- layer 1 on the X tile, once every thread has read the previous tile's layer-3
        // accumulators (the barrier) and the copies have landed
        bool got = true;
        if (tid == 0) {
            got = tc::mbar_wait(tc::smem_u32(bar_x), ph_x, err, 1);
            if (got) {
                ph_x ^= 1u;
                x_pending = false;
            }
        }
        if (!(ok = __syncthreads_and(got ? 1 : 0) != 0)) break;
        if (tid == 0) {
            layer(sW1, NH, XNI / 16, 0u);
            m_pending = true;
        }
        if (!(ok = wait_m(2))) break;
        hidden(0u, bias);
        tc::fence_proxy_async();
        tc::fence_before();
        __syncthreads();
        // ---- layer 2 on h1
        if (tid == 0) {
            layer(sW2, NH, NH / 16, 128u);
            m_pending = true;
        }
        if (!(ok = wait_m(3))) break;
        hidden(128u, bias + NH);
        tc::fence_proxy_async();
        tc::fence_before();
        __syncthreads();
        // ---- layer 3 on h2
        if (tid == 0) {
            layer(sW3, XNO, NH / 16, 0u);
            m_pending = true;
        }
        if (!(ok = wait_m(4))) break;
        // the A tile is free again: the next tile's copies run under this epilogue
        const int next = tile + gridDim.x;
        if (tid == 0 && next < ntiles) {
            load_x(next);
            x_pending = true;
        }
        // tcgen05.ld is warp-collective: every lane reads, lanes past M store nothing
        const int row = tile * 128 + tid;
        float4 *z4 = reinterpret_cast<float4 *>(Z + (size_t)(row < M ? row : 0) * XNO);
#pragma unroll 1
        for (int cc = 0; cc < 3; ++cc) {
            uint32_t v[32];
            tc::tmem_ld32(lane_base + 32u * cc, v);
            tc::tmem_wait_ld();
            if (row < M) {
#pragma unroll
                for (int g = 0; g < 8; ++g)
                    z4[8 * cc + g] = make_float4(__uint_as_float(v[4 * g]), __uint_as_float(v[4 * g + 1]),
                                                 __uint_as_float(v[4 * g + 2]), __uint_as_float(v[4 * g + 3]));
            }
        }
        tc::fence_before();  // these TMEM reads precede the next tile's MMAs
    }
    // after a failed wait: the copies and MMAs already started still write this block's
    // shared and tensor memory; wait for them (bounded) before freeing and exiting
    if (tid == 0 && x_pending) tc::mbar_wait(tc::smem_u32(bar_x), ph_x, err, 5);
    bool drained = true;
    if (tid == 0 && m_pending) drained = tc::mbar_wait(tc::smem_u32(bar_m), ph_m, err, 6);
    drained = __syncthreads_and(drained ? 1 : 0) != 0;
    if (warp == 0) {
        tc::fence_after();
        if (drained) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
    }
}

// ------------------------------------------------------------------------ host side ----
struct XyzLearn {
    ether_ctx *ctx = nullptr;
    uint32_t seed = 0;
    int R = 0, L[3] = {0, 0, 0}, P[3] = {0, 0, 0};
    long long Pc = 0, half = 0;
    float jx = 0.f, jy = 0.f, jz = 0.f;
    // parameters (device): master, quantised, gradient, Adam moments
    float *p = nullptr, *pq = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    int adam_t = 0;
    // data set
    __nv_bfloat16 *X = nullptr;
    float *Y = nullptr;
    long long cap = 0, n = 0, write = 0;
    uint32_t collect_calls = 0;
    // training scratch (max batch)
    int maxB = 0;
    float *Xb = nullptr, *Yb = nullptr, *H1 = nullptr, *H2 = nullptr, *Z = nullptr, *dZ = nullptr,
          *dH1 = nullptr, *dH2 = nullptr;
    double *loss = nullptr;
    // inference: BF16 weights and their swizzled image, one pass of up to `rows` patches
    __nv_bfloat16 *W16 = nullptr;  // W1, W2, W3 (and b1, b2) at their parameter offsets
    uint8_t *ximg = nullptr;       // XIMG_BYTES: xmlp_kernel's shared-memory image
    long long rows = 0;
    __nv_bfloat16 *Xh = nullptr;
    float *Zi = nullptr;
    int *err = nullptr;            // device: first bounded-wait failure of xmlp_kernel
    // sweeps
    uint32_t *lstep = nullptr;
    unsigned long long *acc = nullptr;
    float *dump = nullptr;
    bool dump_on = false;
    int sm_count = 0;
    uint64_t launches = 0, proposed = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float sweep_ms = 0.f, train_ms = 0.f;
    int timed = 0;  // 1: sweep, 2: train pending in e0/e1
    int timed_n = 0;
};

namespace {

int xfail(int code, const std::string &msg) {
    set_error(msg);
    return code;
}

#define XCUDA(expr)                                                                          \
    do {                                                                                     \
        cudaError_t _e = (expr);                                                             \
        if (_e != cudaSuccess)                                                               \
            return xfail(_e == cudaErrorMemoryAllocation ? ETHER_ERR_NOMEM : ETHER_ERR_CUDA,  \
                         std::string(#expr) + ": " + cudaGetErrorString(_e));                \
    } while (0)

XPatchParams patch_params(const XyzLearn &x, int cls, int r0, int nrep) {
    const Ctx &c = x.ctx->c;
    XPatchParams P;
    std::memset(&P, 0, sizeof(P));
    P.spins4 = c.spins4;
    P.L1 = x.L[0]; P.L2 = x.L[1]; P.L3 = x.L[2]; P.H = x.L[0] / 2;
    P.half = x.half;
    P.P1 = x.P[0]; P.P2 = x.P[1]; P.P3 = x.P[2];
    P.cls = cls;
    P.Pc = x.Pc;
    P.r0 = r0;
    P.nrep = nrep;
    P.stream_id = c.stream_id;
    P.lstep = x.lstep;
    P.slot_of_rep = c.slot_of_rep;
    P.beta_slot_f = c.beta_slot_f;
    P.jx = x.jx; P.jy = x.jy; P.jz = x.jz;
    P.seed = c.seed;
    P.K = round_keys(c.seed);
    return P;
}

int warp_grid(const XyzLearn &x, long long warps) {
    return (int)std::max<long long>(1, std::min<long long>((warps + 7) / 8, 8LL * x.sm_count));
}

void xgemm(cudaStream_t st, int M, int N, int K, const float *A, int lda, int ta, const float *B, int ldb, int tb,
           float *C, int ldc) {
    dim3 grid((N + 63) / 64, (M + 63) / 64);
    gemm_kernel<<<grid, 256, 0, st>>>(M, N, K, A, lda, ta, B, ldb, tb, C, ldc, 0.f);
}

int quantise(XyzLearn &x, cudaStream_t st) {
    xquantise_kernel<<<64, 256, 0, st>>>(x.p, x.pq, XNPARAM);
    to_bf16_kernel<<<64, 256, 0, st>>>(x.pq, x.W16, XNPARAM);
    xpack_kernel<<<64, 256, 0, st>>>(x.W16, x.ximg);
    x.launches += 3;
    XCUDA(cudaGetLastError());
    return ETHER_OK;
}

// The inference network on M rows of Xh (BF16, M <= rows): Zi (no output bias), by
// xmlp_kernel: one persistent CTA per SM at most, the X tiles read by TMA.
int infer_rows(XyzLearn &x, cudaStream_t st, int M, const __nv_bfloat16 *Xh, float *Z) {
    auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(tma_encode_tiled_fn());
    if (!encode) return xfail(ETHER_ERR_CUDA, "learned proposal: cuTensorMapEncodeTiled not available");
    CUtensorMap map;
    cuuint64_t gdim[2] = {(cuuint64_t)XNI, (cuuint64_t)M};
    cuuint64_t gstride[1] = {(cuuint64_t)XNI * sizeof(__nv_bfloat16)};
    cuuint32_t box[2] = {64, 128};
    cuuint32_t estride[2] = {1, 1};
    if (encode(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16 *>(Xh), gdim, gstride, box,
               estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return xfail(ETHER_ERR_CUDA, "learned proposal: cuTensorMapEncodeTiled failed");
    XCUDA(cudaFuncSetAttribute(xmlp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, XSM_BYTES));
    const int ntiles = (M + 127) / 128;
    xmlp_kernel<<<std::min(ntiles, x.sm_count), 128, XSM_BYTES, st>>>(map, x.ximg, Z, M, x.err);
    x.launches++;
    XCUDA(cudaGetLastError());
    return ETHER_OK;
}

// The device error flag of xmlp_kernel (synchronises the stream): ETHER_ERR_TIMEOUT once
// after a bounded wait ran out, then cleared.
int xread_err(XyzLearn &x) {
    int e = 0;
    XCUDA(cudaMemcpyAsync(&e, x.err, sizeof(int), cudaMemcpyDeviceToHost, x.ctx->c.stream));
    XCUDA(cudaStreamSynchronize(x.ctx->c.stream));
    if (e) {
        cudaMemsetAsync(x.err, 0, sizeof(int), x.ctx->c.stream);
        return xfail(ETHER_ERR_TIMEOUT, "learned proposal: an inference pipeline wait timed out (stage " +
                                            std::to_string(e) + ")");
    }
    return ETHER_OK;
}

// The network on M rows of X (FP32, BF16 values): H1, H2 (ReLU, BF16) and Z (no output bias).
void forward_rows(XyzLearn &x, cudaStream_t st, int M, const float *X, float *H1, float *H2, float *Z) {
    xgemm(st, M, NH, XNI, X, XNI, 0, x.pq + XOFF_W1, XNI, 1, H1, NH);
    bias_relu_kernel<<<256, 256, 0, st>>>(H1, x.pq + XOFF_B1, M, NH);
    xgemm(st, M, NH, NH, H1, NH, 0, x.pq + XOFF_W2, NH, 1, H2, NH);
    bias_relu_kernel<<<256, 256, 0, st>>>(H2, x.pq + XOFF_B2, M, NH);
    xgemm(st, M, XNO, NH, H2, NH, 0, x.pq + XOFF_W3, NH, 1, Z, XNO);
    x.launches += 5;
}

int ensure_batch(XyzLearn &x, int B) {
    if (B <= x.maxB) return ETHER_OK;
    float **bufs[] = {&x.Xb, &x.Yb, &x.H1, &x.H2, &x.Z, &x.dZ, &x.dH1, &x.dH2};
    const size_t cols[] = {XNI, XNO, NH, NH, XNO, XNO, NH, NH};
    for (int i = 0; i < 8; ++i) {
        cudaFree(*bufs[i]);
        *bufs[i] = nullptr;
        XCUDA(cudaMalloc((void **)bufs[i], (size_t)B * cols[i] * sizeof(float)));
    }
    x.maxB = B;
    return ETHER_OK;
}

// Forward and backward of a batch already in Xb / Yb; gradients into x.g, mean loss added to *x.loss.
int forward_backward(XyzLearn &x, int B, cudaStream_t st) {
    const float *W2 = x.pq + XOFF_W2, *W3 = x.pq + XOFF_W3;
    forward_rows(x, st, B, x.Xb, x.H1, x.H2, x.Z);
    vmf_loss_kernel<<<64, 256, 0, st>>>(x.Z, x.pq + XOFF_B3, x.Yb, x.dZ, B, x.loss);
    xgemm(st, XNO, NH, B, x.dZ, XNO, 1, x.H2, NH, 0, x.g + XOFF_W3, NH);
    colsum_kernel<<<1, 128, 0, st>>>(x.dZ, B, XNO, x.g + XOFF_B3);
    xgemm(st, B, NH, XNO, x.dZ, XNO, 0, W3, NH, 0, x.dH2, NH);
    relu_mask_kernel<<<256, 256, 0, st>>>(x.dH2, x.H2, (long long)B * NH);
    xgemm(st, NH, NH, B, x.dH2, NH, 1, x.H1, NH, 0, x.g + XOFF_W2, NH);
    colsum_kernel<<<1, 128, 0, st>>>(x.dH2, B, NH, x.g + XOFF_B2);
    xgemm(st, B, NH, NH, x.dH2, NH, 0, W2, NH, 0, x.dH1, NH);
    relu_mask_kernel<<<256, 256, 0, st>>>(x.dH1, x.H1, (long long)B * NH);
    xgemm(st, NH, XNI, B, x.dH1, NH, 1, x.Xb, XNI, 0, x.g + XOFF_W1, XNI);
    colsum_kernel<<<1, 128, 0, st>>>(x.dH1, B, NH, x.g + XOFF_B1);
    x.launches += 12;
    XCUDA(cudaGetLastError());
    return ETHER_OK;
}

// One class of a learned sweep, in passes of whole replicas: network inputs, the network, the
// Metropolis-Hastings step.
int class_pass(XyzLearn &x, int cls, float *dump) {
    Ctx &c = x.ctx->c;
    cudaStream_t st = c.stream;
    const int per = (int)std::max<long long>(1, std::min<long long>(x.R, x.rows / x.Pc));
    for (int r0 = 0; r0 < x.R; r0 += per) {
        const int nrep = std::min(per, x.R - r0);
        const XPatchParams P = patch_params(x, cls, r0, nrep);
        const long long M = (long long)nrep * x.Pc;
        xinputs_kernel<<<warp_grid(x, M), 256, 0, st>>>(P, x.Xh);
        int rc = infer_rows(x, st, (int)M, x.Xh, x.Zi);
        if (rc) return rc;
        xpatch_kernel<<<warp_grid(x, M), 256, 0, st>>>(P, x.Zi, x.pq + XOFF_B3, dump, x.acc);
        x.launches += 2;
        XCUDA(cudaGetLastError());
    }
    return ETHER_OK;
}

int learned_sweep(XyzLearn &x, float *dump0) {
    Ctx &c = x.ctx->c;
    for (int cls = 0; cls < 2; ++cls) {
        int rc = class_pass(x, cls, dump0 ? dump0 + (size_t)cls * x.R * x.Pc * XNO : nullptr);
        if (rc) return rc;
    }
    advance_lstep_kernel<<<(x.R + 255) / 256, 256, 0, c.stream>>>(x.lstep, x.R);
    x.launches++;
    x.proposed += 2ull * (uint64_t)x.R * (uint64_t)x.Pc;
    XCUDA(cudaGetLastError());
    return ETHER_OK;
}

}  // namespace

int xyz_create(ether_ctx *h, const ether_learn_desc *d, XyzLearn **out) {
    *out = nullptr;
    Ctx &c = h->c;
    // c.L is set once the lattice is verified to be the periodic simple-cubic one
    if (c.model != ETHER_MODEL_XYZ || c.L[0] <= 0 || c.nsp != 1 || c.nsh != 1 || c.zeeman || c.sia || c.sia_local ||
        c.angle)
        return xfail(ETHER_ERR_UNSUPPORTED,
                     "learned proposal (XYZ): simple cubic, one species, one shell, Marsaglia proposals, no Zeeman or SIA term");
    if (c.L[0] % 8 || c.L[1] % 8 || c.L[2] % 8 || c.L[0] > 1016 || c.L[1] > 1016 || c.L[2] > 1016)
        return xfail(ETHER_ERR_UNSUPPORTED, "learned proposal: every extent a multiple of 8, at most 1016");
    if (d->capacity < 1024) return xfail(ETHER_ERR_ARG, "training capacity below 1024 samples");
    XyzLearn *x = new XyzLearn();
    x->ctx = h;
    x->seed = d->seed;
    x->R = c.R;
    for (int a = 0; a < 3; ++a) {
        x->L[a] = c.L[a];
        x->P[a] = c.L[a] / 4;
    }
    x->Pc = (long long)x->P[0] * x->P[1] * x->P[2] / 2;
    x->half = (long long)(c.L[0] / 2) * c.L[1] * c.L[2];
    x->jx = c.h_Jf[0];
    x->jy = c.h_Jf[1];
    x->jz = c.h_Jf[2];
    x->cap = d->capacity;
    x->rows = std::max<long long>(x->Pc, std::min<long long>((long long)x->R * x->Pc, kChunkPatches));
    cudaError_t e = cudaSuccess;
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&x->sm_count, cudaDevAttrMultiProcessorCount, dev);
    float **pb[] = {&x->p, &x->pq, &x->g, &x->m, &x->v};
    for (float **b : pb)
        if (e == cudaSuccess) e = cudaMalloc((void **)b, XNPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&x->X, (size_t)x->cap * XNI * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc((void **)&x->Y, (size_t)x->cap * XNO * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&x->W16, XNPARAM * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc((void **)&x->Xh, (size_t)x->rows * XNI * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc((void **)&x->ximg, XIMG_BYTES);
    if (e == cudaSuccess) e = cudaMemset(x->ximg, 0, XIMG_BYTES);  // W1's K padding stays zero
    if (e == cudaSuccess) e = cudaMalloc((void **)&x->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(x->err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void **)&x->Zi, (size_t)x->rows * XNO * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&x->loss, sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void **)&x->lstep, x->R * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc((void **)&x->acc, x->R * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(x->lstep, 0, x->R * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(x->acc, 0, x->R * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(x->m, 0, XNPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(x->v, 0, XNPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaEventCreate(&x->e0);
    if (e == cudaSuccess) e = cudaEventCreate(&x->e1);
    if (e == cudaSuccess) {
        // He initialisation, last layer small: the untrained network proposes nearly uniform spins
        std::vector<float> p(XNPARAM, 0.f);
        std::mt19937 gen(d->seed ^ 0x7F4A7C15u);
        std::normal_distribution<float> nd(0.f, 1.f);
        for (int i = 0; i < NH * XNI; ++i) p[XOFF_W1 + i] = nd(gen) * std::sqrt(2.0f / XNI);
        for (int i = 0; i < NH * NH; ++i) p[XOFF_W2 + i] = nd(gen) * std::sqrt(2.0f / NH);
        for (int i = 0; i < XNO * NH; ++i) p[XOFF_W3 + i] = nd(gen) * 0.01f;
        e = cudaMemcpy(x->p, p.data(), XNPARAM * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        xyz_destroy(x);
        return xfail(e == cudaErrorMemoryAllocation ? ETHER_ERR_NOMEM : ETHER_ERR_CUDA,
                     std::string("learned proposal set-up: ") + cudaGetErrorString(e));
    }
    int rc = quantise(*x, c.stream);
    if (rc) {
        xyz_destroy(x);
        return rc;
    }
    // one inference pass of every size a sweep uses, on zero inputs: the kernel's one-time
    // set-up (module load, shared-memory opt-in) happens here, not inside the first sweep
    e = cudaMemsetAsync(x->Xh, 0, (size_t)x->rows * XNI * sizeof(__nv_bfloat16), c.stream);
    if (e != cudaSuccess) {
        xyz_destroy(x);
        return xfail(ETHER_ERR_CUDA, std::string("learned proposal set-up: ") + cudaGetErrorString(e));
    }
    {
        const int per = (int)std::max<long long>(1, std::min<long long>(x->R, x->rows / x->Pc));
        std::vector<int> sizes = {per * (int)x->Pc};
        if (x->R % per) sizes.push_back((x->R % per) * (int)x->Pc);
        for (int M : sizes) {
            rc = infer_rows(*x, c.stream, M, x->Xh, x->Zi);
            if (rc) {
                xyz_destroy(x);
                return rc;
            }
        }
    }
    rc = xread_err(*x);
    if (rc) {
        xyz_destroy(x);
        return rc;
    }
    *out = x;
    return ETHER_OK;
}

void xyz_destroy(XyzLearn *x) {
    if (!x) return;
    if (x->ctx) cudaStreamSynchronize(x->ctx->c.stream);
    void *ptrs[] = {x->p, x->pq, x->g, x->m, x->v, x->X, x->Y, x->Xb, x->Yb, x->H1, x->H2, x->Z, x->dZ, x->dH1,
                    x->dH2, x->loss, x->W16, x->ximg, x->err, x->Xh, x->Zi, x->lstep, x->acc, x->dump};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (x->e0) cudaEventDestroy(x->e0);
    if (x->e1) cudaEventDestroy(x->e1);
    delete x;
}

int xyz_collect(XyzLearn *x, int per_replica) {
    Ctx &c = x->ctx->c;
    const long long total = (long long)x->R * per_replica;
    const XPatchParams P = patch_params(*x, 0, 0, x->R);
    xcollect_kernel<<<warp_grid(*x, total), 256, 0, c.stream>>>(P, per_replica, x->collect_calls, x->X, x->Y,
                                                                 x->write, x->cap);
    XCUDA(cudaGetLastError());
    x->launches++;
    x->collect_calls++;
    x->write = (x->write + total) % x->cap;
    x->n = std::min(x->cap, x->n + total);
    return ETHER_OK;
}

int xyz_train(XyzLearn *x, int steps, int batch, float lr, double *loss_out) {
    if (x->n == 0) return xfail(ETHER_ERR_STATE, "no training samples (ether_learn_collect)");
    int rc = ensure_batch(*x, batch);
    if (rc) return rc;
    cudaStream_t st = x->ctx->c.stream;
    XCUDA(cudaEventRecord(x->e0, st));
    for (int s = 0; s < steps; ++s) {
        XCUDA(cudaMemsetAsync(x->loss, 0, sizeof(double), st));
        xbatch_kernel<<<batch, 128, 0, st>>>(x->X, x->Y, x->n, batch, x->seed, (uint32_t)(x->adam_t + 1), x->Xb, x->Yb);
        x->launches++;
        rc = forward_backward(*x, batch, st);
        if (rc) return rc;
        ++x->adam_t;
        const float c1 = 1.0f - std::pow(0.9f, (float)x->adam_t), c2 = 1.0f - std::pow(0.999f, (float)x->adam_t);
        adam_kernel<<<64, 256, 0, st>>>(x->p, x->g, x->m, x->v, XNPARAM, lr, c1, c2);
        x->launches++;
        rc = quantise(*x, st);
        if (rc) return rc;
    }
    XCUDA(cudaEventRecord(x->e1, st));
    if (loss_out) {
        XCUDA(cudaMemcpyAsync(loss_out, x->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
        XCUDA(cudaStreamSynchronize(st));
    }
    x->timed = 2;
    return ETHER_OK;
}

int xyz_sweep(XyzLearn *x, int nsweeps) {
    Ctx &c = x->ctx->c;
    if (x->dump_on && !x->dump)
        XCUDA(cudaMalloc((void **)&x->dump, 2 * (size_t)x->R * x->Pc * XNO * sizeof(float)));
    XCUDA(cudaEventRecord(x->e0, c.stream));
    for (int s = 0; s < nsweeps; ++s) {
        int rc = learned_sweep(*x, (x->dump_on && s == nsweeps - 1) ? x->dump : nullptr);
        if (rc) return rc;
    }
    XCUDA(cudaEventRecord(x->e1, c.stream));
    x->timed = 1;
    x->timed_n = nsweeps;
    return ETHER_OK;
}

int xyz_record_series(XyzLearn *x, int nsteps, int plain_per_step, int learned_per_step, int stride,
                      double *absM) {
    Ctx &c = x->ctx->c;
    const int nrec = nsteps / stride;
    const size_t bytes = sizeof(double) * (size_t)nrec * x->R;
    double *mser = nullptr;
    XCUDA(cudaMalloc((void **)&mser, bytes));
    int rc = ETHER_OK;
    for (int t = 0; t < nsteps && rc == ETHER_OK; ++t) {
        for (int k = 0; k < plain_per_step && rc == ETHER_OK; ++k) rc = plain_sweep(c);
        for (int k = 0; k < learned_per_step && rc == ETHER_OK; ++k) rc = learned_sweep(*x, nullptr);
        if (rc == ETHER_OK && (t + 1) % stride == 0 && (t + 1) / stride <= nrec) {
            const cudaError_t e = launch_record(c, (t + 1) / stride - 1, false, mser, nullptr);
            if (e != cudaSuccess) rc = xfail(ETHER_ERR_CUDA, std::string("record: ") + cudaGetErrorString(e));
        }
    }
    if (rc == ETHER_OK) {
        cudaError_t e = cudaMemcpyAsync(absM, mser, bytes, cudaMemcpyDeviceToHost, c.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) rc = xfail(ETHER_ERR_CUDA, std::string("series copy: ") + cudaGetErrorString(e));
    }
    cudaFree(mser);
    if (rc == ETHER_OK) rc = xread_err(*x);
    return rc;
}

int xyz_get_accepts(XyzLearn *x, uint64_t *accepted) {
    XCUDA(cudaMemcpyAsync(accepted, x->acc, x->R * sizeof(uint64_t), cudaMemcpyDeviceToHost, x->ctx->c.stream));
    XCUDA(cudaStreamSynchronize(x->ctx->c.stream));
    return xread_err(*x);
}

void xyz_set_dump(XyzLearn *x, bool on) { x->dump_on = on; }

int xyz_get_dump(XyzLearn *x, float *out) {
    if (!x->dump) return xfail(ETHER_ERR_STATE, "no network outputs recorded (ether_learn_set_dump, then a sweep)");
    XCUDA(cudaMemcpyAsync(out, x->dump, 2 * (size_t)x->R * x->Pc * XNO * sizeof(float), cudaMemcpyDeviceToHost,
                          x->ctx->c.stream));
    XCUDA(cudaStreamSynchronize(x->ctx->c.stream));
    return ETHER_OK;
}

int xyz_get_params(XyzLearn *x, float *params) {
    XCUDA(cudaMemcpyAsync(params, x->p, XNPARAM * sizeof(float), cudaMemcpyDeviceToHost, x->ctx->c.stream));
    XCUDA(cudaStreamSynchronize(x->ctx->c.stream));
    return ETHER_OK;
}

int xyz_set_params(XyzLearn *x, const float *params) {
    for (int i = 0; i < XNPARAM; ++i)
        if (!std::isfinite(params[i])) return xfail(ETHER_ERR_ARG, "non-finite parameter " + std::to_string(i));
    cudaStream_t st = x->ctx->c.stream;
    XCUDA(cudaMemcpyAsync(x->p, params, XNPARAM * sizeof(float), cudaMemcpyHostToDevice, st));
    XCUDA(cudaMemsetAsync(x->m, 0, XNPARAM * sizeof(float), st));
    XCUDA(cudaMemsetAsync(x->v, 0, XNPARAM * sizeof(float), st));
    x->adam_t = 0;
    int rc = quantise(*x, st);
    if (rc) return rc;
    XCUDA(cudaStreamSynchronize(st));
    return ETHER_OK;
}

int xyz_loss_grad(XyzLearn *x, const float *xin, const float *y, int B, double *loss, float *grad) {
    int rc = ensure_batch(*x, B);
    if (rc) return rc;
    cudaStream_t st = x->ctx->c.stream;
    XCUDA(cudaMemcpyAsync(x->Xb, xin, (size_t)B * XNI * sizeof(float), cudaMemcpyHostToDevice, st));
    XCUDA(cudaMemcpyAsync(x->Yb, y, (size_t)B * XNO * sizeof(float), cudaMemcpyHostToDevice, st));
    XCUDA(cudaMemsetAsync(x->loss, 0, sizeof(double), st));
    rc = forward_backward(*x, B, st);
    if (rc) return rc;
    double lv = 0.0;
    XCUDA(cudaMemcpyAsync(&lv, x->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
    XCUDA(cudaMemcpyAsync(grad, x->g, XNPARAM * sizeof(float), cudaMemcpyDeviceToHost, st));
    XCUDA(cudaStreamSynchronize(st));
    if (loss) *loss = lv;
    return ETHER_OK;
}

// The inference network (the sweeps' tensor-core path) on B host rows, rounded to BF16 as
// the lattice inputs are: m = Z + b3.
int xyz_forward(XyzLearn *x, const float *xin, int B, float *out) {
    cudaStream_t st = x->ctx->c.stream;
    std::vector<float> b3(XNO);
    XCUDA(cudaMemcpyAsync(b3.data(), x->pq + XOFF_B3, XNO * sizeof(float), cudaMemcpyDeviceToHost, st));
    for (long long r0 = 0; r0 < B; r0 += x->rows) {
        const int M = (int)std::min<long long>(x->rows, B - r0);
        std::vector<__nv_bfloat16> xb((size_t)M * XNI);
        for (size_t i = 0; i < xb.size(); ++i) xb[i] = __float2bfloat16_rn(xin[(size_t)r0 * XNI + i]);
        XCUDA(cudaMemcpyAsync(x->Xh, xb.data(), xb.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, st));
        int rc = infer_rows(*x, st, M, x->Xh, x->Zi);
        if (rc) return rc;
        XCUDA(cudaMemcpyAsync(out + (size_t)r0 * XNO, x->Zi, (size_t)M * XNO * sizeof(float), cudaMemcpyDeviceToHost,
                              st));
        XCUDA(cudaStreamSynchronize(st));
    }
    for (int b = 0; b < B; ++b)
        for (int o = 0; o < XNO; ++o) out[(size_t)b * XNO + o] += b3[o];
    return xread_err(*x);
}

int xyz_info(XyzLearn *x, ether_learn_info *info) {
    if (x->timed) {
        float ms = 0.f;
        XCUDA(cudaEventSynchronize(x->e1));
        XCUDA(cudaEventElapsedTime(&ms, x->e0, x->e1));
        if (x->timed == 1) x->sweep_ms = x->timed_n > 0 ? ms / x->timed_n : 0.f;
        else x->train_ms = ms;
        x->timed = 0;
    }
    info->n_params = XNPARAM;
    info->patches_per_class = x->Pc;
    info->n_samples = x->n;
    info->capacity = x->cap;
    info->train_steps = x->adam_t;
    info->proposed = x->proposed;
    info->kernel_launches = x->launches;
    info->last_sweep_ms = x->sweep_ms;
    info->last_train_ms = x->train_ms;
    return ETHER_OK;
}

void xyz_shape(int *n_inputs, int *n_outputs, int *n_params) {
    *n_inputs = XNI;
    *n_outputs = XNO;
    *n_params = XNPARAM;
}

}  // namespace learn
}  // namespace ether
