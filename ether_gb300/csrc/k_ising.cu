// k_ising.cu -- Ising Metropolis colour phases (src/Metropolis.f90:39-62 with the
// Ising branch of update_spin_details.f90:34-35 and Hamiltonian.f90:34-52).
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
// One thread = one group of eight consecutive sites of the colour class.
__global__ void __launch_bounds__(256)
ising_csr_kernel(uint8_t *__restrict__ spins, int N, int col_off, int n_c, uint32_t colour,
                 const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ nbr,
                 const int32_t *__restrict__ wstride, const uint16_t *__restrict__ itype,
                 const int32_t *__restrict__ type_base, const int32_t *__restrict__ type_half,
                 const uint32_t *__restrict__ thr, int table_entries,
                 const int32_t *__restrict__ slot_of_rep, const uint32_t *__restrict__ stream_id,
                 const uint32_t *__restrict__ step, uint32_t seed,
                 unsigned long long *__restrict__ acc_count) {
    const int r = blockIdx.y;
    uint8_t *sp = spins + (size_t)r * N;
    const uint32_t *tb = thr + (size_t)slot_of_rep[r] * table_entries;
    const uint32_t stream = stream_id[r];
    const uint32_t t = step[r];
    const uint32_t c3 = kMetro | (colour << 8);
    const int ng = (n_c + 7) >> 3;
    unsigned acc = 0;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        const U4 hi = draw((uint32_t)g, t, stream, c3, seed);
        bool have_lo = false;
        U4 lo{0, 0, 0, 0};
        for (int k = 0; k < 8; ++k) {
            const int rho = 8 * g + k;
            if (rho >= n_c) break;
            const int s = col_off + rho;
            int idx = 0;
            for (int q = row_ptr[s]; q < row_ptr[s + 1]; ++q) idx += wstride[q] * (int)sp[nbr[q]];
            const int own = sp[s];
            const int ty = itype[s];
            const uint32_t T = tb[type_base[ty] + own * type_half[ty] + idx];
            const uint32_t uh = half_of(hi, k), th = T >> 16;
            bool flip = uh < th;
            if (uh == th) {
                if (!have_lo) {
                    lo = draw((uint32_t)g, t, stream, c3 | (1u << 16), seed);
                    have_lo = true;
                }
                flip = half_of(lo, k) <= (T & 0xFFFFu);
            }
            if (flip) {
                sp[s] = (uint8_t)(own ^ 1);
                ++acc;
            }
        }
    }
    warp_add_count(acc_count + r, acc);
}

// ------------------------------------------------------- simple cubic, colour-split ----
// Colour c array: rho = (z*L2 + y)*H + xh, H = L1/2, site x = 2*xh + ((y+z+c)&1).
// All six neighbours live in the other colour's array: same xh in rows (y±1,z), (y,z±1),
// and xh, xh∓1 in row (y,z).  A thread takes W (8 or 16) consecutive bytes of one row
// (W | H), i.e. one or two random-number groups.  Byte sums of 0/1 spins never carry
// (max 6); e = n + 7 s (<= 13) is formed for four sites at once; flips are one predicated
// XOR per site and are counted with popc.
template <int W>
struct Vec {
    uint32_t w[W / 4];
};

template <int W>
__device__ __forceinline__ Vec<W> ldv(const uint8_t *p) {
    Vec<W> v;
    if constexpr (W == 8) {
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
    if constexpr (W == 8) {
        *reinterpret_cast<uint2 *>(p) = make_uint2(v.w[0], v.w[1]);
    } else {
        *reinterpret_cast<uint4 *>(p) = make_uint4(v.w[0], v.w[1], v.w[2], v.w[3]);
    }
}

template <int W, int VPT>
__global__ void __launch_bounds__(256)
ising_sc_kernel(uint8_t *__restrict__ spins, int L1, int L2, int L3, uint32_t colour,
                const uint32_t *__restrict__ thr, int table_entries,
                const int32_t *__restrict__ slot_of_rep, const uint32_t *__restrict__ stream_id,
                const uint32_t *__restrict__ step, uint32_t seed,
                unsigned long long *__restrict__ acc_count) {
    static_assert(W == 8 || W == 16, "vector of one or two random-number groups");
    constexpr int NW = W / 4;
    const int r = blockIdx.y;
    const int H = L1 >> 1;
    const int half = H * L2 * L3;
    uint8_t *own_a = spins + (size_t)r * 2 * half + (size_t)colour * half;
    const uint8_t *opp = spins + (size_t)r * 2 * half + (size_t)(colour ^ 1u) * half;
    __shared__ uint32_t s_th[16], s_tl[16];
    if (threadIdx.x < 14) {
        const uint32_t T = thr[(size_t)slot_of_rep[r] * table_entries + threadIdx.x];
        s_th[threadIdx.x] = T >> 16;
        s_tl[threadIdx.x] = T & 0xFFFFu;
    }
    __syncthreads();
    const uint32_t stream = stream_id[r];
    const uint32_t t = step[r];
    const uint32_t c3 = kMetro | (colour << 8);
    const int nvec = half / W;
    unsigned flips = 0;
    // loads of all VPT vectors first, so their latencies overlap
    Vec<W> me[VPT], o0[VPT], a[VPT], b[VPT], c[VPT], d[VPT];
    uint32_t edge[VPT];
    int rho0[VPT], par[VPT];
    bool live[VPT];
#pragma unroll
    for (int j = 0; j < VPT; ++j) {
        const int v = (blockIdx.x * VPT + j) * blockDim.x + threadIdx.x;
        live[j] = v < nvec;
        const int vv = live[j] ? v : 0;
        rho0[j] = vv * W;
        const int row = rho0[j] / H;
        const int xh0 = rho0[j] - row * H;
        const int y = row % L2, z = row / L2;
        par[j] = (y + z + (int)colour) & 1;
        const int ym = (y == 0 ? L2 - 1 : y - 1), yp = (y == L2 - 1 ? 0 : y + 1);
        const int zm = (z == 0 ? L3 - 1 : z - 1), zp = (z == L3 - 1 ? 0 : z + 1);
        me[j] = ldv<W>(own_a + rho0[j]);
        o0[j] = ldv<W>(opp + rho0[j]);
        a[j] = ldv<W>(opp + (z * L2 + ym) * H + xh0);
        b[j] = ldv<W>(opp + (z * L2 + yp) * H + xh0);
        c[j] = ldv<W>(opp + (zm * L2 + y) * H + xh0);
        d[j] = ldv<W>(opp + (zp * L2 + y) * H + xh0);
        if (par[j] == 0) edge[j] = opp[row * H + (xh0 == 0 ? H - 1 : xh0 - 1)];
        else edge[j] = opp[row * H + (xh0 + W == H ? 0 : xh0 + W)];
    }
#pragma unroll
    for (int j = 0; j < VPT; ++j) {
        if (!live[j]) break;
        U4 rh{0, 0, 0, 0};
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            const int grp = (rho0[j] >> 3) + (q >> 1);
            if ((q & 1) == 0) rh = draw((uint32_t)grp, t, stream, c3, seed);
            uint32_t sh;
            if (par[j] == 0) {  // neighbour x-1 -> xh-1: window shifted up by one byte
                uint32_t lo = (q == 0) ? (edge[j] << 24) : o0[j].w[q - 1];
                sh = __funnelshift_l(lo, o0[j].w[q], 8);
            } else {            // neighbour x+1 -> xh+1: window shifted down by one byte
                uint32_t hi = (q == NW - 1) ? edge[j] : o0[j].w[q + 1];
                sh = __funnelshift_r(o0[j].w[q], hi, 8);
            }
            const uint32_t s0 = me[j].w[q];
            const uint32_t n = o0[j].w[q] + sh + a[j].w[q] + b[j].w[q] + c[j].w[q] + d[j].w[q];
            const uint32_t e4 = n + (s0 << 3) - s0;  // bytewise n + 7 s
            const uint32_t wa = (q & 1) ? rh.z : rh.x, wb = (q & 1) ? rh.w : rh.y;
            const uint32_t u0 = wa & 0xFFFFu, u1 = wa >> 16, u2 = wb & 0xFFFFu, u3 = wb >> 16;
            const uint32_t t0 = s_th[e4 & 0xFFu], t1 = s_th[(e4 >> 8) & 0xFFu];
            const uint32_t t2 = s_th[(e4 >> 16) & 0xFFu], t3 = s_th[e4 >> 24];
            uint32_t out = s0;
            if (u0 < t0) out ^= 0x00000001u;
            if (u1 < t1) out ^= 0x00000100u;
            if (u2 < t2) out ^= 0x00010000u;
            if (u3 < t3) out ^= 0x01000000u;
            if ((u0 == t0) | (u1 == t1) | (u2 == t2) | (u3 == t3)) {  // 2^-16 per site
                const U4 rl = draw((uint32_t)grp, t, stream, c3 | (1u << 16), seed);
                const uint32_t la = (q & 1) ? rl.z : rl.x, lb = (q & 1) ? rl.w : rl.y;
                const uint32_t l[4] = {la & 0xFFFFu, la >> 16, lb & 0xFFFFu, lb >> 16};
                const uint32_t uu[4] = {u0, u1, u2, u3}, tt[4] = {t0, t1, t2, t3};
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (uu[k] == tt[k] && l[k] <= s_tl[(e4 >> (8 * k)) & 0xFFu]) out ^= 1u << (8 * k);
            }
            flips += __popc(out ^ s0);
            me[j].w[q] = out;
        }
        stv<W>(own_a + rho0[j], me[j]);
    }
    warp_add_count(acc_count + r, flips);
}

template <int W, int VPT>
static void launch_sc(Ctx &c, int colour) {
    const int bs = 256;
    const int nvec = (c.N / 2) / W;
    dim3 grid((nvec + bs * VPT - 1) / (bs * VPT), c.R);
    ising_sc_kernel<W, VPT><<<grid, bs, 0, c.stream>>>(
        c.spins, c.L[0], c.L[1], c.L[2], (uint32_t)colour, c.thr, c.table_entries, c.slot_of_rep,
        c.stream_id, c.step, c.seed, c.acc_count);
}

static int blocks_for(const Ctx &c, long work, int bs) {
    long need = (work + bs - 1) / bs;
    long cap = (long)c.sm_count * 8 / (c.R > 0 ? c.R : 1);
    if (cap < 1) cap = 1;
    if (need > cap) need = cap;
    if (need < 1) need = 1;
    return (int)need;
}

cudaError_t launch_ising_sweep(Ctx &c, int colour) {
    const int bs = 256;
    if (c.fast) {
        const int key = c.vec_bytes * 10 + c.ising_vpt;
        switch (key) {
            case 161: launch_sc<16, 1>(c, colour); break;
            case 162: launch_sc<16, 2>(c, colour); break;
            case 164: launch_sc<16, 4>(c, colour); break;
            case 81: launch_sc<8, 1>(c, colour); break;
            case 82: launch_sc<8, 2>(c, colour); break;
            default: launch_sc<8, 4>(c, colour); break;
        }
    } else {
        const int n_c = c.col_off[colour + 1] - c.col_off[colour];
        if (n_c == 0) return cudaSuccess;
        dim3 grid(blocks_for(c, (n_c + 7) / 8, bs), c.R);
        ising_csr_kernel<<<grid, bs, 0, c.stream>>>(
            c.spins, c.N, c.col_off[colour], n_c, (uint32_t)colour, c.t.row_ptr, c.t.nbr,
            c.t.wstride, c.t.itype, c.t.type_base, c.t.type_half, c.thr, c.table_entries,
            c.slot_of_rep, c.stream_id, c.step, c.seed, c.acc_count);
    }
    c.launches++;
    return cudaGetLastError();
}

}  // namespace ether
