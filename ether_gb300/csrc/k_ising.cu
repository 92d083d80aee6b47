// k_ising.cu -- per-context launches of the Ising colour phase (bodies in sweep_ising.cuh).
#include <algorithm>

#include "sweep_ising.cuh"
#include "tc_util.cuh"

namespace ether {

// General lattice.  One thread = one group of eight consecutive ranks of the colour class
// (one random-number group).  Neighbours come from the class's ELL block, entry k of rank rho
// at k * n_c + rho: the eight ranks' entries are adjacent and a warp's are contiguous.  The
// neighbour loads are unconditional (padding entries point at valid memory); the threshold
// index idx = sum of stride * up-spin over the site's own entries.  The decision is
// ising_ell_site's: same draws, same thresholds.
__global__ void __launch_bounds__(256)
ising_ell_kernel(uint8_t *__restrict__ spins, int N, int col_off, int n_c, uint32_t colour,
                 const int32_t *__restrict__ ell, const int32_t *__restrict__ ews,
                 const uint16_t *__restrict__ deg, int width, const uint16_t *__restrict__ itype,
                 const int32_t *__restrict__ type_base, const int32_t *__restrict__ type_half,
                 const uint32_t *__restrict__ thr, int table_entries,
                 const int32_t *__restrict__ slot_of_rep, const uint32_t *__restrict__ stream_id,
                 const uint32_t *__restrict__ step, uint32_t seed,
                 unsigned long long *__restrict__ acc_count) {
    const int r = blockIdx.y;
    uint8_t *sp = spins + (size_t)r * N;
    const uint32_t *tb = thr + (size_t)slot_of_rep[r] * table_entries;
    const uint32_t stream = stream_id[r], t = step[r];
    const uint32_t c3 = kMetro | (colour << 8);
    const int ng = (n_c + 7) >> 3;
    unsigned acc = 0;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        const int rho0 = 8 * g;
        int idx[8], dg[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            idx[j] = 0;
            dg[j] = rho0 + j < n_c ? (int)deg[col_off + rho0 + j] : 0;
        }
#pragma unroll 2
        for (int k = 0; k < width; ++k) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int rho = min(rho0 + j, n_c - 1);
                const int e = k * n_c + rho;  // ELL blocks hold < 2^31 entries (checked at creation)
                const int up = sp[ell[e]];
                const int w = ews[e];
                if (k < dg[j]) idx[j] += w * up;
            }
        }
        const U4 hi = draw((uint32_t)g, t, stream, c3, seed);
        bool have_lo = false;
        U4 lo{0, 0, 0, 0};
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int rho = rho0 + j;
            if (rho >= n_c) break;
            const int s = col_off + rho;
            const int own = sp[s];
            const int ty = itype[s];
            const uint32_t T = tb[type_base[ty] + own * type_half[ty] + idx[j]];
            const uint32_t uh = half_of(hi, j), th = T >> 16;
            bool flip = uh < th;
            if (uh == th) {
                if (!have_lo) {
                    lo = draw((uint32_t)g, t, stream, c3 | (1u << 16), seed);
                    have_lo = true;
                }
                flip = half_of(lo, j) <= (T & 0xFFFFu);
            }
            if (flip) {
                sp[s] = (uint8_t)(own ^ 1);
                ++acc;
            }
        }
    }
    warp_add_count(acc_count + r, acc);
}

// The same update with one site per thread, for colour classes too small to fill the GPU
// with groups of eight: every lane draws its group's Philox block itself (the draws, and so
// the decisions, are those of ising_ell_kernel).  W: the class's ELL width at compile time
// (0: at run time).
template <int W>
__global__ void __launch_bounds__(256)
ising_ell_site_kernel(uint8_t *__restrict__ spins, int N, int col_off, int n_c, uint32_t colour,
                      const int32_t *__restrict__ ell, const int32_t *__restrict__ ews,
                      const uint16_t *__restrict__ deg, int width, const uint16_t *__restrict__ itype,
                      const int32_t *__restrict__ type_base, const int32_t *__restrict__ type_half,
                      const uint32_t *__restrict__ thr, int table_entries,
                      const int32_t *__restrict__ slot_of_rep, const uint32_t *__restrict__ stream_id,
                      const uint32_t *__restrict__ step, uint32_t seed,
                      unsigned long long *__restrict__ acc_count) {
    const int r = blockIdx.y;
    uint8_t *sp = spins + (size_t)r * N;
    const uint32_t *tb = thr + (size_t)slot_of_rep[r] * table_entries;
    const uint32_t stream = stream_id[r], t = step[r];
    const uint32_t c3 = kMetro | (colour << 8);
    unsigned acc = 0;
    const IsingEll A{sp, col_off, n_c, width, ell, ews, deg, itype, type_base, type_half, tb};
    for (int rho = blockIdx.x * blockDim.x + threadIdx.x; rho < n_c; rho += gridDim.x * blockDim.x)
        acc += ising_ell_site<W>(A, rho, t, stream, c3, seed) ? 1u : 0u;
    warp_add_count(acc_count + r, acc);
}

template <int W, int VPT, int MINB>
__global__ void __launch_bounds__(256, MINB)
ising_sc_kernel(uint8_t *__restrict__ spins, int L1, int L2, int L3, FastDiv fH, FastDiv fL2,
                uint32_t colour, const uint32_t *__restrict__ thr, int table_entries,
                const int32_t *__restrict__ slot_of_rep, const uint32_t *__restrict__ stream_id,
                const uint32_t *__restrict__ step, uint32_t seed, const RoundKeys K,
                unsigned long long *__restrict__ acc_count) {
    const int r = blockIdx.y;
    const int H = L1 >> 1;
    const int half = H * L2 * L3;
    __shared__ uint32_t s_th[16], s_tl[16];
    load_sc_thresholds(thr + (size_t)slot_of_rep[r] * table_entries, s_th, s_tl);
    __syncthreads();
    const IsingSc A{spins + (size_t)r * 2 * half + (size_t)colour * half,
                    spins + (size_t)r * 2 * half + (size_t)(colour ^ 1u) * half,
                    L1, L2, L3, H, fH, fL2, colour};
    const unsigned flips = byte_sum(ising_sc_vectors<W, VPT>(
        A, blockIdx.x * VPT * blockDim.x + threadIdx.x, blockDim.x, half / W, s_th, s_tl,
        step[r], stream_id[r], kMetro | (colour << 8), seed, K));
    warp_add_count(acc_count + r, flips);
}

// Persistent form: grid = resident blocks x SMs; block b takes the contiguous run of items
// [b items / G, (b + 1) items / G), an item being VPT x 256 vectors of one replica.  The
// thresholds sit in a per-warp slot of shared memory, reloaded when the replica changes, so
// no block barrier is needed; flips are counted per replica and added at each change.
template <int W, int VPT, int MINB>
__global__ void __launch_bounds__(256, MINB)
ising_sc_persist(uint8_t *__restrict__ spins, int L1, int L2, int L3, FastDiv fH, FastDiv fL2,
                 uint32_t colour, const uint32_t *__restrict__ thr, int table_entries,
                 const int32_t *__restrict__ slot_of_rep, const uint32_t *__restrict__ stream_id,
                 const uint32_t *__restrict__ step, uint32_t seed, const RoundKeys K, int R,
                 unsigned long long *__restrict__ acc_count) {
    __shared__ uint32_t s_th[8][16], s_tl[8][16];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int H = L1 >> 1;
    const int half = H * L2 * L3;
    const int nvec = half / W;
    const int per_item = VPT * 256;
    const int items_per_rep = (nvec + per_item - 1) / per_item;
    const long long items = (long long)R * items_per_rep;
    const long long i0 = items * blockIdx.x / gridDim.x, i1 = items * (blockIdx.x + 1) / gridDim.x;
    int cur = -1;
    uint32_t cnt = 0, t = 0, stream = 0;
    for (long long it = i0; it < i1; ++it) {
        const int r = (int)(it / items_per_rep);
        const int v0 = (int)(it - (long long)r * items_per_rep) * per_item;
        if (r != cur) {  // block-uniform
            if (cur >= 0) warp_add_count(acc_count + cur, byte_sum(cnt));
            cnt = 0;
            __syncwarp();
            if (lane < 14) {
                const uint32_t T = thr[(size_t)slot_of_rep[r] * table_entries + lane];
                s_th[warp][lane] = T >> 16;
                s_tl[warp][lane] = T & 0xFFFFu;
            }
            __syncwarp();
            cur = r;
            t = step[r];
            stream = stream_id[r];
        }
        const IsingSc A{spins + (size_t)r * 2 * half + (size_t)colour * half,
                        spins + (size_t)r * 2 * half + (size_t)(colour ^ 1u) * half,
                        L1, L2, L3, H, fH, fL2, colour};
        cnt += ising_sc_vectors<W, VPT>(A, v0 + (int)threadIdx.x, 256, nvec, s_th[warp], s_tl[warp], t,
                                        stream, kMetro | (colour << 8), seed, K);
        // byte lanes hold at most 4 VPT per item: flush before they could reach 256
        if ((it - i0) % (48 / VPT) == (48 / VPT) - 1) {
            warp_add_count(acc_count + cur, byte_sum(cnt));
            cnt = 0;
        }
    }
    if (cur >= 0) warp_add_count(acc_count + cur, byte_sum(cnt));
}

// ---------------------------------------------------------- shared-memory staged form ----
// Persistent; block b owns the contiguous run of steps [b T / G, (b + 1) T / G) of the
// replica-major step sequence (T = R x steps per replica).  A step is S = 4096 / H rows of the
// updated colour (256 threads x 16 bytes).  The other colour's rows that a step reads -- its
// own rows and L2 rows either side (y +- 1 in the same plane, z +- 1) -- are streamed by
// cp.async.bulk into a ring of P stages of S rows (4 KB each) completing on one mbarrier per
// stage, issued P stages ahead by thread 0; the own spins are loaded from global memory one
// step ahead into registers.  All six neighbour words then come from shared memory.
// Requires H = L1 / 2 a power of two >= 16, S dividing L2 L3, and a ring of at most 160 KB.
struct StreamGeo {
    int L1, L2, L3, H, S, rows, spr, h, P;  // rows = L2 L3, spr = rows / S, h = ceil(2 L2 / S)
    FastDiv fL2;
};

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

template <int VS, int MINB>
__global__ void __launch_bounds__(256, MINB)
ising_sc_stream(uint8_t *__restrict__ spins, StreamGeo G, uint32_t colour,
                const uint32_t *__restrict__ thr, int table_entries,
                const int32_t *__restrict__ slot_of_rep, const uint32_t *__restrict__ stream_id,
                const uint32_t *__restrict__ step, uint32_t seed, const RoundKeys K, int R,
                unsigned long long *__restrict__ acc_count, int *__restrict__ err) {
    extern __shared__ __align__(128) uint8_t ring[];  // P stages of S rows, then P mbarriers
    __shared__ uint32_t s_th[8][16], s_tl[8][16];
    const int stage_bytes = G.S * G.H;  // VS x 4096
    uint64_t *full = reinterpret_cast<uint64_t *>(ring + (size_t)G.P * stage_bytes);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long T = (long long)R * G.spr;
    const long long g0 = T * blockIdx.x / gridDim.x, g1 = T * (blockIdx.x + 1) / gridDim.x;
    if (g0 >= g1) return;  // block-uniform
    if (tid == 0) {
        for (int i = 0; i < G.P; ++i) tc::mbar_init(tc::smem_u32(&full[i]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const long long half = (long long)G.H * G.rows;
    const uint32_t ring_rows_mask = (uint32_t)(G.P * G.S - 1);
    const int vrow = G.H >> 4;                    // 16-byte vectors per row
    const int dr = tid / vrow, xh0 = (tid - dr * vrow) * 16;
    const int rows_per_pass = 256 / vrow;         // rows covered by one vector of every thread
    const uint32_t c3 = kMetro | (colour << 8);
    long long issued = 0, waited = 0;             // stages of this block, all segments
    bool ok = true;
    for (long long a = g0; a < g1 && ok;) {
        // ------------------------------------------------------------ one segment ------
        const int r = (int)(a / G.spr);
        const long long e_seg = (long long)(r + 1) * G.spr < g1 ? (long long)(r + 1) * G.spr : g1;
        const int j0 = (int)(a - (long long)r * G.spr), n = (int)(e_seg - a);
        const int nst = n + G.h;                  // stages of this segment
        const long long sbase = issued;           // block stage index of its stage 0
        const int rho_a = j0 * G.S;               // first own row of the segment
        uint8_t *own = spins + (long long)r * 2 * half + (long long)colour * half;
        const uint8_t *opp = spins + (long long)r * 2 * half + (long long)(colour ^ 1u) * half;
        auto issue = [&](int s) {                 // thread 0: ext rows [s S, (s + 1) S)
            const long long gs = sbase + s;
            const uint32_t slot = (uint32_t)(gs % G.P);
            const uint32_t bar = tc::smem_u32(&full[slot]);
            tc::mbar_arrive_tx(bar, (uint32_t)(G.S * G.H));
            int row = rho_a - G.L2 + s * G.S;
            row %= G.rows;
            if (row < 0) row += G.rows;
            const uint32_t dst = tc::smem_u32(ring + (size_t)slot * stage_bytes);
            const int first = G.rows - row < G.S ? G.rows - row : G.S;
            bulk_g2s(dst, opp + (long long)row * G.H, (uint32_t)(first * G.H), bar);
            if (first < G.S) bulk_g2s(dst + first * G.H, opp, (uint32_t)((G.S - first) * G.H), bar);
        };
        if (tid == 0)
            for (int s = 0; s < G.P && s < nst; ++s) issue(s);
        issued += nst;
        // thresholds of this replica in the warp's slot
        __syncwarp();
        if (lane < 14) {
            const uint32_t Tv = thr[(size_t)slot_of_rep[r] * table_entries + lane];
            s_th[warp][lane] = Tv >> 16;
            s_tl[warp][lane] = Tv & 0xFFFFu;
        }
        __syncwarp();
        const uint32_t t = step[r], stream = stream_id[r];
        uint32_t cnt = 0;
        Vec<16> me_next[VS];
#pragma unroll
        for (int u = 0; u < VS; ++u) me_next[u] = ldv<16>(own + (long long)(rho_a + dr + u * rows_per_pass) * G.H + xh0);
        for (int j = 0; j < n; ++j) {
            // stages j .. j + h must have landed
            const long long need = sbase + j + G.h;
            while (waited <= need) {
                if (!tc::mbar_wait(tc::smem_u32(&full[waited % G.P]), (uint32_t)((waited / G.P) & 1), err, 1))
                    ok = false;
                ++waited;
            }
#pragma unroll
            for (int u = 0; u < VS; ++u) {
                const int rho = rho_a + j * G.S + dr + u * rows_per_pass;
                const Vec<16> me = me_next[u];
                if (j + 1 < n) me_next[u] = ldv<16>(own + (long long)(rho + G.S) * G.H + xh0);
                const int z = (int)fdiv((uint32_t)rho, G.fL2), y = rho - z * G.L2;
                const int par = (y + z + (int)colour) & 1;
                const uint32_t e = (uint32_t)(sbase * G.S) + (uint32_t)(j * G.S + dr + u * rows_per_pass + G.L2);
                const uint32_t e_ym = y == 0 ? e + G.L2 - 1 : e - 1;
                const uint32_t e_yp = y == G.L2 - 1 ? e - G.L2 + 1 : e + 1;
                const uint8_t *rowp = ring + (size_t)(e & ring_rows_mask) * G.H;
                const Vec<16> o0 = *reinterpret_cast<const Vec<16> *>(rowp + xh0);
                const Vec<16> va = *reinterpret_cast<const Vec<16> *>(ring + (size_t)(e_ym & ring_rows_mask) * G.H + xh0);
                const Vec<16> vb = *reinterpret_cast<const Vec<16> *>(ring + (size_t)(e_yp & ring_rows_mask) * G.H + xh0);
                const Vec<16> vc = *reinterpret_cast<const Vec<16> *>(ring + (size_t)((e - G.L2) & ring_rows_mask) * G.H + xh0);
                const Vec<16> vd = *reinterpret_cast<const Vec<16> *>(ring + (size_t)((e + G.L2) & ring_rows_mask) * G.H + xh0);
                const uint32_t edge = par == 0 ? rowp[xh0 == 0 ? G.H - 1 : xh0 - 1]
                                               : rowp[xh0 + 16 == G.H ? 0 : xh0 + 16];
                const Vec<16> out = ising_sc_update<16>(me, o0, va, vb, vc, vd, edge, par, rho * G.H + xh0,
                                                        s_th[warp], s_tl[warp], t, stream, c3, seed, K, cnt);
                stv<16>(own + (long long)rho * G.H + xh0, out);
            }
            // every read of stage j is done (its slot may be refilled); a failed wait anywhere
            // stops the whole block
            const int fail = __syncthreads_or(ok ? 0 : 1);
            if (fail) {
                ok = false;
                break;
            }
            if (tid == 0 && j + G.P < nst) issue(j + G.P);
            if (j % (12 / VS) == (12 / VS) - 1) {  // byte lanes stay below 4 x 12
                warp_add_count(acc_count + r, byte_sum(cnt));
                cnt = 0;
            }
        }
        warp_add_count(acc_count + r, byte_sum(cnt));
        a = e_seg;
    }
    // on a failed wait: let the copies already issued land before the block's memory goes
    if (!ok && tid == 0) {
        while (waited < issued) {
            tc::mbar_wait(tc::smem_u32(&full[waited % G.P]), (uint32_t)((waited / G.P) & 1), err, 2);
            ++waited;
        }
    }
}

static bool stream_geometry(const Ctx &c, int vs, StreamGeo &G) {
    G.L1 = c.L[0];
    G.L2 = c.L[1];
    G.L3 = c.L[2];
    G.H = c.L[0] / 2;
    if (G.H < 16 || G.H > 4096 || (G.H & (G.H - 1))) return false;
    G.S = vs * 4096 / G.H;
    G.rows = G.L2 * G.L3;
    if (G.S < 1 || G.rows % G.S || (256 % (G.H / 16) && G.H < 4096)) return false;
    G.spr = G.rows / G.S;
    G.h = (2 * G.L2 + G.S - 1) / G.S;
    int P = 4;
    while (P < G.h + 3) P *= 2;
    G.P = P;
    if ((long)P * G.S * G.H > 160 * 1024) return false;
    G.fL2 = make_fastdiv((uint32_t)G.L2);
    return true;
}

bool ising_stream_supported(const Ctx &c, int vs) {
    StreamGeo G;
    return c.fast && c.model == ETHER_MODEL_ISING && stream_geometry(c, vs, G);
}

template <int VS, int MINB>
static cudaError_t launch_stream(Ctx &c, int colour) {
    StreamGeo G;
    if (!stream_geometry(c, VS, G)) return cudaErrorInvalidValue;
    const int smem = G.P * G.S * G.H + G.P * 8;
    static int occ = 0, occ_smem = 0;  // resident blocks per SM, for the ring size it was found for
    if (occ_smem != smem) {
        cudaFuncSetAttribute(ising_sc_stream<VS, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ising_sc_stream<VS, MINB>, 256, smem) != cudaSuccess || occ < 1)
            occ = 1;
        occ_smem = smem;
    }
    const long long steps = (long long)c.R * G.spr;
    const int grid = (int)std::min<long long>(steps, (long long)occ * c.sm_count);
    ising_sc_stream<VS, MINB><<<grid, 256, smem, c.stream>>>(c.spins, G, (uint32_t)colour, c.thr, c.table_entries,
                                                             c.slot_of_rep, c.stream_id, c.step, c.seed,
                                                             round_keys(c.seed), c.R, c.acc_count, c.err);
    return cudaGetLastError();
}

template <int W, int VPT, int MINB>
static void launch_persist(Ctx &c, int colour) {
    static int occ = 0;  // resident blocks per SM of this instantiation
    if (occ == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ising_sc_persist<W, VPT, MINB>, 256, 0) != cudaSuccess || occ < 1)
            occ = 1;
    }
    const int nvec = (c.N / 2) / W;
    const long long items = (long long)c.R * ((nvec + VPT * 256 - 1) / (VPT * 256));
    const int grid = (int)std::min<long long>(items, (long long)occ * c.sm_count);
    ising_sc_persist<W, VPT, MINB><<<grid, 256, 0, c.stream>>>(
        c.spins, c.L[0], c.L[1], c.L[2], make_fastdiv((uint32_t)(c.L[0] / 2)),
        make_fastdiv((uint32_t)c.L[1]), (uint32_t)colour, c.thr, c.table_entries, c.slot_of_rep,
        c.stream_id, c.step, c.seed, round_keys(c.seed), c.R, c.acc_count);
}

template <int W, int VPT, int MINB>
static void launch_sc(Ctx &c, int colour) {
    const int bs = 256;
    const int nvec = (c.N / 2) / W;
    dim3 grid((nvec + bs * VPT - 1) / (bs * VPT), c.R);
    ising_sc_kernel<W, VPT, MINB><<<grid, bs, 0, c.stream>>>(
        c.spins, c.L[0], c.L[1], c.L[2], make_fastdiv((uint32_t)(c.L[0] / 2)),
        make_fastdiv((uint32_t)c.L[1]), (uint32_t)colour, c.thr, c.table_entries, c.slot_of_rep,
        c.stream_id, c.step, c.seed, round_keys(c.seed), c.acc_count);
}

static int blocks_for(const Ctx &c, long work, int bs) {
    long need = (work + bs - 1) / bs;
    long cap = (long)c.sm_count * 8 / (c.R > 0 ? c.R : 1);
    if (cap < 1) cap = 1;
    if (need > cap) need = cap;
    if (need < 1) need = 1;
    return (int)need;
}

// Resident form for small simple-cubic lattices: one block per replica holds both colour
// arrays in shared memory and runs nsweeps whole sweeps (colour 0, colour 1, counter + 1)
// between two visits to global memory.  The draws, thresholds and vector update are the
// phase kernels' (ising_sc_vectors), so every decision is the same; the sweep counter is
// advanced here instead of by advance_kernel.
template <int W>
__global__ void __launch_bounds__(256)
ising_sc_resident(uint8_t *__restrict__ spins, int L1, int L2, int L3, FastDiv fH, FastDiv fL2,
                  const uint32_t *__restrict__ thr, int table_entries,
                  const int32_t *__restrict__ slot_of_rep, const uint32_t *__restrict__ stream_id,
                  uint32_t *__restrict__ step, uint32_t seed, const RoundKeys K, int nsweeps,
                  unsigned long long *__restrict__ acc_count) {
    extern __shared__ __align__(16) uint8_t s_sp[];  // colour 0 array, then colour 1
    __shared__ uint32_t s_th[16], s_tl[16];
    const int r = blockIdx.x;
    const int H = L1 >> 1;
    const int half = H * L2 * L3;
    const int nvec = half / W;
    uint4 *g = reinterpret_cast<uint4 *>(spins + (size_t)r * 2 * half);
    uint4 *sv = reinterpret_cast<uint4 *>(s_sp);
    const int n16 = (2 * half) >> 4;  // 2 half is a multiple of 16 (W | H)
    for (int i = threadIdx.x; i < n16; i += blockDim.x) sv[i] = g[i];
    load_sc_thresholds(thr + (size_t)slot_of_rep[r] * table_entries, s_th, s_tl);
    const uint32_t stream = stream_id[r];
    const uint32_t t0 = step[r];
    __syncthreads();
    unsigned flips = 0;
    for (int k = 0; k < nsweeps; ++k) {
        const uint32_t t = t0 + (uint32_t)k;
        for (int colour = 0; colour < 2; ++colour) {
            const IsingSc A{s_sp + (size_t)colour * half, s_sp + (size_t)(colour ^ 1) * half,
                            L1, L2, L3, H, fH, fL2, (uint32_t)colour};
            uint32_t cnt = 0;
            for (int v = threadIdx.x; v < nvec; v += blockDim.x)
                cnt += ising_sc_vectors<W, 1>(A, v, 0, nvec, s_th, s_tl, t, stream, kMetro | ((uint32_t)colour << 8),
                                              seed, K);
            flips += byte_sum(cnt);  // each byte <= (W / 4) * ceil(nvec / blockDim) per colour
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n16; i += blockDim.x) g[i] = sv[i];
    if (threadIdx.x == 0) step[r] = t0 + (uint32_t)nsweeps;
    warp_add_count(acc_count + r, flips);
}

bool ising_resident_possible(const Ctx &c, size_t smem_max) {
    if (!c.fast || c.model != ETHER_MODEL_ISING || c.vec_bytes == 0) return false;
    const size_t bytes = (size_t)c.L[0] * c.L[1] * c.L[2];  // both colours
    // (W/4) ceil(nvec/256) flips per byte of a vector count must stay below 256
    const size_t nvec = bytes / 2 / (size_t)c.vec_bytes;
    return bytes <= smem_max && (c.vec_bytes / 4) * ((nvec + 255) / 256) < 256;
}

// Opts the resident kernel into the shared memory a replica needs (once, at creation: not
// during a stream capture).
cudaError_t prepare_ising_resident(const Ctx &c) {
    const int smem = c.L[0] * c.L[1] * c.L[2];
    return c.vec_bytes == 16  ? cudaFuncSetAttribute(ising_sc_resident<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)
           : c.vec_bytes == 8 ? cudaFuncSetAttribute(ising_sc_resident<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)
                              : cudaFuncSetAttribute(ising_sc_resident<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

cudaError_t launch_ising_resident(Ctx &c, int nsweeps) {
    const int smem = c.L[0] * c.L[1] * c.L[2];
    const int bs = 256;
    if (c.vec_bytes == 16) {
        ising_sc_resident<16><<<c.R, bs, smem, c.stream>>>(
            c.spins, c.L[0], c.L[1], c.L[2], make_fastdiv((uint32_t)(c.L[0] / 2)), make_fastdiv((uint32_t)c.L[1]),
            c.thr, c.table_entries, c.slot_of_rep, c.stream_id, c.step, c.seed, round_keys(c.seed), nsweeps,
            c.acc_count);
    } else if (c.vec_bytes == 8) {
        ising_sc_resident<8><<<c.R, bs, smem, c.stream>>>(
            c.spins, c.L[0], c.L[1], c.L[2], make_fastdiv((uint32_t)(c.L[0] / 2)), make_fastdiv((uint32_t)c.L[1]),
            c.thr, c.table_entries, c.slot_of_rep, c.stream_id, c.step, c.seed, round_keys(c.seed), nsweeps,
            c.acc_count);
    } else {
        ising_sc_resident<4><<<c.R, bs, smem, c.stream>>>(
            c.spins, c.L[0], c.L[1], c.L[2], make_fastdiv((uint32_t)(c.L[0] / 2)), make_fastdiv((uint32_t)c.L[1]),
            c.thr, c.table_entries, c.slot_of_rep, c.stream_id, c.step, c.seed, round_keys(c.seed), nsweeps,
            c.acc_count);
    }
    c.launches++;
    return cudaGetLastError();
}

cudaError_t launch_ising_sweep(Ctx &c, int colour) {
    const int bs = 256;
    if (c.fast && c.ising_stream) {
        cudaError_t e;
        switch (c.ising_vpt * 10 + (c.ising_cap ? 4 : 1)) {
            case 11: e = launch_stream<1, 1>(c, colour); break;
            case 14: e = launch_stream<1, 4>(c, colour); break;
            case 21: e = launch_stream<2, 1>(c, colour); break;
            default: e = launch_stream<4, 1>(c, colour); break;
        }
        c.launches++;
        return e;
    }
    if (c.fast) {
        // variant = 1000 persistent + 2000 register cap (four 256-thread blocks per SM)
        //           + 10 bytes per vector + vectors per thread
        const int key = c.ising_cap5 ? 6000 + c.vec_bytes * 10 + c.ising_vpt
                                     : (c.ising_persist ? 1000 : 0) + (c.ising_cap ? 2000 : 0) + c.vec_bytes * 10 + c.ising_vpt;
        switch (key) {
            case 6162: launch_sc<16, 2, 5>(c, colour); break;
            case 161: launch_sc<16, 1, 1>(c, colour); break;
            case 162: launch_sc<16, 2, 1>(c, colour); break;
            case 164: launch_sc<16, 4, 1>(c, colour); break;
            case 81: launch_sc<8, 1, 1>(c, colour); break;
            case 82: launch_sc<8, 2, 1>(c, colour); break;
            case 84: launch_sc<8, 4, 1>(c, colour); break;
            case 41: launch_sc<4, 1, 1>(c, colour); break;
            case 42: launch_sc<4, 2, 1>(c, colour); break;
            case 44: launch_sc<4, 4, 1>(c, colour); break;
            case 2162: launch_sc<16, 2, 4>(c, colour); break;
            case 2164: launch_sc<16, 4, 4>(c, colour); break;
            case 1162: launch_persist<16, 2, 1>(c, colour); break;
            case 1164: launch_persist<16, 4, 1>(c, colour); break;
            case 1082: launch_persist<8, 2, 1>(c, colour); break;
            case 1084: launch_persist<8, 4, 1>(c, colour); break;
            case 1042: launch_persist<4, 2, 1>(c, colour); break;
            case 1044: launch_persist<4, 4, 1>(c, colour); break;
            case 3162: launch_persist<16, 2, 4>(c, colour); break;
            default: launch_persist<16, 4, 4>(c, colour); break;
        }
    } else {
        const int n_c = c.col_off[colour + 1] - c.col_off[colour];
        if (n_c == 0) return cudaSuccess;
        const int32_t *ell = c.t.ell_nbr + c.ell_off[colour];
        const int32_t *ews = c.t.ell_ws + c.ell_off[colour];
        const int r0 = c.rw0, nr = c.rwn ? c.rwn : c.R;  // replica window (the kernel form follows the full R)
        uint8_t *spins = c.spins + (size_t)r0 * c.N;
        const long groups = (long)c.R * ((n_c + 7) / 8);
        if (groups < 2L * c.sm_count * bs) {  // too few groups of eight to fill the GPU
            dim3 grid(blocks_for(c, n_c, bs), nr);
            auto k = ising_ell_site_kernel<0>;
            switch (c.ell_width[colour]) {  // common widths at compile time
                case 4: k = ising_ell_site_kernel<4>; break;
                case 6: k = ising_ell_site_kernel<6>; break;
                case 8: k = ising_ell_site_kernel<8>; break;
                case 12: k = ising_ell_site_kernel<12>; break;
                case 14: k = ising_ell_site_kernel<14>; break;
                case 18: k = ising_ell_site_kernel<18>; break;
                case 24: k = ising_ell_site_kernel<24>; break;
                default: break;
            }
            k<<<grid, bs, 0, c.stream>>>(
                spins, c.N, c.col_off[colour], n_c, (uint32_t)colour, ell, ews, c.t.ell_deg,
                c.ell_width[colour], c.t.itype, c.t.type_base, c.t.type_half, c.thr, c.table_entries,
                c.slot_of_rep + r0, c.stream_id + r0, c.step + r0, c.seed, c.acc_count + r0);
        } else {
            dim3 grid(blocks_for(c, (n_c + 7) / 8, bs), nr);
            ising_ell_kernel<<<grid, bs, 0, c.stream>>>(
                spins, c.N, c.col_off[colour], n_c, (uint32_t)colour, ell, ews, c.t.ell_deg,
                c.ell_width[colour], c.t.itype, c.t.type_base, c.t.type_half, c.thr, c.table_entries,
                c.slot_of_rep + r0, c.stream_id + r0, c.step + r0, c.seed, c.acc_count + r0);
        }
    }
    c.launches++;
    return cudaGetLastError();
}

}  // namespace ether
