// k_ising.cu -- per-context launches of the Ising colour phase (bodies in sweep_ising.cuh).
#include <algorithm>

#include "sweep_ising.cuh"

namespace ether {

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
    IsingCsr A{spins + (size_t)r * N, col_off, n_c, row_ptr, nbr, wstride, itype, type_base,
               type_half, thr + (size_t)slot_of_rep[r] * table_entries};
    const uint32_t stream = stream_id[r], t = step[r];
    const uint32_t c3 = kMetro | (colour << 8);
    const int ng = (n_c + 7) >> 3;
    unsigned acc = 0;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x)
        acc += ising_csr_group(A, g, t, stream, c3, seed);
    warp_add_count(acc_count + r, acc);
}

template <int W, int VPT>
__global__ void __launch_bounds__(256)
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
template <int W, int VPT>
__global__ void __launch_bounds__(256)
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

template <int W, int VPT>
static void launch_persist(Ctx &c, int colour) {
    static int occ = 0;  // resident blocks per SM of this instantiation
    if (occ == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ising_sc_persist<W, VPT>, 256, 0) != cudaSuccess || occ < 1)
            occ = 1;
    }
    const int nvec = (c.N / 2) / W;
    const long long items = (long long)c.R * ((nvec + VPT * 256 - 1) / (VPT * 256));
    const int grid = (int)std::min<long long>(items, (long long)occ * c.sm_count);
    ising_sc_persist<W, VPT><<<grid, 256, 0, c.stream>>>(
        c.spins, c.L[0], c.L[1], c.L[2], make_fastdiv((uint32_t)(c.L[0] / 2)),
        make_fastdiv((uint32_t)c.L[1]), (uint32_t)colour, c.thr, c.table_entries, c.slot_of_rep,
        c.stream_id, c.step, c.seed, round_keys(c.seed), c.R, c.acc_count);
}

template <int W, int VPT>
static void launch_sc(Ctx &c, int colour) {
    const int bs = 256;
    const int nvec = (c.N / 2) / W;
    dim3 grid((nvec + bs * VPT - 1) / (bs * VPT), c.R);
    ising_sc_kernel<W, VPT><<<grid, bs, 0, c.stream>>>(
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

cudaError_t launch_ising_sweep(Ctx &c, int colour) {
    const int bs = 256;
    if (c.fast) {
        const int key = (c.ising_persist ? 1000 : 0) + c.vec_bytes * 10 + c.ising_vpt;
        switch (key) {
            case 161: launch_sc<16, 1>(c, colour); break;
            case 162: launch_sc<16, 2>(c, colour); break;
            case 164: launch_sc<16, 4>(c, colour); break;
            case 81: launch_sc<8, 1>(c, colour); break;
            case 82: launch_sc<8, 2>(c, colour); break;
            case 84: launch_sc<8, 4>(c, colour); break;
            case 1162: launch_persist<16, 2>(c, colour); break;
            case 1164: launch_persist<16, 4>(c, colour); break;
            case 1082: launch_persist<8, 2>(c, colour); break;
            default: launch_persist<8, 4>(c, colour); break;
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
