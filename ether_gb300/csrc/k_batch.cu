// k_batch.cu -- batched Metropolis sweeps over many contexts (ether_batch_* in the C-ABI).
//
// The reference advances one lattice at one temperature per MPI rank (src/ether.f90:112-118,
// one Metropolis sweep at a time: src/Metropolis.f90:34-68).  A batch advances every replica
// of every member context -- mixed lattice sizes, Ising and XYZ, each member with its own
// temperature ladder -- with one kernel per colour phase, member class (the kernel
// specialised for that class) and L2-sized group of members: a grid of blocks walks a table
// of segments (member, replica, first unit, units), each segment a block-sized tile of one
// replica's colour class.  A unit is what one thread updates at a time: a W-byte vector
// (simple-cubic Ising) or one site (general Ising, XYZ; general lattices from the colour
// classes' ELL neighbour blocks).  The per-site arithmetic is the member kernels' own
// (sweep_ising.cuh, sweep_xyz.cuh) with the same random-number counters, so a batch sweep
// reproduces the members' own sweeps bit for bit.  One sweep (the phases and the sweep
// counter advance) is captured once as a CUDA graph and replayed.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "sweep_ising.cuh"
#include "sweep_xyz.cuh"

namespace ether {

enum BatchKind : int32_t { kBIsing16 = 0, kBIsing8 = 1, kBIsingEll = 2, kBXyzSc = 3, kBXyzEll = 4, kBIsing4 = 5 };

// Each colour phase launches one kernel per member class present, specialised for that class
// alone, so that every class gets the registers and occupancy of its own arithmetic.
enum BatchClass : int {
    kCIsing16 = 0,  // simple-cubic Ising, 16-byte vectors
    kCIsing8 = 1,   // simple-cubic Ising, 8-byte vectors
    kCIsingEll = 2, // general Ising, one site per thread from the ELL blocks
    kCXyzScX = 3,   // simple-cubic XYZ, exchange only with Marsaglia proposals
    kCXyzScG = 4,   // simple-cubic XYZ with Zeeman, SIA or ANGLE proposals
    kCXyzEllX = 5,  // general XYZ, exchange only with Marsaglia proposals
    kCXyzEllG = 6,  // general XYZ with Zeeman, SIA or ANGLE proposals
    kCIsing4 = 7,   // simple-cubic Ising, 4-byte vectors
    kNumClasses = 8
};

// Everything a segment needs from its member; copied into shared memory when a block moves
// to another member.  Plain data (no initialisers): it lives in __shared__.
struct BatchMember {
    int32_t kind, N, L1, L2, L3, H;
    FastDiv fH, fL2;
    uint8_t *spins;
    float4 *spins4;
    const uint32_t *thr;
    int32_t table_entries, pad0;
    const int32_t *ell_nbr, *ell_ws, *type_base, *type_half;
    const uint16_t *itype, *ell_j, *ell_deg;
    const int2 *ell_desc;  // per colour: (offset of its ELL block, entries per rank)
    const float4 *J4;
    XyzParams P;
    float jx, jy, jz;
    uint32_t seed;
    RoundKeys K;
    const float *beta_slot_f;
    const int32_t *slot_of_rep;
    const uint32_t *stream_id, *step;
    unsigned long long *acc_count;
    int32_t col_off[kMaxColours + 1];
};
static_assert(sizeof(BatchMember) % 4 == 0, "word copy");

struct BatchSeg {
    uint32_t member, rep, first, count;
};

// One segment of a member of each class.  m lives in shared memory.
template <int W>
__device__ __forceinline__ unsigned batch_ising_sc(const BatchMember &m, uint32_t r, int first, int end,
                                                   uint32_t colour, const uint32_t *s_th, const uint32_t *s_tl,
                                                   uint32_t t, uint32_t stream, int upt) {
    const uint32_t c3 = kMetro | (colour << 8);
    const int half = m.H * m.L2 * m.L3;
    uint8_t *base = m.spins + (size_t)r * 2 * half;
    const IsingSc A{base + (size_t)colour * half, base + (size_t)(colour ^ 1u) * half,
                    m.L1, m.L2, m.L3, m.H, m.fH, m.fL2, colour};
    unsigned acc = 0;
    for (int j = 0; j < upt; ++j) {
        const int v = first + (int)threadIdx.x + j * (int)blockDim.x;
        acc += byte_sum(ising_sc_vectors<W, 1>(A, v, 0, end, s_th, s_tl, t, stream, c3, m.seed, m.K));
    }
    return acc;
}

__device__ __forceinline__ unsigned batch_ising_ell(const BatchMember &m, uint32_t r, int first, int end,
                                                    uint32_t colour, uint32_t t, uint32_t stream) {
    const uint32_t c3 = kMetro | (colour << 8);
    const int off = m.col_off[colour];
    const int2 d = m.ell_desc[colour];
    const IsingEll A{m.spins + (size_t)r * m.N, off, m.col_off[colour + 1] - off, d.y,
                     m.ell_nbr + d.x, m.ell_ws + d.x, m.ell_deg, m.itype, m.type_base, m.type_half,
                     m.thr + (size_t)m.slot_of_rep[r] * m.table_entries};
    unsigned acc = 0;
    for (int rho = first + (int)threadIdx.x; rho < end; rho += blockDim.x)
        acc += ising_ell_site(A, rho, t, stream, c3, m.seed) ? 1u : 0u;
    return acc;
}

template <int OPT>
__device__ __forceinline__ unsigned batch_xyz_sc(const BatchMember &m, uint32_t r, int first, int end,
                                                 uint32_t colour, uint32_t t, uint32_t stream) {
    const uint32_t c3 = kMetro | (colour << 8);
    const int half = m.H * m.L2 * m.L3;
    float4 *base = m.spins4 + (size_t)r * 2 * half;
    const XyzSc A{base + (size_t)colour * half, base + (size_t)(colour ^ 1u) * half,
                  m.L1, m.L2, m.L3, m.H, m.fH, m.fL2, colour, m.jx, m.jy, m.jz};
    const float beta_f = m.beta_slot_f[m.slot_of_rep[r]];
    const RoundKeys &K = m.K;  // read in place from shared memory: no registers held
    // exchange only, Marsaglia proposals: the options fold away at compile time
    XyzParams P = OPT == kXyzExchange ? XyzParams{0, 0, 0, 0.f, nullptr, nullptr, nullptr, 1} : m.P;
    if (P.sia_cls) P.sia_cls += (size_t)colour * half;  // sites are ranks in the colour array
    unsigned acc = 0;
    for (int rho = first + (int)threadIdx.x; rho < end; rho += blockDim.x)
        acc += xyz_sc_site<OPT>(A, P, rho, beta_f, t, c3, K, stream) ? 1u : 0u;
    return acc;
}

template <int OPT>
__device__ __forceinline__ unsigned batch_xyz_ell(const BatchMember &m, uint32_t r, int first, int end,
                                                  uint32_t colour, uint32_t t, uint32_t stream) {
    const uint32_t c3 = kMetro | (colour << 8);
    const int off = m.col_off[colour], n_c = m.col_off[colour + 1] - off;
    const int2 d = m.ell_desc[colour];
    float4 *sp = m.spins4 + (size_t)r * m.N;
    const float beta_f = m.beta_slot_f[m.slot_of_rep[r]];
    const XyzParams P = m.P;
    const RoundKeys &K = m.K;  // read in place from shared memory: no registers held
    unsigned acc = 0;
    for (int rho = first + (int)threadIdx.x; rho < end; rho += blockDim.x)
        acc += xyz_ell_site<OPT>(P, sp, off, n_c, rho, m.ell_nbr + d.x, m.ell_j + d.x, m.ell_deg, d.y, m.J4,
                                 beta_f, t, c3, K, stream) ? 1u : 0u;
    return acc;
}

// Two walks over the segments.  Strided (block_first == nullptr): block b takes segments
// b, b + gridDim.x, ...; the resident blocks sweep through memory together, so the
// neighbour planes one tile reads are the planes its neighbours' tiles read at the same time
// (L2 hits).  Contiguous: block b takes [block_first[b], block_first[b+1]), runs balanced by
// an estimated cost per unit, so member and replica change rarely.  No block barriers: the
// Ising thresholds live in a per-warp slot of shared memory.
template <int CLS, int MINB>
__global__ void __launch_bounds__(256, MINB)
batch_phase_kernel(const BatchMember *__restrict__ members, const BatchSeg *__restrict__ segs,
                   const int32_t *__restrict__ block_first, int n_seg, uint32_t colour, int upt) {
    // Per-warp copies of the current member's parameters and Ising thresholds: a warp moves
    // to another member or replica without waiting for the rest of the block, and the
    // parameters cost no registers.
    constexpr bool kIsingSc = CLS == kCIsing16 || CLS == kCIsing8 || CLS == kCIsing4;
    __shared__ BatchMember s_m[8];
    __shared__ uint32_t s_th[8][kIsingSc ? 16 : 1], s_tl[8][kIsingSc ? 16 : 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    BatchMember &m = s_m[warp];
    uint32_t cur_member = 0xFFFFFFFFu, cur_rep = 0xFFFFFFFFu;
    const bool strided = block_first == nullptr;
    const int s_end = strided ? n_seg : block_first[blockIdx.x + 1];
    const int s_step = strided ? (int)gridDim.x : 1;
    for (int sg = strided ? (int)blockIdx.x : block_first[blockIdx.x]; sg < s_end; sg += s_step) {
        const BatchSeg S = segs[sg];
        const uint32_t r = S.rep;
        if (S.member != cur_member) {  // warp-uniform
            __syncwarp();
            const uint32_t *src = reinterpret_cast<const uint32_t *>(members + S.member);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&m);
            for (int i = lane; i < (int)(sizeof(BatchMember) / 4); i += 32) dst[i] = src[i];
            __syncwarp();
        }
        if constexpr (kIsingSc) {
            if (S.member != cur_member || r != cur_rep) {
                if (lane < 14) {
                    const uint32_t T = m.thr[(size_t)m.slot_of_rep[r] * m.table_entries + lane];
                    s_th[warp][lane] = T >> 16;
                    s_tl[warp][lane] = T & 0xFFFFu;
                }
                __syncwarp();
            }
        }
        cur_member = S.member;
        cur_rep = r;
        const uint32_t t = m.step[r], stream = m.stream_id[r];
        const int first = (int)S.first, end = (int)(S.first + S.count);
        unsigned acc;
        if constexpr (CLS == kCIsing16)
            acc = batch_ising_sc<16>(m, r, first, end, colour, s_th[warp], s_tl[warp], t, stream, upt);
        else if constexpr (CLS == kCIsing8)
            acc = batch_ising_sc<8>(m, r, first, end, colour, s_th[warp], s_tl[warp], t, stream, upt);
        else if constexpr (CLS == kCIsing4)
            acc = batch_ising_sc<4>(m, r, first, end, colour, s_th[warp], s_tl[warp], t, stream, upt);
        else if constexpr (CLS == kCIsingEll)
            acc = batch_ising_ell(m, r, first, end, colour, t, stream);
        else if constexpr (CLS == kCXyzScX)
            acc = batch_xyz_sc<kXyzExchange>(m, r, first, end, colour, t, stream);
        else if constexpr (CLS == kCXyzScG)
            acc = batch_xyz_sc<kXyzGeneral>(m, r, first, end, colour, t, stream);
        else if constexpr (CLS == kCXyzEllX)
            acc = batch_xyz_ell<kXyzExchange>(m, r, first, end, colour, t, stream);
        else
            acc = batch_xyz_ell<kXyzGeneral>(m, r, first, end, colour, t, stream);
        warp_add_count(m.acc_count + r, acc);
    }
}

template <int CLS>
void launch_class(int minb, int grid, int threads, cudaStream_t st, const BatchMember *mem, const BatchSeg *segs,
                  const int32_t *bf, int n_seg, uint32_t colour, int upt) {
    if (minb == 4)
        batch_phase_kernel<CLS, 4><<<grid, threads, 0, st>>>(mem, segs, bf, n_seg, colour, upt);
    else if (minb == 3)
        batch_phase_kernel<CLS, 3><<<grid, threads, 0, st>>>(mem, segs, bf, n_seg, colour, upt);
    else
        batch_phase_kernel<CLS, 1><<<grid, threads, 0, st>>>(mem, segs, bf, n_seg, colour, upt);
}

void launch_phase_class(int cls, int minb, int grid, int threads, cudaStream_t st, const BatchMember *mem,
                        const BatchSeg *segs, const int32_t *bf, int n_seg, uint32_t colour, int upt) {
    switch (cls) {
        case kCIsing16: launch_class<kCIsing16>(minb, grid, threads, st, mem, segs, bf, n_seg, colour, upt); break;
        case kCIsing8: launch_class<kCIsing8>(minb, grid, threads, st, mem, segs, bf, n_seg, colour, upt); break;
        case kCIsingEll: launch_class<kCIsingEll>(minb, grid, threads, st, mem, segs, bf, n_seg, colour, upt); break;
        case kCXyzScX: launch_class<kCXyzScX>(minb, grid, threads, st, mem, segs, bf, n_seg, colour, upt); break;
        case kCXyzScG: launch_class<kCXyzScG>(minb, grid, threads, st, mem, segs, bf, n_seg, colour, upt); break;
        case kCXyzEllX: launch_class<kCXyzEllX>(minb, grid, threads, st, mem, segs, bf, n_seg, colour, upt); break;
        case kCIsing4: launch_class<kCIsing4>(minb, grid, threads, st, mem, segs, bf, n_seg, colour, upt); break;
        default: launch_class<kCXyzEllG>(minb, grid, threads, st, mem, segs, bf, n_seg, colour, upt); break;
    }
}

template <int CLS>
cudaError_t occupancy_class(int *occ, int minb, int threads) {
    return minb == 4   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, batch_phase_kernel<CLS, 4>, threads, 0)
           : minb == 3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, batch_phase_kernel<CLS, 3>, threads, 0)
                       : cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, batch_phase_kernel<CLS, 1>, threads, 0);
}

// Resident blocks per SM of a class kernel (at least 1).
int class_occupancy(int cls, int minb, int threads) {
    int occ = 0;
    cudaError_t e;
    switch (cls) {
        case kCIsing16: e = occupancy_class<kCIsing16>(&occ, minb, threads); break;
        case kCIsing8: e = occupancy_class<kCIsing8>(&occ, minb, threads); break;
        case kCIsingEll: e = occupancy_class<kCIsingEll>(&occ, minb, threads); break;
        case kCXyzScX: e = occupancy_class<kCXyzScX>(&occ, minb, threads); break;
        case kCXyzScG: e = occupancy_class<kCXyzScG>(&occ, minb, threads); break;
        case kCXyzEllX: e = occupancy_class<kCXyzEllX>(&occ, minb, threads); break;
        case kCIsing4: e = occupancy_class<kCIsing4>(&occ, minb, threads); break;
        default: e = occupancy_class<kCXyzEllG>(&occ, minb, threads); break;
    }
    return e == cudaSuccess && occ > 0 ? occ : 1;
}

// Ends a batch sweep: every replica's Metropolis sweep counter advances by one.
__global__ void batch_advance_kernel(uint32_t *const *__restrict__ step_of, int total) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < total) *step_of[i] += 1u;
}

}  // namespace ether

using namespace ether;

struct ether_batch {
    std::vector<ether_ctx *> members;
    cudaStream_t stream = nullptr;
    std::vector<cudaEvent_t> ev_member;
    cudaEvent_t ev_done = nullptr, ev_t0 = nullptr, ev_t1 = nullptr;
    std::vector<BatchMember> h_members;
    std::vector<int> h_variants;       // members' kernel variants when the graph was built
    BatchMember *d_members = nullptr;
    BatchSeg *d_segs = nullptr;
    size_t seg_capacity = 0;
    // runs of segments per (group, colour phase, class): index (g * max_col + p) * kNumClasses + class
    std::vector<int> seg_off, seg_cnt;
    std::vector<int> bf_off, bf_grid;   // per run: block ranges in d_block_first
    // L2-sized groups of members: a group's colour phases run back to back, so that a phase
    // finds in L2 the other colour's spins that the group's previous phase wrote.  Groups are
    // independent and run on n_branch parallel branches of the sweep graph.
    std::vector<int> group_of;          // per member
    std::vector<int> solo;              // per group: a member above the byte budget alone in its group
                                        // (it runs its own phase kernels), else -1
    int n_groups = 1;
    long long group_bytes = 0;          // spin bytes per group; 0: half the L2; 1: every member
                                        // alone, on its own phase kernels
    bool xyz_solo = false;              // every XYZ member alone on its own kernels, Ising members
                                        // in the class kernels
    long long l2_bytes = 0;
    int n_branch = 2;
    std::vector<cudaStream_t> branch;
    std::vector<cudaEvent_t> ev_join;
    cudaEvent_t ev_fork = nullptr;
    int32_t *d_block_first = nullptr;
    size_t bf_capacity = 0;
    float xyz_cost = 20.f;              // estimated cost of an XYZ site, Ising site = 1
    int minb = 1;                       // register cap: 1 = none, 3 or 4 = that many 256-thread blocks
    int walk = 0;                       // 0 strided, 1 contiguous (see batch_phase_kernel), 2 one block per segment
    uint32_t **d_step_of = nullptr;
    int total_R = 0, max_col = 0;
    int threads = 256, upt = 2, bps = 0;  // bps 0: as many as fit
    int grid = 0, sm_count = 0;         // grid: the largest class grid
    int cls_grid[kNumClasses] = {};     // resident blocks per SM x SMs, per class
    long long updates_per_sweep = 0;
    cudaGraphExec_t graph = nullptr;
    std::map<std::string, cudaGraphExec_t> mcs_graphs;  // ether_batch_mcs chunks by gate pattern
    // ether_batch_mcs: the members whose PT and measurement run as batched launches (all but
    // those in the reference-copy PT mode), their table and its offsets
    std::vector<int> obs_in;            // per member: 1 if in the table
    std::vector<ObsMember> h_obs;
    std::vector<int32_t> h_obs_off;     // eoff | roff | poff
    ObsMember *d_obs = nullptr;
    int32_t *d_obs_off = nullptr;
    ObsTable obs;
    bool dirty = true;
    uint64_t launches = 0;
    float last_ms = 0.f;
    int timed_sweeps = 0;  // sweeps between ev_t0 and ev_t1 not yet read
};

namespace {

int bfail(int code, const std::string &msg) {
    set_error(msg);
    return code;
}

#define BCUDA(expr)                                                                          \
    do {                                                                                     \
        cudaError_t _e = (expr);                                                             \
        if (_e != cudaSuccess) {                                                             \
            cudaGetLastError(); /* reported here, not again by a later launch check */       \
            return bfail(_e == cudaErrorMemoryAllocation ? ETHER_ERR_NOMEM : ETHER_ERR_CUDA,  \
                         std::string(#expr) + ": " + cudaGetErrorString(_e));                \
        }                                                                                    \
    } while (0)

BatchMember describe(const Ctx &c) {
    BatchMember m;
    std::memset(&m, 0, sizeof(m));
    if (c.model == ETHER_MODEL_ISING)
        m.kind = !c.fast ? kBIsingEll : c.vec_bytes == 16 ? kBIsing16 : c.vec_bytes == 8 ? kBIsing8 : kBIsing4;
    else
        m.kind = c.fast ? kBXyzSc : kBXyzEll;
    m.N = c.N;
    m.L1 = c.L[0];
    m.L2 = c.L[1];
    m.L3 = c.L[2];
    m.H = c.L[0] / 2;
    if (c.fast) {
        m.fH = make_fastdiv((uint32_t)m.H);
        m.fL2 = make_fastdiv((uint32_t)m.L2);
    }
    m.spins = c.spins;
    m.spins4 = c.spins4;
    m.thr = c.thr;
    m.table_entries = c.table_entries;
    m.ell_nbr = c.t.ell_nbr;
    m.ell_ws = c.t.ell_ws;
    m.type_base = c.t.type_base;
    m.type_half = c.t.type_half;
    m.itype = c.t.itype;
    m.ell_j = c.t.ell_j;
    m.ell_deg = c.t.ell_deg;
    m.ell_desc = c.t.ell_desc;
    m.J4 = c.t.J4;
    m.P.zeeman = c.zeeman;
    m.P.sia = c.sia;
    m.P.sia_local = c.sia_local;
    m.P.sia_cls = c.t.sia_cls;
    m.P.sia_ax = c.t.sia_ax;
    m.P.angle = c.angle;
    m.P.dphi = (float)c.dphi;
    m.P.species = c.t.species;
    m.P.zee = c.t.zee;
    m.P.D = c.t.D;
    m.P.nsp = c.nsp;
    if (!c.h_Jf.empty()) {
        m.jx = c.h_Jf[0];
        m.jy = c.h_Jf[1];
        m.jz = c.h_Jf[2];
    }
    m.seed = c.seed;
    m.K = round_keys(c.seed);
    m.beta_slot_f = c.beta_slot_f;
    m.slot_of_rep = c.slot_of_rep;
    m.stream_id = c.stream_id;
    m.step = c.step;
    m.acc_count = c.acc_count;
    for (int k = 0; k <= c.ncol && k <= kMaxColours; ++k) m.col_off[k] = c.col_off[k];
    return m;
}

// Units of one replica's colour class: vectors (simple-cubic Ising) or sites.
long units_of(const BatchMember &m, const Ctx &c, int colour) {
    if (colour >= c.ncol) return 0;
    const long n_c = c.col_off[colour + 1] - c.col_off[colour];
    switch (m.kind) {
        case kBIsing16: return n_c / 16;
        case kBIsing8: return n_c / 8;
        case kBIsing4: return n_c / 4;
        default: return n_c;
    }
}

int class_of(const BatchMember &m) {
    switch (m.kind) {
        case kBIsing16: return kCIsing16;
        case kBIsing8: return kCIsing8;
        case kBIsing4: return kCIsing4;
        case kBIsingEll: return kCIsingEll;
        case kBXyzSc: return m.P.zeeman || m.P.sia || m.P.sia_local || m.P.angle ? kCXyzScG : kCXyzScX;
        default: return m.P.zeeman || m.P.sia || m.P.sia_local || m.P.angle ? kCXyzEllG : kCXyzEllX;
    }
}

void drop_mcs_graphs(ether_batch &b) {
    for (auto &kv : b.mcs_graphs) cudaGraphExecDestroy(kv.second);
    b.mcs_graphs.clear();
}

int rebuild(ether_batch &b) {
    std::vector<BatchMember> hm;
    hm.reserve(b.members.size());
    for (ether_ctx *h : b.members) {
        if (!h->c.beta_set) return bfail(ETHER_ERR_STATE, "batch member without beta (ether_set_beta / ether_set_ladder)");
        hm.push_back(describe(h->c));
    }
    // a member that runs its own phase kernels is captured with its variant of the moment:
    // a later ether_set_variant / ether_autotune of that member rebuilds the graph
    std::vector<int> hv;
    hv.reserve(b.members.size());
    for (ether_ctx *h : b.members) hv.push_back(ctx_variant(h->c));
    const bool same = hm.size() == b.h_members.size() && hv == b.h_variants &&
                      std::memcmp(hm.data(), b.h_members.data(), hm.size() * sizeof(BatchMember)) == 0;
    if (same && !b.dirty) return ETHER_OK;
    b.h_variants = hv;
    if (b.graph) {
        cudaGraphExecDestroy(b.graph);
        b.graph = nullptr;
    }
    drop_mcs_graphs(b);
    b.h_members = hm;
    if (!b.d_members) BCUDA(cudaMalloc((void **)&b.d_members, hm.size() * sizeof(BatchMember)));
    BCUDA(cudaMemcpyAsync(b.d_members, hm.data(), hm.size() * sizeof(BatchMember), cudaMemcpyHostToDevice, b.stream));
    b.max_col = 0;
    for (ether_ctx *h : b.members) b.max_col = std::max(b.max_col, h->c.ncol);
    // groups: consecutive members up to the byte budget (a larger member is a group alone)
    const long long budget = b.group_bytes > 0 ? b.group_bytes : std::max(1LL, b.l2_bytes / 2);
    b.group_of.assign(b.members.size(), 0);
    b.solo.clear();
    {
        int g = 0;
        long long used = 0;
        b.solo.push_back(-1);
        for (size_t k = 0; k < b.members.size(); ++k) {
            const Ctx &c = b.members[k]->c;
            const long long bytes = (long long)c.R * c.N * (c.model == ETHER_MODEL_ISING ? 1 : (long long)sizeof(float4));
            // a large member, or (xyz_solo) an XYZ member: a group of its own, its own kernels
            const bool alone = bytes > budget || (b.xyz_solo && c.model == ETHER_MODEL_XYZ);
            if (used > 0 && (used + bytes > budget || alone)) {
                ++g;
                used = 0;
                b.solo.push_back(-1);
            }
            b.group_of[k] = g;
            used += bytes;
            if (alone) {
                b.solo[g] = (int)k;  // no segments
                used = budget + 1;   // the next member starts a new group
            }
        }
        b.n_groups = g + 1;
    }
    // segments: group, phase, class, member, replica, tile
    std::vector<BatchSeg> segs;
    const int n_runs = b.n_groups * b.max_col * kNumClasses;
    b.seg_off.assign(n_runs, 0);
    b.seg_cnt.assign(n_runs, 0);
    b.updates_per_sweep = 0;
    const long tile_units = (long)b.threads * b.upt;
    for (int q = 0; q < n_runs; ++q) {
        const int g = q / (b.max_col * kNumClasses), p = (q / kNumClasses) % b.max_col, cls = q % kNumClasses;
        b.seg_off[q] = (int)segs.size();
        for (size_t k = 0; k < b.members.size(); ++k) {
            if (b.group_of[k] != g || class_of(hm[k]) != cls) continue;
            const Ctx &c = b.members[k]->c;
            if (b.solo[g] == (int)k) {
                if (p < c.ncol && cls == class_of(hm[k]))
                    b.updates_per_sweep += (long long)(c.col_off[p + 1] - c.col_off[p]) * c.R;
                continue;
            }
            const long u = units_of(hm[k], c, p);
            if (u == 0) continue;
            for (int r = 0; r < c.R; ++r)
                for (long f = 0; f < u; f += tile_units)
                    segs.push_back(BatchSeg{(uint32_t)k, (uint32_t)r, (uint32_t)f,
                                            (uint32_t)std::min(tile_units, u - f)});
            if (p < c.ncol) b.updates_per_sweep += (long long)(c.col_off[p + 1] - c.col_off[p]) * c.R;
        }
        b.seg_cnt[q] = (int)segs.size() - b.seg_off[q];
    }
    if (segs.size() > b.seg_capacity) {
        if (b.d_segs) cudaFree(b.d_segs);
        b.d_segs = nullptr;
        BCUDA(cudaMalloc((void **)&b.d_segs, std::max<size_t>(1, segs.size()) * sizeof(BatchSeg)));
        b.seg_capacity = segs.size();
    }
    if (!segs.empty())
        BCUDA(cudaMemcpyAsync(b.d_segs, segs.data(), segs.size() * sizeof(BatchSeg), cudaMemcpyHostToDevice, b.stream));
    // grid of each class kernel: its resident blocks per SM x SMs
    b.grid = 0;
    for (int cls = 0; cls < kNumClasses; ++cls) {
        const int occ = class_occupancy(cls, b.minb, b.threads);
        b.cls_grid[cls] = (b.bps > 0 ? std::min(b.bps, occ) : occ) * b.sm_count;
    }
    for (int q = 0; q < n_runs; ++q)
        if (b.seg_cnt[q] > 0) b.grid = std::max(b.grid, b.cls_grid[q % kNumClasses]);
    // per phase: contiguous segment runs of about equal estimated cost, one per block
    std::vector<double> unit_cost(b.members.size());
    for (size_t k = 0; k < b.members.size(); ++k) {
        const Ctx &c = b.members[k]->c;
        const double deg = c.N > 0 ? (double)c.nnz / c.N / 6.0 : 1.0;
        switch (hm[k].kind) {
            case kBIsing16: unit_cost[k] = 16.0; break;
            case kBIsing8: unit_cost[k] = 9.0; break;
            case kBIsing4: unit_cost[k] = 5.5; break;
            case kBIsingEll: unit_cost[k] = 3.0 * deg; break;
            case kBXyzSc: unit_cost[k] = b.xyz_cost; break;
            default: unit_cost[k] = 1.3 * b.xyz_cost * deg; break;
        }
    }
    std::vector<int32_t> bf;
    b.bf_off.assign(n_runs, 0);
    b.bf_grid.assign(n_runs, 0);
    for (int q = 0; q < n_runs; ++q) {
        const int n = b.seg_cnt[q];
        const int G = std::max(1, std::min(b.cls_grid[q % kNumClasses], n));
        b.bf_off[q] = (int)bf.size();
        // walk 2: one block per segment, balanced by the hardware's block scheduler
        b.bf_grid[q] = n > 0 ? (b.walk == 2 ? n : G) : 0;
        std::vector<double> cum(n + 1, 0.0);
        for (int i = 0; i < n; ++i) {
            const BatchSeg &S = segs[b.seg_off[q] + i];
            cum[i + 1] = cum[i] + unit_cost[S.member] * S.count;
        }
        int i = 0;
        for (int blk = 0; blk <= G; ++blk) {
            const double target = cum[n] * blk / G;
            while (i < n && cum[i] < target) ++i;
            bf.push_back(blk == G ? n : i);
        }
    }
    if (bf.size() > b.bf_capacity) {
        if (b.d_block_first) cudaFree(b.d_block_first);
        b.d_block_first = nullptr;
        BCUDA(cudaMalloc((void **)&b.d_block_first, bf.size() * sizeof(int32_t)));
        b.bf_capacity = bf.size();
    }
    if (!bf.empty())
        BCUDA(cudaMemcpyAsync(b.d_block_first, bf.data(), bf.size() * sizeof(int32_t), cudaMemcpyHostToDevice, b.stream));
    BCUDA(cudaStreamSynchronize(b.stream));  // host vectors above go out of scope
    b.dirty = false;
    return ETHER_OK;
}

// Branches 0 .. n-1 exist and wait for the work queued so far on the batch stream.
int fork_branches(ether_batch &b, int n) {
    while ((int)b.branch.size() < n) {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        BCUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        b.branch.push_back(st);
        BCUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        b.ev_join.push_back(ev);
    }
    BCUDA(cudaEventRecord(b.ev_fork, b.stream));
    for (int k = 0; k < n; ++k) BCUDA(cudaStreamWaitEvent(b.branch[k], b.ev_fork, 0));
    return ETHER_OK;
}

// The batch stream waits for branches 0 .. n-1.
int join_branches(ether_batch &b, int n) {
    for (int k = 0; k < n; ++k) {
        BCUDA(cudaEventRecord(b.ev_join[k], b.branch[k]));
        BCUDA(cudaStreamWaitEvent(b.stream, b.ev_join[k], 0));
    }
    return ETHER_OK;
}

int issue_sweep(ether_batch &b) {
    const int nbr = std::min(b.n_branch, b.n_groups);
    if (nbr > 1) {
        const int rc = fork_branches(b, nbr);
        if (rc) return rc;
    }
    const int per_group = b.max_col * kNumClasses;
    for (int g = 0; g < b.n_groups; ++g) {
        cudaStream_t st = nbr > 1 ? b.branch[g % nbr] : b.stream;
        for (int p = 0; p < b.max_col; ++p) {
            if (b.solo[g] >= 0) {
                // the member's own phase kernel (its autotuned variant), on this branch
                Ctx &c = b.members[b.solo[g]]->c;
                if (p >= c.ncol) continue;
                cudaStream_t own = c.stream;
                c.stream = st;
                const cudaError_t e = c.model == ETHER_MODEL_ISING ? launch_ising_sweep(c, p) : launch_xyz_sweep(c, p);
                c.stream = own;
                if (e != cudaSuccess) return bfail(ETHER_ERR_CUDA, std::string("batch member phase: ") + cudaGetErrorString(e));
                continue;
            }
            for (int cls = 0; cls < kNumClasses; ++cls) {
                const int q = g * per_group + p * kNumClasses + cls;
                if (b.seg_cnt[q] == 0) continue;
                const int32_t *bf = b.walk == 1 ? b.d_block_first + b.bf_off[q] : nullptr;
                launch_phase_class(cls, b.minb, b.bf_grid[q], b.threads, st, b.d_members, b.d_segs + b.seg_off[q], bf,
                                   b.seg_cnt[q], (uint32_t)p, b.upt);
                BCUDA(cudaGetLastError());
            }
        }
    }
    if (nbr > 1) {
        const int rc = join_branches(b, nbr);
        if (rc) return rc;
    }
    batch_advance_kernel<<<(b.total_R + 255) / 256, 256, 0, b.stream>>>(b.d_step_of, b.total_R);
    BCUDA(cudaGetLastError());
    return ETHER_OK;
}

int kernels_per_sweep(const ether_batch &b) {
    int n = 1;
    for (int cnt : b.seg_cnt) n += cnt > 0 ? 1 : 0;
    for (int k : b.solo)
        if (k >= 0) n += b.members[k]->c.ncol;
    return n;
}

int capture(ether_batch &b) {
    if (b.graph) return ETHER_OK;
    cudaGraph_t g = nullptr;
    BCUDA(cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal));
    int rc = issue_sweep(b);
    cudaError_t e = cudaStreamEndCapture(b.stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return bfail(ETHER_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b.graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(ETHER_ERR_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(e));
    return ETHER_OK;
}

// The batch stream waits for everything queued on the members' streams.
int join_members(ether_batch &b) {
    for (size_t k = 0; k < b.members.size(); ++k) {
        BCUDA(cudaEventRecord(b.ev_member[k], b.members[k]->c.stream));
        BCUDA(cudaStreamWaitEvent(b.stream, b.ev_member[k], 0));
    }
    return ETHER_OK;
}
// ... and later work on the members' streams waits for the batch.
int release_members(ether_batch &b) {
    BCUDA(cudaEventRecord(b.ev_done, b.stream));
    for (ether_ctx *h : b.members) BCUDA(cudaStreamWaitEvent(h->c.stream, b.ev_done, 0));
    return ETHER_OK;
}

int run_sweeps(ether_batch &b, int nsweeps, bool timed) {
    int rc = rebuild(b);
    if (rc) return rc;
    rc = capture(b);
    if (rc) return rc;
    if (timed) BCUDA(cudaEventRecord(b.ev_t0, b.stream));
    for (int s = 0; s < nsweeps; ++s) BCUDA(cudaGraphLaunch(b.graph, b.stream));
    if (timed) BCUDA(cudaEventRecord(b.ev_t1, b.stream));
    b.launches += (uint64_t)nsweeps * kernels_per_sweep(b);
    return ETHER_OK;
}

// A member's kernels go to a stream of the batch (its stream or a branch) while this is in scope.
struct OnBatchStream {
    Ctx &c;
    cudaStream_t own;
    OnBatchStream(Ctx &ctx, cudaStream_t st) : c(ctx), own(ctx.stream) { c.stream = st; }
    ~OnBatchStream() { c.stream = own; }
};

constexpr int kMemberBranches = 8;

// The table of the batched observables: every member not in the reference-copy PT mode, as
// it is now (ladder shapes can change between calls; the graph key carries them).
int build_obs(ether_batch &b) {
    const int M = (int)b.members.size();
    std::vector<ObsMember> hm;
    std::vector<int32_t> eo{0}, ro{0}, po{0};
    b.obs_in.assign(M, 0);
    for (int m = 0; m < M; ++m) {
        const Ctx &c = b.members[m]->c;
        if (c.flags & ETHER_FLAG_PT_REFERENCE_COPY) continue;
        b.obs_in[m] = 1;
        const ObsMember a = obs_member(c);
        hm.push_back(a);
        eo.push_back(eo.back() + a.R * a.nblk);
        ro.push_back(ro.back() + a.R);
        po.push_back(po.back() + a.n_groups * (a.n_slots / 2 + 1));
    }
    const int Mt = (int)hm.size();
    if (Mt == 0) {
        b.obs = ObsTable();
        return ETHER_OK;
    }
    if (!b.d_obs) {  // sized for every member once: captured graphs keep these addresses
        BCUDA(cudaMalloc((void **)&b.d_obs, (size_t)M * sizeof(ObsMember)));
        BCUDA(cudaMalloc((void **)&b.d_obs_off, (size_t)3 * (M + 1) * sizeof(int32_t)));
    }
    std::vector<int32_t> off(eo);
    off.insert(off.end(), ro.begin(), ro.end());
    off.insert(off.end(), po.begin(), po.end());
    const bool same = hm.size() == b.h_obs.size() && off == b.h_obs_off &&
                      std::memcmp(hm.data(), b.h_obs.data(), hm.size() * sizeof(ObsMember)) == 0;
    if (!same) {
        b.h_obs = hm;
        b.h_obs_off = off;
        BCUDA(cudaMemcpyAsync(b.d_obs, b.h_obs.data(), hm.size() * sizeof(ObsMember), cudaMemcpyHostToDevice, b.stream));
        BCUDA(cudaMemcpyAsync(b.d_obs_off, b.h_obs_off.data(), off.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                              b.stream));
        BCUDA(cudaStreamSynchronize(b.stream));
    }
    b.obs.mem = b.d_obs;
    b.obs.eoff = b.d_obs_off;
    b.obs.roff = b.d_obs_off + (Mt + 1);
    b.obs.poff = b.d_obs_off + 2 * (Mt + 1);
    b.obs.M = Mt;
    b.obs.eblocks = eo.back();
    b.obs.rtotal = ro.back();
    b.obs.ptotal = po.back();
    return ETHER_OK;
}

// The members' own parts of one step (gates g[m]): before the sweep their overrelaxation,
// after it their PT and measurement.  After the sweep the members of the observable table
// take PT and measurement in batched launches, one per kernel for all of them (their gates
// agree: one schedule); the rest -- overrelaxation, members outside the table, spiral
// samples -- is small and independent per member, spread over up to kMemberBranches
// parallel branches.
int issue_member_parts(ether_batch &b, const ether_schedule *sch, const int8_t *g, bool before) {
    const int M = (int)b.members.size();
    const int mask = before ? 1 : 6;
    bool batched = false;
    if (!before && b.obs.M > 0) {
        int gb = -1;
        batched = true;
        for (int m = 0; m < M; ++m)
            if (b.obs_in[m]) {
                if (gb < 0) gb = g[m] & 6;
                else if ((g[m] & 6) != gb) batched = false;
            }
        if (batched && (gb & 2)) {
            BCUDA(launch_batch_energy(b.obs, b.stream));
            BCUDA(launch_batch_pt(b.obs, b.stream));
        }
        if (batched && (gb & 4)) {
            BCUDA(launch_batch_energy(b.obs, b.stream));
            BCUDA(launch_batch_measure(b.obs, b.stream));
        }
    }
    // per member: 1 its own parts, 2 only its spiral sample (src/observable.f90:41)
    std::vector<int8_t> job(M, 0);
    int need = 0;
    for (int m = 0; m < M; ++m) {
        if (!(g[m] & mask)) continue;
        if (batched && b.obs_in[m]) job[m] = ((g[m] & 4) && b.members[m]->c.spiral_ptr) ? 2 : 0;
        else job[m] = 1;
        need += job[m] ? 1 : 0;
    }
    if (need == 0) return ETHER_OK;
    const int nbr = std::min(kMemberBranches, need);
    if (nbr > 1) {
        const int rc = fork_branches(b, nbr);
        if (rc) return rc;
    }
    for (int m = 0, k = 0; m < M; ++m) {
        if (!job[m]) continue;
        OnBatchStream on(b.members[m]->c, nbr > 1 ? b.branch[k++ % nbr] : b.stream);
        if (job[m] == 2) {
            BCUDA(launch_spiral_measure(on.c));
            continue;
        }
        const int rc = before ? mcs_before_sweep(on.c, sch, g[m]) : mcs_after_sweep(on.c, g[m]);
        if (rc) return rc;
    }
    return nbr > 1 ? join_branches(b, nbr) : ETHER_OK;
}

// Steps of the MCS loop, gates sig[k * M + m] for step k and member m: every member's
// overrelaxation, the batch sweep, every member's PT and measurement.
int issue_mcs_steps(ether_batch &b, const ether_schedule *sch, const int8_t *sig, int n) {
    const int M = (int)b.members.size();
    for (int k = 0; k < n; ++k) {
        int rc = issue_member_parts(b, sch, sig + (size_t)k * M, true);
        if (rc) return rc;
        rc = issue_sweep(b);
        if (rc) return rc;
        rc = issue_member_parts(b, sch, sig + (size_t)k * M, false);
        if (rc) return rc;
    }
    b.launches += (uint64_t)n * kernels_per_sweep(b);
    return ETHER_OK;
}

}  // namespace

extern "C" int ether_batch_create(ether_ctx *const *members, int32_t n_members, ether_batch **out) {
    if (!out) return bfail(ETHER_ERR_ARG, "null output handle");
    *out = nullptr;
    if (!members || n_members < 1) return bfail(ETHER_ERR_ARG, "a batch needs at least one member");
    std::vector<ether_ctx *> mem(members, members + n_members);
    for (int i = 0; i < n_members; ++i) {
        if (!mem[i]) return bfail(ETHER_ERR_ARG, "null member context");
        for (int j = 0; j < i; ++j)
            if (mem[j] == mem[i]) return bfail(ETHER_ERR_ARG, "a context appears twice in the batch");
    }
    ether_batch *b = new ether_batch();
    b->members = mem;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
    int l2 = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
    b->l2_bytes = l2;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    b->ev_member.assign(mem.size(), nullptr);
    for (size_t k = 0; e == cudaSuccess && k < mem.size(); ++k)
        e = cudaEventCreateWithFlags(&b->ev_member[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev_t0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev_t1);
    std::vector<uint32_t *> step_of;
    for (ether_ctx *h : mem)
        for (int r = 0; r < h->c.R; ++r) step_of.push_back(h->c.step + r);
    b->total_R = (int)step_of.size();
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_step_of, step_of.size() * sizeof(uint32_t *));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_step_of, step_of.data(), step_of.size() * sizeof(uint32_t *), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        ether_batch_destroy(b);
        return bfail(ETHER_ERR_CUDA, std::string("batch set-up: ") + cudaGetErrorString(e));
    }
    *out = b;
    return ETHER_OK;
}

extern "C" int ether_batch_destroy(ether_batch *b) {
    if (!b) return ETHER_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    drop_mcs_graphs(*b);
    for (cudaEvent_t ev : b->ev_member)
        if (ev) cudaEventDestroy(ev);
    if (b->ev_done) cudaEventDestroy(b->ev_done);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    for (cudaEvent_t ev : b->ev_join) cudaEventDestroy(ev);
    for (cudaStream_t st : b->branch) cudaStreamDestroy(st);
    if (b->ev_t0) cudaEventDestroy(b->ev_t0);
    if (b->ev_t1) cudaEventDestroy(b->ev_t1);
    if (b->d_members) cudaFree(b->d_members);
    if (b->d_segs) cudaFree(b->d_segs);
    if (b->d_step_of) cudaFree(b->d_step_of);
    if (b->d_block_first) cudaFree(b->d_block_first);
    if (b->d_obs) cudaFree(b->d_obs);
    if (b->d_obs_off) cudaFree(b->d_obs_off);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return ETHER_OK;
}

extern "C" int ether_batch_metropolis(ether_batch *b, int32_t nsweeps) {
    if (!b) return bfail(ETHER_ERR_ARG, "null batch");
    if (nsweeps < 0) return bfail(ETHER_ERR_ARG, "negative sweep count");
    if (nsweeps == 0) return ETHER_OK;
    int rc = join_members(*b);
    if (rc) return rc;
    rc = run_sweeps(*b, nsweeps, true);
    if (rc) return rc;
    b->timed_sweeps = nsweeps;
    return release_members(*b);
}

extern "C" int ether_batch_mcs(ether_batch *b, const ether_schedule *sch, int32_t step0, int32_t nsteps,
                               int32_t *swap_counts) {
    if (!b || !sch) return bfail(ETHER_ERR_ARG, "null argument");
    if (sch->coa <= 0 || nsteps < 0 || step0 < 0)
        return bfail(ETHER_ERR_ARG, "coa must be positive, step0 and nsteps >= 0");
    const int M = (int)b->members.size();
    bool ovrr_on = false;
    for (ether_ctx *h : b->members) {
        const int rc = mcs_check(h->c, sch);
        if (rc) return rc;
        ovrr_on = ovrr_on || mcs_ovrr_on(h->c, sch);
    }
    const bool pt_on = sch->pt && sch->exchange_interval > 0;
    int rc = rebuild(*b);
    if (rc) return rc;
    rc = join_members(*b);
    if (rc) return rc;
    rc = build_obs(*b);
    if (rc) return rc;
    // every member's device swap counter starts from the caller's value, as ether_mcs does
    std::vector<int32_t> sc(M, 0);
    if (swap_counts) sc.assign(swap_counts, swap_counts + M);
    for (int m = 0; m < M; ++m)
        BCUDA(cudaMemcpyAsync(b->members[m]->c.swap_dev, &sc[m], sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
    const int chunk = mcs_chunk(mcs_period(sch, ovrr_on, pt_on));
    // the key's tail: what the captured launches take besides the gates
    std::string tail = "/" + std::to_string(sch->ovrr_para);
    for (ether_ctx *h : b->members)
        tail += "/" + std::to_string(h->c.n_slots) + (h->c.spiral_ptr ? "s" : "");
    BCUDA(cudaEventRecord(b->ev_t0, b->stream));
    std::vector<int8_t> sig;
    for (int step = step0 + 1, last = step0 + nsteps; step <= last;) {
        const int n = std::min(chunk, last - step + 1);
        sig.clear();
        for (int k = 0; k < n; ++k)
            for (int m = 0; m < M; ++m) sig.push_back((int8_t)mcs_gates(b->members[m]->c, sch, step + k));
        if (n < 4) {
            rc = issue_mcs_steps(*b, sch, sig.data(), n);
            if (rc) return rc;
        } else {
            std::string key(sig.begin(), sig.end());
            key += tail;
            auto it = b->mcs_graphs.find(key);
            if (it == b->mcs_graphs.end()) {
                if (b->mcs_graphs.size() >= 64) drop_mcs_graphs(*b);
                cudaGraph_t g = nullptr;
                BCUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
                const uint64_t before = b->launches;
                rc = issue_mcs_steps(*b, sch, sig.data(), n);
                b->launches = before;
                cudaError_t e = cudaStreamEndCapture(b->stream, &g);
                if (rc) {
                    if (g) cudaGraphDestroy(g);
                    return rc;
                }
                if (e != cudaSuccess) return bfail(ETHER_ERR_CUDA, std::string("batch MCS capture: ") + cudaGetErrorString(e));
                cudaGraphExec_t ex = nullptr;
                e = cudaGraphInstantiate(&ex, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) return bfail(ETHER_ERR_CUDA, std::string("batch MCS instantiate: ") + cudaGetErrorString(e));
                it = b->mcs_graphs.emplace(key, ex).first;
            }
            BCUDA(cudaGraphLaunch(it->second, b->stream));
            b->launches += (uint64_t)n * kernels_per_sweep(*b);
        }
        step += n;
    }
    BCUDA(cudaEventRecord(b->ev_t1, b->stream));
    b->timed_sweeps = nsteps;
    if (swap_counts) {
        for (int m = 0; m < M; ++m)
            BCUDA(cudaMemcpyAsync(&sc[m], b->members[m]->c.swap_dev, sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream));
        BCUDA(cudaStreamSynchronize(b->stream));
        std::copy(sc.begin(), sc.end(), swap_counts);
    }
    return release_members(*b);
}

extern "C" int ether_batch_set_config(ether_batch *b, int32_t threads, int32_t units_per_thread,
                                      int32_t blocks_per_sm, int32_t walk) {
    if (!b) return bfail(ETHER_ERR_ARG, "null batch");
    if (!(threads == 64 || threads == 128 || threads == 256))
        return bfail(ETHER_ERR_ARG, "threads per block must be 64, 128 or 256");
    if (units_per_thread < 1 || units_per_thread > 64) return bfail(ETHER_ERR_ARG, "units per thread out of [1, 64]");
    if (blocks_per_sm < 0 || blocks_per_sm > 32) return bfail(ETHER_ERR_ARG, "blocks per SM out of [0, 32]");
    if (walk < 0 || walk > 2)
        return bfail(ETHER_ERR_ARG, "walk must be 0 (strided), 1 (contiguous) or 2 (one block per tile)");
    b->walk = walk;
    b->threads = threads;
    b->upt = units_per_thread;
    b->bps = blocks_per_sm;
    b->group_bytes = 0;  // the class kernels over L2-sized groups, with this tile shape
    b->xyz_solo = false;
    b->dirty = true;
    return ETHER_OK;
}

extern "C" int ether_batch_autotune(ether_batch *b, int32_t *config, float *best_ms) {
    if (!b) return bfail(ETHER_ERR_ARG, "null batch");
    int rc = join_members(*b);
    if (rc) return rc;
    // back up every member's spins, sweep counters and acceptance counters
    struct Saved {
        void *src;
        size_t bytes;
        size_t off;
    };
    std::vector<Saved> sv;
    size_t total = 0;
    for (ether_ctx *h : b->members) {
        const Ctx &c = h->c;
        const size_t sb = c.model == ETHER_MODEL_ISING ? (size_t)c.R * c.N : (size_t)c.R * c.N * sizeof(float4);
        void *sp = c.model == ETHER_MODEL_ISING ? (void *)c.spins : (void *)c.spins4;
        for (auto [p, n] : {std::pair<void *, size_t>{sp, sb}, {(void *)c.step, c.R * sizeof(uint32_t)},
                            {(void *)c.acc_count, c.R * sizeof(unsigned long long)}}) {
            sv.push_back(Saved{p, n, total});
            total += (n + 255) / 256 * 256;
        }
    }
    char *backup = nullptr;
    BCUDA(cudaMalloc((void **)&backup, std::max<size_t>(total, 1)));
    for (const Saved &s : sv) BCUDA(cudaMemcpyAsync(backup + s.off, s.src, s.bytes, cudaMemcpyDeviceToDevice, b->stream));
    const int old_t = b->threads, old_u = b->upt, old_b = b->bps;
    const long long old_gb = b->group_bytes;
    const bool old_xs = b->xyz_solo;
    b->group_bytes = 0;  // the class-kernel stages below use L2-sized groups
    b->xyz_solo = false;
    b->timed_sweeps = 0;
    int occ_max = 1;
    float best = 1e30f;
    int bt = old_t, bu = old_u, bb = old_b;
    rc = ETHER_OK;
    const int old_minb = b->minb, old_walk = b->walk;
    int bm = old_minb, bw = old_walk;
    for (int cand = 0; cand < 6 && !rc; ++cand) {
        const int minb = cand < 2 ? 1 : cand < 4 ? 3 : 4, threads = (cand & 1) ? 256 : 128;
        occ_max = 1;  // the largest occupancy among the classes present
        for (ether_ctx *h : b->members)
            occ_max = std::max(occ_max, class_occupancy(class_of(describe(h->c)), minb, threads));
        for (int upt : {1, 2, 4, 8, 16, 32}) {
            // persistent grids of all resident blocks or half of them (strided walk), and
            // one block per tile
            for (int v = 0; v < 3; ++v) {
                if (v == 1 && occ_max == 1) continue;
                const int walk = v == 2 ? 2 : 0;
                const int bps = v == 0 ? occ_max : v == 1 ? occ_max / 2 : 0;
                b->minb = minb;
                b->walk = walk;
                b->threads = threads;
                b->upt = upt;
                b->bps = bps;
                b->dirty = true;
                rc = run_sweeps(*b, 1, false);  // warm-up (also builds and captures)
                if (!rc) rc = run_sweeps(*b, 2, true);
                if (rc) break;
                float ms = 0.f;
                if (cudaEventSynchronize(b->ev_t1) != cudaSuccess ||
                    cudaEventElapsedTime(&ms, b->ev_t0, b->ev_t1) != cudaSuccess) {
                    rc = bfail(ETHER_ERR_CUDA, "batch autotune timing");
                    break;
                }
                ms *= 0.5f;
                if (ms < best) {
                    best = ms;
                    bt = threads;
                    bu = upt;
                    bb = bps;
                    bm = minb;
                    bw = walk;
                }
            }
            if (rc) break;
        }
        if (rc) break;
    }
    // then the contiguous walk with the cost model that splits the segment runs between blocks
    const float old_cost = b->xyz_cost;
    float bc = old_cost;
    for (float cost : {8.f, 14.f, 20.f, 32.f, 48.f}) {
        if (rc) break;
        b->threads = bt;
        b->upt = bu;
        b->bps = bb;
        b->minb = bm;
        b->xyz_cost = cost;
        b->walk = 1;
        b->dirty = true;
        rc = run_sweeps(*b, 1, false);
        if (!rc) rc = run_sweeps(*b, 2, true);
        if (rc) break;
        float ms = 0.f;
        if (cudaEventSynchronize(b->ev_t1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, b->ev_t0, b->ev_t1) != cudaSuccess) {
            rc = bfail(ETHER_ERR_CUDA, "batch autotune timing");
            break;
        }
        ms *= 0.5f;
        if (ms < best) {
            best = ms;
            bc = cost;
            bw = 1;
        }
    }
    // then the number of parallel graph branches the member groups are spread over
    const int old_nb = b->n_branch;
    int bnb = old_nb;
    for (int nb : {1, 2, 4, 8}) {
        if (rc) break;
        b->threads = bt;
        b->upt = bu;
        b->bps = bb;
        b->minb = bm;
        b->xyz_cost = bc;
        b->walk = bw;
        b->n_branch = nb;
        b->dirty = true;
        rc = run_sweeps(*b, 1, false);
        if (!rc) rc = run_sweeps(*b, 2, true);
        if (rc) break;
        float ms = 0.f;
        if (cudaEventSynchronize(b->ev_t1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, b->ev_t0, b->ev_t1) != cudaSuccess) {
            rc = bfail(ETHER_ERR_CUDA, "batch autotune timing");
            break;
        }
        ms *= 0.5f;
        if (ms < best) {
            best = ms;
            bnb = nb;
        }
    }
    // last, every member on its own phase kernels (each member a group of its own, on the
    // graph's parallel branches): the batch is then never slower than the members' own launches
    // by more than the graph's own cost; and the hybrid of XYZ members on their own kernels
    // with Ising members in the class kernels
    long long bgb = 0;
    bool bxs = false;
    bool have_xyz = false, have_ising = false;
    for (ether_ctx *h : b->members) (h->c.model == ETHER_MODEL_XYZ ? have_xyz : have_ising) = true;
    for (int cand = 0; cand < 6; ++cand) {
        if (rc) break;
        const int nb = (cand % 3 == 0) ? 4 : (cand % 3 == 1) ? 8 : 16;
        const bool hybrid = cand >= 3;
        if (hybrid && !(have_xyz && have_ising)) continue;
        b->threads = bt;
        b->upt = bu;
        b->bps = bb;
        b->minb = bm;
        b->xyz_cost = bc;
        b->walk = bw;
        b->n_branch = nb;
        b->group_bytes = hybrid ? 0 : 1;
        b->xyz_solo = hybrid;
        b->dirty = true;
        rc = run_sweeps(*b, 1, false);
        if (!rc) rc = run_sweeps(*b, 2, true);
        if (rc) break;
        float ms = 0.f;
        if (cudaEventSynchronize(b->ev_t1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, b->ev_t0, b->ev_t1) != cudaSuccess) {
            rc = bfail(ETHER_ERR_CUDA, "batch autotune timing");
            break;
        }
        ms *= 0.5f;
        if (ms < best) {
            best = ms;
            bnb = nb;
            bgb = hybrid ? 0 : 1;
            bxs = hybrid;
        }
    }
    b->group_bytes = rc ? old_gb : bgb;
    b->xyz_solo = rc ? old_xs : bxs;
    b->n_branch = rc ? old_nb : bnb;
    for (const Saved &s : sv) cudaMemcpyAsync(s.src, backup + s.off, s.bytes, cudaMemcpyDeviceToDevice, b->stream);
    cudaStreamSynchronize(b->stream);
    cudaFree(backup);
    b->threads = rc ? old_t : bt;
    b->upt = rc ? old_u : bu;
    b->bps = rc ? old_b : bb;
    b->xyz_cost = rc ? old_cost : bc;
    b->minb = rc ? old_minb : bm;
    b->walk = rc ? old_walk : bw;
    b->dirty = true;
    if (rc) return rc;
    int rr = release_members(*b);
    if (rr) return rr;
    if (config) {
        config[0] = b->threads;
        config[1] = b->upt;
        config[2] = b->bps;
        config[3] = b->walk;
    }
    if (best_ms) *best_ms = best;
    return ETHER_OK;
}

extern "C" int ether_batch_get_info(ether_batch *b, ether_batch_info *info) {
    if (!b || !info) return bfail(ETHER_ERR_ARG, "null argument");
    int rc = rebuild(*b);
    if (rc) return rc;
    if (b->timed_sweeps > 0) {
        float ms = 0.f;
        BCUDA(cudaEventSynchronize(b->ev_t1));
        BCUDA(cudaEventElapsedTime(&ms, b->ev_t0, b->ev_t1));
        b->last_ms = ms / b->timed_sweeps;
        b->timed_sweeps = 0;
    }
    info->n_members = (int32_t)b->members.size();
    info->n_replicas = b->total_R;
    info->threads = b->threads;
    info->units_per_thread = b->upt;
    info->blocks_per_sm = b->grid / std::max(1, b->sm_count);
    info->grid = b->grid;
    info->walk = b->walk;
    info->n_segments = 0;
    for (int n : b->seg_cnt) info->n_segments += n;
    info->kernels_per_sweep = kernels_per_sweep(*b);
    info->site_updates_per_sweep = b->updates_per_sweep;
    info->kernel_launches = b->launches;
    info->last_sweep_ms = b->last_ms;
    return ETHER_OK;
}

extern "C" int ether_batch_get_stream(ether_batch *b, void **stream) {
    if (!b || !stream) return bfail(ETHER_ERR_ARG, "null argument");
    *stream = (void *)b->stream;
    return ETHER_OK;
}
