// internal.h -- context layout shared by the C-ABI implementation and the kernels.
//
// Device layout (all replicas of one context share the lattice tables):
//   * Sites are stored colour-major: storage index s = col_off[colour[i]] + rank_in_colour[i].
//     For an even simple-cubic lattice this is the two-array checkerboard split
//     (colour 0 = even x+y+z), and the rank inside a colour class is
//     (z*L2 + y)*(L1/2) + x/2, so kernels address neighbours arithmetically.
//   * Ising spins: uint8 0/1 (1 = Sz=+1), spins[r*N + s].  3 B of HBM traffic per update.
//   * XYZ spins:  float4 (Sx, Sy, Sz, phi), spins4[r*N + s].  48 B per update.
//   * Neighbours: CSR in storage order (row of s = its reference nn list, shells in
//     order, neighbours in the reference's increasing-index order), values = storage
//     indices; per slot a coupling index jidx = b*nsp*nsp + (si-1)*nsp + (sj-1) and, for
//     Ising, a threshold-table stride.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <map>
#include <string>
#include <vector>

#include "../../include/ether_gpu.h"

namespace ether {

constexpr int kMaxColours = 64;

// Division by a loop-invariant divisor d >= 1 for 0 <= n < 2^31, by multiply and shift
// (Granlund & Montgomery, "Division by invariant integers using multiplication", PLDI 1994;
// round-up variant): l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1,
// n / d = (umulhi(n, m) + n) >> l.  The sum cannot overflow because n < 2^31.
struct FastDiv {
    uint32_t d, m, l;
};
inline FastDiv make_fastdiv(uint32_t d) {
    uint32_t l = 0;
    while ((1ull << l) < d) ++l;
    const uint64_t m = ((1ull << 32) * ((1ull << l) - d)) / d + 1;
    return FastDiv{d, (uint32_t)m, l};
}
#if defined(__CUDACC__)
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
    return (__umulhi(n, f.m) + n) >> f.l;
}
#endif

struct DevTables {
    // lattice (storage order)
    int32_t *row_ptr = nullptr;   // N+1
    int32_t *nbr = nullptr;       // nnz, storage indices
    uint16_t *jidx = nullptr;     // nnz
    int32_t *wstride = nullptr;   // nnz (Ising table strides)
    uint8_t *species = nullptr;   // N (1-based)
    uint16_t *itype = nullptr;    // N (Ising table site type)
    int32_t *type_base = nullptr; // n_types: offset of a type's table inside one slot's table
    int32_t *type_half = nullptr; // n_types: entries per own-spin half
    float *J = nullptr;           // nJ * 3 (FP32 couplings)
    double *Jd = nullptr;         // nJ * 3 (FP64 couplings, Ising energy)
    float *zee = nullptr;         // nsp * 3: -g mb s H
    double *zeed = nullptr;       // nsp * 3
    float *D = nullptr;           // nsp * 3 (SIA)
    double *mweight = nullptr;    // N: stgg * s(species)
    float *mweight_f = nullptr;   // N: the same in FP32 when every weight is exact in FP32
    int32_t *site_of_storage = nullptr;  // N: 0-based site number of a storage index
    int32_t *storage = nullptr;          // N: storage index of a 0-based site number
    // neighbour lists per colour class in ELL form: entry k of rank rho of colour c at
    // ell_off[c] + k * n_c + rho (same order as the CSR), padded to the class's widest site
    int32_t *ell_nbr = nullptr;   // storage indices
    uint16_t *ell_j = nullptr;    // XYZ: coupling index (into J4)
    int32_t *ell_ws = nullptr;    // Ising: stride of the threshold-table index
    uint16_t *ell_deg = nullptr;  // N: neighbours of a storage index
    int2 *ell_desc = nullptr;     // per colour: (offset of its ELL block, entries per rank)
    float4 *J4 = nullptr;         // nJ: (Jxx, Jyy, Jzz, 0) in FP32
    uint8_t *sia_cls = nullptr;   // N: local-axis anisotropy class of a storage index
    float4 *sia_ax = nullptr;     // classes: (a_x, a_y, a_z, D) in FP32
};

struct Ctx {
    // configuration
    int N = 0, nsp = 0, nsh = 0, cap = 0, model = 0, angle = 0, zeeman = 0, sia = 0;
    int sia_local = 0;  // per-site local-axis anisotropy classes present (XYZ)
    double dphi = 0, h[3] = {0, 0, 0}, g = 0, mb = 0;
    int R = 0;
    uint32_t seed = 0;
    int flags = 0;
    // colouring
    int ncol = 0;
    int col_off[kMaxColours + 1] = {0};
    long nnz = 0;  // neighbour-list entries (CSR)
    std::vector<long> ell_off;    // per colour: offset of its ELL block
    std::vector<int> ell_width;   // per colour: entries per rank
    std::vector<int32_t> colour, rank, storage;  // per site (0-based index)
    std::vector<int32_t> site_of_storage;
    // fast simple-cubic path
    bool fast = false;
    int L[3] = {0, 0, 0};
    int vec_bytes = 0;  // Ising bytes per thread in the SC kernel
    // Ising tables
    int n_types = 0, table_entries = 0;
    std::vector<int32_t> h_type_base, h_type_half;
    std::vector<std::vector<int>> type_groupcount;  // per type: neighbours per group
    std::vector<int32_t> type_species;
    std::vector<double> s_len;     // spin length per species
    std::vector<double> pos;       // 3N cartesian positions ion(6:8), storage order
    std::vector<float> h_Jf;       // nJ * 3 FP32 couplings (host copy)
    std::vector<double> h_Jd;      // nJ * 3 FP64 couplings
    // PT ladder
    int n_slots = 0, n_groups = 1;
    std::vector<double> beta_slots;  // n_slots
    bool beta_set = false;
    // device
    cudaStream_t stream = nullptr;
    DevTables t;
    uint8_t *spins = nullptr;    // Ising
    float4 *spins4 = nullptr;    // XYZ
    double *beta_slot = nullptr; // n_slots
    float *beta_slot_f = nullptr;
    int32_t *slot_of_rep = nullptr;  // R (slot within group)
    int32_t *rep_of_slot = nullptr;  // R (group*n_slots + slot -> replica)
    uint32_t *thr = nullptr;     // n_slots * table_entries: flip iff u32 <= thr
    int ising_vpt = 1;           // vectors per thread of the simple-cubic Ising kernel
    bool ising_persist = false;  // persistent simple-cubic Ising kernel
    bool ising_cap = false;      // register-capped (four blocks per SM) instantiation
    bool ising_cap5 = false;     // register-capped to five blocks per SM (48 registers)
    bool ising_stream = false;   // shared-memory staged simple-cubic Ising kernel
    int xyz_variant = 11;        // simple-cubic XYZ kernel: 10 * sites per thread + blocks per SM cap
    bool resident = false;       // ether_mcs runs runs of sweeps with ising_sc_resident
    int *err = nullptr;          // device: first bounded-wait failure of a kernel (0 = none)
    unsigned long long *acc_before = nullptr;  // R: acceptance counts at the start of a call
    double *acc_ratio = nullptr;               // R: device acceptance ratios of a call
    double *acc_host = nullptr;                // R: pinned host copy
    void *stage = nullptr;                     // pinned staging of ether_{set,get}_spins_batch
    bool ion_direct = false;                   // the device reads / writes the host records in place
    // ether_{set,get}_spins_batch where ion_direct: measured rates (replicas per second) of the
    // in-place kernel and of the host's staged conversion, per direction (0 read-back, 1
    // upload), the replicas the kernel moved in the last call, and the kernel's timing events
    double ion_rate_k[2] = {0.0, 0.0}, ion_rate_h[2] = {0.0, 0.0};
    int ion_last_kernel[2] = {0, 0};
    int ion_gets = 0;  // read-backs so far (the first three try the kernel, the cores, the kernel)
    cudaEvent_t ion_ev[2] = {nullptr, nullptr};
    cudaStream_t ion_copy = nullptr;  // the host's staged copies beside the in-place kernel
    size_t stage_bytes = 0;
    int32_t *spiral_ptr = nullptr, *spiral_nbr = nullptr;  // spiral partners, CSR in storage order
    long spiral_count = 0;
    double *spiral_part = nullptr;  // R * spiral_blocks * 3: block partials of the spiral sum
    double *spiral_sums = nullptr;  // 4R per (group, slot): samples, x, x^2, x^4
    int spiral_blocks = 0;
    // acceptance by temperature: acc_count is per replica; acc_slot[g * n_slots + slot]
    // collects each replica's accepts at the slot it held, binned before every PT swap
    unsigned long long *acc_slot = nullptr;  // R
    unsigned long long *acc_mark = nullptr;  // R: acc_count at the last binning
    uint32_t *stream_id = nullptr;  // R
    uint32_t *step = nullptr;       // R (Metropolis sweep counter)
    uint32_t *ovrr_step = nullptr;  // R
    uint32_t *fresh_call = nullptr; // R
    unsigned long long *acc_count = nullptr;  // R
    double *E = nullptr;         // 2R: raw energy, exchange part
    double *M = nullptr;         // 3R
    double *sums = nullptr;      // 7R (per group*n_slots + slot)
    double *partials = nullptr;  // scratch for reductions
    int partial_blocks = 0;
    // exact shortcuts of the energy reduction (k_obs.cu): every bond's z coupling equal
    // (ising_juni, Ising), every |weight| equal (mw_abs), every weight exact in FP32
    bool juni_set = false, mw_pos = false;
    double ising_juni = 0.0, mw_abs = 0.0;
    int32_t *pt_accepts = nullptr;  // 1
    int32_t *swap_dev = nullptr;    // 1: PT swap counter
    int32_t *copy_from = nullptr;   // R (reference-copy PT mode)
    std::map<std::string, cudaGraphExec_t> graphs;  // ether_mcs chunks by gate pattern
    // replica window of the general-lattice sweep launchers and launch_advance: replicas
    // rw0 .. rw0 + rwn - 1 (rwn 0: all); ether_mcs runs parts of a general lattice's replicas
    // on c.stream and the aux streams side by side between its PT and measurement steps
    static constexpr int kMaxParts = 4;
    int rw0 = 0, rwn = 0;
    int n_parts = 0;
    cudaStream_t aux[kMaxParts - 1] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev_fork = nullptr, ev_join[kMaxParts - 1] = {nullptr, nullptr, nullptr};
    size_t device_bytes = 0;
    uint64_t launches = 0;
    float sq_ms = 0.f;  // last structure-factor kernel time (CUDA events)
    int sm_count = 0;
};

// One context's observables and PT state as the batched observable kernels see it
// (obs_member, k_obs.cu): a member of a device table.
struct ObsMember {
    const uint8_t *spins;
    const float4 *spins4;
    int N, model, zeeman, sia;
    const int32_t *row_ptr, *nbr;
    const uint16_t *jidx;
    const float *J;
    const double *Jd;
    const uint8_t *species;
    const float *zee;
    const double *zeed;
    const float *D;
    const uint8_t *sia_cls;  // null unless local-axis anisotropy
    const float4 *sia_ax;
    const double *mweight;
    const float *mweight_f;  // null unless every weight is exact in FP32
    // simple-cubic contexts (sc_xyz = 1 XYZ, sc_ising = 1 Ising in the counting form):
    // neighbours in closed form from the colour arrays; mw_pos: every weight is +mw_abs
    int sc_xyz, sc_L1, sc_L2, sc_L3, sc_ising, mw_pos;
    FastDiv sc_fH, sc_fL2;
    float sc_jx, sc_jy, sc_jz;
    float mw_abs_f;          // mw_abs in FP32 (exact when mweight_f is set)
    int sc_pad2, sc_pad3;
    double juni, mw_abs;     // Ising counting form: the one bond coupling, the one |weight|
    int count_form, nsp;     // count_form: Ising sums by integer counts (juni, mw_abs, one species)
    double *partials;
    int nblk, R;             // energy blocks per replica, replicas
    double *E, *M, *sums;
    int n_slots, n_groups;
    const double *beta_slot;
    int32_t *rep_of_slot, *slot_of_rep, *copy_from, *swap_dev, *pt_accepts;
    uint32_t seed;
    int true_energy;
    const unsigned long long *acc_count;
    unsigned long long *acc_mark, *acc_slot;
};

// A device table of members and the prefix offsets the batched kernels index it by:
// eoff energy blocks (R * nblk), roff replicas, poff PT pairs (n_groups * (n_slots/2 + 1)),
// each of length M + 1.
struct ObsTable {
    const ObsMember *mem = nullptr;
    const int32_t *eoff = nullptr, *roff = nullptr, *poff = nullptr;
    int M = 0, eblocks = 0, rtotal = 0, ptotal = 0;
};
ObsMember obs_member(const Ctx &c);
// The per-member sequences of launch_energy_mag, launch_pt(c, -1) (true-swap mode) and
// launch_measure for every member of the table, one launch per kernel on stream st.
cudaError_t launch_batch_energy(const ObsTable &t, cudaStream_t st);
cudaError_t launch_batch_pt(const ObsTable &t, cudaStream_t st);
cudaError_t launch_batch_measure(const ObsTable &t, cudaStream_t st);

// kernel launchers (k_*.cu)
cudaError_t launch_ising_sweep(Ctx &c, int colour);
bool ising_resident_possible(const Ctx &c, size_t smem_max);
cudaError_t prepare_ising_resident(const Ctx &c);
cudaError_t launch_ising_resident(Ctx &c, int nsweeps);
bool ising_stream_supported(const Ctx &c, int vectors_per_step);
cudaError_t launch_xyz_sweep(Ctx &c, int colour);
bool xyz_variant_valid(int variant);
cudaError_t launch_overrelax(Ctx &c, int colour, int pass, float part);
cudaError_t launch_fresh(Ctx &c);
cudaError_t launch_advance(Ctx &c, uint32_t *counter);
cudaError_t launch_accept_ratio(Ctx &c, double *out);
cudaError_t launch_broadcast(Ctx &c, void *base, size_t bytes_per_replica);
// k_ion.cu: whether device dev addresses pageable host memory through the host's page tables;
// replicas r0 .. r0+n-1 from (to_device) or into the ion(0:8, N, n) records at ion, on c.stream
bool ion_direct_possible(int dev);
cudaError_t launch_ion_copy(Ctx &c, int r0, int n, double *ion, bool to_device);
cudaError_t launch_energy_mag(Ctx &c, bool want_energy);
cudaError_t launch_measure(Ctx &c);
// Row t of the |M| (and E) series; with t_dev the row is read from device memory and
// advanced afterwards (for captured graphs).
cudaError_t launch_record(Ctx &c, int t, bool want_e, double *mser, double *eser, int32_t *t_dev = nullptr);
cudaError_t launch_pt(Ctx &c, int set_swap_count);
cudaError_t launch_acc_bin(Ctx &c);
cudaError_t launch_spiral_measure(Ctx &c);
int energy_blocks(const Ctx &c);
int plain_sweep(Ctx &c);  // one Metropolis sweep of every replica (ETHER_OK or an error code)
int ctx_variant(const Ctx &c);  // the context's kernel variant code (ether_set_variant's numbering)
void *tma_encode_tiled_fn();    // cuTensorMapEncodeTiled (PFN_cuTensorMapEncodeTiled_v12000), or null

// Pieces of one MCS of src/ether.f90:159-203, shared by ether_mcs and ether_batch_mcs.  The
// launches go to c.stream.
bool mcs_ovrr_on(const Ctx &c, const ether_schedule *sch);     // overrelaxes at all
int mcs_check(const Ctx &c, const ether_schedule *sch);        // beta set, PT ladder
int mcs_gates(const Ctx &c, const ether_schedule *sch, int step);  // 1 OVRR, 2 PT, 4 measure
int mcs_before_sweep(Ctx &c, const ether_schedule *sch, int gates);
int mcs_after_sweep(Ctx &c, int gates);
long mcs_period(const ether_schedule *sch, bool ovrr_on, bool pt_on);
int mcs_chunk(long period);
void set_error(const std::string &msg);
int structure_factor_launch(Ctx &c, const double *frac, const int nq[3], const double q0[3],
                            const double dq[3], float *sq_host, float *comp_host, std::string &msg);

}  // namespace ether

// The opaque handle of the C-ABI.
struct ether_ctx {
    ether::Ctx c;
};

namespace ether {
}  // namespace ether
