/*
 * ether_gpu.h -- C-ABI of the GB300 Monte Carlo sweep for ETHER (mukkelian/Ether).
 *
 * The reference has no plugin or FFI layer: its hot path is a set of Fortran subroutine
 * calls inside the MCS loop of src/ether.f90 that share state through `module init`
 * (src/init.f90:20-98).  Each entry point below replaces one of those calls; the comment
 * on each names the reference routine (file:line) it stands in for.  A Fortran host binds
 * them with ISO_C_BINDING (fortran/ether_gpu_mod.f90); C, C++ and Python (ctypes) bind
 * them directly.
 *
 * Conventions
 *   - Every call returns int: ETHER_OK (0) or a negative ETHER_ERR_* code.  No exception
 *     crosses the ABI.  ether_last_error() returns a message for the last failure.
 *   - Arrays are passed in the reference's own Fortran layouts (column-major, 1-based
 *     values where the reference stores indices):
 *         ion(0:8, N)              real(8)   ion[c + 9*i]
 *         nn(nsh, N, 0:cap, 0:1)   integer   nn[b + nsh*(i + N*(k + (cap+1)*t))]
 *         j_exc(nsh, nsp, nsp, 3)  real(8)   j_exc[b + nsh*(si + nsp*(sj + nsp*c))]
 *         sia_vec(3, nsp)          real(8)
 *     j_exc, sia_vec, h are the values after parameters.f90 (eV or J_para units).
 *   - Host buffers belong to the caller and are never retained after a call returns.
 *   - A context owns all of its device memory and one CUDA stream.  One host thread per
 *     context; calls on one context are not re-entrant.
 *   - A context holds R replicas of the lattice.  A replica is what one MPI rank held in
 *     the reference (one temperature of one REPEAT); R replicas advance together.
 */
#ifndef ETHER_GPU_H
#define ETHER_GPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ETHER_ABI_VERSION 2

enum {
    ETHER_OK = 0,
    ETHER_ERR_ARG = -1,         /* invalid argument or inconsistent descriptor            */
    ETHER_ERR_CUDA = -2,        /* CUDA runtime error (message in ether_last_error)        */
    ETHER_ERR_NOMEM = -3,       /* device or host allocation failed                       */
    ETHER_ERR_UNSUPPORTED = -4, /* valid input outside what the kernels implement          */
    ETHER_ERR_CAPACITY = -5,    /* a table outgrew its fixed capacity                      */
    ETHER_ERR_TIMEOUT = -6,     /* a bounded device-side wait ran out                      */
    ETHER_ERR_STATE = -7,       /* call out of order (e.g. no beta set)                    */
    ETHER_ERR_NODEV = -8,       /* no CUDA device                                          */
    ETHER_ERR_PARSE = -9        /* malformed input deck (in.ether, j_exchange, ...)         */
};

enum { ETHER_MODEL_ISING = 0, ETHER_MODEL_XYZ = 1 };

/* Descriptor flags. */
enum {
    ETHER_FLAG_FORCE_GENERAL = 1 << 0, /* never use the simple-cubic fast kernels           */
    ETHER_FLAG_PT_TRUE_ENERGY = 1 << 1,/* PT exponent uses the Hamiltonian energy (bonds
                                          once) instead of the reference's raw sum          */
    ETHER_FLAG_PT_REFERENCE_COPY = 1 << 2,/* PT acceptance copies the lower slot's
                                          configuration into the higher slot (what
                                          parallel_tempering.f90:92-106 effectively does)
                                          instead of exchanging the two                     */
    ETHER_FLAG_NO_GRAPHS = 1 << 3,        /* ether_mcs launches kernels one by one instead of
                                          replaying captured CUDA graphs                    */
    ETHER_FLAG_NO_RESIDENT = 1 << 4,      /* ether_mcs never runs a small simple-cubic Ising
                                          lattice's sweeps in the shared-memory resident
                                          kernel (same results, one launch per phase)        */
    ETHER_FLAG_STAGED_SPINS = 1 << 5      /* ether_{set,get}_spins_batch convert on the host's
                                          cores through pinned staging even where the device
                                          could read and write the ion records in place
                                          (same results)                                     */
};

typedef struct ether_ctx ether_ctx;

/* Everything `module init` holds that the sweep reads (src/init.f90:28-92). */
typedef struct ether_desc {
    int32_t n_sites;      /* total_ions                                                    */
    int32_t n_species;    /* nspecies                                                      */
    int32_t n_shells;     /* no_of_nbd                                                     */
    int32_t nbd_capacity; /* nbd_capacity (nn's third extent is cap+1)                     */
    int32_t model;        /* ETHER_MODEL_ISING / ETHER_MODEL_XYZ                           */
    int32_t angle;        /* ANGLE proposal (otherwise Marsaglia)                          */
    double dphi;          /* ANGLE step in radians                                         */
    int32_t zeeman;       /* Zeeman term on                                                */
    double h[3];          /* field                                                         */
    double g_factor, mb;  /* g and Bohr magneton in the run's units                        */
    int32_t sia;          /* single-ion anisotropy on (used only for XYZ, as the reference) */
    const double *ion;    /* ion(0:8, N): ID, Sx, Sy, Sz, species, phi, x, y, z            */
    const int32_t *nn;    /* nn(nsh, N, 0:cap, 0:1)                                        */
    const double *j_exc;  /* j_exc(nsh, nsp, nsp, 3)                                       */
    const double *sia_vec;/* sia_vec(3, nsp) or NULL                                       */
    const double *s;      /* s(nsp): spin length per species                               */
    const double *stgg;   /* stgg_ion(N) or NULL (all 1)                                   */
    int32_t n_replicas;   /* R                                                             */
    uint32_t seed;        /* SEED tag (src/read_input.f90:119-121)                         */
    int32_t sc[3];        /* supercell (0 = unknown); enables the simple-cubic kernels     */
    int32_t basis;        /* lattice_per_unit_cell (0 = unknown)                           */
    int32_t flags;        /* ETHER_FLAG_*                                                  */
    const double *sia_local; /* sia_local(4, N) or NULL: per-site single-ion anisotropy
                             D (a . S)^2 about a local unit axis a = sia_local(1:3, i) with
                             D = sia_local(4, i) (energy units after parameters.f90), XYZ only,
                             added to the sia_vec term.  No counterpart in the reference, whose
                             anisotropy is diagonal per species (src/get_sia_values.f90:57-58):
                             it expresses easy axes along local directions such as the
                             pyrochlore's <111>.  At most 256 distinct (a, D) per context
                             (ETHER_ERR_CAPACITY beyond).  Turns overrelaxation off in
                             ether_mcs, as the reference's SIA does (src/ether.f90:163-168). */
} ether_desc;

/* Library version / last error (thread-local message of the last failing call). */
int ether_abi_version(void);
const char *ether_last_error(void);

/* Replaces the module-init set-up that precedes the MCS loop (src/ether.f90:62-86): copies
 * the lattice, couplings and initial spins of every replica to the device, colours the
 * neighbour graph, and builds the kernels' tables. */
int ether_create(const ether_desc *desc, ether_ctx **out);
int ether_destroy(ether_ctx *ctx);

/* beta(R): 1/(kB T) per replica (src/ether.f90:142-144).  Replica r sits at temperature
 * slot r % n_slots of PT group r / n_slots; n_slots = R unless set by ether_set_ladder. */
int ether_set_beta(ether_ctx *ctx, const double *beta);
/* PT ladders: R = n_groups * n_slots replicas, each group an independent ladder (one per
 * REPEAT).  beta_slots(n_slots).  Resets the slot permutation to the identity. */
int ether_set_ladder(ether_ctx *ctx, int32_t n_slots, const double *beta_slots);
/* Random streams: replica r draws from Philox key (seed, stream[r]); step[r] is its sweep
 * counter (NULL keeps the current value).  Plays the role of random_seed(put=...) at
 * src/ether.f90:154. */
int ether_set_streams(ether_ctx *ctx, const uint32_t *stream, const uint32_t *step);

/* ion(0:8,N) <-> replica spins.  replica = -1 addresses every replica (set) / replica 0
 * (get).  Only ion(1:3,:) and ion(5,:) are read or written. */
int ether_set_spins(ether_ctx *ctx, int32_t replica, const double *ion);
int ether_get_spins(ether_ctx *ctx, int32_t replica, double *ion);
/* The same for replicas r0 .. r0+n-1 at once: ion(0:8, N, n), one reference ion array per
 * replica back to back (what a driver holds when the replica batch replaces the MPI ranks
 * of src/ether.f90:112-118, each of which owned one ion).  Where the device addresses
 * pageable host memory through the host's page tables (ether_info.ion_direct: a Grace CPU's
 * memory over NVLink-C2C), a kernel reads and writes the records' spin fields in place (an
 * XYZ set reads whole records in tiles; only the spin fields are written), beside or instead
 * of the host's conversion as measured (ether_spins_batch_split);
 * otherwise the layout conversion runs on the host's cores into pinned staging memory (up to
 * 512 MB, allocated on the first call and kept by the context), overlapped with the copies.
 * Returns when the data is in place; ion must stay valid for the call.  On the in-place path
 * ion must be host memory mapped for all n records (device memory or an unmapped page gives
 * ETHER_ERR_ARG before any launch). */
int ether_set_spins_batch(ether_ctx *ctx, int32_t r0, int32_t n, const double *ion);
int ether_get_spins_batch(ether_ctx *ctx, int32_t r0, int32_t n, double *ion);
/* How the last ether_get_spins_batch / ether_set_spins_batch divided its replicas: the number
 * moved in place by a kernel (the rest went through the host's staging).  Where both ways are
 * open, a call is shared as it runs: the kernel takes chunks of replicas from the front while
 * the host's cores take chunks from the back, until they meet (a call larger than the 512 MB
 * staging area is divided by rates measured in earlier calls). */
int ether_spins_batch_split(ether_ctx *ctx, int32_t *get_kernel, int32_t *set_kernel);

/* fresh_spins (src/fresh_spins.f90:31-38), called at src/ether.f90:155: Ising flips every
 * spin, XYZ draws a new Marsaglia / ANGLE state, on every replica. */
int ether_fresh_spins(ether_ctx *ctx);

/* Metropolis (src/Metropolis.f90:34-68), called at src/ether.f90:172: nsweeps full
 * colour-ordered sweeps of every replica.  accept(R) (may be NULL) receives the summed
 * per-sweep acceptance ratios accepted/N. */
int ether_metropolis(ether_ctx *ctx, int32_t nsweeps, double *accept);

/* overrelaxation (src/overrelaxation.f90:30-61), called at src/ether.f90:168, on every
 * replica: colour-ordered reflection S' = 2(A.S)/(A.A) A - S, normalised, of each site
 * with probability ovrr_para (ovrr_para >= 1: floor(ovrr_para) full passes first). */
int ether_overrelaxation(ether_ctx *ctx, double ovrr_para);

/* get_tot_energy (src/get_tot_energy.f90:33-47), called at src/ether.f90:177: raw sum of
 * site energies per replica (exchange counted twice, Zeeman and SIA once). E(R). */
int ether_tot_energy(ether_ctx *ctx, double *E);
/* get_tot_magnetisation (src/get_tot_magnetisation.f90:32-40): M(3,R). */
int ether_tot_magnetisation(ether_ctx *ctx, double *M);

/* observable (src/observable.f90:30-43), called at src/ether.f90:201: when
 * step > tmcs_eq and step % coa == 0, computes E and M and adds e = E/(2N), m = |M|/N,
 * and their squares and fourth powers to the accumulators of each replica's current
 * temperature slot (get_eng.f90:36-40, get_mag.f90:36-41). */
int ether_observable(ether_ctx *ctx, int32_t step, int32_t tmcs_eq, int32_t coa);
/* zeroes('avg') (src/zeroes.f90:48-55). */
int ether_zero_avg(ether_ctx *ctx);
/* Accumulators per temperature slot and group: sums(7, R) = (count, e, e2, e4, m, m2, m4),
 * slot-major within each group (index = group*n_slots + slot).  get_eng/get_mag('avg_*')
 * (src/get_eng.f90:42-60, src/get_mag.f90:43-59) and observables_per_repeat
 * (src/observables_per_repeat.f90:29-69) are ether_avg / ether_per_repeat below. */
int ether_get_sums(ether_ctx *ctx, double *sums);
/* 'avg' reductions for every slot: out(6, R) = (<e>, U_E, C_v, <|m|>, U_M, chi). */
int ether_avg(ether_ctx *ctx, double *out);
/* observables_per_repeat: mean and error over the n_groups REPEAT groups, per slot.
 * mean(6, n_slots), err(6, n_slots). */
int ether_per_repeat(ether_ctx *ctx, double *mean, double *err);

/* parallel_tempering (src/parallel_tempering.f90:39-108), called at src/ether.f90:189-198:
 * odd/even neighbour pairs of temperature slots in every group, FP64 exponent
 * delta = -(beta_hi - beta_lo)(E_lo - E_hi), swap of configurations as a swap of slot
 * indices.  Uses the energies of the last ether_tot_energy / ether_mcs step.  accepted
 * (may be NULL) receives the number of accepted pairs. */
int ether_parallel_tempering(ether_ctx *ctx, int32_t swap_count, int32_t *accepted);
/* slot_of_replica(R). */
int ether_get_slots(ether_ctx *ctx, int32_t *slot_of_replica);

/* The whole per-MCS body of src/ether.f90:159-203 for steps step0+1 .. step0+nsteps,
 * on device, replayed from CUDA graphs: OVRR gate (:163-169), Metropolis (:172),
 * total energy when PT needs it (:177), PT (:189-198), observable (:201). */
typedef struct ether_schedule {
    int32_t tmcs_eq;           /* equilibration MCS                                        */
    int32_t coa;               /* measure every coa steps                                  */
    int32_t ovrr;              /* OVRR logical                                             */
    double ovrr_para;          /* fraction of N                                            */
    int32_t ovrr_mcs;          /* OVRR every ovrr_mcs steps                                */
    int32_t pt;                /* PT logical                                               */
    int32_t exchange_interval; /* PT every exchange_interval steps                         */
} ether_schedule;
int ether_mcs(ether_ctx *ctx, const ether_schedule *sch, int32_t step0, int32_t nsteps,
              int32_t *swap_count);

/* Time series for the integrated autocorrelation time: nsweeps Metropolis sweeps; after
 * every stride-th sweep |M| (get_tot_magnetisation, src/get_tot_magnetisation.f90:32-40) and,
 * if E is not NULL, the raw energy (get_tot_energy) of every replica.  absM(R, nsweeps/stride)
 * and E(R, nsweeps/stride) are host arrays, record-major (index = t*R + r). */
int ether_record_series(ether_ctx *ctx, int32_t nsweeps, int32_t stride, double *absM, double *E);

/* Acceptance counters (accepted site updates per replica since the last reset). */
int ether_get_accept_counts(ether_ctx *ctx, uint64_t *counts);
int ether_reset_accept_counts(ether_ctx *ctx);
/* The same counts per temperature: counts(R) indexed group * n_slots + slot, each replica's
 * accepts credited to the slot it held when it made them (PT moves replicas between slots).
 * src/ether.f90:173 accumulates this count on the rank that owns a temperature. */
int ether_get_slot_accept_counts(ether_ctx *ctx, uint64_t *counts);

/* Introspection used by tests and tools. */
typedef struct ether_info {
    int32_t n_colours;       /* colour classes of the Checkerboard order                   */
    int32_t fast_path;       /* 1 when the simple-cubic kernels run                        */
    int32_t n_types;         /* Ising threshold-table site types                           */
    int32_t table_entries;   /* Ising threshold entries per temperature slot               */
    int32_t n_slots, n_groups;
    size_t device_bytes;     /* device memory owned by the context                         */
    uint64_t kernel_launches;/* kernels launched by this context so far                    */
    float sq_kernel_ms;      /* CUDA-event time of the last ether_structure_factor's kernels */
    int32_t ion_direct;      /* 1 when ether_{set,get}_spins_batch move the records by a kernel
                                in place (takes the struct's former tail padding)              */
} ether_info;
int ether_get_info(ether_ctx *ctx, ether_info *info);
/* colour(N) and rank_in_colour(N) of the Checkerboard order. */
int ether_get_colouring(ether_ctx *ctx, int32_t *colour, int32_t *rank_in_colour);
/* Block until all work on the context's stream has finished. */
int ether_sync(ether_ctx *ctx);
/* The cudaStream_t every kernel of this context is launched on (for event timing or for
 * ordering a caller's own work after the sweep). */
int ether_get_stream(ether_ctx *ctx, void **stream);
/* One colour phase of the Metropolis sweep (the inner part of ether_metropolis), without
 * advancing the sweep counter; colour in [0, n_colours).  For per-kernel timing and for
 * hosts that interleave their own work between colour classes. */
int ether_metropolis_phase(ether_ctx *ctx, int32_t colour);
/* Advance every replica's sweep counter by one (ends a sweep built from phases). */
int ether_end_sweep(ether_ctx *ctx);

/* Autotuner: times the kernel variants of this context's fast path on its own data
 * (spins and counters are restored) and keeps the fastest; the choice is cached per size
 * class for the process.  Ising simple cubic: variant = 1000 (persistent) + 2000 (register
 * cap) + bytes per vector (4, 8, 16) * 10 + vectors per thread, or 4000 + 10 * vectors per step + 1 / 4
 * (shared-memory staged kernel).  XYZ simple cubic: variant = 5000 + 10 * sites per thread +
 * blocks per SM of the register cap (5011 .. 5015, 5021 .. 5024, 5041, 5042).  best_ms = one colour
 * phase.  Either
 * output may be NULL. */
int ether_autotune(ether_ctx *ctx, int32_t *variant, float *best_ms);
/* Force a kernel variant (same encoding as ether_autotune). */
int ether_set_variant(ether_ctx *ctx, int32_t variant);

/* structure_factor (utility/Structure_Factor/structure_factor.f90:99-183) of every replica's
 * current configuration on a 3-D grid of q, on the tensor cores (BF16 high/low split
 * products, FP32 accumulation; about 16 significant bits per product).
 *   q(h) = sum_a (q0[a] + h_a dq[a]) b_a,  h_a = 0 .. nq[a]-1,  b_a the reciprocal vectors of
 *   the cell abc (rows a1, a2, a3; b_a . a_b = 2 pi delta_ab), nq[0] a multiple of 64.
 *   sq(Q, R)      = |S(q)|^2 / N^2     (the reference's real(dot_product(Cq, Cq))/N^2)
 *   comp(3, Q, R) = |S_a(q)| / N        (the reference's abs(S_q_a)/N)
 *   with q index h1 + nq[0]*(h2 + nq[1]*h3), S_a(q) = sum_i S_i,a exp(i q.r_i). */
int ether_structure_factor(ether_ctx *ctx, const double *abc, const int32_t nq[3],
                           const double q0[3], const double dq[3], float *sq, float *comp);

/* ------------------------------------------- moment vectors and the spiral state ---- */
/* get_moment_vectors (src/get_moment_vectors.f90:20-38), called at src/ether.f90:219:
 * mm(3, nsp, R) = sum over the sites of each species of stgg_i s(sp) S_i, per replica. */
int ether_moment_vectors(ether_ctx *ctx, double *mm);
/* get_spiral_state 'ions_for_spiral' (src/get_spiral_state.f90:45-77), called at
 * src/ether.f90:69 for XYZ: every site's partners j != i with |r_j - r_i| <= ss_dis and
 * angle(r_j - r_i, ss_direc) <= ss_latency degrees (ss_direc used as given, not normalised;
 * no periodic images), at most `capacity` per site (spiral_capacity; ETHER_ERR_CAPACITY
 * beyond, where the reference would write past its array).  count = spiral_count. */
int ether_spiral_setup(ether_ctx *ctx, double ss_dis, const double ss_direc[3], double ss_latency,
                       int32_t capacity, int64_t *count);
/* get_spiral_state 'spiral_state' (src/get_spiral_state.f90:79-108): ss(R) =
 * |sum_i sum_j S_i x S_j| / spiral_count per replica (the per-sample value the reference
 * accumulates into spiral_state_avg, _2_avg, _4_avg). */
int ether_spiral_state(ether_ctx *ctx, double *ss);
/* Once ether_spiral_setup has run, every measurement step of ether_mcs also accumulates the
 * spiral state per (group, slot) (src/observable.f90:41, src/get_spiral_state.f90:118-123);
 * ether_zero_avg clears it.  get_spiral_state 'avg_spiral_state'
 * (src/get_spiral_state.f90:127-140) per (group, slot): out(3, R) = <x>,
 * U = 1.5 - 0.5 <x^4>/<x^2>^2, chi = beta (<x^2> - <x>^2) spiral_count. */
int ether_spiral_avg(ether_ctx *ctx, double *out);

/* ------------------------------------------------------------------- batched sweeps ---- */
/* The reference advances one lattice at one temperature per MPI rank (src/ether.f90:112-118,
 * src/Metropolis.f90:34-68).  A batch advances the Metropolis sweeps of many contexts --
 * different lattice sizes, Ising and XYZ, each with its own ladder and replicas -- with one
 * persistent kernel per colour phase (grid = resident blocks per SM x SMs) over a table of
 * block-sized tiles, one CUDA graph per sweep.  Spins, sweep counters, random streams and
 * acceptance counters are the members' own: a batch sweep leaves every member exactly as
 * ether_metropolis(member, 1) would.  Members are distinct contexts on the current device,
 * each with beta set; they stay owned by the caller and must outlive the batch.  Batch work
 * runs on the batch's stream, after all work already queued on the members' streams and
 * before any work queued on them later. */
typedef struct ether_batch ether_batch;
int ether_batch_create(ether_ctx *const *members, int32_t n_members, ether_batch **batch);
int ether_batch_destroy(ether_batch *batch);
/* nsweeps Metropolis sweeps of every member (no overrelaxation, no PT: those stay per
 * member).  Asynchronous; ether_batch_get_info reads the time it took. */
int ether_batch_metropolis(ether_batch *batch, int32_t nsweeps);
/* The MCS loop body of src/ether.f90:159-203 (as ether_mcs) for every member at once, steps
 * step0+1 .. step0+nsteps under one schedule: each step runs every member's overrelaxation
 * where its gate is open (:163-169), one batch sweep (:172), then every member's total energy
 * + PT (:177, :189-198) and observable (:201) where theirs are; members that cannot
 * overrelax (Ising, field, anisotropy) skip that part, as in ether_mcs.  Chunks of steps are
 * captured once per gate pattern and replayed.  swap_counts(n_members), in and out, is each
 * member's PT swap counter (NULL: all start at 0).  Leaves every member exactly as
 * ether_mcs(member, sch, step0, nsteps, &swap_counts[m]) would.  Synchronous only when
 * swap_counts is given.  ether_batch_get_info's last_sweep_ms gives the time per MCS step. */
int ether_batch_mcs(ether_batch *batch, const ether_schedule *sch, int32_t step0, int32_t nsteps,
                    int32_t *swap_counts);
/* Tile shape: threads per block (64/128/256), units per thread (1..64; a unit is a 16-, 8-
 * or 4-byte vector of simple-cubic Ising sites, or one site of a general Ising lattice or of
 * XYZ), resident blocks per SM (0 = as many as fit) and the walk over the tiles (0: block b
 * of a persistent grid takes tiles b, b + grid, ...; 1: contiguous runs of equal estimated
 * cost; 2: one block per tile, blocks per SM ignored). */
int ether_batch_set_config(ether_batch *batch, int32_t threads, int32_t units_per_thread,
                           int32_t blocks_per_sm, int32_t walk);
/* Autotuner: times the tile shapes, register caps and walks on the members' data (spins
 * and counters are restored) and keeps the fastest; its last candidates run every member, or
 * every XYZ member, on its own phase kernels inside the batch graph (ether_batch_set_config
 * returns to the class kernels).  config(4) = threads, units per thread,
 * blocks per SM, walk; best_ms = one sweep.  Either output may be NULL. */
int ether_batch_autotune(ether_batch *batch, int32_t *config, float *best_ms);
typedef struct ether_batch_info {
    int32_t n_members, n_replicas;
    int32_t threads, units_per_thread, blocks_per_sm, grid, walk;
    int32_t n_segments;        /* tiles per sweep, all colour phases                        */
    int32_t kernels_per_sweep; /* colour phases + the counter advance                       */
    int64_t site_updates_per_sweep;
    uint64_t kernel_launches;  /* kernels launched by this batch so far                     */
    float last_sweep_ms;       /* CUDA-event time per sweep of the last ether_batch_metropolis
                                  (per MCS step of the last ether_batch_mcs)                */
} ether_batch_info;
int ether_batch_get_info(ether_batch *batch, ether_batch_info *info);
/* The cudaStream_t the batch launches on. */
int ether_batch_get_stream(ether_batch *batch, void **stream);

/* ------------------------------------------------------- learned patch proposal ---- */
/* No counterpart in the reference (which only has single-site moves, src/Metropolis.f90);
 * its target distribution is kept exactly: every learned move is accepted or rejected by
 * Metropolis-Hastings against the reference's energy.  Simple-cubic Ising contexts with one
 * species, one shell, no Zeeman term, or simple-cubic XYZ contexts with one species, one
 * shell, Marsaglia proposals and no Zeeman or SIA term; extents multiples of 8.
 * XYZ: the network (96 boundary spins x 3 components + beta (Jxx, Jyy, Jzz), padded to 304
 * -> 128 -> 128 -> 96, BF16 weights, CUDA cores) gives each colour-0 site a von Mises-Fisher
 * parameter m (3 outputs); the colour-1 spins are drawn from their exact heat-bath vMF
 * conditionals; params, forward outputs and dumps have the widths ether_learn_get_shape
 * returns.  Ising:
 * A learned sweep tiles each replica with 4^3 patches (a fresh random offset per sweep) and
 * updates the two patch classes in turn: the network (96 boundary spins + 4 beta J -> 128 ->
 * 128 -> 32, BF16 weights, tensor cores) proposes the patch's 32 colour-0 spins, the 32
 * colour-1 spins are drawn from their exact heat-bath conditionals, and the whole patch is
 * accepted with probability min(1, pi(new) q(old) / (pi(old) q(new))).  The plain
 * ether_metropolis sweep stays the fallback; interleave the two. */
typedef struct ether_learn ether_learn;
typedef struct ether_learn_desc {
    int32_t patch;     /* patch edge: 4                                                    */
    int32_t hidden;    /* hidden width: 128                                                */
    uint32_t seed;     /* weight initialisation and training minibatches                   */
    int64_t capacity;  /* training samples kept on the device (ring buffer), >= 1024        */
} ether_learn_desc;
int ether_learn_create(ether_ctx *ctx, const ether_learn_desc *desc, ether_learn **learn);
int ether_learn_destroy(ether_learn *learn);
/* Training data: per_replica random patches (boundary, colour-0 spins, 4 beta J) of every
 * replica's current configuration -- configurations the plain sweep produced, at every
 * temperature of the context's ladder. */
int ether_learn_collect(ether_learn *learn, int32_t per_replica);
/* steps of Adam (learning rate lr) on minibatches of `batch` samples, maximum likelihood of
 * the colour-0 spins given the boundary; loss (may be NULL) = last minibatch's mean loss. */
int ether_learn_train(ether_learn *learn, int32_t steps, int32_t batch, float lr, double *loss);
/* nsweeps learned sweeps of every replica (asynchronous, on the context's stream). */
int ether_learn_sweep(ether_learn *learn, int32_t nsweeps);
/* No counterpart in the reference (its moves are single-site).  The learned form batched over
 * contexts: n learners of n distinct contexts (any mix of models and sizes) advance together,
 * nsweeps steps of plain_per_sweep Metropolis sweeps then one learned sweep each, the steps of
 * all contexts issued in turn without waiting, so the contexts' work overlaps on the GPU.
 * Leaves every context exactly as its own calls (ether_metropolis, ether_learn_sweep) would.
 * Asynchronous. */
int ether_learn_batch_sweep(ether_learn *const *learns, int32_t n, int32_t nsweeps,
                            int32_t plain_per_sweep);
/* Device-side series for tau_int: nsteps steps of plain_per_step Metropolis sweeps then
 * learned_per_step learned sweeps, |M| of every replica after every stride-th step:
 * absM(R, nsteps / stride) host array, record-major (index = t*R + r). */
int ether_learn_record_series(ether_learn *learn, int32_t nsteps, int32_t plain_per_step,
                              int32_t learned_per_step, int32_t stride, double *absM);
/* Accepted patches per replica since creation (accepted(R)). */
int ether_learn_get_accepts(ether_learn *learn, uint64_t *accepted);
/* Parameters: W1(n_inputs,128), b1(128), W2(128,128), b2(128), W3(128,n_outputs),
 * b3(n_outputs), FP32, row = output unit; n = n_params (Ising 37152, XYZ 67936).  Setting them
 * resets the optimiser. */
int ether_learn_get_params(ether_learn *learn, float *params);
int ether_learn_set_params(ether_learn *learn, const float *params);
/* The training kernels on a given batch (Ising): x(128, B) inputs, y(B) colour-0 spins as
 * bits; loss = mean BCE, grad(37152) = its gradient (no update). */
int ether_learn_loss_grad(ether_learn *learn, const float *x, const uint32_t *y, int32_t B,
                          double *loss, float *grad);
/* The same with targets as floats y(n_outputs, B): Ising 0 / 1 per colour-0 site, XYZ the
 * colour-0 spins' components (loss = mean von Mises-Fisher negative log density). */
int ether_learn_loss_grad_f(ether_learn *learn, const float *x, const float *y, int32_t B,
                            double *loss, float *grad);
/* The inference network on x(n_inputs, B): outputs(n_outputs, B) (Ising: logits, tensor
 * cores; XYZ: the vMF parameters with the output bias). */
int ether_learn_forward(ether_learn *learn, const float *x, int32_t B, float *logits);
/* Widths of the network: inputs, outputs, parameters (Ising 128, 32, 37152). */
int ether_learn_get_shape(ether_learn *learn, int32_t *n_inputs, int32_t *n_outputs, int32_t *n_params);
/* Record the network outputs of the last sweep of the next ether_learn_sweep (Ising: the 32
 * logits; XYZ: the 96 vMF parameters with the output bias); get_dump returns them as
 * out(n_outputs, Pc, R, 2) (class, replica, patch of the class). */
int ether_learn_set_dump(ether_learn *learn, int32_t on);
int ether_learn_get_dump(ether_learn *learn, float *logits);
typedef struct ether_learn_info {
    int32_t n_params;
    int32_t train_steps;
    int64_t patches_per_class;  /* Pc per replica                                          */
    int64_t n_samples, capacity;
    uint64_t proposed;          /* patch proposals so far, all replicas                    */
    uint64_t kernel_launches;
    float last_sweep_ms;        /* CUDA-event time per learned sweep of the last call      */
    float last_train_ms;        /* CUDA-event time of the last ether_learn_train          */
} ether_learn_info;
int ether_learn_get_info(ether_learn *learn, ether_learn_info *info);

/* ------------------------------------------------------------- no-allocation energy ---- */
/* No counterpart in the reference.  Energy and magnetisation of n_replicas simple-cubic
 * configurations already in device memory, for callers that cannot allocate device memory
 * where they need the result (a framework that owns every allocation through its own pool,
 * an OpenACC / OpenMP-target Fortran driver, a service whose fixed device budget is spent):
 * ether_tot_energy needs a context, and creating one allocates.  This call allocates nothing.
 *   spins: device pointer, sites in the reference's order (x fastest), replicas one after
 *          another; int8 Sz = +-1 (Ising) or float4 (Sx, Sy, Sz, phi) (XYZ).
 *   L(3): periodic extents (>= 3 each); J(3) = diagonal exchange of the six nearest
 *   neighbours (j_exc after parameters.f90); zee(3) = -g mB s H (Zeeman), zero if off.
 *   E(n_replicas), M(3, n_replicas): host arrays, the raw sums of get_tot_energy and
 *   get_tot_magnetisation (unit stagger and spin length).  stream: cudaStream_t or NULL.
 * Scratch is 1 MiB of the library's static device memory, shared by all calls: at most 992
 * replicas per call (ETHER_ERR_CAPACITY beyond, before any memory is touched), and calls
 * that overlap on the GPU race.  The first call on a device looks up the scratch address
 * (cudaGetSymbolAddress).  Every call synchronizes `stream` before it returns (the results
 * are then in E and M), so it must not be made while that stream is being captured into a
 * CUDA graph.  `spins` that the current device cannot address (pageable host memory,
 * another device's memory, an unknown pointer) give ETHER_ERR_ARG before any launch. */
int ether_sc_energy_noalloc(int32_t model, const void *spins, const int32_t L[3],
                            int32_t n_replicas, const double J[3], const double zee[3],
                            double *E, double *M, void *stream);

/* ---------------------------------------------------------------- lattice builder ---- */
/* generate_supercell + getting_nbd (src/generate_supercell.f90:38-132,
 * src/getting_nbd.f90:34-82, src/search_nbd.f90:20-64) in O(N) with a cell list, giving
 * the same neighbour sets in the same order as the reference's O(N^2) search.
 *   basis_cart(3, nbasis), basis_species(nbasis) 1-based, abc(3,3) rows = lattice vectors,
 *   bc: 'c' closed / 'o' open per axis, nbd_dis(nsh), tol = nbdfc.
 *   ion(0:8, N) receives ID, initial spins ((-1)**l for the z component, as
 *   generate_supercell.f90:42 does for Ising), species and positions;
 *   stgg(N) (may be NULL) receives the Checkerboard signs (-1)**(i+j+k+l) when
 *   checkerboard != 0, else 1; nn(nsh, N, 0:cap, 0:1). */
int ether_build_lattice(int32_t nbasis, const double *basis_cart, const int32_t *basis_species,
                        const double *abc, const int32_t sc[3], const char bc[3],
                        int32_t checkerboard, int32_t n_shells, const double *nbd_dis,
                        double tol, int32_t cap, double *ion, double *stgg, int32_t *nn);

/* ------------------------------------------------------------------ the program ---- */
/* src/ether.f90 for one input directory: reads in.ether, structure.vasp, j_exchange and,
 * when asked for, single_ion_anisotropy and staggered from indir exactly as the reference's
 * readers do, runs the temperature scan (every temperature a PT slot, every REPEAT a group
 * of replicas, one ether_mcs loop) and writes the reference's output files into outdir:
 * ETHER.obs, ETHER.spn, data/{magnetization,energy,moment_vectors,spiral_state_parameters,
 * gss,nbd}.dat, data/fetched_lattice_network.xsf, data/graph.sh, spins/<T>spK.xsf, plus
 * deck.txt (everything read, after src/parameters.f90).  A malformed deck gives
 * ETHER_ERR_PARSE with the reference's message in ether_last_error. */
enum {
    ETHER_RUN_PARSE_ONLY = 1 << 0, /* read the deck, build the lattice, write deck.txt,
                                      nbd.dat and the network file; no GPU work          */
    ETHER_RUN_QUIET = 1 << 1,      /* nothing on stdout                                  */
    ETHER_RUN_RESUME = 1 << 2      /* start every temperature from its record of
                                      outdir/ETHER.spn, without fresh_spins: continue an
                                      earlier run of the same deck                        */
};
typedef struct ether_run_info {
    int32_t ranks;          /* in: temperatures per PT round, as mpirun -np (0 = all at once) */
    int32_t model;          /* out: ETHER_MODEL_*                                             */
    int32_t n_sites, n_species, n_shells, n_temperatures, repeat, n_rounds; /* out            */
    uint64_t site_updates;  /* out: Metropolis attempts of the run                            */
    double seconds;         /* out: wall time of the MCS loops                                */
} ether_run_info;
int ether_run(const char *indir, const char *outdir, int32_t flags, ether_run_info *info);

#ifdef __cplusplus
}
#endif
#endif
