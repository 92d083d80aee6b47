/*
 * ether_oracle.h -- CPU restatement of ETHER's Monte Carlo sweep (TEST INFRASTRUCTURE ONLY).
 *
 * This library is the checker for the GPU path.  Only the tests, the smoke check and the
 * CPU-baseline leg of bench.py load it.  The product library (libether_gpu.so) never links,
 * loads or calls it.
 *
 * Every routine restates one Fortran routine of the reference (mukkelian/Ether); the
 * citation (file:line) is given next to each declaration.  Arrays use the reference's own
 * Fortran column-major layouts so the same buffers can be fed to the oracle and to the
 * GPU library:
 *   ion(0:8, N)                 -> ion[c + 9*i]                          (src/init.f90:73)
 *   nn(nsh, N, 0:cap, 0:1)      -> nn[b + nsh*(i + N*(k + (cap+1)*t))]   (src/init.f90:42)
 *   j_exc(nsh, nsp, nsp, 3)     -> j_exc[b + nsh*(si + nsp*(sj + nsp*c))] (src/j_values.f90:83)
 *   sia_vec(3, nsp)             -> sia_vec[c + 3*sp]                     (src/get_sia_values.f90:57)
 * with 0-based b, i, k, c, si, sj here; the *values* stored in nn(...,1) are 1-based site
 * numbers and ion(4,i) holds the 1-based species number, exactly as in the reference.
 *
 * Parity status: the reference has no tests, fixtures or golden outputs, and its random
 * numbers come from libgfortran's random_number (a third-party dependency absent from the
 * reference tree, version unpinned).  Parity is therefore pinned by (a) Philox known-answer
 * vectors, (b) exact enumeration of tiny lattices, (c) analytic two-spin results and
 * (d) literature critical points -- not by reference-produced outputs ("parity unpinned"
 * against the reference binary itself, which cannot be built without gfortran/MPI).
 */
#ifndef ETHER_ORACLE_H
#define ETHER_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- Philox4x32-10 ---- */
/* Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ------------------------------------------------------------------ system ---------- */
typedef struct orc_sys {
    int n_sites, n_species, n_shells, cap;
    int model;            /* 0 = Ising, 1 = XYZ (src/read_input.f90:62-66)            */
    int angle;            /* ANGLE proposal (src/update_spin_details.f90:36-47)        */
    double dphi;          /* radians (src/read_input.f90:95-97)                        */
    int zeeman;           /* src/Hamiltonian.f90:48                                    */
    double h[3], g_factor, mb;
    int sia;              /* src/Hamiltonian.f90:50                                    */
    const int32_t *nn;    /* nn(nsh, N, 0:cap, 0:1)                                    */
    const double *j_exc;  /* already scaled by parameters.f90                          */
    const double *sia_vec;/* may be NULL when !sia                                      */
    const double *s;      /* spin length per species                                   */
    const double *stgg;   /* stgg_ion(N) (src/get_tot_magnetisation.f90:37); NULL = 1  */
    const double *sia_local; /* sia_local(4, N) or NULL: a site term D (a . S)^2 with the
                             unit axis a = sia_local(0:2, i) and D = sia_local(3, i), XYZ only.
                             Not expressible in the reference (its SIA is the diagonal
                             sia_vec per species, src/get_sia_values.f90:57-58); it adds to
                             that term like siaS2 (src/Hamiltonian.f90:127-143) adds D S^2. */
} orc_sys;

/* ------------------------------------------------------------- lattice build -------- */
/* generate_supercell (src/generate_supercell.f90:38-132) for the geometry: positions,
 * species and the Checkerboard stagger sign (-1)^(i+j+k+l) (:127).  Initial spins are
 * written as generate_supercell.f90:42 writes them for Ising (Sz = (-1)**l).  basis_cart[3*l+d] are cartesian basis positions, abc[3*a+d]
 * lattice vector a.  Returns N. */
int orc_supercell(int nbasis, const double *basis_cart, const int *basis_species,
                  const double *abc, const int sc[3], int checkerboard,
                  double *ion, double *stgg);

/* getting_nbd + search_nbd (src/getting_nbd.f90:34-82, src/search_nbd.f90:20-64):
 * brute force O(N^2 * 27).  Returns 0, or -1 when a shell overflows cap (the reference
 * has no overflow check; we report it). */
int orc_neighbours_bruteforce(int N, const double *ion, const double *abc, const int sc[3],
                              const char bc[3], int nsh, const double *nbd_dis, double tol,
                              int cap, int32_t *nn);

/* Greedy colouring by site index over the symmetric closure of all shells.  The colour
 * classes define the update order of our Checkerboard mode. Returns number of colours. */
int orc_greedy_colouring(int N, int nsh, int cap, const int32_t *nn, int32_t *colour,
                         int32_t *rank_in_colour);

/* ------------------------------------------------------------- Hamiltonian ---------- */
/* Hamiltonian(.TRUE./.FALSE.) (src/Hamiltonian.f90:20-143) in FP64 on ion(0:8,N). */
double orc_hamiltonian(const orc_sys *sy, const double *ion, int i, const double *s_trial,
                       const double *s_old, int trial);
/* get_tot_energy (src/get_tot_energy.f90:33-47): raw sum of site energies. */
double orc_tot_energy(const orc_sys *sy, const double *ion);
/* get_tot_magnetisation (src/get_tot_magnetisation.f90:32-40). */
void orc_tot_magnetisation(const orc_sys *sy, const double *ion, double m[3]);
/* Same two quantities for the FP32 spin mirror (float4 x,y,z,phi per site). */
double orc_tot_energy_f32(const orc_sys *sy, const double *ion, const float *spin4);
void orc_tot_magnetisation_f32(const orc_sys *sy, const double *ion, const float *spin4,
                               double m[3]);

/* --------------------------------------------------------- sequential stream -------- */
/* Stand-in for libgfortran's random_number in the typewriter (reference-order) mode:
 * a sequential Philox stream, 53-bit doubles in [0,1). */
typedef struct orc_stream { uint32_t key[2]; uint64_t n; } orc_stream;
void orc_stream_init(orc_stream *st, uint32_t seed, uint32_t stream_id);
double orc_stream_uniform(orc_stream *st);

/* -------------------------------------------------- reference-order Metropolis ------ */
/* Metropolis (src/Metropolis.f90:34-68) run in site order i = 1..N on one thread, FP64,
 * acceptance -beta*dE > log(eta); proposals as update_spin_details
 * (src/update_spin_details.f90:30-51) and George_Marsaglia (src/George_Marsaglia.f90:29-39).
 * Returns accepted / N. */
double orc_metropolis_typewriter(const orc_sys *sy, double *ion, double beta, orc_stream *st);
/* fresh_spins (src/fresh_spins.f90:31-38). */
void orc_fresh_spins_typewriter(const orc_sys *sy, double *ion, orc_stream *st);
/* overrelaxation (src/overrelaxation.f90:30-61) with get_random_indices
 * (src/get_random_indices.f90:31-36): n_steps reflections at random sites. */
void orc_overrelaxation_typewriter(const orc_sys *sy, double *ion, int n_steps, orc_stream *st);

/* -------------------------------------------- colour-ordered (Checkerboard) mode ---- */
/* The same Metropolis step, with the site loop visiting colour 0, 1, ... in order and the
 * random numbers replayed from the counter-based stream shared with the GPU:
 *   key = (seed, 0x45544852), counter = (c0, t, stream, purpose | colour<<8 | block<<16).
 * Ising: c0 = rank>>3; u = (halfword (rank&7) of block 0) << 16 | (same halfword of
 *        block 1); accept iff u <= T where
 *        T = max(ceil(2^32 exp(-beta dE)), 1) - 1 (clamped to 2^32-1) -- the reference's
 *        -beta dE > log(eta) for eta = u 2^-32, eta = 0 included -- and dE is evaluated
 *        per (shell, neighbour-species) group.  Spins live in ion(3,:) (= +-1).
 * XYZ:   c0 = rank, block = 0, 1, ... (pairs of the Marsaglia rejection loop).  `prec` = 32 runs the FP32 mirror on spin4 (x,y,z,phi);
 *        prec = 64 runs the same draws in FP64 on ion.
 * Returns accepted / N. */
double orc_metropolis_colour(const orc_sys *sy, double *ion, float *spin4, int prec,
                             double beta, uint32_t seed, uint32_t stream, uint32_t t,
                             const int32_t *colour, const int32_t *rank_in_colour, int ncol);
/* Colour-ordered overrelaxation: pass p < floor(frac) reflects every site; the last
 * pass reflects a site iff its uniform < frac - floor(frac).  FP32 mirror only. */
void orc_overrelax_colour(const orc_sys *sy, const double *ion, float *spin4, double frac,
                          uint32_t seed,
                          uint32_t stream, uint32_t t, const int32_t *colour,
                          const int32_t *rank_in_colour, int ncol);
/* Fresh random spins (src/fresh_spins.f90) from the counter stream (purpose 2):
 * Ising flips every spin; XYZ draws Marsaglia / ANGLE states. FP32 mirror + ion. */
void orc_fresh_spins_colour(const orc_sys *sy, double *ion, float *spin4, uint32_t seed,
                            uint32_t stream, uint32_t call);

/* --------------------------------------------------------- parallel tempering ------- */
/* parallel_tempering (src/parallel_tempering.f90:39-108) on a ladder of n slots.
 * slot_of_rep / rep_of_slot: permutation; energy[rep]; beta[slot].  Pairs (s, s+1) with
 * s even when swap_count is even, odd otherwise.  The lower slot decides; delta =
 * -(beta[s+1]-beta[s])*(E_lo - E_hi); accept iff delta > 0 or u < exp(delta), u from
 * the counter stream key=(seed, 0x45544852), ctr=(s, swap_count, 0x50540000 + group, 3).
 * mode 0: exchange configurations (swap the permutation); mode 1: the reference's
 * effective behaviour, where only the higher slot adopts the lower slot's configuration
 * (copy_from[hi] = lo).  Returns the number of accepted pairs. */
int orc_parallel_tempering(int n_slots, const double *beta, const double *energy,
                           int32_t *rep_of_slot, int swap_count, uint32_t seed,
                           uint32_t group, int mode, int32_t *copy_from);

/* ------------------------------------------------------------- observables ---------- */
/* Accumulators of get_eng('eng') / get_mag('mag') (src/get_eng.f90:36-40,
 * src/get_mag.f90:36-41) and the 'avg' reductions (get_eng.f90:42-60, get_mag.f90:43-59). */
typedef struct orc_acc {
    double n, e, e2, e4, m, m2, m4;
} orc_acc;
void orc_acc_sample(orc_acc *a, double e_raw, const double mag[3], int N);
/* out[0..5] = <e>, U_E, C_v, <|m|>, U_M, chi */
void orc_acc_average(const orc_acc *a, double beta, int N, double out[6]);
/* observables_per_repeat (src/observables_per_repeat.f90:29-69) over `rep` repeats of
 * vals[rep*6] -> mean[6], err[6]. */
void orc_per_repeat(int rep, const double *vals, double mean[6], double err[6]);

/* ---------------------------------------------------------- structure factor -------- */
/* structure_factor (utility/Structure_Factor/structure_factor.f90:99-183) in FP64 for an
 * arbitrary list of q vectors: S_a(q) = sum_i S_i,a exp(i q.r_i).  out[6*iq] = Re/Im of
 * S_x, S_y, S_z. */
void orc_structure_factor(int N, const double *pos /*3N*/, const double *spin /*3N*/,
                          int nq, const double *q /*3*nq*/, double *out /*6*nq*/);

/* ---------------------------------------------------------- reference driver -------- */
/* The per-temperature body of src/ether.f90:147-214 for one rank, typewriter sweeps.
 * Runs `repeat` repeats of tmcs MCS at beta, with OVRR/PT gating as ether.f90:163-198
 * (PT needs several ranks, so it is not part of this single-rank loop).  ion is carried
 * across repeats as in the reference (fresh_spins at each repeat start).  Returns the
 * per-repeat observables vals[6*repeat] and the acceptance ratio. */
typedef struct orc_run_cfg {
    int tmcs, tmcs_eq, coa, repeat;
    int ovrr; double ovrr_para; int ovrr_mcs;
    uint32_t seed; int itemp, rank;
} orc_run_cfg;
double orc_run_temperature(const orc_sys *sy, double *ion, double beta, const orc_run_cfg *cfg,
                           double *vals);
/* Same, on `nthreads` OpenMP threads, one temperature per thread (the reference's
 * MPI-over-temperatures decomposition with one temperature per rank).  ion0 is the
 * initial state shared by all temperatures; vals[6*repeat*nT]; acc[nT]. */
void orc_run_temperatures(const orc_sys *sy, const double *ion0, int nT, const double *beta,
                          const orc_run_cfg *cfg, int nthreads, double *vals, double *acc);
/* One round of nT temperatures with parallel tempering every `ex` MCS (0: none), the ranks
 * of src/ether.f90 in lockstep; configurations move between slots on an accepted swap.
 * vals[6*repeat*nT], acc[nT], *n_accepted = accepted swaps of the run. */
void orc_run_ladder(const orc_sys *sy, const double *ion0, int nT, const double *beta,
                    const orc_run_cfg *cfg, int ex, int nthreads, double *vals, double *acc,
                    long *n_accepted);

/* ---------------------------------------------------------- own float math ---------- */
/* exp / sincos used by the FP32 mirror (same algorithm as the GPU kernels: Cody-Waite
 * range reduction + Taylor polynomial).  Exposed for accuracy tests against libm. */
float orc_expf_neg(float x);
void orc_sincosf(float x, float *s, float *c);


/* ---- learned patch proposal (learn_oracle.c) ---- */
float orc_bf16_round(float f);
float orc_logf_own(float x);
int orc_mlp_n_params(void);
void orc_mlp_forward(const float *params, const float *x, int B, int quant, float *logits);
double orc_mlp_loss_grad(const float *params, const float *x, const uint32_t *y, int B, int quant,
                         double *grad);
void orc_patch_tables(int32_t *A, int32_t *B, int32_t *Bn, int32_t *Ab);
void orc_patch_gather(const uint8_t *sp, const int L[3], const int off[3], int pi, int pj, int pk,
                      float k4, float *x, uint32_t bnd[3], uint32_t *abits, uint32_t *bbits);
void orc_patch_btables(double betaJ, uint32_t TB[7], float LBup[7], float LBdn[7]);
void orc_patch_offsets(uint32_t seed, uint32_t stream, uint32_t t, int off[3]);
long orc_patch_sweep(uint8_t *sp, const int L[3], double betaJ, const float *logits,
                     uint32_t seed, uint32_t stream, uint32_t t);
void orc_patch_chain(const int L[3], double betaJ, long nsteps, long nequil, int use_patch,
                     float zscale, float zbias, uint32_t seed, double out[5]);


/* ---- moment vectors and spiral state ---- */
void orc_moment_vectors(const orc_sys *sy, const double *ion, double *mm);
long orc_spiral_pairs(int N, const double *ion, double ss_dis, const double ss_direc[3],
                      double ss_latency, int cap, int32_t *ifs);
double orc_spiral_state(int N, const double *ion, int cap, const int32_t *ifs, long count);

#ifdef __cplusplus
}
#endif
#endif
