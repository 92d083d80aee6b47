/*
 * ether_oracle.c -- CPU restatement of ETHER's Monte Carlo sweep.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py as the checker.  The product library never uses it.
 *
 * Build (see oracle/build.sh):  cc -O2 -fopenmp -ffp-contract=off -fPIC -shared
 * -ffp-contract=off is required: the FP32 mirror must round every operation exactly as
 * the CUDA kernels do (they are compiled with --fmad=false and use explicit fmaf).
 */
#include "ether_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ Philox ---------- */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += PHILOX_W0; k1 += PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Counter-based draws of the Checkerboard mode, shared with the GPU kernels:
 *   key = (seed, 0x45544852), counter = (c0, t, stream, purpose | colour << 8 | block << 16).
 * The key is the same for every replica of a run, the replica's stream id sits in the
 * counter. */
#define ETHER_KEY1 0x45544852u
static void draw(uint32_t c0, uint32_t t, uint32_t stream, uint32_t tag, uint32_t seed,
                 uint32_t out[4]) {
    uint32_t c[4] = {c0, t, stream, tag}, k[2] = {seed, ETHER_KEY1};
    orc_philox4x32_10(c, k, out);
}

/* Counter-stream purposes (fourth counter word, low byte). */
enum { P_METRO = 0, P_OVRR = 1, P_FRESH = 2, P_PT = 3 };

/* u32 -> float maps shared with the GPU kernels. */
static inline float u01f(uint32_t u) { return (float)(u >> 8) * 0x1p-24f; }
static inline float upm1f(uint32_t u) { return (float)(u >> 8) * 0x1p-23f - 1.0f; }
static inline double u01d(uint32_t u) { return (double)(u >> 8) * 0x1p-24; }
static inline double upm1d(uint32_t u) { return (double)(u >> 8) * 0x1p-23 - 1.0; }

/* ------------------------------------------------------------- own float math ------- */
/* exp(x) for x <= 0: Cody-Waite reduction x = n ln2 + r, |r| <= ln2/2, then the degree-7
 * Taylor polynomial of e^r in Horner form, scaled by 2^n built from the exponent bits.
 * Below -87 the result is the smallest normal float, so that a uniform eta = 0 (log eta =
 * -inf in the reference) is still accepted and every larger eta is rejected. */
float orc_expf_neg(float x) {
    if (x < -87.0f) return 0x1p-126f;
    float n = rintf(x * 1.44269502f);
    float r = x - n * 0.693359375f;
    r = r - n * -2.12194440e-4f;
    float p = 1.98412698e-4f;
    p = fmaf(p, r, 1.38888889e-3f);
    p = fmaf(p, r, 8.33333333e-3f);
    p = fmaf(p, r, 4.16666667e-2f);
    p = fmaf(p, r, 1.66666667e-1f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    int ni = (int)n;
    uint32_t bits = (uint32_t)(ni + 127) << 23;
    float scale;
    memcpy(&scale, &bits, 4);
    return p * scale;
}

/* sin/cos for |x| <= ~4: quadrant reduction by pi/2 (two-term constant), Taylor
 * polynomials on |r| <= pi/4 (sin to r^9, cos to r^8). */
void orc_sincosf(float x, float *s, float *c) {
    float q = rintf(x * 0.636619772f);
    float r = x - q * 1.5703125f;
    r = r - q * 4.83826792e-4f;
    float r2 = r * r;
    float sp = 2.75573192e-6f;
    sp = fmaf(sp, r2, -1.98412698e-4f);
    sp = fmaf(sp, r2, 8.33333333e-3f);
    sp = fmaf(sp, r2, -1.66666667e-1f);
    float r3 = r * r2;
    float sn = fmaf(r3, sp, r);
    float cp = 2.48015873e-5f;
    cp = fmaf(cp, r2, -1.38888889e-3f);
    cp = fmaf(cp, r2, 4.16666667e-2f);
    cp = fmaf(cp, r2, -0.5f);
    float cs = fmaf(cp, r2, 1.0f);
    int iq = ((int)q) & 3;
    switch (iq) {
        case 0: *s = sn; *c = cs; break;
        case 1: *s = cs; *c = -sn; break;
        case 2: *s = -sn; *c = -cs; break;
        default: *s = -cs; *c = sn; break;
    }
}

#define PI_F 3.14159274f
#define TWO_PI_F 6.28318548f

/* ---------------------------------------------------------------- indexing ---------- */
#define ION(ion, c, i) ((ion)[(c) + 9 * (size_t)(i)])
static inline int nn_count(const orc_sys *sy, int b, int i) {
    return sy->nn[b + (size_t)sy->n_shells * ((size_t)i)];
}
static inline int nn_site(const orc_sys *sy, int b, int i, int k) { /* 0-based site */
    size_t N = sy->n_sites, nsh = sy->n_shells, cap1 = sy->cap + 1;
    return sy->nn[b + nsh * ((size_t)i + N * ((size_t)k + cap1 * 1))] - 1;
}
static inline double jex(const orc_sys *sy, int b, int si, int sj, int c) {
    /* si, sj 1-based species */
    size_t nsh = sy->n_shells, nsp = sy->n_species;
    return sy->j_exc[b + nsh * ((size_t)(si - 1) + nsp * ((size_t)(sj - 1) + nsp * c))];
}
static inline int species_of(const double *ion, int i) { return (int)ION(ion, 4, i); }

/* ------------------------------------------------------------- lattice build -------- */
int orc_supercell(int nbasis, const double *basis_cart, const int *basis_species,
                  const double *abc, const int sc[3], int checkerboard, double *ion,
                  double *stgg) {
    int n = 0;
    for (int k = 1; k <= sc[2]; ++k)
        for (int j = 1; j <= sc[1]; ++j)
            for (int i = 1; i <= sc[0]; ++i)
                for (int l = 1; l <= nbasis; ++l) {
                    double *r = ion + 9 * (size_t)n;
                    r[0] = n + 1;
                    r[1] = 0.0; r[2] = 0.0;
                    r[3] = (l % 2 == 0) ? 1.0 : -1.0; /* (-1)**l, generate_supercell.f90:42 */
                    r[4] = basis_species[l - 1];
                    r[5] = 0.0;
                    for (int d = 0; d < 3; ++d)
                        r[6 + d] = abc[0 * 3 + d] * (i - 1) + abc[1 * 3 + d] * (j - 1) +
                                   abc[2 * 3 + d] * (k - 1) + basis_cart[3 * (l - 1) + d];
                    if (stgg) stgg[n] = checkerboard ? (((i + j + k + l) % 2 == 0) ? 1.0 : -1.0) : 1.0;
                    ++n;
                }
    return n;
}

int orc_neighbours_bruteforce(int N, const double *ion, const double *abc, const int sc[3],
                              const char bc[3], int nsh, const double *nbd_dis, double tol,
                              int cap, int32_t *nn) {
    double SC[3][3];
    for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 3; ++d) SC[a][d] = sc[a] * abc[3 * a + d];
    int to[3];
    for (int a = 0; a < 3; ++a) to[a] = (bc[a] == 'o' || bc[a] == 'O') ? 1 : 3;
    const int shift[3] = {0, 1, -1};
    size_t cap1 = (size_t)cap + 1;
    memset(nn, 0, sizeof(int32_t) * (size_t)nsh * N * cap1 * 2);
    int overflow = 0;
    for (int i = 0; i < N; ++i) {
        const double *p0 = ion + 9 * (size_t)i + 6;
        for (int b = 0; b < nsh; ++b) {
            int cnt = 0;
            for (int j = 0; j < N; ++j) {
                if (j == i) continue;
                const double *p1 = ion + 9 * (size_t)j + 6;
                int captured = 0;
                for (int a = 0; a < to[0] && !captured; ++a)
                    for (int bb = 0; bb < to[1] && !captured; ++bb)
                        for (int c = 0; c < to[2] && !captured; ++c) {
                            double r[3], d2 = 0.0;
                            for (int d = 0; d < 3; ++d) {
                                double q = SC[0][d] * shift[a] + SC[1][d] * shift[bb] +
                                           SC[2][d] * shift[c] + p1[d];
                                r[d] = p0[d] - q;
                            }
                            d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
                            if (fabs(nbd_dis[b] - sqrt(d2)) <= tol) captured = 1;
                        }
                if (captured) {
                    ++cnt;
                    if (cnt > cap) { overflow = 1; continue; }
                    nn[b + nsh * ((size_t)i + N * ((size_t)cnt + cap1 * 0))] = j + 1;
                    nn[b + nsh * ((size_t)i + N * ((size_t)cnt + cap1 * 1))] = j + 1;
                }
            }
            nn[b + nsh * ((size_t)i)] = cnt > cap ? cap : cnt;
        }
    }
    return overflow ? -1 : 0;
}

static int cmp_i64(const void *a, const void *b) {
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

int orc_greedy_colouring(int N, int nsh, int cap, const int32_t *nn, int32_t *colour,
                         int32_t *rank_in_colour) {
    size_t cap1 = (size_t)cap + 1;
    size_t ne = 0;
    for (int i = 0; i < N; ++i)
        for (int b = 0; b < nsh; ++b) ne += 2 * (size_t)nn[b + nsh * (size_t)i];
    int64_t *e = (int64_t *)malloc(sizeof(int64_t) * (ne + 1));
    size_t m = 0;
    for (int i = 0; i < N; ++i)
        for (int b = 0; b < nsh; ++b) {
            int cnt = nn[b + nsh * (size_t)i];
            for (int k = 1; k <= cnt; ++k) {
                int j = nn[b + nsh * ((size_t)i + N * ((size_t)k + cap1))] - 1;
                e[m++] = (int64_t)i * N + j;
                e[m++] = (int64_t)j * N + i;
            }
        }
    qsort(e, m, sizeof(int64_t), cmp_i64);
    size_t *start = (size_t *)calloc((size_t)N + 1, sizeof(size_t));
    for (size_t q = 0; q < m; ++q) start[e[q] / N + 1]++;
    for (int i = 0; i < N; ++i) start[i + 1] += start[i];
    int ncol = 0;
    int used[256];
    for (int i = 0; i < N; ++i) {
        memset(used, 0, sizeof(used));
        for (size_t q = start[i]; q < start[i + 1]; ++q) {
            int j = (int)(e[q] % N);
            if (j < i && colour[j] < 256) used[colour[j]] = 1;
        }
        int c = 0;
        while (used[c]) ++c;
        colour[i] = c;
        if (c + 1 > ncol) ncol = c + 1;
    }
    int cnt[256] = {0};
    for (int i = 0; i < N; ++i) rank_in_colour[i] = cnt[colour[i]]++;
    free(start);
    free(e);
    return ncol;
}

/* The local-axis anisotropy of site i in FP32 as the GPU holds it: (a_x, a_y, a_z, D). */
static void sia_local_f32(const orc_sys *sy, int i, float a[4]) {
    for (int c = 0; c < 4; ++c) a[c] = (float)sy->sia_local[4 * (size_t)i + c];
}

/* ------------------------------------------------------------- Hamiltonian ---------- */
double orc_hamiltonian(const orc_sys *sy, const double *ion, int i, const double *s_trial,
                       const double *s_old, int trial) {
    double Sd[3], S2d[3];
    for (int c = 0; c < 3; ++c) {
        if (trial) {
            Sd[c] = s_trial[c] - s_old[c];
            S2d[c] = s_trial[c] * s_trial[c] - s_old[c] * s_old[c];
        } else {
            Sd[c] = s_old[c];
            S2d[c] = s_old[c] * s_old[c];
        }
    }
    int si = species_of(ion, i);
    double tot = 0.0;
    for (int b = 0; b < sy->n_shells; ++b) { /* JSiSj, Hamiltonian.f90:72-103 */
        int cnt = nn_count(sy, b, i);
        for (int k = 1; k <= cnt; ++k) {
            int j = nn_site(sy, b, i, k);
            int sj = species_of(ion, j);
            if (sj == 0) continue;
            double e = 0.0;
            for (int c = 0; c < 3; ++c) e += (Sd[c] * ION(ion, 1 + c, j)) * jex(sy, b, si, sj, c);
            tot += e;
        }
    }
    if (sy->zeeman) { /* gmbSH, Hamiltonian.f90:118-121 */
        double d = Sd[0] * sy->h[0] + Sd[1] * sy->h[1] + Sd[2] * sy->h[2];
        tot += -(sy->g_factor * sy->mb * sy->s[si - 1] * d);
    }
    if (sy->sia && sy->model == 1) { /* siaS2, Hamiltonian.f90:137-141 */
        const double *D = sy->sia_vec + 3 * (size_t)(si - 1);
        tot += D[0] * S2d[0] + D[1] * S2d[1] + D[2] * S2d[2];
    }
    if (sy->sia_local && sy->model == 1) { /* D (a . S)^2 about the site's own axis */
        const double *a = sy->sia_local + 4 * (size_t)i;
        const double pn = a[0] * s_trial[0] + a[1] * s_trial[1] + a[2] * s_trial[2];
        const double po = a[0] * s_old[0] + a[1] * s_old[1] + a[2] * s_old[2];
        tot += trial ? a[3] * (pn * pn - po * po) : a[3] * (po * po);
    }
    return tot;
}

double orc_tot_energy(const orc_sys *sy, const double *ion) {
    double t = 0.0;
    for (int i = 0; i < sy->n_sites; ++i) {
        const double *S = ion + 9 * (size_t)i + 1;
        t += orc_hamiltonian(sy, ion, i, S, S, 0);
    }
    return t;
}

void orc_tot_magnetisation(const orc_sys *sy, const double *ion, double m[3]) {
    m[0] = m[1] = m[2] = 0.0;
    for (int i = 0; i < sy->n_sites; ++i) {
        double st = sy->stgg ? sy->stgg[i] : 1.0;
        double sl = sy->s[species_of(ion, i) - 1];
        for (int c = 0; c < 3; ++c) m[c] += st * ION(ion, 1 + c, i) * sl;
    }
}

/* ---------------------------------------------------- FP32 mirror: site fields ------ */
static void field_f32(const orc_sys *sy, const double *ion, const float *sp4, int i,
                      float h[3]) {
    int si = species_of(ion, i);
    float hx = 0.0f, hy = 0.0f, hz = 0.0f;
    for (int b = 0; b < sy->n_shells; ++b) {
        int cnt = nn_count(sy, b, i);
        for (int k = 1; k <= cnt; ++k) {
            int j = nn_site(sy, b, i, k);
            int sj = species_of(ion, j);
            if (sj == 0) continue;
            float Jx = (float)jex(sy, b, si, sj, 0);
            float Jy = (float)jex(sy, b, si, sj, 1);
            float Jz = (float)jex(sy, b, si, sj, 2);
            hx = fmaf(Jx, sp4[4 * (size_t)j + 0], hx);
            hy = fmaf(Jy, sp4[4 * (size_t)j + 1], hy);
            hz = fmaf(Jz, sp4[4 * (size_t)j + 2], hz);
        }
    }
    h[0] = hx; h[1] = hy; h[2] = hz;
}

static void zee_f32(const orc_sys *sy, int si, float z[3]) {
    double gms = sy->g_factor * sy->mb * sy->s[si - 1];
    for (int c = 0; c < 3; ++c) z[c] = (float)(-(gms * sy->h[c]));
}

double orc_tot_energy_f32(const orc_sys *sy, const double *ion, const float *sp4) {
    /* Per-site energy in FP32 (same expression as the GPU energy kernel), summed in FP64. */
    double t = 0.0;
    for (int i = 0; i < sy->n_sites; ++i) {
        int si = species_of(ion, i);
        float h[3];
        field_f32(sy, ion, sp4, i, h);
        const float *S = sp4 + 4 * (size_t)i;
        float e = S[0] * h[0];
        e = fmaf(S[1], h[1], e);
        e = fmaf(S[2], h[2], e);
        if (sy->zeeman) {
            float z[3];
            zee_f32(sy, si, z);
            e = fmaf(S[0], z[0], e);
            e = fmaf(S[1], z[1], e);
            e = fmaf(S[2], z[2], e);
        }
        if (sy->sia && sy->model == 1) {
            const double *D = sy->sia_vec + 3 * (size_t)(si - 1);
            e = fmaf((float)D[0], S[0] * S[0], e);
            e = fmaf((float)D[1], S[1] * S[1], e);
            e = fmaf((float)D[2], S[2] * S[2], e);
        }
        if (sy->sia_local && sy->model == 1) {
            float a[4];
            sia_local_f32(sy, i, a);
            float ps = a[0] * S[0];
            ps = fmaf(a[1], S[1], ps);
            ps = fmaf(a[2], S[2], ps);
            e = fmaf(a[3], ps * ps, e);
        }
        t += (double)e;
    }
    return t;
}

void orc_tot_magnetisation_f32(const orc_sys *sy, const double *ion, const float *sp4,
                               double m[3]) {
    m[0] = m[1] = m[2] = 0.0;
    for (int i = 0; i < sy->n_sites; ++i) {
        double st = sy->stgg ? sy->stgg[i] : 1.0;
        double sl = sy->s[species_of(ion, i) - 1];
        for (int c = 0; c < 3; ++c) m[c] += st * (double)sp4[4 * (size_t)i + c] * sl;
    }
}

/* --------------------------------------------------------- sequential stream -------- */
void orc_stream_init(orc_stream *st, uint32_t seed, uint32_t stream_id) {
    st->key[0] = seed;
    st->key[1] = stream_id;
    st->n = 0;
}
double orc_stream_uniform(orc_stream *st) {
    uint32_t c[4] = {(uint32_t)st->n, (uint32_t)(st->n >> 32), 0u, 0xF0u}, o[4];
    orc_philox4x32_10(c, st->key, o);
    st->n++;
    return ((double)(o[0] >> 5) * 67108864.0 + (double)(o[1] >> 6)) * 0x1p-53;
}
static double get_random_num(orc_stream *st, double from, double to) {
    return (to - from) * orc_stream_uniform(st) + from;
}

/* -------------------------------------------------- reference-order Metropolis ------ */
static void george_marsaglia(orc_stream *st, double *sx, double *sy_, double *sz) {
    double v1, v2, s;
    do {
        v1 = get_random_num(st, -1.0, 1.0);
        v2 = get_random_num(st, -1.0, 1.0);
        s = v1 * v1 + v2 * v2;
    } while (s >= 1.0);
    *sx = 2 * v1 * sqrt(1 - s);
    *sy_ = 2 * v2 * sqrt(1 - s);
    *sz = 1 - 2 * s;
}

/* update_spin_details (src/update_spin_details.f90:30-51); ref = ion(1:5,i). */
static void update_spin_details(const orc_sys *sy, const double *ref1, double *ref2,
                                orc_stream *st) {
    for (int c = 0; c < 5; ++c) ref2[c] = ref1[c];
    if (sy->model == 0) {
        ref2[2] = -ref1[2];
    } else if (!sy->angle) {
        george_marsaglia(st, &ref2[0], &ref2[1], &ref2[2]);
        ref2[4] = 0.0;
    } else {
        ref2[4] = ref1[4];
        ref2[2] = get_random_num(st, -1.0, 1.0);
        double rn = get_random_num(st, -1.0, 1.0);
        double phi = ref2[4] + sy->dphi * rn;
        ref2[0] = sqrt(1 - ref2[2] * ref2[2]) * cos(phi);
        ref2[1] = sqrt(1 - ref2[2] * ref2[2]) * sin(phi);
        ref2[4] = phi;
    }
    double n = sqrt(ref2[0] * ref2[0] + ref2[1] * ref2[1] + ref2[2] * ref2[2]);
    for (int c = 0; c < 3; ++c) ref2[c] = ref2[c] / n;
}

double orc_metropolis_typewriter(const orc_sys *sy, double *ion, double beta, orc_stream *st) {
    double acc = 0.0;
    for (int i = 0; i < sy->n_sites; ++i) {
        double prev[5], upd[5];
        for (int c = 0; c < 5; ++c) prev[c] = ION(ion, 1 + c, i);
        update_spin_details(sy, prev, upd, st);
        double dE = orc_hamiltonian(sy, ion, i, upd, prev, 1);
        double eta = get_random_num(st, 0.0, 1.0);
        if (-beta * dE > log(eta)) {
            for (int c = 0; c < 5; ++c) ION(ion, 1 + c, i) = upd[c];
            acc += 1.0;
        }
    }
    return acc / sy->n_sites;
}

void orc_fresh_spins_typewriter(const orc_sys *sy, double *ion, orc_stream *st) {
    for (int i = 0; i < sy->n_sites; ++i) {
        double prev[5], upd[5];
        for (int c = 0; c < 5; ++c) prev[c] = ION(ion, 1 + c, i);
        update_spin_details(sy, prev, upd, st);
        for (int c = 0; c < 5; ++c) ION(ion, 1 + c, i) = upd[c];
    }
}

static void ovrr_vec_f64(const orc_sys *sy, const double *ion, int i, double A[3]) {
    int si = species_of(ion, i);
    A[0] = A[1] = A[2] = 0.0;
    for (int b = 0; b < sy->n_shells; ++b) {
        int cnt = nn_count(sy, b, i);
        for (int k = 1; k <= cnt; ++k) {
            int j = nn_site(sy, b, i, k);
            int sj = species_of(ion, j);
            if (sj == 0) continue;
            for (int c = 0; c < 3; ++c) A[c] += jex(sy, b, si, sj, c) * ION(ion, 1 + c, j);
        }
    }
}

void orc_overrelaxation_typewriter(const orc_sys *sy, double *ion, int n_steps, orc_stream *st) {
    int N = sy->n_sites;
    for (int m = 0; m < n_steps; ++m) {
        double rn = get_random_num(st, 1.0, (double)N);
        int i = (int)lround(rn); /* nint: half away from zero */
        if (i < 1) i = 1;
        if (i > N) i = N;
        --i;
        double A[3], S[3];
        for (int c = 0; c < 3; ++c) S[c] = ION(ion, 1 + c, i);
        ovrr_vec_f64(sy, ion, i, A);
        double ad = A[0] * S[0] + A[1] * S[1] + A[2] * S[2];
        double aa = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
        for (int c = 0; c < 3; ++c) S[c] = (2 * (ad / aa) * A[c]) - S[c];
        double n = sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
        for (int c = 0; c < 3; ++c) ION(ion, 1 + c, i) = S[c] / n;
    }
}

/* -------------------------------------------- colour-ordered (Checkerboard) mode ---- */
#define MARSAGLIA_MAX_PAIRS 64

/* Pair p of the Metropolis proposal stream: p=0 -> words 1,2 of block 0; p>=1 -> block
 * (p+1)/2, words 0,1 (p odd) or 2,3 (p even). */
static void metro_pair(uint32_t c0, uint32_t t, uint32_t c3, uint32_t seed, uint32_t stream,
                       const uint32_t blk0[4], int p, uint32_t *a, uint32_t *b) {
    if (p == 0) { *a = blk0[1]; *b = blk0[2]; return; }
    uint32_t o[4];
    draw(c0, t, stream, c3 | ((uint32_t)((p + 1) / 2) << 16), seed, o);
    if (p & 1) { *a = o[0]; *b = o[1]; } else { *a = o[2]; *b = o[3]; }
}

/* Canonical FP64 Ising energy change used by the colour mode (and by the GPU library's
 * threshold tables): field = sum over groups (shell b ascending, neighbour species sj
 * ascending) of Jzz(b,si,sj) * m_g, m_g = sum of Sz over the group's neighbours. */
static double ising_dE(const orc_sys *sy, const double *ion, int i) {
    int si = species_of(ion, i);
    int nsp = sy->n_species;
    double field = 0.0;
    int m[64];
    for (int b = 0; b < sy->n_shells; ++b) {
        for (int q = 0; q < nsp; ++q) m[q] = 0;
        int cnt = nn_count(sy, b, i);
        for (int k = 1; k <= cnt; ++k) {
            int j = nn_site(sy, b, i, k);
            int sj = species_of(ion, j);
            if (sj == 0) continue;
            m[sj - 1] += (ION(ion, 3, j) > 0) ? 1 : -1;
        }
        for (int q = 0; q < nsp; ++q) field += jex(sy, b, si, q + 1, 2) * (double)m[q];
    }
    double sig = ION(ion, 3, i) > 0 ? 1.0 : -1.0;
    double dE = (-2.0 * sig) * field;
    if (sy->zeeman) {
        double gms = sy->g_factor * sy->mb * sy->s[si - 1];
        dE += -(gms * ((-2.0 * sig) * sy->h[2]));
    }
    return dE;
}

/* Replay acceptance of -beta*dE > log(eta) with eta = u * 2^-32: accept iff u <= T,
 * T = max(ceil(p * 2^32), 1) - 1, p = exp(-beta*dE).  u = 0 (eta = 0, log = -inf) is always
 * accepted, exactly as in the reference. */
static uint32_t ising_thr(double beta, double dE) {
    double q = exp(-beta * dE) * 4294967296.0;
    if (q >= 4294967296.0) return 0xFFFFFFFFu;
    double c = ceil(q);
    return c < 1.0 ? 0u : (uint32_t)(c - 1.0);
}

/* One XYZ site update on the FP32 mirror.  Returns 1 when accepted. */
static int xyz_site_f32(const orc_sys *sy, const double *ion, float *sp4, int i, float beta_f,
                        uint32_t seed, uint32_t stream, uint32_t t, uint32_t rho, uint32_t c3) {
    int si = species_of(ion, i);
    float h[3];
    field_f32(sy, ion, sp4, i, h);
    float *S = sp4 + 4 * (size_t)i;
    uint32_t blk[4];
    draw(rho, t, stream, c3, seed, blk);
    float eta = u01f(blk[0]);
    float nx, ny, nz, nphi;
    if (!sy->angle) {
        int ok = 0;
        float v1 = 0, v2 = 0, s = 0;
        for (int p = 0; p < MARSAGLIA_MAX_PAIRS; ++p) {
            uint32_t a, b;
            metro_pair(rho, t, c3, seed, stream, blk, p, &a, &b);
            v1 = upm1f(a);
            v2 = upm1f(b);
            s = v1 * v1 + v2 * v2;
            if (s < 1.0f) { ok = 1; break; }
        }
        if (!ok) return 0;
        float tq = sqrtf(1.0f - s);
        nx = (2.0f * v1) * tq;
        ny = (2.0f * v2) * tq;
        nz = 1.0f - 2.0f * s;
        nphi = 0.0f;
    } else {
        nz = upm1f(blk[1]);
        nphi = S[3] + (float)sy->dphi * upm1f(blk[2]);
        if (nphi >= PI_F) nphi = nphi - TWO_PI_F;
        else if (nphi < -PI_F) nphi = nphi + TWO_PI_F;
        float r = sqrtf(1.0f - nz * nz);
        float sn, cs;
        orc_sincosf(nphi, &sn, &cs);
        nx = r * cs;
        ny = r * sn;
    }
    /* no division by the norm: the FP32 kernels leave out update_spin_details.f90:50-51,
     * whose effect on these unit-length proposals is a few ulp (the FP64 replay keeps it) */
    float dx = nx - S[0], dy = ny - S[1], dz = nz - S[2];
    float e = dx * h[0];
    e = fmaf(dy, h[1], e);
    e = fmaf(dz, h[2], e);
    if (sy->zeeman) {
        float z[3];
        zee_f32(sy, si, z);
        e = fmaf(dx, z[0], e);
        e = fmaf(dy, z[1], e);
        e = fmaf(dz, z[2], e);
    }
    if (sy->sia) {
        const double *D = sy->sia_vec + 3 * (size_t)(si - 1);
        float qx = nx * nx - S[0] * S[0];
        float qy = ny * ny - S[1] * S[1];
        float qz = nz * nz - S[2] * S[2];
        e = fmaf((float)D[0], qx, e);
        e = fmaf((float)D[1], qy, e);
        e = fmaf((float)D[2], qz, e);
    }
    if (sy->sia_local) {
        float a[4];
        sia_local_f32(sy, i, a);
        float pn = a[0] * nx;
        pn = fmaf(a[1], ny, pn);
        pn = fmaf(a[2], nz, pn);
        float ps = a[0] * S[0];
        ps = fmaf(a[1], S[1], ps);
        ps = fmaf(a[2], S[2], ps);
        e = fmaf(a[3], pn * pn - ps * ps, e);
    }
    int acc = (e <= 0.0f) || (eta < orc_expf_neg(-(beta_f * e)));
    if (acc) { S[0] = nx; S[1] = ny; S[2] = nz; S[3] = nphi; }
    return acc;
}

/* One XYZ site update with the same draws in FP64 on ion. */
static int xyz_site_f64(const orc_sys *sy, double *ion, int i, double beta, uint32_t seed,
                        uint32_t stream, uint32_t t, uint32_t rho, uint32_t c3) {
    uint32_t blk[4];
    draw(rho, t, stream, c3, seed, blk);
    double eta = u01d(blk[0]);
    double prev[5], upd[5];
    for (int c = 0; c < 5; ++c) prev[c] = ION(ion, 1 + c, i);
    for (int c = 0; c < 5; ++c) upd[c] = prev[c];
    if (!sy->angle) {
        int ok = 0;
        double v1 = 0, v2 = 0, s = 0;
        for (int p = 0; p < MARSAGLIA_MAX_PAIRS; ++p) {
            uint32_t a, b;
            metro_pair(rho, t, c3, seed, stream, blk, p, &a, &b);
            v1 = upm1d(a);
            v2 = upm1d(b);
            s = v1 * v1 + v2 * v2;
            if (s < 1.0) { ok = 1; break; }
        }
        if (!ok) return 0;
        upd[0] = 2 * v1 * sqrt(1 - s);
        upd[1] = 2 * v2 * sqrt(1 - s);
        upd[2] = 1 - 2 * s;
        upd[4] = 0.0;
    } else {
        upd[2] = upm1d(blk[1]);
        double phi = prev[4] + sy->dphi * upm1d(blk[2]);
        if (phi >= M_PI) phi -= 2 * M_PI;
        else if (phi < -M_PI) phi += 2 * M_PI;
        upd[0] = sqrt(1 - upd[2] * upd[2]) * cos(phi);
        upd[1] = sqrt(1 - upd[2] * upd[2]) * sin(phi);
        upd[4] = phi;
    }
    double n = sqrt(upd[0] * upd[0] + upd[1] * upd[1] + upd[2] * upd[2]);
    for (int c = 0; c < 3; ++c) upd[c] /= n;
    double dE = orc_hamiltonian(sy, ion, i, upd, prev, 1);
    int acc = (dE <= 0.0) || (eta < exp(-beta * dE));
    if (acc)
        for (int c = 0; c < 5; ++c) ION(ion, 1 + c, i) = upd[c];
    return acc;
}

/* Site lists per colour in increasing index order. */
static int **colour_lists(int N, const int32_t *colour, int ncol, int **counts_out) {
    int *cnt = (int *)calloc((size_t)ncol, sizeof(int));
    for (int i = 0; i < N; ++i) cnt[colour[i]]++;
    int **lists = (int **)malloc(sizeof(int *) * (size_t)ncol);
    int *fill = (int *)calloc((size_t)ncol, sizeof(int));
    for (int c = 0; c < ncol; ++c) lists[c] = (int *)malloc(sizeof(int) * (size_t)(cnt[c] + 1));
    for (int i = 0; i < N; ++i) lists[colour[i]][fill[colour[i]]++] = i;
    free(fill);
    *counts_out = cnt;
    return lists;
}
static void free_lists(int **l, int *cnt, int ncol) {
    for (int c = 0; c < ncol; ++c) free(l[c]);
    free(l);
    free(cnt);
}

double orc_metropolis_colour(const orc_sys *sy, double *ion, float *spin4, int prec,
                             double beta, uint32_t seed, uint32_t stream, uint32_t t,
                             const int32_t *colour, const int32_t *rank_in_colour, int ncol) {
    int N = sy->n_sites;
    int *cnt;
    int **lists = colour_lists(N, colour, ncol, &cnt);
    double acc = 0.0;
    float beta_f = (float)beta;
    for (int c = 0; c < ncol; ++c) {
        uint32_t c3 = (uint32_t)P_METRO | ((uint32_t)c << 8);
        for (int q = 0; q < cnt[c]; ++q) {
            int i = lists[c][q];
            uint32_t rho = (uint32_t)rank_in_colour[i];
            if (sy->model == 0) {
                /* u32 of site rho: high half = halfword (rho & 7) of block 0, low half =
                 * the same halfword of block 1, of the group rho >> 3. */
                uint32_t hi[4], lo[4];
                draw(rho >> 3, t, stream, c3, seed, hi);
                draw(rho >> 3, t, stream, c3 | (1u << 16), seed, lo);
                const uint32_t k = rho & 7, sh = 16u * (k & 1u);
                uint32_t u = (((hi[k >> 1] >> sh) & 0xFFFFu) << 16) | ((lo[k >> 1] >> sh) & 0xFFFFu);
                double dE = ising_dE(sy, ion, i);
                if (u <= ising_thr(beta, dE)) {
                    ION(ion, 3, i) = -ION(ion, 3, i);
                    acc += 1.0;
                }
            } else if (prec == 32) {
                acc += xyz_site_f32(sy, ion, spin4, i, beta_f, seed, stream, t, rho, c3);
            } else {
                acc += xyz_site_f64(sy, ion, i, beta, seed, stream, t, rho, c3);
            }
        }
    }
    free_lists(lists, cnt, ncol);
    return acc / N;
}

void orc_overrelax_colour(const orc_sys *sy, const double *ion, float *spin4, double frac,
                          uint32_t seed, uint32_t stream, uint32_t t, const int32_t *colour,
                          const int32_t *rank_in_colour, int ncol) {
    int N = sy->n_sites;
    int *cnt;
    int **lists = colour_lists(N, colour, ncol, &cnt);
    int full = (int)floor(frac);
    float part = (float)(frac - full);
    int npass = full + (part > 0.0f ? 1 : 0);
    for (int p = 0; p < npass; ++p) {
        for (int c = 0; c < ncol; ++c) {
            uint32_t c3 = (uint32_t)P_OVRR | ((uint32_t)c << 8);
            for (int q = 0; q < cnt[c]; ++q) {
                int i = lists[c][q];
                if (p == full) {
                    uint32_t o[4];
                    draw((uint32_t)rank_in_colour[i], t, stream, c3 | ((uint32_t)p << 16), seed, o);
                    if (!(u01f(o[0]) < part)) continue;
                }
                float h[3];
                field_f32(sy, ion, spin4, i, h);
                float *S = spin4 + 4 * (size_t)i;
                float d = h[0] * S[0];
                d = fmaf(h[1], S[1], d);
                d = fmaf(h[2], S[2], d);
                float a2 = h[0] * h[0];
                a2 = fmaf(h[1], h[1], a2);
                a2 = fmaf(h[2], h[2], a2);
                if (!(a2 > 0.0f)) continue;
                float f = 2.0f * (d / a2);
                float nx = f * h[0] - S[0];
                float ny = f * h[1] - S[1];
                float nz = f * h[2] - S[2];
                float inv = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
                S[0] = nx * inv; S[1] = ny * inv; S[2] = nz * inv;
            }
        }
    }
    free_lists(lists, cnt, ncol);
}

/* Fresh spins from the counter stream: key (seed, stream), ctr (site, call, block, 2). */
void orc_fresh_spins_colour(const orc_sys *sy, double *ion, float *spin4, uint32_t seed,
                            uint32_t stream, uint32_t call) {
    for (int i = 0; i < sy->n_sites; ++i) {
        if (sy->model == 0) {
            ION(ion, 3, i) = -ION(ion, 3, i);
            continue;
        }
        uint32_t o[4];
        draw((uint32_t)i, call, stream, P_FRESH, seed, o);
        float *S = spin4 + 4 * (size_t)i;
        float nx, ny, nz, nphi;
        if (!sy->angle) {
            int ok = 0;
            float v1 = 0, v2 = 0, s = 0;
            for (int p = 0; p < MARSAGLIA_MAX_PAIRS; ++p) {
                uint32_t w[4];
                if (p < 2) memcpy(w, o, sizeof(w));
                else draw((uint32_t)i, call, stream, P_FRESH | ((uint32_t)(p / 2) << 16), seed, w);
                v1 = upm1f(w[2 * (p & 1)]);
                v2 = upm1f(w[2 * (p & 1) + 1]);
                s = v1 * v1 + v2 * v2;
                if (s < 1.0f) { ok = 1; break; }
            }
            if (!ok) continue;
            float tq = sqrtf(1.0f - s);
            nx = (2.0f * v1) * tq;
            ny = (2.0f * v2) * tq;
            nz = 1.0f - 2.0f * s;
            nphi = 0.0f;
        } else {
            nz = upm1f(o[0]);
            nphi = S[3] + (float)sy->dphi * upm1f(o[1]);
            if (nphi >= PI_F) nphi = nphi - TWO_PI_F;
            else if (nphi < -PI_F) nphi = nphi + TWO_PI_F;
            float r = sqrtf(1.0f - nz * nz);
            float sn, cs;
            orc_sincosf(nphi, &sn, &cs);
            nx = r * cs;
            ny = r * sn;
        }
        float inv = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
        S[0] = nx * inv; S[1] = ny * inv; S[2] = nz * inv; S[3] = nphi;
        for (int c = 0; c < 3; ++c) ION(ion, 1 + c, i) = (double)S[c];
        ION(ion, 5, i) = (double)nphi;
    }
}

/* --------------------------------------------------------- parallel tempering ------- */
int orc_parallel_tempering(int n_slots, const double *beta, const double *energy,
                           int32_t *rep_of_slot, int swap_count, uint32_t seed,
                           uint32_t group, int mode, int32_t *copy_from) {
    int nacc = 0;
    if (copy_from)
        for (int s = 0; s < n_slots; ++s) copy_from[s] = -1;
    for (int s = (swap_count % 2 == 0) ? 0 : 1; s + 1 < n_slots; s += 2) {
        int lo = rep_of_slot[s], hi = rep_of_slot[s + 1];
        double delta = -(beta[s + 1] - beta[s]) * (energy[lo] - energy[hi]);
        int acc;
        if (delta > 0.0) acc = 1;
        else {
            uint32_t o[4];
            draw((uint32_t)s, (uint32_t)swap_count, 0x50540000u + group, P_PT, seed, o);
            double r = (double)o[0] * 0x1p-32;
            acc = r < exp(delta);
        }
        if (!acc) continue;
        ++nacc;
        if (mode == 0) {
            rep_of_slot[s] = hi;
            rep_of_slot[s + 1] = lo;
        } else if (copy_from) {
            copy_from[s + 1] = s;
        }
    }
    return nacc;
}

/* ------------------------------------------------------------- observables ---------- */
void orc_acc_sample(orc_acc *a, double e_raw, const double mag[3], int N) {
    double e = e_raw / (2.0 * N);
    double mv = sqrt(mag[0] * mag[0] + mag[1] * mag[1] + mag[2] * mag[2]);
    double m = mv / N;
    a->n += 1.0;
    a->e += e; a->e2 += e * e; a->e4 += (e * e) * (e * e);
    a->m += m; a->m2 += m * m; a->m4 += (m * m) * (m * m);
}

void orc_acc_average(const orc_acc *a, double beta, int N, double out[6]) {
    double e = a->e / a->n, e2 = a->e2 / a->n, e4 = a->e4 / a->n;
    double m = a->m / a->n, m2 = a->m2 / a->n, m4 = a->m4 / a->n;
    out[0] = e;
    out[1] = 1.0 - (1.0 / 3.0) * (e4 / (e2 * e2));
    out[2] = (beta * beta) * (e2 - e * e) * N;
    out[3] = m;
    out[4] = 1.0 - (1.0 / 3.0) * (m4 / (m2 * m2));
    out[5] = beta * (m2 - m * m) * N;
}

void orc_per_repeat(int rep, const double *vals, double mean[6], double err[6]) {
    double r1 = 1.0 / (rep * (rep - 1.0));
    for (int q = 0; q < 6; ++q) {
        double s = 0.0;
        for (int r = 0; r < rep; ++r) s += vals[6 * r + q];
        mean[q] = s / rep;
        double e = 0.0;
        for (int r = 0; r < rep; ++r) e += (vals[6 * r + q] - mean[q]) * (vals[6 * r + q] - mean[q]);
        err[q] = sqrt(r1 * e);
    }
}

/* ---------------------------------------------------------- structure factor -------- */
void orc_structure_factor(int N, const double *pos, const double *spin, int nq, const double *q,
                          double *out) {
    for (int iq = 0; iq < nq; ++iq) {
        double re[3] = {0, 0, 0}, im[3] = {0, 0, 0};
        for (int i = 0; i < N; ++i) {
            double ph = q[3 * iq] * pos[3 * i] + q[3 * iq + 1] * pos[3 * i + 1] +
                        q[3 * iq + 2] * pos[3 * i + 2];
            double c = cos(ph), s = sin(ph);
            for (int a = 0; a < 3; ++a) {
                re[a] += spin[3 * i + a] * c;
                im[a] += spin[3 * i + a] * s;
            }
        }
        for (int a = 0; a < 3; ++a) {
            out[6 * iq + 2 * a] = re[a];
            out[6 * iq + 2 * a + 1] = im[a];
        }
    }
}

/* ---------------------------------------------------------- reference driver -------- */
double orc_run_temperature(const orc_sys *sy, double *ion, double beta, const orc_run_cfg *cfg,
                           double *vals) {
    int N = sy->n_sites;
    int ovrr_steps = (int)lround(N * cfg->ovrr_para);
    int ovrr_on = cfg->ovrr && sy->model == 1 && !sy->zeeman && !sy->sia && !sy->sia_local && cfg->ovrr_mcs > 0;
    double acc_total = 0.0;
    for (int r = 1; r <= cfg->repeat; ++r) {
        orc_stream st;
        orc_stream_init(&st, cfg->seed, (uint32_t)(cfg->itemp + 175 * cfg->rank + 666 * r));
        orc_fresh_spins_typewriter(sy, ion, &st);
        orc_acc a;
        memset(&a, 0, sizeof(a));
        for (int step = 1; step <= cfg->tmcs; ++step) {
            if (ovrr_on && step % cfg->ovrr_mcs == 0 && step % cfg->coa != 0)
                orc_overrelaxation_typewriter(sy, ion, ovrr_steps, &st);
            acc_total += orc_metropolis_typewriter(sy, ion, beta, &st);
            double E = orc_tot_energy(sy, ion); /* ether.f90:177, every MCS */
            if (step > cfg->tmcs_eq && step % cfg->coa == 0) {
                double M[3];
                orc_tot_magnetisation(sy, ion, M);
                orc_acc_sample(&a, E, M, N);
            }
        }
        orc_acc_average(&a, beta, N, vals + 6 * (size_t)(r - 1));
    }
    return acc_total / ((double)cfg->repeat * cfg->tmcs);
}

void orc_run_temperatures(const orc_sys *sy, const double *ion0, int nT, const double *beta,
                          const orc_run_cfg *cfg, int nthreads, double *vals, double *acc) {
    size_t nb = sizeof(double) * 9 * (size_t)sy->n_sites;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int it = 0; it < nT; ++it) {
        double *ion = (double *)malloc(nb);
        memcpy(ion, ion0, nb);
        orc_run_cfg c = *cfg;
        c.itemp = it + 1;
        acc[it] = orc_run_temperature(sy, ion, beta[it], &c, vals + 6 * (size_t)cfg->repeat * it);
        free(ion);
    }
    (void)nthreads;
}

/* One round of temperatures with parallel tempering: src/ether.f90:150-214 as the nT MPI
 * ranks of comm_ei execute it in lockstep (rank k holds temperature slot k, itemp = k + 1),
 * with src/parallel_tempering.f90:39-108 every `ex` MCS except at measurement steps
 * (ether.f90:189-198) and swap_count reset every REPEAT (:158).  Per MCS and slot: the OVRR
 * gate (:163-168), Metropolis in typewriter order, get_tot_energy (:177); then the swap
 * attempts over the ladder with those raw energies; then observable (:201) on each slot's
 * configuration.  On an accepted swap the two configurations change slots and each slot
 * keeps its own random stream (seeded as :154).  Slots are updated on `nthreads` OpenMP
 * threads between the swap steps.  vals(6, repeat, nT) as orc_run_temperatures; acc[nT]
 * the acceptance ratio per slot; the number of accepted swaps goes to *n_accepted. */
void orc_run_ladder(const orc_sys *sy, const double *ion0, int nT, const double *beta,
                    const orc_run_cfg *cfg, int ex, int nthreads, double *vals, double *acc,
                    long *n_accepted) {
    const int N = sy->n_sites;
    const size_t nb = sizeof(double) * 9 * (size_t)N;
    const int ovrr_steps = (int)lround(N * cfg->ovrr_para);
    const int ovrr_on = cfg->ovrr && sy->model == 1 && !sy->zeeman && !sy->sia && !sy->sia_local && cfg->ovrr_mcs > 0;
    double **cfgs = (double **)malloc(sizeof(double *) * nT);
    double *E = (double *)malloc(sizeof(double) * nT);
    int32_t *conf_of_slot = (int32_t *)malloc(sizeof(int32_t) * nT);
    orc_stream *st = (orc_stream *)malloc(sizeof(orc_stream) * nT);
    orc_acc *a = (orc_acc *)malloc(sizeof(orc_acc) * nT);
    for (int k = 0; k < nT; ++k) {
        cfgs[k] = (double *)malloc(nb);
        memcpy(cfgs[k], ion0, nb);
        conf_of_slot[k] = k;
        acc[k] = 0.0;
    }
    long nacc = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (int r = 1; r <= cfg->repeat; ++r) {
        int swap_count = 0;
        for (int k = 0; k < nT; ++k) {
            orc_stream_init(&st[k], cfg->seed, (uint32_t)((k + 1) + 175 * cfg->rank + 666 * r));
            orc_fresh_spins_typewriter(sy, cfgs[conf_of_slot[k]], &st[k]);
            memset(&a[k], 0, sizeof(orc_acc));
        }
        for (int step = 1; step <= cfg->tmcs; ++step) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static, 1)
#endif
            for (int k = 0; k < nT; ++k) {
                double *ion = cfgs[conf_of_slot[k]];
                if (ovrr_on && step % cfg->ovrr_mcs == 0 && step % cfg->coa != 0)
                    orc_overrelaxation_typewriter(sy, ion, ovrr_steps, &st[k]);
                acc[k] += orc_metropolis_typewriter(sy, ion, beta[k], &st[k]);
                E[conf_of_slot[k]] = orc_tot_energy(sy, ion);
            }
            if (ex > 0 && step % ex == 0 && step % cfg->coa != 0) {
                ++swap_count;
                nacc += orc_parallel_tempering(nT, beta, E, conf_of_slot, swap_count, cfg->seed,
                                               (uint32_t)r, 0, NULL);
            }
            if (step > cfg->tmcs_eq && step % cfg->coa == 0)
                for (int k = 0; k < nT; ++k) {
                    double M[3];
                    orc_tot_magnetisation(sy, cfgs[conf_of_slot[k]], M);
                    orc_acc_sample(&a[k], E[conf_of_slot[k]], M, N);
                }
        }
        for (int k = 0; k < nT; ++k)
            orc_acc_average(&a[k], beta[k], N, vals + 6 * ((size_t)cfg->repeat * k + (r - 1)));
    }
    for (int k = 0; k < nT; ++k) {
        acc[k] /= (double)cfg->repeat * cfg->tmcs;
        free(cfgs[k]);
    }
    free(cfgs); free(E); free(conf_of_slot); free(st); free(a);
    if (n_accepted) *n_accepted = nacc;
    (void)nthreads;
}

/* ------------------------------------------------------ moment vectors, spiral state ---- */
/* get_moment_vectors (src/get_moment_vectors.f90:20-38): mm(3, nsp) = sum over sites of
 * stgg_i * s(species_i) * S_i, sites in order. */
void orc_moment_vectors(const orc_sys *sy, const double *ion, double *mm) {
    for (int k = 0; k < 3 * sy->n_species; ++k) mm[k] = 0.0;
    for (int i = 0; i < sy->n_sites; ++i) {
        const int sp = (int)ion[9 * i + 4];
        const double w = (sy->stgg ? sy->stgg[i] : 1.0) * sy->s[sp - 1];
        for (int a = 0; a < 3; ++a) mm[3 * (sp - 1) + a] += w * ion[9 * i + 1 + a];
    }
}

/* get_spiral_state 'ions_for_spiral' (src/get_spiral_state.f90:45-77): for every site i the
 * sites j != i (increasing j) with |r_j - r_i| <= ss_dis and
 * acos((r_j - r_i)/|r_j - r_i| . ss_direc) * 180/pi <= ss_latency; no periodic images.
 * ifs(cap, N) receives 1-based j (0 = none).  Returns the total count, or -1 if a site has
 * more than cap (the reference writes past its array then). */
long orc_spiral_pairs(int N, const double *ion, double ss_dis, const double ss_direc[3],
                      double ss_latency, int cap, int32_t *ifs) {
    const double to_angle = 180.0 / 3.14159265358979323846;
    long count = 0;
    for (long k = 0; k < (long)cap * N; ++k) ifs[k] = 0;
    for (int i = 0; i < N; ++i) {
        int found = 0;
        for (int j = 0; j < N; ++j) {
            if (j == i) continue;
            double r[3];
            for (int a = 0; a < 3; ++a) r[a] = ion[9 * j + 6 + a] - ion[9 * i + 6 + a];
            const double dis = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            if (!(dis <= ss_dis)) continue;
            const double u[3] = {r[0] / dis, r[1] / dis, r[2] / dis};
            const double ang = acos(u[0] * ss_direc[0] + u[1] * ss_direc[1] + u[2] * ss_direc[2]) * to_angle;
            if (!(ang <= ss_latency)) continue;
            if (found == cap) return -1;
            ifs[(long)i * cap + found++] = j + 1;
            ++count;
        }
    }
    return count;
}

/* get_spiral_state 'spiral_state' (:79-108): |sum_i sum_j S_i x S_j| / spiral_count. */
double orc_spiral_state(int N, const double *ion, int cap, const int32_t *ifs, long count) {
    double ss[3] = {0, 0, 0};
    for (int i = 0; i < N; ++i) {
        const double *a = ion + 9 * i + 1;
        for (int k = 0; k < cap; ++k) {
            const int j = ifs[(long)i * cap + k];
            if (j == 0) break;
            const double *b = ion + 9 * (j - 1) + 1;
            ss[0] += a[1] * b[2] - a[2] * b[1];
            ss[1] += a[2] * b[0] - a[0] * b[2];
            ss[2] += a[0] * b[1] - a[1] * b[0];
        }
    }
    return sqrt(ss[0] * ss[0] + ss[1] * ss[1] + ss[2] * ss[2]) / (double)count;
}
