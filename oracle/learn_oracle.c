/*
 * learn_oracle.c -- TEST INFRASTRUCTURE: CPU restatement of the learned patch proposals
 * (the product's ether_learn_* in ether_gb300/csrc/k_learn.cu for Ising and
 * ether_gb300/csrc/k_learn_xyz.cu for Heisenberg; the Heisenberg part is at the end of this
 * file).  Only tests/, smoke() and bench.py's CPU legs call it.  The reference has no learned proposal; what must match the
 * reference is the stationary distribution, which exact Metropolis-Hastings preserves: the
 * acceptance below uses the reference's Ising energy (src/Hamiltonian.f90:57-105, pair
 * energy J s_i s_j with s = +-1, J the z component of j_exc) and its Boltzmann weight
 * exp(-beta E) (src/Metropolis.f90:50-56).
 *
 * Patch update (simple-cubic Ising, checkerboard storage, L1, L2, L3 multiples of 8):
 *   * a learned sweep draws an offset (ox, oy, oz) in [0,4)^3 per replica and tiles the
 *     lattice with 4^3 patches at (4i + ox, 4j + oy, 4k + oz); patch class (i + j + k) & 1;
 *     class 0 then class 1 (patches of one class share no bond);
 *   * canonical frame: local (a, b, c) in [0,4)^3 with real x = ox_p + (par ? 3 - a : a),
 *     par = (ox + oy + oz) & 1, so A-sites ((a + b + c) even) are always colour 0;
 *     A- and B-sites are numbered by a + 4b + 16c;
 *   * network input x[128]: the 96 boundary spins (faces a = -1, 4, b = -1, 4, c = -1, 4;
 *     16 sites each, index by the two other coordinates), x[96] = bf16(4 beta J), rest 0;
 *     MLP 128 -> 128 (ReLU) -> 128 (ReLU) -> 32 logits, BF16 weights and activations,
 *     FP32 accumulation; logit k is the log-odds of A-site k being up;
 *   * proposal: A-site k up iff u_k < T_k, T_k = clamp(sigmoid(z_k) 2^32, 1, 2^32 - 256)
 *     (so q_A = T/2^32 exactly); then every B-site from its exact conditional given its six
 *     neighbours (A-sites just drawn, boundary): up iff u < TB[n], TB from FP64 per
 *     temperature (table of the 7 neighbour sums);
 *   * accept with log alpha = (log q(old) - log q(new)) - beta J dB, dB the change of the
 *     patch's bond sum.  log q(new) - log q(old) = d, accumulated in FP32 in this order:
 *     A-sites k = 0..31 that changed add +z_k (now up) or -z_k (now down) -- the log-odds
 *     of the proposal, whose sampler realises sigmoid(z) to FP32 rounding and 2^-32 --, then
 *     B-sites m = 0..31 add (log q_B(new_m) - log q_B(old_m)); log alpha = (0 - d) - beta J dB.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ether_oracle.h"

/* ----------------------------------------------------------------- patch geometry ---- */
/* For A-site k: canonical (a, b, c); for B-site m likewise. */
static int g_ready = 0;
static int g_A[32][3], g_B[32][3];
/* neighbours of B-site m: code >= 0 -> A-site index, code < 0 -> boundary -(1 + idx) */
static int g_Bn[32][6];
/* boundary neighbours of A-site k (-1 = none), up to 3 */
static int g_Ab[32][3];

static int face_index(int a, int b, int c) {
    /* (a, b, c) with exactly one coordinate in {-1, 4}; returns the boundary index */
    if (a == -1) return 0 * 16 + b + 4 * c;
    if (a == 4) return 1 * 16 + b + 4 * c;
    if (b == -1) return 2 * 16 + a + 4 * c;
    if (b == 4) return 3 * 16 + a + 4 * c;
    if (c == -1) return 4 * 16 + a + 4 * b;
    return 5 * 16 + a + 4 * b;
}

static int a_index(int a, int b, int c) { /* index among A- or B-sites of its parity */
    const int lin = a + 4 * b + 16 * c;
    int n = 0;
    for (int t = 0; t < lin; ++t) {
        const int ta = t & 3, tb = (t >> 2) & 3, tc = t >> 4;
        if (((ta + tb + tc) & 1) == ((a + b + c) & 1)) ++n;
    }
    return n;
}

static void geometry(void) {
    if (g_ready) return;
    int na = 0, nb = 0;
    for (int lin = 0; lin < 64; ++lin) {
        const int a = lin & 3, b = (lin >> 2) & 3, c = lin >> 4;
        if (((a + b + c) & 1) == 0) { g_A[na][0] = a; g_A[na][1] = b; g_A[na][2] = c; ++na; }
        else { g_B[nb][0] = a; g_B[nb][1] = b; g_B[nb][2] = c; ++nb; }
    }
    static const int d[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
    for (int m = 0; m < 32; ++m)
        for (int q = 0; q < 6; ++q) {
            const int a = g_B[m][0] + d[q][0], b = g_B[m][1] + d[q][1], c = g_B[m][2] + d[q][2];
            if (a < 0 || a > 3 || b < 0 || b > 3 || c < 0 || c > 3) g_Bn[m][q] = -(1 + face_index(a, b, c));
            else g_Bn[m][q] = a_index(a, b, c);
        }
    for (int k = 0; k < 32; ++k) {
        int n = 0;
        for (int q = 0; q < 3; ++q) g_Ab[k][q] = -1;
        for (int q = 0; q < 6; ++q) {
            const int a = g_A[k][0] + d[q][0], b = g_A[k][1] + d[q][1], c = g_A[k][2] + d[q][2];
            if (a < 0 || a > 3 || b < 0 || b > 3 || c < 0 || c > 3) g_Ab[k][n++] = face_index(a, b, c);
        }
    }
    g_ready = 1;
}

void orc_patch_tables(int32_t *A, int32_t *B, int32_t *Bn, int32_t *Ab) {
    geometry();
    memcpy(A, g_A, sizeof g_A);
    memcpy(B, g_B, sizeof g_B);
    memcpy(Bn, g_Bn, sizeof g_Bn);
    memcpy(Ab, g_Ab, sizeof g_Ab);
}

/* storage index of real site (x, y, z) in one replica's colour-split array */
static long sc_index(const int L[3], int x, int y, int z) {
    x = ((x % L[0]) + L[0]) % L[0];
    y = ((y % L[1]) + L[1]) % L[1];
    z = ((z % L[2]) + L[2]) % L[2];
    const long H = L[0] / 2, half = H * L[1] * L[2];
    return ((x + y + z) & 1) * half + ((long)z * L[1] + y) * H + (x >> 1);
}

/* real coordinates of canonical (a, b, c) of the patch at origin o with reflection par */
static long site_of(const int L[3], const int o[3], int par, int a, int b, int c) {
    return sc_index(L, o[0] + (par ? 3 - a : a), o[1] + b, o[2] + c);
}

static float bf16r(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    memcpy(&f, &u, 4);
    return f;
}
float orc_bf16_round(float f) { return bf16r(f); }

/* Patch (pi, pj, pk) of a replica with offsets off[3]: boundary bits bnd[3] (bit f*16+idx of
 * word idx>>5), A bits, B bits (bit k = up) and the network input row x[128]. */
void orc_patch_gather(const uint8_t *sp, const int L[3], const int off[3], int pi, int pj, int pk,
                      float k4, float *x, uint32_t bnd[3], uint32_t *abits, uint32_t *bbits) {
    geometry();
    const int o[3] = {4 * pi + off[0], 4 * pj + off[1], 4 * pk + off[2]};
    const int par = (off[0] + off[1] + off[2]) & 1;
    bnd[0] = bnd[1] = bnd[2] = 0;
    for (int f = 0; f < 6; ++f)
        for (int u = 0; u < 4; ++u)
            for (int v = 0; v < 4; ++v) {
                int a, b, c;
                const int e = (f & 1) ? 4 : -1;
                if (f < 2) { a = e; b = u; c = v; }
                else if (f < 4) { a = u; b = e; c = v; }
                else { a = u; b = v; c = e; }
                const int idx = face_index(a, b, c);
                if (sp[site_of(L, o, par, a, b, c)]) bnd[idx >> 5] |= 1u << (idx & 31);
            }
    *abits = *bbits = 0;
    for (int k = 0; k < 32; ++k) {
        if (sp[site_of(L, o, par, g_A[k][0], g_A[k][1], g_A[k][2])]) *abits |= 1u << k;
        if (sp[site_of(L, o, par, g_B[k][0], g_B[k][1], g_B[k][2])]) *bbits |= 1u << k;
    }
    if (x) {
        for (int i = 0; i < 96; ++i) x[i] = ((bnd[i >> 5] >> (i & 31)) & 1u) ? 1.0f : -1.0f;
        x[96] = bf16r(k4);
        for (int i = 97; i < 128; ++i) x[i] = 0.0f;
    }
}

/* ------------------------------------------------------------------------ the MLP ---- */
/* params: W1[128][128], b1[128], W2[128][128], b2[128], W3[32][128], b3[32] (fp32 master,
 * row = output unit).  quant != 0: BF16 weights and BF16 hidden activations (what the GPU
 * computes); quant == 0: plain FP64 (for finite differences). */
enum { NI = 128, NH = 128, NO = 32 };
#define OFF_W1 0
#define OFF_B1 (OFF_W1 + NH * NI)
#define OFF_W2 (OFF_B1 + NH)
#define OFF_B2 (OFF_W2 + NH * NH)
#define OFF_W3 (OFF_B2 + NH)
#define OFF_B3 (OFF_W3 + NO * NH)
#define NPARAM (OFF_B3 + NO)

int orc_mlp_n_params(void) { return NPARAM; }

static double wq(const float *p, int i, int quant) { return quant ? (double)bf16r(p[i]) : (double)p[i]; }

static void forward1(const float *p, const float *x, int quant, double *h1, double *h2, double *z) {
    for (int o = 0; o < NH; ++o) {
        double s = 0.0;
        for (int i = 0; i < NI; ++i) s += wq(p, OFF_W1 + o * NI + i, quant) * (double)x[i];
        s += p[OFF_B1 + o];
        s = s > 0.0 ? s : 0.0;
        h1[o] = quant ? (double)bf16r((float)s) : s;
    }
    for (int o = 0; o < NH; ++o) {
        double s = 0.0;
        for (int i = 0; i < NH; ++i) s += wq(p, OFF_W2 + o * NH + i, quant) * h1[i];
        s += p[OFF_B2 + o];
        s = s > 0.0 ? s : 0.0;
        h2[o] = quant ? (double)bf16r((float)s) : s;
    }
    for (int o = 0; o < NO; ++o) {
        double s = 0.0;
        for (int i = 0; i < NH; ++i) s += wq(p, OFF_W3 + o * NH + i, quant) * h2[i];
        z[o] = s + p[OFF_B3 + o];
    }
}

void orc_mlp_forward(const float *params, const float *x, int B, int quant, float *logits) {
    double h1[NH], h2[NH], z[NO];
    for (int b = 0; b < B; ++b) {
        forward1(params, x + (size_t)b * NI, quant, h1, h2, z);
        for (int o = 0; o < NO; ++o) logits[(size_t)b * NO + o] = (float)z[o];
    }
}

/* Mean over the batch of sum_k BCE(z_k, y_k) (y bit k of y[b]); grad = d loss / d params
 * (straight-through for the BF16 rounding). */
double orc_mlp_loss_grad(const float *p, const float *x, const uint32_t *y, int B, int quant,
                         double *grad) {
    double h1[NH], h2[NH], z[NO], dz[NO], dh2[NH], dh1[NH];
    double loss = 0.0;
    memset(grad, 0, sizeof(double) * NPARAM);
    for (int b = 0; b < B; ++b) {
        const float *xb = x + (size_t)b * NI;
        forward1(p, xb, quant, h1, h2, z);
        for (int o = 0; o < NO; ++o) {
            const double t = (double)((y[b] >> o) & 1u);
            /* BCE with logits: softplus(z) - t z */
            const double sp = z[o] > 0 ? z[o] + log1p(exp(-z[o])) : log1p(exp(z[o]));
            loss += sp - t * z[o];
            dz[o] = (1.0 / (1.0 + exp(-z[o])) - t) / B;
        }
        for (int i = 0; i < NH; ++i) dh2[i] = 0.0;
        for (int o = 0; o < NO; ++o) {
            grad[OFF_B3 + o] += dz[o];
            for (int i = 0; i < NH; ++i) {
                grad[OFF_W3 + o * NH + i] += dz[o] * h2[i];
                dh2[i] += dz[o] * wq(p, OFF_W3 + o * NH + i, quant);
            }
        }
        for (int i = 0; i < NH; ++i) dh2[i] = h2[i] > 0.0 ? dh2[i] : 0.0;
        for (int i = 0; i < NH; ++i) dh1[i] = 0.0;
        for (int o = 0; o < NH; ++o) {
            grad[OFF_B2 + o] += dh2[o];
            for (int i = 0; i < NH; ++i) {
                grad[OFF_W2 + o * NH + i] += dh2[o] * h1[i];
                dh1[i] += dh2[o] * wq(p, OFF_W2 + o * NH + i, quant);
            }
        }
        for (int i = 0; i < NH; ++i) dh1[i] = h1[i] > 0.0 ? dh1[i] : 0.0;
        for (int o = 0; o < NH; ++o) {
            grad[OFF_B1 + o] += dh1[o];
            for (int i = 0; i < NI; ++i) grad[OFF_W1 + o * NI + i] += dh1[o] * (double)xb[i];
        }
    }
    return loss / B;
}

/* --------------------------------------------------------------- exact MH replay ---- */
/* FP32 log of x in (0, 1]: x = m 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s),
 * s = (m - 1)/(m + 1), series through s^9 (|s| < 0.172: truncation < 1e-9). */
float orc_logf_own(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    int e = (int)((u >> 23) & 0xFFu) - 127;
    u = (u & 0x007FFFFFu) | 0x3F800000u;
    float m;
    memcpy(&m, &u, 4);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = 0.111111111f;
    p = fmaf(p, s2, 0.142857143f);
    p = fmaf(p, s2, 0.2f);
    p = fmaf(p, s2, 0.333333333f);
    p = fmaf(p, s2, 1.0f);
    const float lm = 2.0f * (s * p);
    return fmaf((float)e, 0.693147182f, lm);
}

/* sigmoid(z) = r or e r with e = exp(-|z|), r = 1 / (1 + e) correctly rounded */
static float sigmoid_own(float z) {
    const float e = orc_expf_neg(-fabsf(z));
    const float r = 1.0f / (1.0f + e);
    return z >= 0.0f ? r : e * r;
}

static uint32_t thr_of_logit(float z) {
    float t = sigmoid_own(z) * 4294967296.0f;
    if (t < 1.0f) t = 1.0f;
    if (t > 4294967040.0f) t = 4294967040.0f;
    return (uint32_t)t;
}

static uint32_t word_of(const uint32_t w[4], int i) { return w[i & 3]; }

/* Heat-bath tables of the B-sites for beta J (FP64 -> u32 threshold, FP32 logs).
 * Index (n + 6) / 2, n = sum of the six neighbours (+-1). */
void orc_patch_btables(double betaJ, uint32_t TB[7], float LBup[7], float LBdn[7]) {
    for (int q = 0; q < 7; ++q) {
        const int n = 2 * q - 6;
        const double p = 1.0 / (1.0 + exp(2.0 * betaJ * n));  /* P(up) ~ exp(-beta J n) */
        double t = floor(p * 4294967296.0 + 0.5);
        if (t < 1.0) t = 1.0;
        if (t > 4294967295.0) t = 4294967295.0;
        TB[q] = (uint32_t)t;
        LBup[q] = (float)log(t / 4294967296.0);
        LBdn[q] = (float)log((4294967296.0 - t) / 4294967296.0);
    }
}

static void draw4(uint32_t c0, uint32_t t, uint32_t stream, uint32_t tag, uint32_t seed, uint32_t out[4]) {
    const uint32_t ctr[4] = {c0, t, stream, tag};
    const uint32_t key[2] = {seed, 0x45544852u};
    orc_philox4x32_10(ctr, key, out);
}

#define K_LEARN 4u

void orc_patch_offsets(uint32_t seed, uint32_t stream, uint32_t t, int off[3]) {
    uint32_t w[4];
    draw4(0xFFFFFFFFu, t, stream, K_LEARN | (0xFFu << 8), seed, w);
    off[0] = (int)(w[0] & 3u);
    off[1] = (int)((w[0] >> 2) & 3u);
    off[2] = (int)((w[0] >> 4) & 3u);
}

/* One patch update; returns 1 if accepted (spins written). */
static int patch_update(uint8_t *sp, const int L[3], const int off[3], int pi, int pj, int pk,
                        uint32_t pidx, const float *z, float betaJf, const uint32_t TB[7],
                        const float LBup[7], const float LBdn[7], uint32_t seed, uint32_t stream,
                        uint32_t t) {
    uint32_t bnd[3], ao, bo;
    orc_patch_gather(sp, L, off, pi, pj, pk, 0.0f, NULL, bnd, &ao, &bo);
    uint32_t an = 0, bn = 0;
    float d = 0.0f;
    uint32_t w[4];
    for (int k = 0; k < 32; ++k) {
        if ((k & 3) == 0) draw4(pidx, t, stream, K_LEARN | ((uint32_t)(k >> 2) << 16), seed, w);
        const uint32_t T = thr_of_logit(z[k]);
        const int up = word_of(w, k) < T;
        if (up) an |= 1u << k;
        if (up != (int)((ao >> k) & 1u)) d += up ? z[k] : -z[k];
    }
    int bond_o = 0, bond_n = 0;
    for (int m = 0; m < 32; ++m) {
        if ((m & 3) == 0) draw4(pidx, t, stream, K_LEARN | ((uint32_t)(8 + (m >> 2)) << 16), seed, w);
        int nn = 0, no = 0;
        for (int q = 0; q < 6; ++q) {
            const int cd = g_Bn[m][q];
            if (cd >= 0) {
                nn += ((an >> cd) & 1u) ? 1 : -1;
                no += ((ao >> cd) & 1u) ? 1 : -1;
            } else {
                const int bi = -cd - 1;
                const int s = ((bnd[bi >> 5] >> (bi & 31)) & 1u) ? 1 : -1;
                nn += s;
                no += s;
            }
        }
        const int qn = (nn + 6) >> 1, qo = (no + 6) >> 1;
        const int up = word_of(w, m) < TB[qn];
        if (up) bn |= 1u << m;
        const int upo = (int)((bo >> m) & 1u);
        const float lbn = up ? LBup[qn] : LBdn[qn];
        const float lbo = upo ? LBup[qo] : LBdn[qo];
        d += lbn - lbo;
        bond_n += (up ? 1 : -1) * nn;
        bond_o += (upo ? 1 : -1) * no;
    }
    for (int k = 0; k < 32; ++k) {
        int sb = 0;
        for (int q = 0; q < 3; ++q) {
            const int bi = g_Ab[k][q];
            if (bi < 0) continue;
            sb += ((bnd[bi >> 5] >> (bi & 31)) & 1u) ? 1 : -1;
        }
        bond_n += (((an >> k) & 1u) ? 1 : -1) * sb;
        bond_o += (((ao >> k) & 1u) ? 1 : -1) * sb;
    }
    draw4(pidx, t, stream, K_LEARN | (16u << 16), seed, w);
    const float la = (0.0f - d) - betaJf * (float)(bond_n - bond_o);
    int acc = la >= 0.0f;
    if (!acc) acc = (float)(w[0] >> 8) * 5.9604644775390625e-08f < orc_expf_neg(la);
    if (acc) {
        const int o[3] = {4 * pi + off[0], 4 * pj + off[1], 4 * pk + off[2]};
        const int par = (off[0] + off[1] + off[2]) & 1;
        for (int k = 0; k < 32; ++k) {
            sp[site_of(L, o, par, g_A[k][0], g_A[k][1], g_A[k][2])] = (uint8_t)((an >> k) & 1u);
            sp[site_of(L, o, par, g_B[k][0], g_B[k][1], g_B[k][2])] = (uint8_t)((bn >> k) & 1u);
        }
    }
    return acc;
}

/* One learned sweep of one replica (class 0 then class 1).  logits: [2][Pc][32] in the
 * order the GPU processes the class's patches: q = t + (P1/2) (j + P2 k),
 * i = 2t + ((cls + j + k) & 1).  Returns the number of accepted patches. */
long orc_patch_sweep(uint8_t *sp, const int L[3], double betaJ, const float *logits,
                     uint32_t seed, uint32_t stream, uint32_t t) {
    geometry();
    uint32_t TB[7];
    float LBup[7], LBdn[7];
    orc_patch_btables(betaJ, TB, LBup, LBdn);
    const float betaJf = (float)betaJ;
    int off[3];
    orc_patch_offsets(seed, stream, t, off);
    const int P1 = L[0] / 4, P2 = L[1] / 4, P3 = L[2] / 4;
    const long Pc = (long)P1 * P2 * P3 / 2;
    long acc = 0;
    for (int cls = 0; cls < 2; ++cls)
        for (long q = 0; q < Pc; ++q) {
            const int tt = (int)(q % (P1 / 2));
            const long row = q / (P1 / 2);
            const int j = (int)(row % P2), k = (int)(row / P2);
            const int i = 2 * tt + ((cls + j + k) & 1);
            const uint32_t pidx = (uint32_t)(i + P1 * (j + P2 * k));
            acc += patch_update(sp, L, off, i, j, k, pidx, logits + ((size_t)cls * Pc + q) * 32,
                                betaJf, TB, LBup, LBdn, seed, stream, t);
        }
    return acc;
}

/* ------------------------------------------------------ statistical check on the CPU ---- */
/* A chain of one L^3 replica at beta J: every step one typewriter Metropolis sweep (exact
 * thresholds in FP64) and, if use_patch, one learned sweep whose logits come from a fixed
 * stand-in "network" z_k = zscale * (sum of A-site k's boundary neighbours) + zbias -- any
 * proposal leaves the Boltzmann distribution invariant under the exact acceptance.
 * Returns <e>, err(e), <|m|>, err(|m|) per site (batch means over 20 batches) and the
 * patch acceptance ratio. */
void orc_patch_chain(const int L[3], double betaJ, long nsteps, long nequil, int use_patch,
                     float zscale, float zbias, uint32_t seed, double out[5]) {
    geometry();
    const long N = (long)L[0] * L[1] * L[2];
    uint8_t *sp = (uint8_t *)calloc((size_t)N, 1);
    orc_stream st;
    orc_stream_init(&st, seed, 77u);
    for (long s = 0; s < N; ++s) sp[s] = orc_stream_uniform(&st) < 0.5 ? 1 : 0;
    const int P1 = L[0] / 4, P2 = L[1] / 4, P3 = L[2] / 4;
    const long Pc = (long)P1 * P2 * P3 / 2;
    uint32_t TB[7];
    float LBup[7], LBdn[7];
    orc_patch_btables(betaJ, TB, LBup, LBdn);
    enum { NB = 20 };
    double be[NB] = {0}, bm[NB] = {0};
    long acc = 0, prop = 0;
    const long per = (nsteps / NB) > 0 ? nsteps / NB : 1;
    for (long step = 0; step < nequil + nsteps; ++step) {
        /* typewriter Metropolis with the exact FP64 acceptance */
        for (int zc = 0; zc < L[2]; ++zc)
            for (int yc = 0; yc < L[1]; ++yc)
                for (int xc = 0; xc < L[0]; ++xc) {
                    const long i = sc_index(L, xc, yc, zc);
                    int n = 0;
                    n += sp[sc_index(L, xc + 1, yc, zc)] ? 1 : -1;
                    n += sp[sc_index(L, xc - 1, yc, zc)] ? 1 : -1;
                    n += sp[sc_index(L, xc, yc + 1, zc)] ? 1 : -1;
                    n += sp[sc_index(L, xc, yc - 1, zc)] ? 1 : -1;
                    n += sp[sc_index(L, xc, yc, zc + 1)] ? 1 : -1;
                    n += sp[sc_index(L, xc, yc, zc - 1)] ? 1 : -1;
                    const int s = sp[i] ? 1 : -1;
                    const double bdE = -2.0 * betaJ * s * n; /* beta (E_new - E_old) */
                    if (bdE <= 0.0 || orc_stream_uniform(&st) < exp(-bdE)) sp[i] ^= 1u;
                }
        if (use_patch) {
            int off[3];
            orc_patch_offsets(seed, 5u, (uint32_t)step, off);
            for (int cls = 0; cls < 2; ++cls)
                for (long q = 0; q < Pc; ++q) {
                    const int tt = (int)(q % (P1 / 2));
                    const long row = q / (P1 / 2);
                    const int j = (int)(row % P2), k = (int)(row / P2);
                    const int i = 2 * tt + ((cls + j + k) & 1);
                    uint32_t bnd[3], ao, bo;
                    orc_patch_gather(sp, L, off, i, j, k, 0.0f, NULL, bnd, &ao, &bo);
                    float zz[32];
                    for (int a = 0; a < 32; ++a) {
                        int sb = 0;
                        for (int qq = 0; qq < 3; ++qq) {
                            const int bi = g_Ab[a][qq];
                            if (bi >= 0) sb += ((bnd[bi >> 5] >> (bi & 31)) & 1u) ? 1 : -1;
                        }
                        zz[a] = zscale * (float)sb + zbias;
                    }
                    const uint32_t pidx = (uint32_t)(i + P1 * (j + P2 * k));
                    acc += patch_update(sp, L, off, i, j, k, pidx, zz, (float)betaJ, TB, LBup, LBdn,
                                        seed, 5u, (uint32_t)step);
                    ++prop;
                }
        }
        if (step >= nequil) {
            long bond = 0, mag = 0;
            for (int zc = 0; zc < L[2]; ++zc)
                for (int yc = 0; yc < L[1]; ++yc)
                    for (int xc = 0; xc < L[0]; ++xc) {
                        const int s = sp[sc_index(L, xc, yc, zc)] ? 1 : -1;
                        mag += s;
                        bond += s * ((sp[sc_index(L, xc + 1, yc, zc)] ? 1 : -1) +
                                     (sp[sc_index(L, xc, yc + 1, zc)] ? 1 : -1) +
                                     (sp[sc_index(L, xc, yc, zc + 1)] ? 1 : -1));
                    }
            const long b = (step - nequil) / per;
            if (b < NB) {
                be[b] += (double)bond / N;
                bm[b] += fabs((double)mag) / N;
            }
        }
    }
    double me = 0, mm = 0, ve = 0, vm = 0;
    for (int b = 0; b < NB; ++b) {
        be[b] /= per;
        bm[b] /= per;
        me += be[b] / NB;
        mm += bm[b] / NB;
    }
    for (int b = 0; b < NB; ++b) {
        ve += (be[b] - me) * (be[b] - me);
        vm += (bm[b] - mm) * (bm[b] - mm);
    }
    out[0] = me;
    out[1] = sqrt(ve / (NB * (NB - 1.0)));
    out[2] = mm;
    out[3] = sqrt(vm / (NB * (NB - 1.0)));
    out[4] = prop > 0 ? (double)acc / prop : 0.0;
    free(sp);
}

/* ============================================== the Heisenberg (XYZ) learned proposal ==== */
/* Restatement of the XYZ learner (the product's k_learn_xyz.cu).  Target: exp(-beta E),
 * E = sum over bonds of S_i . (J o S_j), J = (Jxx, Jyy, Jzz) (src/Hamiltonian.f90:57-105).
 * Patch tiling, offsets, canonical frame and A/B numbering as the Ising learner above.
 *   * network input x[304]: boundary site i (face order) at 3i .. 3i+2 (BF16-rounded
 *     components), x[288..290] = bf16(beta Jxx), bf16(beta Jyy), bf16(beta Jzz), rest 0;
 *     MLP 304 -> 128 -> 128 -> 96 (ReLU, BF16 weights and hidden activations);
 *     m_k = outputs 3k .. 3k+2 + bias: the von Mises-Fisher parameter of A-site k;
 *   * A-site k ~ vMF(m_k) from draw(pidx, t, stream, 4 | (32 + k) << 16): u01(.x), upm1(.y);
 *     B-site k ~ vMF(-beta J o g_k), g_k = sum of its six neighbours (q order), from .z, .w;
 *     |m| < 1e-3 is the uniform distribution (sampler and density);
 *   * log alpha = sum_k [(s_A,new + s_B,new) - (s_A,old + s_B,old)], summed over k = 0..31 by
 *     the xor butterfly (offsets 16, 8, 4, 2, 1), with s_A = (-beta) (x_A . (J o b_A)) -
 *     log q_A(x_A), b_A the sum of A-site k's boundary neighbours, and s_B = m_B . y_B -
 *     log q_B(y_B); accept if log alpha >= 0 or u01(draw(pidx, t, stream, 4 | 16 << 16).x) <
 *     exp(log alpha).  FP32 throughout, the operations in the product's order. */
enum { XNI = 304, XNO = 96 };
#define XOFF_W1 0
#define XOFF_B1 (XOFF_W1 + NH * XNI)
#define XOFF_W2 (XOFF_B1 + NH)
#define XOFF_B2 (XOFF_W2 + NH * NH)
#define XOFF_W3 (XOFF_B2 + NH)
#define XOFF_B3 (XOFF_W3 + XNO * NH)
#define XNPARAM (XOFF_B3 + XNO)

int orc_xmlp_n_params(void) { return XNPARAM; }

/* quant 1: BF16 weights and hidden activations (the training kernels); quant 2: also BF16
 * hidden-layer biases (the inference path, cuBLASLt's bias epilogue in BF16). */
static void xforward1(const float *p, const float *x, int quant, double *h1, double *h2, double *z) {
    for (int o = 0; o < NH; ++o) {
        double s = 0.0;
        for (int i = 0; i < XNI; ++i) s += wq(p, XOFF_W1 + o * XNI + i, quant) * (double)x[i];
        s += quant == 2 ? (double)bf16r(p[XOFF_B1 + o]) : (double)p[XOFF_B1 + o];
        s = s > 0.0 ? s : 0.0;
        h1[o] = quant ? (double)bf16r((float)s) : s;
    }
    for (int o = 0; o < NH; ++o) {
        double s = 0.0;
        for (int i = 0; i < NH; ++i) s += wq(p, XOFF_W2 + o * NH + i, quant) * h1[i];
        s += quant == 2 ? (double)bf16r(p[XOFF_B2 + o]) : (double)p[XOFF_B2 + o];
        s = s > 0.0 ? s : 0.0;
        h2[o] = quant ? (double)bf16r((float)s) : s;
    }
    for (int o = 0; o < XNO; ++o) {
        double s = 0.0;
        for (int i = 0; i < NH; ++i) s += wq(p, XOFF_W3 + o * NH + i, quant) * h2[i];
        z[o] = s + p[XOFF_B3 + o];
    }
}

void orc_xmlp_forward(const float *params, const float *x, int B, int quant, float *out) {
    double h1[NH], h2[NH], z[XNO];
    for (int b = 0; b < B; ++b) {
        xforward1(params, x + (size_t)b * XNI, quant, h1, h2, z);
        for (int o = 0; o < XNO; ++o) out[(size_t)b * XNO + o] = (float)z[o];
    }
}

/* log C(kappa) = log(kappa / (4 pi sinh kappa)) and A(kappa) = (1/kappa - coth kappa) / kappa */
static void vmf_terms(double kap, double *logc, double *A) {
    if (kap < 1e-4) {
        *logc = -log(4.0 * M_PI) - kap * kap / 6.0;
        *A = -1.0 / 3.0 + kap * kap / 45.0;
    } else {
        *logc = log(kap) - kap - log(-expm1(-2.0 * kap)) - log(2.0 * M_PI);
        *A = (1.0 / kap - 1.0 / tanh(kap)) / kap;
    }
}

/* Mean over the batch of sum_k -log vMF(y_k; m_k) (y: 96 spin components per row); grad =
 * d loss / d params (straight-through for the BF16 rounding). */
double orc_xmlp_loss_grad(const float *p, const float *x, const float *y, int B, int quant, double *grad) {
    double h1[NH], h2[NH], z[XNO], dz[XNO], dh2[NH], dh1[NH];
    double loss = 0.0;
    memset(grad, 0, sizeof(double) * XNPARAM);
    for (int b = 0; b < B; ++b) {
        const float *xb = x + (size_t)b * XNI;
        const float *yb = y + (size_t)b * XNO;
        xforward1(p, xb, quant, h1, h2, z);
        for (int k = 0; k < 32; ++k) {
            const double mx = z[3 * k], my = z[3 * k + 1], mz = z[3 * k + 2];
            const double kap = sqrt(mx * mx + my * my + mz * mz);
            double logc, A;
            vmf_terms(kap, &logc, &A);
            loss += -(logc + mx * yb[3 * k] + my * yb[3 * k + 1] + mz * yb[3 * k + 2]);
            dz[3 * k] = -(yb[3 * k] + A * mx) / B;
            dz[3 * k + 1] = -(yb[3 * k + 1] + A * my) / B;
            dz[3 * k + 2] = -(yb[3 * k + 2] + A * mz) / B;
        }
        for (int i = 0; i < NH; ++i) dh2[i] = 0.0;
        for (int o = 0; o < XNO; ++o) {
            grad[XOFF_B3 + o] += dz[o];
            for (int i = 0; i < NH; ++i) {
                grad[XOFF_W3 + o * NH + i] += dz[o] * h2[i];
                dh2[i] += dz[o] * wq(p, XOFF_W3 + o * NH + i, quant);
            }
        }
        for (int i = 0; i < NH; ++i) dh2[i] = h2[i] > 0.0 ? dh2[i] : 0.0;
        for (int i = 0; i < NH; ++i) dh1[i] = 0.0;
        for (int o = 0; o < NH; ++o) {
            grad[XOFF_B2 + o] += dh2[o];
            for (int i = 0; i < NH; ++i) {
                grad[XOFF_W2 + o * NH + i] += dh2[o] * h1[i];
                dh1[i] += dh2[o] * wq(p, XOFF_W2 + o * NH + i, quant);
            }
        }
        for (int i = 0; i < NH; ++i) dh1[i] = h1[i] > 0.0 ? dh1[i] : 0.0;
        for (int o = 0; o < NH; ++o) {
            grad[XOFF_B1 + o] += dh1[o];
            for (int i = 0; i < XNI; ++i) grad[XOFF_W1 + o * XNI + i] += dh1[o] * (double)xb[i];
        }
    }
    return loss / B;
}

static float xu01(uint32_t u) { return (float)(u >> 8) * 0x1p-24f; }
static float xupm1(uint32_t u) { return (float)(u >> 8) * 0x1p-23f - 1.0f; }

static float xdot3(float ax, float ay, float az, float bx, float by, float bz) {
    float d = ax * bx;
    d = fmaf(ay, by, d);
    return fmaf(az, bz, d);
}

/* log(1 - y), y in [0, 1): 2 atanh(-y / (2 - y)) through s^15 below 1/2, else log(1 - y) */
static float xlog1m(float y) {
    if (y >= 0.5f) return orc_logf_own(1.0f - y);
    const float s = -y / (2.0f - y);
    const float s2 = s * s;
    float p = 0.0666666667f;
    p = fmaf(p, s2, 0.0769230769f);
    p = fmaf(p, s2, 0.0909090909f);
    p = fmaf(p, s2, 0.111111111f);
    p = fmaf(p, s2, 0.142857143f);
    p = fmaf(p, s2, 0.2f);
    p = fmaf(p, s2, 0.333333333f);
    p = fmaf(p, s2, 1.0f);
    return 2.0f * (s * p);
}

/* 1 - e^{-2 kappa}: series of 1 - e^{-y} through y^8 for y = 2 kappa < 1/2 */
static float xoneminus(float kappa) {
    const float y = 2.0f * kappa;
    if (y >= 0.5f) return 1.0f - orc_expf_neg(-y);
    float p = 2.48015873e-5f;
    p = fmaf(p, y, -1.98412698e-4f);
    p = fmaf(p, y, 1.38888889e-3f);
    p = fmaf(p, y, -8.33333333e-3f);
    p = fmaf(p, y, 4.16666667e-2f);
    p = fmaf(p, y, -1.66666667e-1f);
    p = fmaf(p, y, 0.5f);
    p = fmaf(p, y, -1.0f);
    return -(y * p);
}

#define XKAPPA_MIN 1e-3f
#define XLOG4PI 2.53102425f
#define XLOG2PI 1.83787707f

/* vMF(m): kappa = |m|, rk = 1 / kappa, c = log(kappa / (1 - e^{-2 kappa})) - log 2 pi; the
 * uniform distribution below XKAPPA_MIN.  log density at x = c + (m . x - kappa). */
typedef struct {
    float mx, my, mz, kappa, rk, c;
    int uni;
} Vmf;

static Vmf vmf_prep(float mx, float my, float mz) {
    Vmf V;
    V.mx = mx;
    V.my = my;
    V.mz = mz;
    V.kappa = sqrtf(xdot3(mx, my, mz, mx, my, mz));
    V.uni = V.kappa < XKAPPA_MIN;
    V.rk = V.uni ? 0.0f : 1.0f / V.kappa;
    V.c = V.uni ? -XLOG4PI : orc_logf_own(V.kappa * (1.0f / xoneminus(V.kappa))) - XLOG2PI;
    return V;
}

static float vmf_lp(const Vmf *V, float x, float y, float z) {
    return V->uni ? -XLOG4PI : V->c + (xdot3(V->mx, V->my, V->mz, x, y, z) - V->kappa);
}

float orc_vmf_logpdf(float mx, float my, float mz, float x, float y, float z) {
    const Vmf V = vmf_prep(mx, my, mz);
    return vmf_lp(&V, x, y, z);
}

/* Wood's sampler: 1 - w = -log(1 - (1 - u)(1 - e^{-2 kappa})) / kappa, azimuth pi v */
static void vmf_draw(const Vmf *V, float u, float v, float out[3]) {
    float ux = 0.0f, uy = 0.0f, uz = 1.0f, om;
    if (V->uni) {
        om = 2.0f * (1.0f - u);
    } else {
        ux = V->mx * V->rk;
        uy = V->my * V->rk;
        uz = V->mz * V->rk;
        om = -xlog1m((1.0f - u) * xoneminus(V->kappa)) * V->rk;
    }
    om = fminf(fmaxf(om, 0.0f), 2.0f);
    const float w = 1.0f - om;
    const float r = sqrtf(om * (2.0f - om));
    float e1x, e1y, e1z;
    if (fabsf(uz) < 0.9f) {
        const float rn = 1.0f / sqrtf(xdot3(uy, ux, 0.0f, uy, ux, 0.0f));
        e1x = -uy * rn;
        e1y = ux * rn;
        e1z = 0.0f;
    } else {
        const float rn = 1.0f / sqrtf(xdot3(0.0f, uz, uy, 0.0f, uz, uy));
        e1x = 0.0f;
        e1y = uz * rn;
        e1z = -uy * rn;
    }
    const float e2x = uy * e1z - uz * e1y, e2y = uz * e1x - ux * e1z, e2z = ux * e1y - uy * e1x;
    float sn, cs;
    orc_sincosf(3.14159265f * v, &sn, &cs);
    const float px = cs * e1x + sn * e2x, py = cs * e1y + sn * e2y, pz = cs * e1z + sn * e2z;
    const float x = w * ux + r * px, y = w * uy + r * py, z = w * uz + r * pz;
    const float rnn = 1.0f / sqrtf(xdot3(x, y, z, x, y, z));
    out[0] = x * rnn;
    out[1] = y * rnn;
    out[2] = z * rnn;
}

void orc_vmf_sample(float mx, float my, float mz, float u, float v, float out[3]) {
    const Vmf V = vmf_prep(mx, my, mz);
    vmf_draw(&V, u, v, out);
}

static void bnd_coords(int i, int *a, int *b, int *c) {
    const int f = i >> 4, u = i & 3, v = (i >> 2) & 3, e = (f & 1) ? 4 : -1;
    if (f < 2) { *a = e; *b = u; *c = v; }
    else if (f < 4) { *a = u; *b = e; *c = v; }
    else { *a = u; *b = v; *c = e; }
}

/* One XYZ patch update; sp4: one replica's spins, 4 floats per storage index (x, y, z, phi). */
static int xpatch_update(float *sp4, const int L[3], const int off[3], int pi, int pj, int pk, uint32_t pidx,
                         const float *m96, float beta, const float J[3], uint32_t seed, uint32_t stream,
                         uint32_t t) {
    const int o[3] = {4 * pi + off[0], 4 * pj + off[1], 4 * pk + off[2]};
    const int par = (off[0] + off[1] + off[2]) & 1;
    const float nbeta = -beta;
    float nA[32][3], oA[32][3], nB[32][3], d[32];
    long ia[32], ib[32];
    float sa_new[32], sa_old[32];
    for (int k = 0; k < 32; ++k) {
        ia[k] = site_of(L, o, par, g_A[k][0], g_A[k][1], g_A[k][2]);
        for (int c = 0; c < 3; ++c) oA[k][c] = sp4[4 * ia[k] + c];
        const float mx = m96[3 * k], my = m96[3 * k + 1], mz = m96[3 * k + 2];
        float bx = 0.0f, by = 0.0f, bz = 0.0f;
        for (int n = 0; n < 3; ++n) {
            const int bi = g_Ab[k][n];
            if (bi < 0) continue;
            int a, b, c;
            bnd_coords(bi, &a, &b, &c);
            const long s = site_of(L, o, par, a, b, c);
            bx += sp4[4 * s];
            by += sp4[4 * s + 1];
            bz += sp4[4 * s + 2];
        }
        const float hx = J[0] * bx, hy = J[1] * by, hz = J[2] * bz;
        uint32_t w[4];
        draw4(pidx, t, stream, K_LEARN | ((32u + (uint32_t)k) << 16), seed, w);
        const Vmf VA = vmf_prep(mx, my, mz);
        vmf_draw(&VA, xu01(w[0]), xupm1(w[1]), nA[k]);
        sa_new[k] = nbeta * xdot3(nA[k][0], nA[k][1], nA[k][2], hx, hy, hz) - vmf_lp(&VA, nA[k][0], nA[k][1], nA[k][2]);
        sa_old[k] = nbeta * xdot3(oA[k][0], oA[k][1], oA[k][2], hx, hy, hz) - vmf_lp(&VA, oA[k][0], oA[k][1], oA[k][2]);
    }
    for (int k = 0; k < 32; ++k) {
        ib[k] = site_of(L, o, par, g_B[k][0], g_B[k][1], g_B[k][2]);
        const float yo[3] = {sp4[4 * ib[k]], sp4[4 * ib[k] + 1], sp4[4 * ib[k] + 2]};
        float gn[3] = {0.0f, 0.0f, 0.0f}, go[3] = {0.0f, 0.0f, 0.0f};
        for (int q = 0; q < 6; ++q) {
            const int cd = g_Bn[k][q];
            float sn[3], so[3];
            if (cd >= 0) {
                for (int c = 0; c < 3; ++c) {
                    sn[c] = nA[cd][c];
                    so[c] = oA[cd][c];
                }
            } else {
                int a, b, c;
                bnd_coords(-cd - 1, &a, &b, &c);
                const long s = site_of(L, o, par, a, b, c);
                for (int e = 0; e < 3; ++e) sn[e] = so[e] = sp4[4 * s + e];
            }
            for (int c = 0; c < 3; ++c) {
                gn[c] += sn[c];
                go[c] += so[c];
            }
        }
        const float mbn[3] = {nbeta * (J[0] * gn[0]), nbeta * (J[1] * gn[1]), nbeta * (J[2] * gn[2])};
        const float mbo[3] = {nbeta * (J[0] * go[0]), nbeta * (J[1] * go[1]), nbeta * (J[2] * go[2])};
        uint32_t w[4];
        draw4(pidx, t, stream, K_LEARN | ((32u + (uint32_t)k) << 16), seed, w);
        const Vmf VBn = vmf_prep(mbn[0], mbn[1], mbn[2]), VBo = vmf_prep(mbo[0], mbo[1], mbo[2]);
        vmf_draw(&VBn, xu01(w[2]), xupm1(w[3]), nB[k]);
        const float sb_new = xdot3(mbn[0], mbn[1], mbn[2], nB[k][0], nB[k][1], nB[k][2]) -
                             vmf_lp(&VBn, nB[k][0], nB[k][1], nB[k][2]);
        const float sb_old = xdot3(mbo[0], mbo[1], mbo[2], yo[0], yo[1], yo[2]) - vmf_lp(&VBo, yo[0], yo[1], yo[2]);
        d[k] = (sa_new[k] + sb_new) - (sa_old[k] + sb_old);
    }
    for (int off2 = 16; off2 >= 1; off2 >>= 1) {
        float nd[32];
        for (int l = 0; l < 32; ++l) nd[l] = d[l] + d[l ^ off2];
        memcpy(d, nd, sizeof(nd));
    }
    const float la = d[0];
    uint32_t w[4];
    draw4(pidx, t, stream, K_LEARN | (16u << 16), seed, w);
    const int acc = la >= 0.0f || xu01(w[0]) < orc_expf_neg(la);
    if (acc)
        for (int k = 0; k < 32; ++k)
            for (int c = 0; c < 3; ++c) {
                sp4[4 * ia[k] + c] = nA[k][c];
                sp4[4 * ib[k] + c] = nB[k][c];
            }
    return acc;
}

/* One XYZ learned sweep of one replica (class 0 then class 1); mdump: [2][Pc][96] vMF
 * parameters in the GPU's patch order.  Returns the number of accepted patches. */
long orc_xpatch_sweep(float *sp4, const int L[3], float beta, const float J[3], const float *mdump,
                      uint32_t seed, uint32_t stream, uint32_t t) {
    geometry();
    int off[3];
    orc_patch_offsets(seed, stream, t, off);
    const int P1 = L[0] / 4, P2 = L[1] / 4, P3 = L[2] / 4;
    const long Pc = (long)P1 * P2 * P3 / 2;
    long acc = 0;
    for (int cls = 0; cls < 2; ++cls)
        for (long q = 0; q < Pc; ++q) {
            const int tt = (int)(q % (P1 / 2));
            const long row = q / (P1 / 2);
            const int j = (int)(row % P2), k = (int)(row / P2);
            const int i = 2 * tt + ((cls + j + k) & 1);
            const uint32_t pidx = (uint32_t)(i + P1 * (j + P2 * k));
            acc += xpatch_update(sp4, L, off, i, j, k, pidx, mdump + ((size_t)cls * Pc + q) * XNO, beta, J, seed,
                                 stream, t);
        }
    return acc;
}
