// k_obs.cu -- energy / magnetisation reductions (src/get_tot_energy.f90:33-47,
// src/get_tot_magnetisation.f90:32-40), the observable accumulators (src/observable.f90,
// src/get_eng.f90:36-40, src/get_mag.f90:36-41) and parallel tempering
// (src/parallel_tempering.f90:39-108).
//
// Site energies are FP32 (XYZ) or exact sums of ±J (Ising); every per-replica total and
// every accumulator is FP64.  Reductions write per-block partials to scratch memory and a
// second kernel adds them in a fixed order, so results do not depend on timing.
//
// GB300 issues about 2 FP64 instructions per SM and clock against 128 FP32, so the running
// sums avoid FP64 per site: Ising bond terms s_i s_j J are +-J exactly, so with one coupling,
// one species and one |weight| a thread counts them in integers and the warp and the block
// add the counts (else it adds +-J, one FP64 add per bond); XYZ sums are kept as FP32
// double-single pairs (Knuth's TwoSum, products split exactly with fmaf), about 48
// significant bits, summed over the warp and the block the same way and turned into FP64 once
// per block.
#include "internal.h"
#include "rng_math.cuh"
#include "sweep_xyz.cuh"

namespace ether {

constexpr int kRedBs = 256;
constexpr int kNq = 5;  // E_raw, E_exchange, Mx, My, Mz

// A running sum hi + lo of FP32 terms (double-single): TwoSum keeps hi's rounding error
// exactly, lo collects those errors.
struct DS {
    float hi = 0.f, lo = 0.f;
};
__device__ __forceinline__ void ds_add(DS &a, float x) {
    const float s = a.hi + x;
    const float bp = s - a.hi;
    const float err = (a.hi - (s - bp)) + (x - bp);
    a.hi = s;
    a.lo += err;
}
// a += w x, the product split exactly (p + fmaf(w, x, -p) = w x)
__device__ __forceinline__ void ds_add_prod(DS &a, float w, float x) {
    const float p = w * x;
    const float e = fmaf(w, x, -p);
    ds_add(a, p);
    a.lo += e;
}
__device__ __forceinline__ double ds_value(const DS &a) { return (double)a.hi + (double)a.lo; }
// Warp sum of double-single values (lane 0 holds it): FP32 shuffles and TwoSums, no FP64.
__device__ __forceinline__ DS warp_sum_ds(DS v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h = __shfl_down_sync(0xffffffffu, v.hi, o);
        const float l = __shfl_down_sync(0xffffffffu, v.lo, o);
        ds_add(v, h);
        v.lo += l;
    }
    return v;
}

// Simple cubic, colour-split arrays: sum over the six bonds of rank rho of colour `colour`
// of s_i s_j (+1 aligned, -1 not), neighbours in closed form from the other colour's bytes.
__device__ __forceinline__ int sc_ising_bonds(const uint8_t *__restrict__ opp, const ObsMember &a, int H,
                                              int colour, int rho, uint8_t own) {
    const int row = (int)fdiv((uint32_t)rho, a.sc_fH);
    const int xh = rho - row * H;
    const int z = (int)fdiv((uint32_t)row, a.sc_fL2), y = row - z * a.sc_L2;
    const int p = (y + z + colour) & 1;
    const int L2 = a.sc_L2, L3 = a.sc_L3;
    const int ym = (y == 0 ? L2 - 1 : y - 1), yp = (y == L2 - 1 ? 0 : y + 1);
    const int zm = (z == 0 ? L3 - 1 : z - 1), zp = (z == L3 - 1 ? 0 : z + 1);
    const int xh_m = p == 0 ? (xh == 0 ? H - 1 : xh - 1) : xh;
    const int xh_p = p == 0 ? xh : (xh == H - 1 ? 0 : xh + 1);
    const uint8_t v0 = opp[row * H + xh_m], v1 = opp[row * H + xh_p];
    const uint8_t v2 = opp[(z * L2 + ym) * H + xh], v3 = opp[(z * L2 + yp) * H + xh];
    const uint8_t v4 = opp[(zm * L2 + y) * H + xh], v5 = opp[(zp * L2 + y) * H + xh];
    const int same = (v0 == own) + (v1 == own) + (v2 == own) + (v3 == own) + (v4 == own) + (v5 == own);
    return 2 * same - 6;
}

// Sign flip of an FP64 value by its sign bit (no FP64 instruction).
__device__ __forceinline__ double neg_if(double v, bool neg) {
    return __longlong_as_double(__double_as_longlong(v) ^ (neg ? (long long)0x8000000000000000ULL : 0LL));
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// How a block's per-thread sums are kept until the block total: integer counts (Ising
// counting form), double-single pairs for all kNq (or only the two energies) quantities, or
// FP64.  Integers and pairs are summed over the warp and then over the block's warps, and
// turned into FP64 once per block: the FP64 pipe, 1/64 of the FP32 rate, then carries one
// conversion per block instead of one per warp.
enum { kFormDouble = 0, kFormCount = 1, kFormDS = 2, kFormDSEnergy = 3 };

// Block totals of three per-warp integer sums (lane 0 of each warp holds its warp's) into
// t[0..2] of thread 0 (the whole block calls it).
__device__ __forceinline__ void block_sum_ints(const int (&ci)[3], int (&t)[3]) {
    __shared__ int si[kRedBs / 32][3];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int j = 0; j < 3; ++j) si[wid][j] = ci[j];
    __syncthreads();
    t[0] = t[1] = t[2] = 0;
    if (threadIdx.x == 0)
        for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2)
            for (int j = 0; j < 3; ++j) t[j] += si[w2][j];
}

// Block totals of Q quantities into out[0..Q-1] (thread j writes quantity j; the whole block
// calls it): quantities j < nds come as per-warp double-single sums in qd (lane 0 holds the
// warp's), the others as per-thread FP64 values in q, summed over the warp here.
template <int Q>
__device__ __forceinline__ void block_sum_mixed(const double (&q)[Q], const DS (&qd)[Q], int nds,
                                                double *__restrict__ out) {
    __shared__ float2 sd[kRedBs / 32][Q];
    __shared__ double sm[kRedBs / 32][Q];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        if (j < nds) {
            if (lane == 0) sd[wid][j] = make_float2(qd[j].hi, qd[j].lo);
        } else {
            const double v = warp_sum_d(q[j]);
            if (lane == 0) sm[wid][j] = v;
        }
    }
    __syncthreads();
    const int j = threadIdx.x;
    if (j < Q) {
        const int nw = (int)(blockDim.x >> 5);
        if (j < nds) {
            DS acc;
            for (int w2 = 0; w2 < nw; ++w2) {
                ds_add(acc, sd[w2][j].x);
                acc.lo += sd[w2][j].y;
            }
            out[j] = ds_value(acc);
        } else {
            double v = 0.0;
            for (int w2 = 0; w2 < nw; ++w2) v += sm[w2][j];
            out[j] = v;
        }
    }
}

// Partial sums of block b (of a.nblk) of replica r into a.partials[(r * nblk + b) * kNq ..]:
// the whole block calls it.
__device__ __forceinline__ void energy_block(const ObsMember &a, int r, int b) {
    const int N = a.N;
    const int stride = a.nblk * blockDim.x;
    double q[kNq] = {0, 0, 0, 0, 0};
    int ci[3] = {0, 0, 0};
    DS qd[kNq];
    int form = kFormDouble;
    if (a.model == 0 && a.count_form) {
        // E_ex = J sum s_i s_j, the field term z sum s_i, M = |w| sum sign(w_i) s_i
        const uint8_t *sp = a.spins + (size_t)r * N;
        int cb = 0, cz = 0, cm = 0;
        const int H = a.sc_L1 >> 1, half = N >> 1;
        for (int s = b * blockDim.x + threadIdx.x; s < N; s += stride) {
            const uint8_t own = sp[s];
            if (a.sc_ising) {
                const int colour = s >= half ? 1 : 0;
                cb += sc_ising_bonds(sp + (size_t)(colour ^ 1) * half, a, H, colour, s - colour * half, own);
            } else {
                for (int k = a.row_ptr[s]; k < a.row_ptr[s + 1]; ++k) cb += (sp[a.nbr[k]] == own) ? 1 : -1;
            }
            cz += own ? 1 : -1;
            const bool wneg = a.mw_pos ? false : __double_as_longlong(a.mweight[s]) < 0;
            cm += ((own != 0) != wneg) ? 1 : -1;
        }
        // counts summed over the warp and the block in integers, FP64 once per block
        ci[0] = __reduce_add_sync(0xffffffffu, cb);
        ci[1] = __reduce_add_sync(0xffffffffu, cz);
        ci[2] = __reduce_add_sync(0xffffffffu, cm);
        form = kFormCount;
    } else if (a.model == 0) {
        const uint8_t *sp = a.spins + (size_t)r * N;
        for (int s = b * blockDim.x + threadIdx.x; s < N; s += stride) {
            const uint8_t own = sp[s];
            double e = 0.0;
            for (int k = a.row_ptr[s]; k < a.row_ptr[s + 1]; ++k)
                e += neg_if(a.Jd[3 * a.jidx[k] + 2], sp[a.nbr[k]] != own);  // (s_i s_j) J
            q[1] += e;
            if (a.zeeman) e += neg_if(a.zeed[3 * (a.species[s] - 1) + 2], !own);
            q[0] += e;
            q[4] += neg_if(a.mweight[s], !own);
        }
    } else {
        const float4 *sp = a.spins4 + (size_t)r * N;
        DS e0, e1, m0, m1, m2;
        const bool mwf = a.mweight_f != nullptr;
        // no Zeeman or anisotropy term: e0 would add the same values as e1
        const bool fields = a.zeeman || a.sia || a.sia_cls;
        const int H = a.sc_L1 >> 1, half = N >> 1;
        for (int s = b * blockDim.x + threadIdx.x; s < N; s += stride) {
            const float4 S = sp[s];
            float hx = 0.f, hy = 0.f, hz = 0.f;
            if (a.sc_xyz) {
                // simple cubic: storage index s = colour * half + rank; the six neighbours in
                // closed form from the other colour's array, summed in the CSR's order
                const int colour = s >= half ? 1 : 0, rho = s - colour * half;
                const int row = (int)fdiv((uint32_t)rho, a.sc_fH);
                const int xh = rho - row * H;
                const int z = (int)fdiv((uint32_t)row, a.sc_fL2), y = row - z * a.sc_L2;
                const int p = (y + z + colour) & 1;
                const Acc3 h = sc_field(sp + (size_t)(colour ^ 1) * half, a.sc_L1, a.sc_L2, a.sc_L3, H, xh, y, z, p,
                                        a.sc_jx, a.sc_jy, a.sc_jz);
                hx = h.x;
                hy = h.y;
                hz = h.z;
            } else {
                for (int k = a.row_ptr[s]; k < a.row_ptr[s + 1]; ++k) {
                    float4 Sj = sp[a.nbr[k]];
                    const float *Jp = a.J + 3 * a.jidx[k];
                    hx = fmaf(Jp[0], Sj.x, hx);
                    hy = fmaf(Jp[1], Sj.y, hy);
                    hz = fmaf(Jp[2], Sj.z, hz);
                }
            }
            float e = S.x * hx;
            e = fmaf(S.y, hy, e);
            e = fmaf(S.z, hz, e);
            ds_add(e1, e);
            if (fields) {
                if (a.zeeman || a.sia) {
                    const int si = a.species[s] - 1;
                    if (a.zeeman) {
                        const float *z = a.zee + 3 * si;
                        e = fmaf(S.x, z[0], e);
                        e = fmaf(S.y, z[1], e);
                        e = fmaf(S.z, z[2], e);
                    }
                    if (a.sia) {
                        const float *d = a.D + 3 * si;
                        e = fmaf(d[0], S.x * S.x, e);
                        e = fmaf(d[1], S.y * S.y, e);
                        e = fmaf(d[2], S.z * S.z, e);
                    }
                }
                if (a.sia_cls) {  // local-axis anisotropy D (a . S)^2
                    const float4 ax = a.sia_ax[a.sia_cls[s]];
                    float ps = ax.x * S.x;
                    ps = fmaf(ax.y, S.y, ps);
                    ps = fmaf(ax.z, S.z, ps);
                    e = fmaf(ax.w, ps * ps, e);
                }
                ds_add(e0, e);
            }
            if (mwf) {
                const float wf = a.mw_pos ? a.mw_abs_f : a.mweight_f[s];  // mw_pos: all weights +mw_abs
                ds_add_prod(m0, wf, S.x);
                ds_add_prod(m1, wf, S.y);
                ds_add_prod(m2, wf, S.z);
            } else {
                const double w = a.mweight[s];
                q[2] += w * (double)S.x;
                q[3] += w * (double)S.y;
                q[4] += w * (double)S.z;
            }
        }
        // double-single sums over the warp and the block, FP64 once per block
        qd[1] = warp_sum_ds(e1);
        qd[0] = fields ? warp_sum_ds(e0) : qd[1];
        if (mwf) {
            qd[2] = warp_sum_ds(m0);
            qd[3] = warp_sum_ds(m1);
            qd[4] = warp_sum_ds(m2);
        }
        form = mwf ? kFormDS : kFormDSEnergy;
    }
    double *out = a.partials + ((size_t)r * a.nblk + b) * kNq;
    if (form == kFormCount) {
        int t[3];
        block_sum_ints(ci, t);
        if (threadIdx.x == 0) {
            const double e_ex = a.juni * (double)t[0];
            out[0] = a.zeeman ? e_ex + a.zeed[2] * (double)t[1] : e_ex;
            out[1] = e_ex;
            out[2] = 0.0;
            out[3] = 0.0;
            out[4] = a.mw_abs * (double)t[2];
        }
    } else {
        block_sum_mixed<kNq>(q, qd, form == kFormDS ? kNq : form == kFormDSEnergy ? 2 : 0, out);
    }
}

__global__ void __launch_bounds__(kRedBs) energy_mag_kernel(const ObsMember a) {
    energy_block(a, blockIdx.y, blockIdx.x);
}

// Replica r: sums the partials in index order (a block of 128 threads).
__device__ __forceinline__ void finish_block(const double *__restrict__ partials, int nblk, int R, int r,
                                             double *__restrict__ E, double *__restrict__ M) {
    __shared__ double sm[kNq][128];
    for (int j = 0; j < kNq; ++j) {
        double v = 0.0;
        for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += partials[((size_t)r * nblk + b) * kNq + j];
        sm[j][threadIdx.x] = v;
    }
    __syncthreads();
    for (int w = 64; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int j = 0; j < kNq; ++j) sm[j][threadIdx.x] += sm[j][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        E[r] = sm[0][0];
        E[R + r] = sm[1][0];
        M[3 * r + 0] = sm[2][0];
        M[3 * r + 1] = sm[3][0];
        M[3 * r + 2] = sm[4][0];
    }
}

// One block per replica.
__global__ void finish_energy_kernel(const double *__restrict__ partials, int nblk, int R,
                                     double *__restrict__ E, double *__restrict__ M) {
    finish_block(partials, nblk, R, blockIdx.x, E, M);
}

// get_eng('eng') / get_mag('mag') of replica r, into its (group, slot) accumulator.
__device__ __forceinline__ void measure_one(const double *__restrict__ E, const double *__restrict__ M,
                                            int N, int n_slots, const int32_t *__restrict__ slot_of_rep,
                                            double *__restrict__ sums, int r) {
    const int idx = (r / n_slots) * n_slots + slot_of_rep[r];
    const double e = E[r] / (2.0 * N);
    const double mx = M[3 * r], my = M[3 * r + 1], mz = M[3 * r + 2];
    const double m = sqrt(mx * mx + my * my + mz * mz) / N;
    double *a = sums + (size_t)idx * 7;
    a[0] += 1.0;
    a[1] += e;
    a[2] += e * e;
    a[3] += (e * e) * (e * e);
    a[4] += m;
    a[5] += m * m;
    a[6] += (m * m) * (m * m);
}

__global__ void measure_kernel(const double *__restrict__ E, const double *__restrict__ M, int N,
                               int R, int n_slots, const int32_t *__restrict__ slot_of_rep,
                               double *__restrict__ sums) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < R) measure_one(E, M, N, n_slots, slot_of_rep, sums, r);
}

// parallel_tempering: pair tid = (group, pair) of one ladder set.  Exponent in FP64.
__device__ __forceinline__ void pt_pair(const double *__restrict__ E, int R, int n_slots, int n_groups,
                                        const double *__restrict__ beta_slot, int32_t *__restrict__ rep_of_slot,
                                        int32_t *__restrict__ slot_of_rep, int32_t *__restrict__ copy_from,
                                        const int32_t *__restrict__ swap_ptr, uint32_t seed, int true_energy,
                                        int copy_mode, int32_t *__restrict__ n_acc, int tid) {
    const int swap_count = *swap_ptr;
    const int npairs = n_slots / 2 + 1;
    if (tid >= npairs * n_groups) return;
    const int g = tid / npairs, q = tid - g * npairs;
    const int s = ((swap_count & 1) ? 1 : 0) + 2 * q;
    if (s + 1 >= n_slots) return;
    int32_t *ros = rep_of_slot + (size_t)g * n_slots;
    const int lo = ros[s], hi = ros[s + 1];
    double elo = E[lo], ehi = E[hi];
    if (true_energy) {  // bonds once: E = E_ex/2 + (E_raw - E_ex)
        elo = 0.5 * E[R + lo] + (E[lo] - E[R + lo]);
        ehi = 0.5 * E[R + hi] + (E[hi] - E[R + hi]);
    }
    const double delta = -(beta_slot[s + 1] - beta_slot[s]) * (elo - ehi);
    bool acc;
    if (delta > 0.0) acc = true;
    else {
        U4 o = draw((uint32_t)s, (uint32_t)swap_count, 0x50540000u + (uint32_t)g, kPT, seed);
        acc = ((double)o.x * 0x1p-32) < exp(delta);
    }
    if (!acc) return;
    atomicAdd(n_acc, 1);
    if (copy_mode) {
        copy_from[hi] = lo;
    } else {
        ros[s] = hi;
        ros[s + 1] = lo;
        slot_of_rep[lo] = s + 1;
        slot_of_rep[hi] = s;
    }
}

// One thread per (group, pair).
__global__ void pt_kernel(const double *__restrict__ E, int R, int n_slots, int n_groups,
                          const double *__restrict__ beta_slot, int32_t *__restrict__ rep_of_slot,
                          int32_t *__restrict__ slot_of_rep, int32_t *__restrict__ copy_from,
                          const int32_t *__restrict__ swap_ptr, uint32_t seed, int true_energy, int copy_mode,
                          int32_t *__restrict__ n_acc) {
    pt_pair(E, R, n_slots, n_groups, beta_slot, rep_of_slot, slot_of_rep, copy_from, swap_ptr, seed,
            true_energy, copy_mode, n_acc, blockIdx.x * blockDim.x + threadIdx.x);
}

// Reference-copy PT mode: replica r takes the configuration of replica copy_from[r].
__global__ void pt_copy_kernel(uint8_t *__restrict__ spins, float4 *__restrict__ spins4, int N,
                               int model, const int32_t *__restrict__ copy_from) {
    const int r = blockIdx.y;
    const int src = copy_from[r];
    if (src < 0) return;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += gridDim.x * blockDim.x) {
        if (model == 0) spins[(size_t)r * N + s] = spins[(size_t)src * N + s];
        else spins4[(size_t)r * N + s] = spins4[(size_t)src * N + s];
    }
}

// Blocks per replica of the reductions: no more than four blocks per SM over all replicas
// (the context's own launch fills the GPU once, each thread running through many sites), and
// at least eight sites per thread, so that the per-warp and per-block sums stay a small part
// of a thread's work also for the many small contexts of a batch.  The same number serves the
// context's own launches and the batched ones, so the two sum in the same order.
int energy_blocks(const Ctx &c) {
    long need = (c.N + kRedBs * 8 - 1) / (kRedBs * 8);
    long cap = (long)c.sm_count * 4 / (c.R > 0 ? c.R : 1);
    if (cap < 1) cap = 1;
    if (need > cap) need = cap;
    if (need > 4096) need = 4096;
    return (int)(need < 1 ? 1 : need);
}

ObsMember obs_member(const Ctx &c) {
    ObsMember a{};
    a.spins = c.spins;
    a.spins4 = c.spins4;
    a.N = c.N;
    a.model = c.model;
    a.zeeman = c.zeeman;
    a.sia = c.sia && c.model == 1;
    a.row_ptr = c.t.row_ptr;
    a.nbr = c.t.nbr;
    a.jidx = c.t.jidx;
    a.J = c.t.J;
    a.Jd = c.t.Jd;
    a.species = c.t.species;
    a.zee = c.t.zee;
    a.zeed = c.t.zeed;
    a.D = c.t.D;
    a.sia_cls = c.sia_local && c.model == 1 ? c.t.sia_cls : nullptr;
    a.sia_ax = c.t.sia_ax;
    a.mweight = c.t.mweight;
    a.mweight_f = c.t.mweight_f;
    a.juni = c.ising_juni;
    a.mw_abs = c.mw_abs;
    a.nsp = c.nsp;
    a.count_form = (c.model == 0 && c.juni_set && c.mw_abs > 0.0 && (!c.zeeman || c.nsp == 1)) ? 1 : 0;
    a.sc_xyz = (c.fast && c.model == 1) ? 1 : 0;
    a.sc_ising = (c.fast && c.model == 0 && a.count_form) ? 1 : 0;
    a.mw_pos = (c.mw_pos && c.mw_abs > 0.0) ? 1 : 0;
    a.sc_pad2 = a.sc_pad3 = 0;
    a.sc_L1 = c.L[0];
    a.sc_L2 = c.L[1];
    a.sc_L3 = c.L[2];
    a.sc_fH = make_fastdiv((uint32_t)std::max(1, c.L[0] / 2));
    a.sc_fL2 = make_fastdiv((uint32_t)std::max(1, c.L[1]));
    a.sc_jx = a.sc_xyz ? c.h_Jf[0] : 0.f;
    a.sc_jy = a.sc_xyz ? c.h_Jf[1] : 0.f;
    a.sc_jz = a.sc_xyz ? c.h_Jf[2] : 0.f;
    a.mw_abs_f = (float)c.mw_abs;
    a.partials = c.partials;
    a.nblk = c.partial_blocks;
    a.R = c.R;
    a.E = c.E;
    a.M = c.M;
    a.sums = c.sums;
    a.n_slots = c.n_slots;
    a.n_groups = c.n_groups;
    a.beta_slot = c.beta_slot;
    a.rep_of_slot = c.rep_of_slot;
    a.slot_of_rep = c.slot_of_rep;
    a.copy_from = c.copy_from;
    a.swap_dev = c.swap_dev;
    a.pt_accepts = c.pt_accepts;
    a.seed = c.seed;
    a.true_energy = (c.flags & ETHER_FLAG_PT_TRUE_ENERGY) ? 1 : 0;
    a.acc_count = c.acc_count;
    a.acc_mark = c.acc_mark;
    a.acc_slot = c.acc_slot;
    return a;
}

cudaError_t launch_energy_mag(Ctx &c, bool) {
    const int nblk = c.partial_blocks;
    dim3 grid(nblk, c.R);
    energy_mag_kernel<<<grid, kRedBs, 0, c.stream>>>(obs_member(c));
    finish_energy_kernel<<<c.R, 128, 0, c.stream>>>(c.partials, nblk, c.R, c.E, c.M);
    c.launches += 2;
    return cudaGetLastError();
}

// Magnetisation only (src/get_tot_magnetisation.f90:32-40), no neighbour reads: per-block
// partial sums of w_s S_s into partials[(r*nblk + b)*kNq + 2..4], summed per thread and
// warp as energy_block sums them (so the two give the same M).
__global__ void __launch_bounds__(kRedBs) mag_kernel(const ObsMember a) {
    const int r = blockIdx.y;
    const int N = a.N;
    const int stride = gridDim.x * blockDim.x;
    double q[3] = {0, 0, 0};
    DS qd[3];
    int form = kFormDouble;
    double *out = a.partials + ((size_t)r * gridDim.x + blockIdx.x) * kNq + 2;
    if (a.model == 0 && a.count_form) {
        const uint8_t *sp = a.spins + (size_t)r * N;
        int cm = 0;
        if (a.mw_pos && gridDim.x == 1 && (N & 15) == 0 && (reinterpret_cast<uintptr_t>(sp) & 15) == 0) {
            // every weight +|w| and one block per replica: M / |w| = 2 (up spins) - N, counted
            // 16 bytes (0 or 1 each) at a time -- the same integer as the per-site loop
            const uint4 *v = reinterpret_cast<const uint4 *>(sp);
            int ones = 0, sites = 0;
            for (int k = threadIdx.x; k < (N >> 4); k += blockDim.x) {
                const uint4 q = v[k];
                ones = __dp4a((int)q.x, 0x01010101, ones);
                ones = __dp4a((int)q.y, 0x01010101, ones);
                ones = __dp4a((int)q.z, 0x01010101, ones);
                ones = __dp4a((int)q.w, 0x01010101, ones);
                sites += 16;
            }
            cm = 2 * ones - sites;
        } else {
            for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += stride) {
                const bool wneg = a.mw_pos ? false : __double_as_longlong(a.mweight[s]) < 0;
                cm += ((sp[s] != 0) != wneg) ? 1 : -1;
            }
        }
        const int ci[3] = {0, 0, __reduce_add_sync(0xffffffffu, cm)};
        int t[3];
        block_sum_ints(ci, t);
        if (threadIdx.x == 0) {
            out[0] = 0.0;
            out[1] = 0.0;
            out[2] = a.mw_abs * (double)t[2];
        }
        return;
    } else if (a.model == 0) {
        const uint8_t *sp = a.spins + (size_t)r * N;
        for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += stride)
            q[2] += neg_if(a.mweight[s], !sp[s]);
    } else if (a.mweight_f) {
        const float4 *sp = a.spins4 + (size_t)r * N;
        DS m0, m1, m2;
        for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += stride) {
            const float4 S = sp[s];
            const float wf = a.mw_pos ? a.mw_abs_f : a.mweight_f[s];
            ds_add_prod(m0, wf, S.x);
            ds_add_prod(m1, wf, S.y);
            ds_add_prod(m2, wf, S.z);
        }
        qd[0] = warp_sum_ds(m0);
        qd[1] = warp_sum_ds(m1);
        qd[2] = warp_sum_ds(m2);
        form = kFormDS;
    } else {
        const float4 *sp = a.spins4 + (size_t)r * N;
        for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += stride) {
            const double w = a.mweight[s];
            const float4 S = sp[s];
            q[0] += w * (double)S.x;
            q[1] += w * (double)S.y;
            q[2] += w * (double)S.z;
        }
    }
    block_sum_mixed<3>(q, qd, form == kFormDS ? 3 : 0, out);
}

// One row t of the time series: |M| (and E) of every replica.  from_partials: M is summed
// here from mag_kernel's partials (in block order); otherwise M and E come from the last
// energy / magnetisation reduction.
__global__ void record_kernel(const double *__restrict__ partials, int nblk, int R,
                              int from_partials, double *__restrict__ M,
                              const double *__restrict__ E, double *__restrict__ mser,
                              double *__restrict__ eser, int t_arg, const int32_t *__restrict__ t_dev) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const int t = t_dev ? *t_dev : t_arg;  // t_dev: the row from device memory (graph replays)
    double m[3];
    if (from_partials) {
        m[0] = m[1] = m[2] = 0.0;
        for (int b = 0; b < nblk; ++b)
            for (int j = 0; j < 3; ++j) m[j] += partials[((size_t)r * nblk + b) * kNq + 2 + j];
        for (int j = 0; j < 3; ++j) M[3 * r + j] = m[j];
    } else {
        for (int j = 0; j < 3; ++j) m[j] = M[3 * r + j];
    }
    mser[(size_t)t * R + r] = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
    if (eser) eser[(size_t)t * R + r] = E[r];
}

// The next row of a series whose row index lives in device memory.
__global__ void record_bump_kernel(int32_t *__restrict__ t_dev) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *t_dev += 1;
}

cudaError_t launch_record(Ctx &c, int t, bool want_e, double *mser, double *eser, int32_t *t_dev) {
    if (want_e) {
        cudaError_t e = launch_energy_mag(c, true);
        if (e != cudaSuccess) return e;
        record_kernel<<<(c.R + 127) / 128, 128, 0, c.stream>>>(c.partials, c.partial_blocks, c.R, 0,
                                                                c.M, c.E, mser, eser, t, t_dev);
        c.launches++;
    } else {
        dim3 grid(c.partial_blocks, c.R);
        mag_kernel<<<grid, kRedBs, 0, c.stream>>>(obs_member(c));
        record_kernel<<<(c.R + 127) / 128, 128, 0, c.stream>>>(c.partials, c.partial_blocks, c.R, 1,
                                                                c.M, c.E, mser, nullptr, t, t_dev);
        c.launches += 2;
    }
    if (t_dev) {
        record_bump_kernel<<<1, 32, 0, c.stream>>>(t_dev);
        c.launches++;
    }
    return cudaGetLastError();
}

cudaError_t launch_measure(Ctx &c) {
    measure_kernel<<<(c.R + 127) / 128, 128, 0, c.stream>>>(c.E, c.M, c.N, c.R, c.n_slots,
                                                            c.slot_of_rep, c.sums);
    c.launches++;
    return cudaGetLastError();
}

// PT swap counter, kept on the device so that captured graphs replay correctly.
__device__ __forceinline__ void pt_bump(int32_t *__restrict__ swap, int32_t *__restrict__ n_acc, int set,
                                        int32_t value) {
    *swap = set ? value : *swap + 1;
    *n_acc = 0;
}

__global__ void pt_bump_kernel(int32_t *__restrict__ swap, int32_t *__restrict__ n_acc, int set,
                               int32_t value) {
    if (threadIdx.x == 0 && blockIdx.x == 0) pt_bump(swap, n_acc, set, value);
}

// Accepts since the last binning go to the (group, slot) position each replica holds now;
// positions are a permutation of the replicas within a group, so no two threads collide.
__device__ __forceinline__ void acc_bin_one(const unsigned long long *__restrict__ acc_count,
                                            unsigned long long *__restrict__ acc_mark,
                                            const int32_t *__restrict__ slot_of_rep, int n_slots,
                                            unsigned long long *__restrict__ acc_slot, int r) {
    const unsigned long long now = acc_count[r];
    const int pos = (r / n_slots) * n_slots + slot_of_rep[r];
    acc_slot[pos] += now - acc_mark[r];
    acc_mark[r] = now;
}

__global__ void acc_bin_kernel(const unsigned long long *__restrict__ acc_count,
                               unsigned long long *__restrict__ acc_mark,
                               const int32_t *__restrict__ slot_of_rep, int n_slots, int R,
                               unsigned long long *__restrict__ acc_slot) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < R) acc_bin_one(acc_count, acc_mark, slot_of_rep, n_slots, acc_slot, r);
}

cudaError_t launch_acc_bin(Ctx &c) {
    acc_bin_kernel<<<(c.R + 127) / 128, 128, 0, c.stream>>>(c.acc_count, c.acc_mark, c.slot_of_rep,
                                                            c.n_slots, c.R, c.acc_slot);
    c.launches++;
    return cudaGetLastError();
}

// set >= 0: use swap_count = set (ether_parallel_tempering); set < 0: increment the device
// counter first (the loop of src/ether.f90:190-192 inside ether_mcs).
cudaError_t launch_pt(Ctx &c, int set_swap_count) {
    const int copy_mode = (c.flags & ETHER_FLAG_PT_REFERENCE_COPY) ? 1 : 0;
    const int npairs = c.n_slots / 2 + 1;
    const int nt = npairs * c.n_groups;
    {
        cudaError_t e = launch_acc_bin(c);  // accepts so far belong to the slots held before the swap
        if (e != cudaSuccess) return e;
    }
    pt_bump_kernel<<<1, 32, 0, c.stream>>>(c.swap_dev, c.pt_accepts, set_swap_count >= 0 ? 1 : 0,
                                           set_swap_count);
    c.launches++;
    if (copy_mode) cudaMemsetAsync(c.copy_from, 0xFF, sizeof(int32_t) * c.R, c.stream);
    pt_kernel<<<(nt + 127) / 128, 128, 0, c.stream>>>(
        c.E, c.R, c.n_slots, c.n_groups, c.beta_slot, c.rep_of_slot, c.slot_of_rep, c.copy_from,
        c.swap_dev, c.seed, (c.flags & ETHER_FLAG_PT_TRUE_ENERGY) ? 1 : 0, copy_mode,
        c.pt_accepts);
    c.launches++;
    if (copy_mode) {
        dim3 grid(energy_blocks(c), c.R);
        pt_copy_kernel<<<grid, 256, 0, c.stream>>>(c.spins, c.spins4, c.N, c.model, c.copy_from);
        c.launches++;
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------- batched forms ----
// The same bodies over a table of members: item idx belongs to member m with
// off[m] <= idx < off[m + 1] (members with no items are skipped).
__device__ __forceinline__ int member_of(const int32_t *__restrict__ off, int M, int idx) {
    int lo = 0, hi = M;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= idx) lo = mid;
        else hi = mid;
    }
    return lo;
}

// One block per (member, replica, energy block); capped at four resident blocks per SM (the
// kernel waits on neighbour gathers, so more warps hide more of it).
__global__ void __launch_bounds__(kRedBs, 4)
batch_energy_kernel(const ObsMember *__restrict__ mem, const int32_t *__restrict__ eoff, int M) {
    // the member's record in shared memory: its fields are read in every site's iteration
    __shared__ ObsMember a;
    const int m = member_of(eoff, M, blockIdx.x);
    {
        static_assert(sizeof(ObsMember) % 8 == 0, "ObsMember is copied in 8-byte words");
        const unsigned long long *src = reinterpret_cast<const unsigned long long *>(mem + m);
        unsigned long long *dst = reinterpret_cast<unsigned long long *>(&a);
        for (int k = threadIdx.x; k < (int)(sizeof(ObsMember) / 8); k += blockDim.x) dst[k] = src[k];
    }
    __syncthreads();
    const int local = blockIdx.x - eoff[m];
    energy_block(a, local / a.nblk, local % a.nblk);
}

// One block of 128 per (member, replica).
__global__ void batch_finish_kernel(const ObsMember *__restrict__ mem, const int32_t *__restrict__ roff, int M) {
    const int m = member_of(roff, M, blockIdx.x);
    const ObsMember &a = mem[m];
    finish_block(a.partials, a.nblk, a.R, blockIdx.x - roff[m], a.E, a.M);
}

// One thread per (member, replica): what = 0 acceptance binning, 1 measurement.
__global__ void batch_replica_kernel(const ObsMember *__restrict__ mem, const int32_t *__restrict__ roff,
                                     int M, int total, int what) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int m = member_of(roff, M, idx);
    const ObsMember &a = mem[m];
    const int r = idx - roff[m];
    if (what == 0) acc_bin_one(a.acc_count, a.acc_mark, a.slot_of_rep, a.n_slots, a.acc_slot, r);
    else measure_one(a.E, a.M, a.N, a.n_slots, a.slot_of_rep, a.sums, r);
}

// One thread per member.
__global__ void batch_pt_bump_kernel(const ObsMember *__restrict__ mem, int M) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < M) pt_bump(mem[m].swap_dev, mem[m].pt_accepts, 0, 0);
}

// One thread per (member, group, pair).
__global__ void batch_pt_kernel(const ObsMember *__restrict__ mem, const int32_t *__restrict__ poff, int M,
                                int total) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int m = member_of(poff, M, idx);
    const ObsMember &a = mem[m];
    pt_pair(a.E, a.R, a.n_slots, a.n_groups, a.beta_slot, a.rep_of_slot, a.slot_of_rep, a.copy_from,
            a.swap_dev, a.seed, a.true_energy, 0, a.pt_accepts, idx - poff[m]);
}

cudaError_t launch_batch_energy(const ObsTable &t, cudaStream_t st) {
    if (t.M == 0) return cudaSuccess;
    batch_energy_kernel<<<t.eblocks, kRedBs, 0, st>>>(t.mem, t.eoff, t.M);
    batch_finish_kernel<<<t.rtotal, 128, 0, st>>>(t.mem, t.roff, t.M);
    return cudaGetLastError();
}

cudaError_t launch_batch_pt(const ObsTable &t, cudaStream_t st) {
    if (t.M == 0) return cudaSuccess;
    // accepts so far belong to the slots held before the swap
    batch_replica_kernel<<<(t.rtotal + 127) / 128, 128, 0, st>>>(t.mem, t.roff, t.M, t.rtotal, 0);
    batch_pt_bump_kernel<<<(t.M + 127) / 128, 128, 0, st>>>(t.mem, t.M);
    if (t.ptotal > 0) batch_pt_kernel<<<(t.ptotal + 127) / 128, 128, 0, st>>>(t.mem, t.poff, t.M, t.ptotal);
    return cudaGetLastError();
}

cudaError_t launch_batch_measure(const ObsTable &t, cudaStream_t st) {
    if (t.M == 0) return cudaSuccess;
    batch_replica_kernel<<<(t.rtotal + 127) / 128, 128, 0, st>>>(t.mem, t.roff, t.M, t.rtotal, 1);
    return cudaGetLastError();
}

}  // namespace ether
