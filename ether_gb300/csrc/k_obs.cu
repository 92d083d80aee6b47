// k_obs.cu -- energy / magnetisation reductions (src/get_tot_energy.f90:33-47,
// src/get_tot_magnetisation.f90:32-40), the observable accumulators (src/observable.f90,
// src/get_eng.f90:36-40, src/get_mag.f90:36-41) and parallel tempering
// (src/parallel_tempering.f90:39-108).
//
// Site energies are FP32 (XYZ) or exact FP64 sums of ±J (Ising); every per-replica total
// and every accumulator is FP64.  Reductions write per-block partials to scratch memory
// and a second kernel adds them in a fixed order, so results do not depend on timing.
#include "internal.h"
#include "rng_math.cuh"

namespace ether {

constexpr int kRedBs = 256;
constexpr int kNq = 5;  // E_raw, E_exchange, Mx, My, Mz

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kRedBs)
energy_mag_kernel(const uint8_t *__restrict__ spins, const float4 *__restrict__ spins4, int N,
                  int model, int zeeman, int sia, const int32_t *__restrict__ row_ptr,
                  const int32_t *__restrict__ nbr, const uint16_t *__restrict__ jidx,
                  const float *__restrict__ J, const double *__restrict__ Jd,
                  const uint8_t *__restrict__ species, const float *__restrict__ zee,
                  const double *__restrict__ zeed, const float *__restrict__ D,
                  const uint8_t *__restrict__ sia_cls, const float4 *__restrict__ sia_ax,
                  const double *__restrict__ mweight, double *__restrict__ partials) {
    const int r = blockIdx.y;
    double q[kNq] = {0, 0, 0, 0, 0};
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += gridDim.x * blockDim.x) {
        const double w = mweight[s];
        if (model == 0) {
            const uint8_t *sp = spins + (size_t)r * N;
            const double si = sp[s] ? 1.0 : -1.0;
            double e = 0.0;
            for (int k = row_ptr[s]; k < row_ptr[s + 1]; ++k) {
                double sj = sp[nbr[k]] ? 1.0 : -1.0;
                e += (si * sj) * Jd[3 * jidx[k] + 2];
            }
            q[1] += e;
            if (zeeman) e += si * zeed[3 * (species[s] - 1) + 2];
            q[0] += e;
            q[4] += w * si;
        } else {
            const float4 *sp = spins4 + (size_t)r * N;
            const float4 S = sp[s];
            float hx = 0.f, hy = 0.f, hz = 0.f;
            for (int k = row_ptr[s]; k < row_ptr[s + 1]; ++k) {
                float4 Sj = sp[nbr[k]];
                const float *Jp = J + 3 * jidx[k];
                hx = fmaf(Jp[0], Sj.x, hx);
                hy = fmaf(Jp[1], Sj.y, hy);
                hz = fmaf(Jp[2], Sj.z, hz);
            }
            float e = S.x * hx;
            e = fmaf(S.y, hy, e);
            e = fmaf(S.z, hz, e);
            q[1] += (double)e;
            if (zeeman || sia) {
                const int si = species[s] - 1;
                if (zeeman) {
                    const float *z = zee + 3 * si;
                    e = fmaf(S.x, z[0], e);
                    e = fmaf(S.y, z[1], e);
                    e = fmaf(S.z, z[2], e);
                }
                if (sia) {
                    const float *d = D + 3 * si;
                    e = fmaf(d[0], S.x * S.x, e);
                    e = fmaf(d[1], S.y * S.y, e);
                    e = fmaf(d[2], S.z * S.z, e);
                }
            }
            if (sia_cls) {  // local-axis anisotropy D (a . S)^2
                const float4 a = sia_ax[sia_cls[s]];
                float ps = a.x * S.x;
                ps = fmaf(a.y, S.y, ps);
                ps = fmaf(a.z, S.z, ps);
                e = fmaf(a.w, ps * ps, e);
            }
            q[0] += (double)e;
            q[2] += w * (double)S.x;
            q[3] += w * (double)S.y;
            q[4] += w * (double)S.z;
        }
    }
    __shared__ double sm[kRedBs / 32][kNq];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < kNq; ++j) {
        double v = warp_sum_d(q[j]);
        if (lane == 0) sm[wid][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < kNq) {
        double v = 0.0;
        for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) v += sm[w2][threadIdx.x];
        partials[((size_t)r * gridDim.x + blockIdx.x) * kNq + threadIdx.x] = v;
    }
}

// One block per replica: sums the partials in index order.
__global__ void finish_energy_kernel(const double *__restrict__ partials, int nblk, int R,
                                     double *__restrict__ E, double *__restrict__ M) {
    const int r = blockIdx.x;
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

// get_eng('eng') / get_mag('mag') for every replica, into its (group, slot) accumulator.
__global__ void measure_kernel(const double *__restrict__ E, const double *__restrict__ M, int N,
                               int R, int n_slots, const int32_t *__restrict__ slot_of_rep,
                               double *__restrict__ sums) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
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

// parallel_tempering: one thread per (group, pair).  Exponent in FP64.
__global__ void pt_kernel(const double *__restrict__ E, int R, int n_slots, int n_groups,
                          const double *__restrict__ beta_slot, int32_t *__restrict__ rep_of_slot,
                          int32_t *__restrict__ slot_of_rep, int32_t *__restrict__ copy_from,
                          const int32_t *__restrict__ swap_ptr, uint32_t seed, int true_energy, int copy_mode,
                          int32_t *__restrict__ n_acc) {
    const int swap_count = *swap_ptr;
    const int npairs = n_slots / 2 + 1;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
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

int energy_blocks(const Ctx &c) {
    long need = (c.N + kRedBs - 1) / kRedBs;
    long cap = (long)c.sm_count * 4 / (c.R > 0 ? c.R : 1);
    if (cap < 1) cap = 1;
    if (need > cap) need = cap;
    if (need > 4096) need = 4096;
    return (int)(need < 1 ? 1 : need);
}

cudaError_t launch_energy_mag(Ctx &c, bool) {
    const int nblk = c.partial_blocks;
    dim3 grid(nblk, c.R);
    energy_mag_kernel<<<grid, kRedBs, 0, c.stream>>>(
        c.spins, c.spins4, c.N, c.model, c.zeeman, c.sia && c.model == 1, c.t.row_ptr, c.t.nbr,
        c.t.jidx, c.t.J, c.t.Jd, c.t.species, c.t.zee, c.t.zeed, c.t.D,
        c.sia_local && c.model == 1 ? c.t.sia_cls : nullptr, c.t.sia_ax, c.t.mweight, c.partials);
    finish_energy_kernel<<<c.R, 128, 0, c.stream>>>(c.partials, nblk, c.R, c.E, c.M);
    c.launches += 2;
    return cudaGetLastError();
}

// Magnetisation only (src/get_tot_magnetisation.f90:32-40), no neighbour reads: per-block
// partial sums of w_s S_s into partials[(r*nblk + b)*kNq + 2..4].
__global__ void __launch_bounds__(kRedBs)
mag_kernel(const uint8_t *__restrict__ spins, const float4 *__restrict__ spins4, int N, int model,
           const double *__restrict__ mweight, double *__restrict__ partials) {
    const int r = blockIdx.y;
    double q[3] = {0, 0, 0};
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += gridDim.x * blockDim.x) {
        const double w = mweight[s];
        if (model == 0) {
            q[2] += w * (spins[(size_t)r * N + s] ? 1.0 : -1.0);
        } else {
            const float4 S = spins4[(size_t)r * N + s];
            q[0] += w * (double)S.x;
            q[1] += w * (double)S.y;
            q[2] += w * (double)S.z;
        }
    }
    __shared__ double sm[kRedBs / 32][3];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        double v = warp_sum_d(q[j]);
        if (lane == 0) sm[wid][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0.0;
        for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) v += sm[w2][threadIdx.x];
        partials[((size_t)r * gridDim.x + blockIdx.x) * kNq + 2 + threadIdx.x] = v;
    }
}

// One row t of the time series: |M| (and E) of every replica.  from_partials: M is summed
// here from mag_kernel's partials (in block order); otherwise M and E come from the last
// energy / magnetisation reduction.
__global__ void record_kernel(const double *__restrict__ partials, int nblk, int R,
                              int from_partials, double *__restrict__ M,
                              const double *__restrict__ E, double *__restrict__ mser,
                              double *__restrict__ eser, int t) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
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

cudaError_t launch_record(Ctx &c, int t, bool want_e, double *mser, double *eser) {
    if (want_e) {
        cudaError_t e = launch_energy_mag(c, true);
        if (e != cudaSuccess) return e;
        record_kernel<<<(c.R + 127) / 128, 128, 0, c.stream>>>(c.partials, c.partial_blocks, c.R, 0,
                                                                c.M, c.E, mser, eser, t);
        c.launches++;
    } else {
        dim3 grid(c.partial_blocks, c.R);
        mag_kernel<<<grid, kRedBs, 0, c.stream>>>(c.spins, c.spins4, c.N, c.model, c.t.mweight,
                                                  c.partials);
        record_kernel<<<(c.R + 127) / 128, 128, 0, c.stream>>>(c.partials, c.partial_blocks, c.R, 1,
                                                                c.M, c.E, mser, nullptr, t);
        c.launches += 2;
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
__global__ void pt_bump_kernel(int32_t *__restrict__ swap, int32_t *__restrict__ n_acc, int set,
                               int32_t value) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        *swap = set ? value : *swap + 1;
        *n_acc = 0;
    }
}

// Accepts since the last binning go to the (group, slot) position each replica holds now;
// positions are a permutation of the replicas within a group, so no two threads collide.
__global__ void acc_bin_kernel(const unsigned long long *__restrict__ acc_count,
                               unsigned long long *__restrict__ acc_mark,
                               const int32_t *__restrict__ slot_of_rep, int n_slots, int R,
                               unsigned long long *__restrict__ acc_slot) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const unsigned long long now = acc_count[r];
    const int pos = (r / n_slots) * n_slots + slot_of_rep[r];
    acc_slot[pos] += now - acc_mark[r];
    acc_mark[r] = now;
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

}  // namespace ether
