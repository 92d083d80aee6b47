// k_moments.cu -- per-species moment vectors (src/get_moment_vectors.f90:20-38) and the
// spiral-state observable (src/get_spiral_state.f90:45-108) on the GPU.
//
//   mm(sp) = sum over sites of species sp of stgg_i s(sp) S_i           (per replica)
//   ss     = | sum_i sum_{j in ifs(i)} S_i x S_j | / spiral_count        (per replica)
//
// ifs(i) (the reference's 'ions_for_spiral') is built once on the host from the site
// positions with the reference's tests -- |r_j - r_i| <= ss_dis and the angle between
// r_j - r_i and ss_direc at most ss_latency degrees, no periodic images -- and kept as CSR in
// storage order.  Both reductions use fixed-order block partials (FP64 accumulation of the
// FP32 / int8 spins), summed per replica in block order.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "internal.h"

namespace ether {
namespace {

constexpr int kBs = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block partial of three sums into out[(r * gridDim.x + blockIdx.x) * 3 + 0..2]
__device__ __forceinline__ void block_store3(const double q[3], double *out, int r) {
    __shared__ double sm[kBs / 32][3];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const double v = warp_sum(q[j]);
        if (lane == 0) sm[wid][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0.0;
        for (int w = 0; w < kBs / 32; ++w) v += sm[w][threadIdx.x];
        out[((size_t)r * gridDim.x + blockIdx.x) * 3 + threadIdx.x] = v;
    }
}

__global__ void __launch_bounds__(kBs)
moment_kernel(const uint8_t *__restrict__ spins, const float4 *__restrict__ spins4, int N, int model,
              const double *__restrict__ mweight, const uint8_t *__restrict__ species, int sp,
              double *__restrict__ part) {
    const int r = blockIdx.y;
    double q[3] = {0, 0, 0};
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += gridDim.x * blockDim.x) {
        if (species[s] != sp) continue;
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
    block_store3(q, part, r);
}

__global__ void __launch_bounds__(kBs)
spiral_kernel(const float4 *__restrict__ spins4, int N, const int32_t *__restrict__ ptr,
              const int32_t *__restrict__ nbr, double *__restrict__ part) {
    const int r = blockIdx.y;
    const float4 *sp = spins4 + (size_t)r * N;
    double q[3] = {0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const float4 a = sp[i];
        for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
            const float4 b = sp[nbr[k]];
            q[0] += (double)a.y * b.z - (double)a.z * b.y;
            q[1] += (double)a.z * b.x - (double)a.x * b.z;
            q[2] += (double)a.x * b.y - (double)a.y * b.x;
        }
    }
    block_store3(q, part, r);
}

// out[r * stride + off + 0..2] = sum of the replica's block partials, in block order
__global__ void finish3_kernel(const double *__restrict__ part, int nblk, int R, double *__restrict__ out,
                               int stride, int off) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    double m[3] = {0, 0, 0};
    for (int b = 0; b < nblk; ++b)
        for (int j = 0; j < 3; ++j) m[j] += part[((size_t)r * nblk + b) * 3 + j];
    for (int j = 0; j < 3; ++j) out[(size_t)r * stride + off + j] = m[j];
}

// src/get_spiral_state.f90:118-123 at one measurement step: x = |sum| / spiral_count,
// accumulated at the (group, slot) position of each replica.
__global__ void spiral_measure_kernel(const double *__restrict__ part, int nblk, int R, int n_slots,
                                      const int32_t *__restrict__ slot_of_rep, double inv_count,
                                      double *__restrict__ sums) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    double m[3] = {0, 0, 0};
    for (int b = 0; b < nblk; ++b)
        for (int j = 0; j < 3; ++j) m[j] += part[((size_t)r * nblk + b) * 3 + j];
    const double x = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]) * inv_count;
    double *a = sums + 4 * ((size_t)(r / n_slots) * n_slots + slot_of_rep[r]);
    a[0] += 1.0;
    a[1] += x;
    a[2] += x * x;
    a[3] += (x * x) * (x * x);
}

int nblocks(const Ctx &c) {
    long need = (c.N + kBs - 1) / kBs;
    long cap = (long)c.sm_count * 4 / (c.R > 0 ? c.R : 1);
    return (int)std::max<long>(1, std::min(need, std::max<long>(cap, 1)));
}

}  // namespace

cudaError_t launch_spiral_measure(Ctx &c) {
    spiral_kernel<<<dim3(c.spiral_blocks, c.R), kBs, 0, c.stream>>>(c.spins4, c.N, c.spiral_ptr, c.spiral_nbr,
                                                                   c.spiral_part);
    spiral_measure_kernel<<<(c.R + 127) / 128, 128, 0, c.stream>>>(
        c.spiral_part, c.spiral_blocks, c.R, c.n_slots, c.slot_of_rep, 1.0 / (double)c.spiral_count, c.spiral_sums);
    c.launches += 2;
    return cudaGetLastError();
}

}  // namespace ether

using namespace ether;

namespace {
int mfail(int code, const std::string &msg) {
    set_error(msg);
    return code;
}
#define MCUDA(expr)                                                                          \
    do {                                                                                     \
        cudaError_t _e = (expr);                                                             \
        if (_e != cudaSuccess)                                                               \
            return mfail(_e == cudaErrorMemoryAllocation ? ETHER_ERR_NOMEM : ETHER_ERR_CUDA,  \
                         std::string(#expr) + ": " + cudaGetErrorString(_e));                \
    } while (0)
}  // namespace

extern "C" int ether_moment_vectors(ether_ctx *h, double *mm) {
    if (!h || !mm) return mfail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    const int nblk = nblocks(c);
    double *part = nullptr, *out = nullptr;
    const size_t out_n = (size_t)c.R * c.nsp * 3;
    MCUDA(cudaMallocAsync((void **)&part, (size_t)c.R * nblk * 3 * sizeof(double), c.stream));
    cudaError_t e = cudaMallocAsync((void **)&out, out_n * sizeof(double), c.stream);
    for (int sp = 1; e == cudaSuccess && sp <= c.nsp; ++sp) {
        moment_kernel<<<dim3(nblk, c.R), kBs, 0, c.stream>>>(c.spins, c.spins4, c.N, c.model, c.t.mweight,
                                                            c.t.species, sp, part);
        finish3_kernel<<<(c.R + 127) / 128, 128, 0, c.stream>>>(part, nblk, c.R, out, 3 * c.nsp, 3 * (sp - 1));
        c.launches += 2;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(mm, out, out_n * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    cudaFreeAsync(part, c.stream);
    if (out) cudaFreeAsync(out, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return mfail(ETHER_ERR_CUDA, std::string("moment vectors: ") + cudaGetErrorString(e));
    return ETHER_OK;
}

extern "C" int ether_spiral_setup(ether_ctx *h, double ss_dis, const double ss_direc[3], double ss_latency,
                                  int32_t capacity, int64_t *count) {
    if (!h || !ss_direc) return mfail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    if (c.model != ETHER_MODEL_XYZ)
        return mfail(ETHER_ERR_UNSUPPORTED, "the spiral state is an XYZ observable (src/ether.f90:69 skips Ising)");
    if (!(ss_dis > 0.0) || !std::isfinite(ss_dis) || capacity < 1 || capacity > 1024)
        return mfail(ETHER_ERR_ARG, "ss_dis must be positive and capacity in [1, 1024]");
    const int N = c.N;
    // positions in site order (c.pos is in storage order)
    std::vector<double> pos((size_t)3 * N);
    for (int s = 0; s < N; ++s)
        for (int a = 0; a < 3; ++a) pos[3 * (size_t)c.site_of_storage[s] + a] = c.pos[3 * (size_t)s + a];
    // cell list of edge ss_dis over the bounding box
    double lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = 1e300;
        hi[a] = -1e300;
    }
    for (int i = 0; i < N; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], pos[3 * (size_t)i + a]);
            hi[a] = std::max(hi[a], pos[3 * (size_t)i + a]);
        }
    int nc[3];
    for (int a = 0; a < 3; ++a) nc[a] = (int)std::min<double>(std::floor((hi[a] - lo[a]) / ss_dis) + 1.0, 512.0);
    auto cell_of = [&](int i, int a) {
        int k = (int)std::floor((pos[3 * (size_t)i + a] - lo[a]) / ss_dis);
        return std::max(0, std::min(nc[a] - 1, k));
    };
    std::vector<std::vector<int>> cells((size_t)nc[0] * nc[1] * nc[2]);
    for (int i = 0; i < N; ++i)
        cells[((size_t)cell_of(i, 2) * nc[1] + cell_of(i, 1)) * nc[0] + cell_of(i, 0)].push_back(i);
    const double to_angle = 180.0 / 3.14159265358979323846;
    std::vector<std::vector<int>> ifs(N);
    long total = 0;
    std::vector<int> cand;
    for (int i = 0; i < N; ++i) {
        cand.clear();
        const int ci[3] = {cell_of(i, 0), cell_of(i, 1), cell_of(i, 2)};
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int x = ci[0] + dx, y = ci[1] + dy, z = ci[2] + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= nc[0] || y >= nc[1] || z >= nc[2]) continue;
                    for (int j : cells[((size_t)z * nc[1] + y) * nc[0] + x]) cand.push_back(j);
                }
        std::sort(cand.begin(), cand.end());  // the reference's increasing j
        for (int j : cand) {
            if (j == i) continue;
            double r[3];
            for (int a = 0; a < 3; ++a) r[a] = pos[3 * (size_t)j + a] - pos[3 * (size_t)i + a];
            const double dis = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            if (!(dis <= ss_dis)) continue;
            const double u[3] = {r[0] / dis, r[1] / dis, r[2] / dis};
            const double ang = std::acos(u[0] * ss_direc[0] + u[1] * ss_direc[1] + u[2] * ss_direc[2]) * to_angle;
            if (!(ang <= ss_latency)) continue;
            if ((int)ifs[i].size() == capacity)
                return mfail(ETHER_ERR_CAPACITY, "site " + std::to_string(i + 1) + " has more than " +
                                                     std::to_string(capacity) + " spiral partners (spiral_capacity)");
            ifs[i].push_back(j);
            ++total;
        }
    }
    if (total == 0) return mfail(ETHER_ERR_ARG, "no spiral pairs within ss_dis and ss_latency");
    // CSR in storage order
    std::vector<int32_t> ptr(N + 1, 0), nbr;
    nbr.reserve(total);
    for (int s = 0; s < N; ++s) {
        for (int j : ifs[c.site_of_storage[s]]) nbr.push_back(c.storage[j]);
        ptr[s + 1] = (int32_t)nbr.size();
    }
    if (c.spiral_ptr) cudaFree(c.spiral_ptr);
    if (c.spiral_nbr) cudaFree(c.spiral_nbr);
    c.spiral_ptr = c.spiral_nbr = nullptr;
    MCUDA(cudaMalloc((void **)&c.spiral_ptr, ptr.size() * sizeof(int32_t)));
    MCUDA(cudaMalloc((void **)&c.spiral_nbr, std::max<size_t>(1, nbr.size()) * sizeof(int32_t)));
    MCUDA(cudaMemcpy(c.spiral_ptr, ptr.data(), ptr.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    MCUDA(cudaMemcpy(c.spiral_nbr, nbr.data(), nbr.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    c.spiral_count = total;
    // accumulators of the per-sample spiral state (src/get_spiral_state.f90:118-123), read
    // at every measurement step of ether_mcs from now on
    if (c.spiral_part) cudaFree(c.spiral_part);
    if (c.spiral_sums) cudaFree(c.spiral_sums);
    c.spiral_part = c.spiral_sums = nullptr;
    c.spiral_blocks = nblocks(c);
    MCUDA(cudaMalloc((void **)&c.spiral_part, (size_t)c.R * c.spiral_blocks * 3 * sizeof(double)));
    MCUDA(cudaMalloc((void **)&c.spiral_sums, (size_t)c.R * 4 * sizeof(double)));
    MCUDA(cudaMemset(c.spiral_sums, 0, (size_t)c.R * 4 * sizeof(double)));
    // captured MCS chunks hold the old partner tables: capture again
    for (auto &kv : c.graphs) cudaGraphExecDestroy(kv.second);
    c.graphs.clear();
    if (count) *count = total;
    return ETHER_OK;
}

extern "C" int ether_spiral_state(ether_ctx *h, double *ss) {
    if (!h || !ss) return mfail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    if (!c.spiral_ptr) return mfail(ETHER_ERR_STATE, "ether_spiral_setup first");
    const int nblk = nblocks(c);
    double *part = nullptr, *out = nullptr;
    MCUDA(cudaMallocAsync((void **)&part, (size_t)c.R * nblk * 3 * sizeof(double), c.stream));
    cudaError_t e = cudaMallocAsync((void **)&out, (size_t)c.R * 3 * sizeof(double), c.stream);
    if (e == cudaSuccess) {
        spiral_kernel<<<dim3(nblk, c.R), kBs, 0, c.stream>>>(c.spins4, c.N, c.spiral_ptr, c.spiral_nbr, part);
        finish3_kernel<<<(c.R + 127) / 128, 128, 0, c.stream>>>(part, nblk, c.R, out, 3, 0);
        c.launches += 2;
        e = cudaGetLastError();
    }
    std::vector<double> v((size_t)3 * c.R);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v.data(), out, v.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    cudaFreeAsync(part, c.stream);
    if (out) cudaFreeAsync(out, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return mfail(ETHER_ERR_CUDA, std::string("spiral state: ") + cudaGetErrorString(e));
    for (int r = 0; r < c.R; ++r) {
        const double *m = v.data() + 3 * r;
        ss[r] = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]) / (double)c.spiral_count;
    }
    return ETHER_OK;
}

// get_spiral_state 'avg_spiral_state' (src/get_spiral_state.f90:127-140) per (group, slot):
// out(3, R) = <x>, U = 1.5 - 0.5 <x^4> / <x^2>^2, chi = beta (<x^2> - <x>^2) spiral_count.
extern "C" int ether_spiral_avg(ether_ctx *h, double *out) {
    if (!h || !out) return mfail(ETHER_ERR_ARG, "null argument");
    Ctx &c = h->c;
    if (!c.spiral_sums) return mfail(ETHER_ERR_STATE, "ether_spiral_setup first");
    std::vector<double> s((size_t)4 * c.R);
    MCUDA(cudaMemcpyAsync(s.data(), c.spiral_sums, s.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    MCUDA(cudaStreamSynchronize(c.stream));
    for (int g = 0; g < c.n_groups; ++g)
        for (int sl = 0; sl < c.n_slots; ++sl) {
            const size_t idx = (size_t)g * c.n_slots + sl;
            const double *a = s.data() + 4 * idx;
            const double x = a[1] / a[0], x2 = a[2] / a[0], x4 = a[3] / a[0];
            double *o = out + 3 * idx;
            o[0] = x;
            o[1] = 1.5 - 0.5 * (x4 / (x2 * x2));
            o[2] = c.beta_slots[sl] * (x2 - x * x) * (double)c.spiral_count;
        }
    return ETHER_OK;
}
