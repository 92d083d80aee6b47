// k_ion.cu -- the reference's per-replica ion(0:8, N) records read and written by the GPU in
// place, for ether_set_spins_batch / ether_get_spins_batch on a device that addresses the
// host's pageable memory through the host's own page tables (a Grace CPU's memory seen over
// NVLink-C2C).  The records never pass through the host's cores or a staging copy: a thread
// per (site, replica) takes ion(3) (Ising) or ion(1:3), ion(5) (XYZ) of its record and writes
// the spin at its storage index, or the other way round.  Only those fields are written; the
// conversions are the host path's (ion(3) > 0 for an Ising spin, round to nearest FP32 for
// an XYZ component, FP32 -> FP64 exactly on the way back).
//
// Blocks walk sites in the records' order, so the host lines are read or written once and in
// sequence; the device side is scattered over the colour classes' storage ranges, which stay
// in whole sectors per warp (two colour segments per warp on a simple-cubic lattice).
#include <algorithm>

#include "internal.h"

namespace ether {
namespace {

constexpr int kIonBs = 256;  // threads per block (XYZ reading: sites per record tile)

// Reading Ising: a thread per site reads ion(3) alone; the lines holding no spin field are
// never fetched (measured faster than reading whole records for an 8-byte field in 72).
__global__ void __launch_bounds__(kIonBs)
ion_in_ising_kernel(const double *__restrict__ ion, int N, const int32_t *__restrict__ storage,
                    uint8_t *__restrict__ spins) {
    const int i = blockIdx.x * kIonBs + threadIdx.x;
    if (i >= N) return;
    const size_t r = blockIdx.y;
    spins[r * N + storage[i]] = ion[9 * ((size_t)r * N + i) + 3] > 0.0 ? 1 : 0;
}

// Reading XYZ: a block stages the records of kIonBs consecutive sites (9 doubles each, read as
// consecutive doubles, so each warp's load covers 256 contiguous bytes) in shared memory, then
// each thread takes its site's fields.  The spin fields span bytes 8-48 of each 72-byte record,
// so the whole tile is read; only the spin fields are used.
__global__ void __launch_bounds__(kIonBs)
ion_in_xyz_kernel(const double *__restrict__ ion, int N, const int32_t *__restrict__ storage,
                  float4 *__restrict__ spins4) {
    __shared__ double rec[9 * kIonBs];
    const int t = threadIdx.x;
    const int i0 = blockIdx.x * kIonBs;
    const int n = min(kIonBs, N - i0);
    const size_t r = blockIdx.y;
    const double *src = ion + 9 * ((size_t)r * N + i0);
    if (n == kIonBs) {
        double v[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) v[j] = src[j * kIonBs + t];
#pragma unroll
        for (int j = 0; j < 9; ++j) rec[j * kIonBs + t] = v[j];
    } else {
        for (int k = t; k < 9 * n; k += kIonBs) rec[k] = src[k];
    }
    __syncthreads();
    if (t >= n) return;
    const double *p = rec + 9 * t;
    spins4[r * N + storage[i0 + t]] = make_float4((float)p[1], (float)p[2], (float)p[3], (float)p[5]);
}

__global__ void __launch_bounds__(kIonBs)
ion_out_ising_kernel(const uint8_t *__restrict__ spins, int N, const int32_t *__restrict__ storage,
                     double *__restrict__ ion) {
    const int i = blockIdx.x * kIonBs + threadIdx.x;
    if (i >= N) return;
    const size_t r = blockIdx.y;
    ion[9 * ((size_t)r * N + i) + 3] = spins[r * N + storage[i]] ? 1.0 : -1.0;
}

// Writing XYZ: a warp's 32 sites x 4 fields go out as four stores in address order (store k
// of lane l writes field (32k + l) % 4 of site (32k + l) / 4), so one store instruction covers
// the records of 8 consecutive sites instead of touching 32 records.
__global__ void __launch_bounds__(kIonBs)
ion_out_xyz_kernel(const float4 *__restrict__ spins4, int N, const int32_t *__restrict__ storage,
                   double *__restrict__ ion) {
    const int lane = threadIdx.x & 31;
    const int w0 = blockIdx.x * kIonBs + (threadIdx.x & ~31);
    const int i = w0 + lane;
    const size_t r = blockIdx.y;
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < N) q = spins4[r * N + storage[i]];
    double *base = ion + 9 * ((size_t)r * N + w0);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int g = 32 * k + lane;
        const int src = g >> 2, f = g & 3;
        const float x = __shfl_sync(0xffffffffu, q.x, src);
        const float y = __shfl_sync(0xffffffffu, q.y, src);
        const float z = __shfl_sync(0xffffffffu, q.z, src);
        const float w = __shfl_sync(0xffffffffu, q.w, src);
        const float v = f == 0 ? x : f == 1 ? y : f == 2 ? z : w;
        if (w0 + src < N) base[9 * src + (f == 3 ? 5 : f + 1)] = (double)v;
    }
}

}  // namespace

bool ion_direct_possible(int dev) {
    int pageable = 0, host_tables = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) !=
        cudaSuccess)
        return false;
    return pageable == 1 && host_tables == 1;
}

cudaError_t launch_ion_copy(Ctx &c, int r0, int n, double *ion, bool to_device) {
    const int N = c.N;
    const unsigned gx = (unsigned)((N + kIonBs - 1) / kIonBs);
    for (int a = 0; a < n; a += 65535) {
        const int m = std::min(n - a, 65535);
        const dim3 grid(gx, (unsigned)m);
        double *rec = ion + (size_t)9 * N * a;
        const size_t off = (size_t)(r0 + a) * N;
        if (c.model == ETHER_MODEL_ISING) {
            if (to_device)
                ion_in_ising_kernel<<<grid, kIonBs, 0, c.stream>>>(rec, N, c.t.storage, c.spins + off);
            else
                ion_out_ising_kernel<<<grid, kIonBs, 0, c.stream>>>(c.spins + off, N, c.t.storage, rec);
        } else {
            if (to_device)
                ion_in_xyz_kernel<<<grid, kIonBs, 0, c.stream>>>(rec, N, c.t.storage, c.spins4 + off);
            else
                ion_out_xyz_kernel<<<grid, kIonBs, 0, c.stream>>>(c.spins4 + off, N, c.t.storage, rec);
        }
        c.launches++;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace ether
