// noalloc.cu -- energy and magnetisation of simple-cubic spin configurations that the caller
// already holds in device memory, computed without allocating any memory.
//
// Who needs it.  ether_tot_energy works on a context, and creating a context allocates device
// memory.  Some callers cannot allocate at the point where they need an energy: a host
// framework that owns every device allocation through its own pool and hands this library
// only pointers into it (its accounting would not see a cudaMalloc of ours, and a full pool
// would make ours fail); a Fortran driver whose device arrays are mapped by an OpenACC or
// OpenMP-target runtime; a long-running service with a fixed device-memory budget that is
// already spent on spin configurations.  This entry point takes the configurations and
// returns E and M in the caller's host arrays, and allocates nothing: its scratch memory is
// a fixed array in the library's static device memory.
//
// Scratch.  kScratchDoubles doubles (1 MiB) of static __device__ memory, held by every GPU
// that loads the library until the process exits.  A call needs
// n_replicas * (blocks + 1) * 4 doubles, blocks = clamp(ceil(N / 2048), 1, 32), which fits
// for any N when n_replicas <= kMaxReplicas = 992; larger requests return ETHER_ERR_CAPACITY
// before touching any memory.  Every call shares the same array and leaves its contents behind: two calls
// whose work overlaps on the GPU (different streams or host threads without ordering) race on
// it and give wrong results.  Every partial sum is written before it is read, so nothing has to
// be cleared between calls.
//
// Set-up.  Host code cannot use the array's name as a device address (it names a host-side
// stand-in).  The first call on each device, with that device current, looks the address up
// with cudaGetSymbolAddress and caches it.
//
// Streams.  Every call ends with cudaStreamSynchronize on the caller's stream, so no call may
// be made while that stream is being captured into a CUDA graph (the synchronisation would
// break the caller's capture).
//
// Input memory.  `spins` must be memory the current device can address: a device allocation
// of this device, managed memory, or page-locked host memory mapped for the device.  Anything
// else (pageable host memory, another device's memory, a pointer the runtime does not know)
// is rejected with ETHER_ERR_ARG before any kernel is launched, since a kernel given it would
// fault or read unrelated memory.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "internal.h"

namespace ether {
namespace {

constexpr int kScratchDoubles = 1 << 17;  // 1 MiB
constexpr int kMaxReplicas = 992;         // 992 * (32 + 1) * 4 <= kScratchDoubles
constexpr int kMaxDevices = 64;
constexpr int kBs = 256;

static __device__ __align__(256) double g_scratch[kScratchDoubles];

std::mutex g_mu;
double *g_addr[kMaxDevices] = {nullptr};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Site energies as get_tot_energy (src/get_tot_energy.f90:33-47): exchange with the six
// periodic neighbours (bonds counted from both ends) plus the Zeeman term; M as
// get_tot_magnetisation (src/get_tot_magnetisation.f90:32-40) with unit stagger and spin
// length.  Spins in the reference's site order (x fastest), replicas one after another.
__global__ void __launch_bounds__(kBs)
noalloc_partials(int model, const void *__restrict__ spins, int L1, int L2, int L3, double jx,
                 double jy, double jz, double zx, double zy, double zz, double *__restrict__ scr) {
    const int r = blockIdx.y;
    const int N = L1 * L2 * L3;
    double q[4] = {0.0, 0.0, 0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const int x = i % L1, y = (i / L1) % L2, z = i / (L1 * L2);
        const int nb[6] = {(x + 1) % L1 + L1 * (y + L2 * z), (x + L1 - 1) % L1 + L1 * (y + L2 * z),
                           x + L1 * ((y + 1) % L2 + L2 * z), x + L1 * ((y + L2 - 1) % L2 + L2 * z),
                           x + L1 * (y + L2 * ((z + 1) % L3)), x + L1 * (y + L2 * ((z + L3 - 1) % L3))};
        if (model == 0) {
            const int8_t *s = static_cast<const int8_t *>(spins) + (size_t)r * N;
            const double si = s[i] > 0 ? 1.0 : -1.0;
            double e = 0.0;
            for (int k = 0; k < 6; ++k) e += (si * (s[nb[k]] > 0 ? 1.0 : -1.0)) * jz;
            e += si * zz;
            q[0] += e;
            q[3] += si;
        } else {
            const float4 *s = static_cast<const float4 *>(spins) + (size_t)r * N;
            const float4 S = s[i];
            double hx = 0.0, hy = 0.0, hz = 0.0;
            for (int k = 0; k < 6; ++k) {
                const float4 Sj = s[nb[k]];
                hx += Sj.x;
                hy += Sj.y;
                hz += Sj.z;
            }
            q[0] += S.x * (jx * hx + zx) + S.y * (jy * hy + zy) + S.z * (jz * hz + zz);
            q[1] += S.x;
            q[2] += S.y;
            q[3] += S.z;
        }
    }
    __shared__ double sm[kBs / 32][4];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const double v = warp_sum(q[j]);
        if (lane == 0) sm[wid][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0.0;
        for (int w = 0; w < kBs / 32; ++w) v += sm[w][threadIdx.x];
        scr[((size_t)r * gridDim.x + blockIdx.x) * 4 + threadIdx.x] = v;
    }
}

// Per replica, the partials in index order -> E at out[r], M at out[R + 3r ..].
__global__ void noalloc_finish(const double *__restrict__ scr, int nblk, int R,
                               double *__restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    double q[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < nblk; ++b)
        for (int j = 0; j < 4; ++j) q[j] += scr[((size_t)r * nblk + b) * 4 + j];
    out[r] = q[0];
    out[R + 3 * r + 0] = q[1];
    out[R + 3 * r + 1] = q[2];
    out[R + 3 * r + 2] = q[3];
}

}  // namespace
}  // namespace ether

using namespace ether;

extern "C" int ether_sc_energy_noalloc(int32_t model, const void *spins, const int32_t L[3],
                                       int32_t n_replicas, const double J[3], const double zee[3],
                                       double *E, double *M, void *stream) {
    if (!spins || !L || !J || !zee || !E || !M || n_replicas <= 0 ||
        (model != ETHER_MODEL_ISING && model != ETHER_MODEL_XYZ)) {
        set_error("ether_sc_energy_noalloc: invalid argument");
        return ETHER_ERR_ARG;
    }
    if (L[0] < 3 || L[1] < 3 || L[2] < 3 || (long)L[0] * L[1] * L[2] > 0x7FFFFFFFL / 16) {
        set_error("ether_sc_energy_noalloc: extents must be >= 3 and L1*L2*L3 < 2^27");
        return ETHER_ERR_ARG;
    }
    const long N = (long)L[0] * L[1] * L[2];
    long nblk = (N + 2047) / 2048;
    if (nblk < 1) nblk = 1;
    if (nblk > 32) nblk = 32;
    if (n_replicas > kMaxReplicas || (long)n_replicas * (nblk + 1) * 4 > kScratchDoubles) {
        set_error("ether_sc_energy_noalloc: " + std::to_string(n_replicas) +
                  " replicas: the 1 MiB of static scratch takes at most 992 per call");
        return ETHER_ERR_CAPACITY;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        set_error(std::string("ether_sc_energy_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return ETHER_ERR_NODEV;
    }
    {
        cudaPointerAttributes pa{};
        e = cudaPointerGetAttributes(&pa, spins);
        if (e != cudaSuccess) {
            cudaGetLastError();  // the failed query is not a lasting error: clear it
            set_error(std::string("ether_sc_energy_noalloc: spins is not a pointer the CUDA "
                                  "runtime knows: ") + cudaGetErrorString(e));
            return ETHER_ERR_ARG;
        }
        const bool ok = (pa.type == cudaMemoryTypeDevice && pa.device == dev) ||
                        pa.type == cudaMemoryTypeManaged ||
                        (pa.type == cudaMemoryTypeHost && pa.devicePointer == spins);
        if (!ok) {
            set_error("ether_sc_energy_noalloc: spins must be memory this device can address "
                      "(its own device memory, managed memory or mapped page-locked host "
                      "memory); got " +
                      std::string(pa.type == cudaMemoryTypeUnregistered ? "pageable host memory"
                                  : pa.type == cudaMemoryTypeDevice ? "another device's memory"
                                                                    : "unmapped host memory"));
            return ETHER_ERR_ARG;
        }
    }
    double *scr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_scratch);
            if (e != cudaSuccess || !p) {
                set_error(std::string("ether_sc_energy_noalloc: cudaGetSymbolAddress: ") +
                          cudaGetErrorString(e));
                return ETHER_ERR_CUDA;
            }
            g_addr[dev] = static_cast<double *>(p);
        }
        scr = g_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *fin = scr + (size_t)n_replicas * nblk * 4;
    dim3 grid((unsigned)nblk, (unsigned)n_replicas);
    noalloc_partials<<<grid, kBs, 0, st>>>(model, spins, L[0], L[1], L[2], J[0], J[1], J[2],
                                           zee[0], zee[1], zee[2], scr);
    noalloc_finish<<<(n_replicas + 127) / 128, 128, 0, st>>>(scr, (int)nblk, n_replicas, fin);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(E, fin, sizeof(double) * n_replicas, cudaMemcpyDeviceToHost, st);
    // Ising spins have x and y components 0, so M = (0, 0, sum of Sz) for them
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(M, fin + n_replicas, sizeof(double) * 3 * n_replicas,
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_error(std::string("ether_sc_energy_noalloc: ") + cudaGetErrorString(e));
        return ETHER_ERR_CUDA;
    }
    return ETHER_OK;
}
