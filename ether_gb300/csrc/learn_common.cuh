// learn_common.cuh -- what the two learned patch proposals share: the 4^3 patch geometry in
// closed form, the FP32 training kernels (defined in k_learn.cu), and the entry points of
// the Heisenberg learner (k_learn_xyz.cu) that the ether_learn_* functions hand an XYZ
// context over to.
#pragma once
#include <cstdint>

#include <cuda_bf16.h>

#include "internal.h"

namespace ether {
namespace learn {

constexpr uint32_t kLearn = 4;  // Philox purpose
constexpr int NH = 128;         // hidden width of both networks

// ------------------------------------------------------------------ patch geometry ----
// Canonical frame of a patch: local (a, b, c) in [0, 4)^3; A-sites ((a + b + c) even) and
// B-sites numbered 0..31 each in order of a + 4b + 16c.  Row = b + 4c; the two A-sites
// (B-sites) of a row sit at a = p, p + 2 (a = 1 - p, 3 - p), p = (b + c) & 1, and have
// indices 2 row + (a >> 1).  Boundary sites (faces a = -1, 4, b = -1, 4, c = -1, 4) are
// numbered face * 16 + (the two other coordinates u + 4 v).
__host__ __device__ constexpr int geo_b_a(int m) { return (1 - ((((m >> 1) & 3) + ((m >> 1) >> 2)) & 1)) + 2 * (m & 1); }
__host__ __device__ constexpr int geo_a_a(int k) { return ((((k >> 1) & 3) + ((k >> 1) >> 2)) & 1) + 2 * (k & 1); }
// Neighbour q (-x, +x, -y, +y, -z, +z) of B-site m: A-site index (>= 0) or -(1 + boundary index).
__host__ __device__ constexpr int geo_bn(int m, int q) {
    const int row = m >> 1, b = row & 3, c = row >> 2, a = geo_b_a(m);
    return q == 0 ? (a == 0 ? -(1 + b + 4 * c) : 2 * row + ((a - 1) >> 1))
         : q == 1 ? (a == 3 ? -(1 + 16 + b + 4 * c) : 2 * row + ((a + 1) >> 1))
         : q == 2 ? (b == 0 ? -(1 + 32 + a + 4 * c) : 2 * (row - 1) + (a >> 1))
         : q == 3 ? (b == 3 ? -(1 + 48 + a + 4 * c) : 2 * (row + 1) + (a >> 1))
         : q == 4 ? (c == 0 ? -(1 + 64 + a + 4 * b) : 2 * (row - 4) + (a >> 1))
                  : (c == 3 ? -(1 + 80 + a + 4 * b) : 2 * (row + 4) + (a >> 1));
}
// Boundary neighbour q of A-site k (-1 if that neighbour is inside the patch).
__host__ __device__ constexpr int geo_ab(int k, int q) {
    const int row = k >> 1, b = row & 3, c = row >> 2, a = geo_a_a(k);
    return q == 0 ? (a == 0 ? b + 4 * c : -1)
         : q == 1 ? (a == 3 ? 16 + b + 4 * c : -1)
         : q == 2 ? (b == 0 ? 32 + a + 4 * c : -1)
         : q == 3 ? (b == 3 ? 48 + a + 4 * c : -1)
         : q == 4 ? (c == 0 ? 64 + a + 4 * b : -1)
                  : (c == 3 ? 80 + a + 4 * b : -1);
}
// Canonical coordinates of boundary site i (the inverse of the numbering above).
__host__ __device__ inline void geo_bnd(int i, int &a, int &b, int &c) {
    const int f = i >> 4, u = i & 3, v = (i >> 2) & 3, e = (f & 1) ? 4 : -1;
    if (f < 2) { a = e; b = u; c = v; }
    else if (f < 4) { a = u; b = e; c = v; }
    else { a = u; b = v; c = e; }
}

// --------------------------------------------------- FP32 training kernels (k_learn.cu) ----
// C (M x N, ldc) = beta C + sum_k A(m, k) B(k, n), A(m, k) = ta ? A[k lda + m] : A[m lda + k],
// B(k, n) = tb ? B[n ldb + k] : B[k ldb + n]; fixed summation order.
__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, const float *__restrict__ A, int lda, int ta,
                            const float *__restrict__ B, int ldb, int tb, float *__restrict__ C, int ldc,
                            float beta);
// H = bf16(max(H + b, 0)) row-wise
__global__ void bias_relu_kernel(float *__restrict__ Hm, const float *__restrict__ b, int rows, int cols);
__global__ void colsum_kernel(const float *__restrict__ D, int rows, int cols, float *__restrict__ out);
__global__ void relu_mask_kernel(float *__restrict__ dH, const float *__restrict__ Hm, long long n);
__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, int n, float lr, float c1, float c2);
__global__ void advance_lstep_kernel(uint32_t *c, int R);

// ------------------------------------------------ the Heisenberg learner (k_learn_xyz.cu) ----
struct XyzLearn;
int xyz_create(ether_ctx *h, const ether_learn_desc *d, XyzLearn **out);
void xyz_destroy(XyzLearn *x);
int xyz_collect(XyzLearn *x, int per_replica);
int xyz_train(XyzLearn *x, int steps, int batch, float lr, double *loss);
int xyz_sweep(XyzLearn *x, int nsweeps);
int xyz_record_series(XyzLearn *x, int nsteps, int plain_per_step, int learned_per_step, int stride,
                      double *absM);
int xyz_get_accepts(XyzLearn *x, uint64_t *accepted);
void xyz_set_dump(XyzLearn *x, bool on);
int xyz_get_dump(XyzLearn *x, float *out);
int xyz_get_params(XyzLearn *x, float *params);
int xyz_set_params(XyzLearn *x, const float *params);
int xyz_loss_grad(XyzLearn *x, const float *xin, const float *y, int B, double *loss, float *grad);
int xyz_forward(XyzLearn *x, const float *xin, int B, float *out);
int xyz_info(XyzLearn *x, ether_learn_info *info);
void xyz_shape(int *n_inputs, int *n_outputs, int *n_params);

}  // namespace learn
}  // namespace ether
