// Two-level preconditioner application (the learned preconditioner's
// per-iteration operator), float32 inside, FP64 residual in and correction out:
//     y_c  = K_c^-1 P^T r
//     s    = S (r - (K P) y_c)                 S = diag(w) D^-1
//     y_c2 = K_c^-1 P^T (K s)
//     z    = P (y_c - y_c2) + s                = C r + (I - C K) S (I - K C) r
// P is piecewise constant over aggregates; P^T is a per-aggregate sum (one warp
// per aggregate, fixed lane order and shuffle tree, so the result is
// deterministic); K_c^-1 is a dense float32 matrix (one warp per row).
#include "spmv.cuh"
#include "../../include/tensormesh_gb300.h"

namespace tmg {
namespace tl {

constexpr int kThreads = 256;

template <class T>
__global__ void restrict_kernel(int32_t nc, const int64_t* __restrict__ ptr, const int32_t* __restrict__ perm,
                                const T* __restrict__ r, float* __restrict__ rc) {
  const int c = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= nc) return;  // the whole warp leaves together
  float s = 0.f;
  for (int64_t k = ptr[c] + lane; k < ptr[c + 1]; k += 32) s += (float)r[perm[k]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) rc[c] = s;
}

__global__ void gemv_kernel(int32_t nc, const float* __restrict__ A, const float* __restrict__ x,
                            float* __restrict__ y) {
  const int row = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= nc) return;
  const float* a = A + (int64_t)row * nc;
  float s = 0.f;
  for (int j = lane; j < nc; j += 32) s += a[j] * x[j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[row] = s;
}

__global__ void smooth_kernel(int64_t n, const int64_t* __restrict__ kp_ptr, const int32_t* __restrict__ kp_idx,
                              const float* __restrict__ kp_val, const float* __restrict__ yc,
                              const double* __restrict__ r, const float* __restrict__ sw, float* __restrict__ s1) {
  const int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x;
  if (i >= n) return;
  float acc = (float)r[i];
  for (int64_t k = kp_ptr[i]; k < kp_ptr[i + 1]; ++k) acc -= kp_val[k] * yc[kp_idx[k]];
  s1[i] = sw[i] * acc;
}

__global__ void finish_kernel(int64_t n, const int32_t* __restrict__ agg, const float* __restrict__ yc,
                              const float* __restrict__ yc2, const float* __restrict__ s1, double* __restrict__ z) {
  const int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x;
  if (i >= n) return;
  const int c = agg[i];
  z[i] = (double)((yc[c] - yc2[c]) + s1[i]);
}

}  // namespace tl
}  // namespace tmg

extern "C" int tm_twolevel_apply(const tm_twolevel* t, const double* r, double* z, void* stream) {
  if (!t || !r || !z) return TM_ERR_INVALID;
  if (t->n < 0 || t->nc < 1 || t->k_nnz < 0) return TM_ERR_INVALID;
  if (t->n == 0) return TM_OK;
  if (!t->agg || !t->agg_ptr || !t->agg_perm || !t->kc_inv || !t->kp_indptr || !t->kp_indices || !t->kp_values ||
      !t->k_indptr || !t->k_indices || !t->k_values || !t->sw || !t->work)
    return TM_ERR_INVALID;
  using namespace tmg::tl;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t n = t->n;
  const int32_t nc = t->nc;
  float* s1 = t->work;
  float* r2 = s1 + n;
  float* rc = r2 + n;
  float* yc = rc + nc;
  float* rc2 = yc + nc;
  float* yc2 = rc2 + nc;
  const int gc = (nc + kThreads / 32 - 1) / (kThreads / 32);
  const int gn = (int)((n + kThreads - 1) / kThreads);
  restrict_kernel<double><<<gc, kThreads, 0, s>>>(nc, t->agg_ptr, t->agg_perm, r, rc);
  gemv_kernel<<<gc, kThreads, 0, s>>>(nc, t->kc_inv, rc, yc);
  smooth_kernel<<<gn, kThreads, 0, s>>>(n, t->kp_indptr, t->kp_indices, t->kp_values, yc, r, t->sw, s1);
  tmg::launch_spmv<float>(n, t->k_nnz, t->k_indptr, t->k_indices, t->k_values, s1, r2, s);
  restrict_kernel<float><<<gc, kThreads, 0, s>>>(nc, t->agg_ptr, t->agg_perm, r2, rc2);
  gemv_kernel<<<gc, kThreads, 0, s>>>(nc, t->kc_inv, rc2, yc2);
  finish_kernel<<<gn, kThreads, 0, s>>>(n, t->agg, yc, yc2, s1, z);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}
