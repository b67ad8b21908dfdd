// CSR sparse matrix-vector product, shared by the C entry tm_spmv_csr and the
// two-level preconditioner.
#pragma once
#include "tm_common.cuh"

namespace tmg {

// CSR SpMV: a group of G lanes per row, FP accumulation in the value type.
template <class T, int G>
__global__ void spmv_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                            const T* __restrict__ val, const T* __restrict__ x, T* __restrict__ y) {
  // G lanes per row; lane l sums entries b + l, b + l + G, ... in order, and
  // issues four of them (index and value loads, then the x gathers) at a time
  const int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t row = gid / G;
  const int lane = threadIdx.x % G;
  T s = 0;
  if (row < n) {
    const int64_t b = indptr[row], e = indptr[row + 1];
    for (int64_t k = b + lane; k < e; k += 4 * G) {
      T v[4];
      int c[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const bool ok = k + j * G < e;
        v[j] = ok ? val[k + j * G] : T(0);
        c[j] = ok ? idx[k + j * G] : idx[b];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) s += v[j] * x[c[j]];
    }
  }
  if (G > 1) {
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off, G);
  }
  if (row < n && lane == 0) y[row] = s;
}

// lanes per row for a mean row length (about 4 entries per lane)
inline int spmv_lanes(int64_t n_rows, int64_t nnz) {
  const double avg = n_rows > 0 ? (double)nnz / (double)n_rows : 0.0;
  return avg <= 4.0 ? 1 : avg <= 8.0 ? 2 : avg <= 16.0 ? 4 : avg <= 32.0 ? 8 : 16;
}

template <class T>
inline void launch_spmv(int64_t n_rows, int64_t nnz, const int64_t* indptr, const int32_t* idx, const T* val,
                        const T* x, T* y, cudaStream_t s) {
  const int G = spmv_lanes(n_rows, nnz);
  const int grid = (int)((n_rows * G + 255) / 256);
  switch (G) {
    case 1: spmv_kernel<T, 1><<<grid, 256, 0, s>>>(n_rows, indptr, idx, val, x, y); break;
    case 2: spmv_kernel<T, 2><<<grid, 256, 0, s>>>(n_rows, indptr, idx, val, x, y); break;
    case 4: spmv_kernel<T, 4><<<grid, 256, 0, s>>>(n_rows, indptr, idx, val, x, y); break;
    case 8: spmv_kernel<T, 8><<<grid, 256, 0, s>>>(n_rows, indptr, idx, val, x, y); break;
    default: spmv_kernel<T, 16><<<grid, 256, 0, s>>>(n_rows, indptr, idx, val, x, y); break;
  }
}

}  // namespace tmg
