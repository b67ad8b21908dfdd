// C-ABI entry points: argument validation and dispatch.
#include <cstdio>
#include "tm_common.cuh"
#include "spmv.cuh"
#include "../../include/tensormesh_gb300.h"

namespace tmg {
int assemble_tri3(const tm_patch_plan&, const tm_assemble_args&, cudaStream_t);
int assemble_tri6(const tm_patch_plan&, const tm_assemble_args&, cudaStream_t);
int assemble_tet4(const tm_patch_plan&, const tm_assemble_args&, cudaStream_t);
int assemble_tet10(const tm_patch_plan&, const tm_assemble_args&, cudaStream_t);
int backward_tri3(const tm_patch_plan&, const tm_assemble_args&, const tm_backward_args&, cudaStream_t);
int backward_tri6(const tm_patch_plan&, const tm_assemble_args&, const tm_backward_args&, cudaStream_t);
int backward_tet4(const tm_patch_plan&, const tm_assemble_args&, const tm_backward_args&, cudaStream_t);
int backward_tet10(const tm_patch_plan&, const tm_assemble_args&, const tm_backward_args&, cudaStream_t);

template <class T>
__global__ void segment_sum_kernel(int64_t n_seg, const int64_t* __restrict__ ptr, const int64_t* __restrict__ perm,
                                   int width, const T* __restrict__ src, T* __restrict__ dst) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n_seg * width) return;
  int64_t s = i / width;
  int w = (int)(i - s * width);
  T acc = 0;
  for (int64_t k = ptr[s]; k < ptr[s + 1]; ++k) acc += src[perm[k] * width + w];
  dst[i] = acc;
}

static int n_basis(int el) {
  switch (el) {
    case TM_TRI3: return 3;
    case TM_TRI6: return 6;
    case TM_TET4: return 4;
    case TM_TET10: return 10;
  }
  return -1;
}

template <class T, int D, int B>
__global__ void quad_points_kernel(int Q, const double* __restrict__ tables, const T* __restrict__ pts,
                                   const int32_t* __restrict__ elems, int64_t n_el, T* __restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n_el * Q) return;
  int64_t e = i / Q;
  int q = (int)(i - e * Q);
  const double* N = tables + Q + q * B;
  double acc[D];
#pragma unroll
  for (int d = 0; d < D; ++d) acc[d] = 0.0;
#pragma unroll
  for (int b = 0; b < B; ++b) {
    int v = elems[e * B + b];
#pragma unroll
    for (int d = 0; d < D; ++d) acc[d] += N[b] * (double)pts[(int64_t)v * D + d];
  }
#pragma unroll
  for (int d = 0; d < D; ++d) out[i * D + d] = (T)acc[d];
}

}  // namespace tmg

extern "C" int tm_assemble(const tm_patch_plan* plan, const tm_assemble_args* args, void* stream) {
  if (!plan || !args) return TM_ERR_INVALID;
  const int B = tmg::n_basis(args->element);
  if (B < 0) return TM_ERR_UNSUPPORTED;
  if (plan->n_basis != B) return TM_ERR_INVALID;
  if (args->dtype != TM_F32 && args->dtype != TM_F64) return TM_ERR_INVALID;
  if (args->n_quad < 1 || args->n_quad > 11) return TM_ERR_INVALID;
  if (!args->tables || !args->points || !args->out) return TM_ERR_INVALID;
  if (args->coef_kind != TM_COEF_SCALAR && !args->coef) return TM_ERR_INVALID;
  if (args->coef_kind < TM_COEF_SCALAR || args->coef_kind > TM_COEF_QUAD) return TM_ERR_INVALID;
  if (args->form == TM_FORM_LOAD && (args->n_comp < 1 || args->n_comp > 3)) return TM_ERR_INVALID;
  if (args->form != TM_FORM_LOAD && args->coef_kind == TM_COEF_POINT && args->n_comp != 1) return TM_ERR_INVALID;
  if (plan->n_patches <= 0) return TM_OK;
  if (plan->max_rows > 4096 || plan->max_vtx > 65535) return TM_ERR_INDEX;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (args->element) {
    case TM_TRI3: return tmg::assemble_tri3(*plan, *args, s);
    case TM_TRI6: return tmg::assemble_tri6(*plan, *args, s);
    case TM_TET4: return tmg::assemble_tet4(*plan, *args, s);
    case TM_TET10: return tmg::assemble_tet10(*plan, *args, s);
  }
  return TM_ERR_UNSUPPORTED;
}

static int check_assemble_args(const tm_patch_plan* plan, const tm_assemble_args* args) {
  if (!plan || !args) return TM_ERR_INVALID;
  const int B = tmg::n_basis(args->element);
  if (B < 0) return TM_ERR_UNSUPPORTED;
  if (plan->n_basis != B) return TM_ERR_INVALID;
  if (args->dtype != TM_F32 && args->dtype != TM_F64) return TM_ERR_INVALID;
  if (args->n_quad < 1 || args->n_quad > 11) return TM_ERR_INVALID;
  if (!args->tables || !args->points) return TM_ERR_INVALID;
  if (args->coef_kind < TM_COEF_SCALAR || args->coef_kind > TM_COEF_QUAD) return TM_ERR_INVALID;
  if (args->coef_kind != TM_COEF_SCALAR && !args->coef) return TM_ERR_INVALID;
  if (args->form == TM_FORM_LOAD && (args->n_comp < 1 || args->n_comp > 3)) return TM_ERR_INVALID;
  if (args->form != TM_FORM_LOAD && args->coef_kind == TM_COEF_POINT && args->n_comp != 1) return TM_ERR_INVALID;
  if (plan->max_rows > 4096 || plan->max_vtx > 65535) return TM_ERR_INDEX;
  return TM_OK;
}

extern "C" int tm_assemble_backward(const tm_patch_plan* plan, const tm_assemble_args* args,
                                    const tm_backward_args* bw, void* stream) {
  int st = check_assemble_args(plan, args);
  if (st != TM_OK) return st;
  if (!bw || !bw->grad_out) return TM_ERR_INVALID;
  if (plan->n_patches <= 0) return TM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (args->element) {
    case TM_TRI3: return tmg::backward_tri3(*plan, *args, *bw, s);
    case TM_TRI6: return tmg::backward_tri6(*plan, *args, *bw, s);
    case TM_TET4: return tmg::backward_tet4(*plan, *args, *bw, s);
    case TM_TET10: return tmg::backward_tet10(*plan, *args, *bw, s);
  }
  return TM_ERR_UNSUPPORTED;
}

extern "C" int tm_segment_sum(int32_t dtype, int64_t n_segments, const int64_t* ptr, const int64_t* perm,
                              int32_t width, const void* src, void* dst, void* stream) {
  if (n_segments == 0) return TM_OK;
  if (n_segments < 0 || width < 1 || !ptr || !perm || !src || !dst) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int64_t total = n_segments * width;
  unsigned grid = (unsigned)((total + 255) / 256);
  if (dtype == TM_F64)
    tmg::segment_sum_kernel<double><<<grid, 256, 0, s>>>(n_segments, ptr, perm, width, (const double*)src, (double*)dst);
  else if (dtype == TM_F32)
    tmg::segment_sum_kernel<float><<<grid, 256, 0, s>>>(n_segments, ptr, perm, width, (const float*)src, (float*)dst);
  else
    return TM_ERR_INVALID;
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_quadrature_points(int32_t element, int32_t dtype, int32_t n_quad, const double* tables,
                                    const void* points, const int32_t* elements, int64_t n_elements,
                                    void* out, void* stream) {
  const int B = tmg::n_basis(element);
  if (B < 0) return TM_ERR_UNSUPPORTED;
  if (!tables || !points || !elements || !out || n_quad < 1 || n_quad > 11 || n_elements < 0) return TM_ERR_INVALID;
  if (n_elements == 0) return TM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int64_t total = n_elements * n_quad;
  int grid = (int)((total + 255) / 256);
#define TM_QP(T, D, BB) \
  tmg::quad_points_kernel<T, D, BB><<<grid, 256, 0, s>>>(n_quad, tables, (const T*)points, elements, n_elements, (T*)out)
  if (dtype == TM_F64) {
    switch (element) {
      case TM_TRI3: TM_QP(double, 2, 3); break;
      case TM_TRI6: TM_QP(double, 2, 6); break;
      case TM_TET4: TM_QP(double, 3, 4); break;
      case TM_TET10: TM_QP(double, 3, 10); break;
    }
  } else if (dtype == TM_F32) {
    switch (element) {
      case TM_TRI3: TM_QP(float, 2, 3); break;
      case TM_TRI6: TM_QP(float, 2, 6); break;
      case TM_TET4: TM_QP(float, 3, 4); break;
      case TM_TET10: TM_QP(float, 3, 10); break;
    }
  } else {
    return TM_ERR_INVALID;
  }
#undef TM_QP
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_spmv_csr(int32_t dtype, int64_t n_rows, int64_t nnz, const int64_t* indptr, const int32_t* indices,
                           const void* values, const void* x, void* y, void* stream) {
  if (n_rows < 0 || nnz < 0) return TM_ERR_INVALID;
  if (n_rows == 0) return TM_OK;
  if (!indptr || (nnz > 0 && (!indices || !values)) || !x || !y) return TM_ERR_INVALID;
  if (dtype != TM_F64 && dtype != TM_F32) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // nnz only picks the lanes per row; the rows' extents come from indptr
  if (dtype == TM_F64)
    tmg::launch_spmv<double>(n_rows, nnz, indptr, indices, (const double*)values, (const double*)x, (double*)y, s);
  else
    tmg::launch_spmv<float>(n_rows, nnz, indptr, indices, (const float*)values, (const float*)x, (float*)y, s);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}
