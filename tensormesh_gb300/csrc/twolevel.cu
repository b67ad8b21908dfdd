// Two-level preconditioner application (the learned preconditioner's
// per-iteration operator), float32 inside, FP64 residual in and correction out:
//     y_c  = K_c^-1 P^T r
//     s    = S (r - (K P) y_c)                 S = diag(w) D^-1
//     y_c2 = K_c^-1 P^T (K s)
//     z    = P (y_c - y_c2) + s                = C r + (I - C K) S (I - K C) r
// P is piecewise constant over aggregates; P^T is a per-aggregate sum (one warp
// per aggregate, fixed lane order and shuffle tree, so the result is
// deterministic); K_c^-1 is a dense matrix (one warp per row), float32 or
// its half-precision unit-diagonal form with a float32 diagonal scale.
#include <cuda_fp16.h>
#include "spmv.cuh"
#include "../../include/tensormesh_gb300.h"

namespace tmg {
namespace tl {

constexpr int kThreads = 256;

// Loads in flight per lane in the restriction and the coarse matvec: the
// index loads of a round are all issued before the value loads that depend
// on them.
constexpr int kTlIlp = 8;

// rc[c] = sum of r over aggregate c (times scale[c] when scale is given):
// lane l adds entries l, l + 32, ... of the aggregate in that order, then a
// shuffle tree (deterministic).
template <class T>
__global__ void restrict_kernel(int32_t nc, const int64_t* __restrict__ ptr, const int32_t* __restrict__ perm,
                                const T* __restrict__ r, const float* __restrict__ scale, float* __restrict__ rc) {
  const int c = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= nc) return;  // the whole warp leaves together
  const int64_t k1 = ptr[c + 1];
  float s = 0.f;
  for (int64_t kb = ptr[c] + lane; kb < k1; kb += 32 * kTlIlp) {
    int id[kTlIlp];
#pragma unroll
    for (int u = 0; u < kTlIlp; ++u) id[u] = kb + 32 * u < k1 ? __ldg(perm + kb + 32 * u) : -1;
    T v[kTlIlp];
#pragma unroll
    for (int u = 0; u < kTlIlp; ++u) v[u] = id[u] >= 0 ? r[id[u]] : T(0);
#pragma unroll
    for (int u = 0; u < kTlIlp; ++u)
      if (id[u] >= 0) s += (float)v[u];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) rc[c] = scale ? s * scale[c] : s;
}

// y = A x with A dense nc x nc (row-major), one warp per row.  kVec (nc a
// multiple of 4 and A 16-byte aligned): the row is read as float4, lane l
// taking quads l, l + 32, ...; kVecX: x is 16-byte aligned too.
template <bool kVec, bool kVecX>
__global__ void gemv_kernel(int32_t nc, const float* __restrict__ A, const float* __restrict__ x,
                            float* __restrict__ y) {
  const int row = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= nc) return;
  const float* a = A + (int64_t)row * nc;
  float s = 0.f;
  if constexpr (kVec) {
    const float4* a4 = reinterpret_cast<const float4*>(a);
    const int n4 = nc >> 2;
    for (int jb = lane; jb < n4; jb += 32 * kTlIlp) {
      float4 v[kTlIlp];
#pragma unroll
      for (int u = 0; u < kTlIlp; ++u) v[u] = jb + 32 * u < n4 ? __ldg(a4 + jb + 32 * u) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int u = 0; u < kTlIlp; ++u) {
        const int j = jb + 32 * u;
        if (j < n4) {
          float4 xv;
          if constexpr (kVecX) {
            xv = __ldg(reinterpret_cast<const float4*>(x) + j);
          } else {
            xv = make_float4(__ldg(x + 4 * j), __ldg(x + 4 * j + 1), __ldg(x + 4 * j + 2), __ldg(x + 4 * j + 3));
          }
          s = fmaf(v[u].x, xv.x, s);
          s = fmaf(v[u].y, xv.y, s);
          s = fmaf(v[u].z, xv.z, s);
          s = fmaf(v[u].w, xv.w, s);
        }
      }
    }
  } else {
    for (int j = lane; j < nc; j += 32) s += a[j] * x[j];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[row] = s;
}

inline void launch_gemv(int32_t nc, const float* A, const float* x, float* y, cudaStream_t s) {
  const int grid = (nc + kThreads / 32 - 1) / (kThreads / 32);
  const bool vec = (nc & 3) == 0 && ((uintptr_t)A & 15u) == 0;
  const bool vecx = ((uintptr_t)x & 15u) == 0;
  if (vec && vecx) gemv_kernel<true, true><<<grid, kThreads, 0, s>>>(nc, A, x, y);
  else if (vec) gemv_kernel<true, false><<<grid, kThreads, 0, s>>>(nc, A, x, y);
  else gemv_kernel<false, false><<<grid, kThreads, 0, s>>>(nc, A, x, y);
}

// y = D H D x with H the half-precision unit-diagonal form of K_c^-1 and
// D = diag(scale): x arrives multiplied by D already (the restriction applies
// it), so row i is y_i = scale_i sum_j H_ij x_j, one warp per row.  kVec (nc
// a multiple of 8, H 16-byte aligned): eight halves per 16-byte load, lane l
// taking octets l, l + 32, ...; kVecX: x is 16-byte aligned too.  Half the
// bytes of the float32 matvec; the rounding of H (2^-11 of the diagonal
// scale) left the flexible-CG iteration counts of the 128^3 C5 system
// unchanged.
template <bool kVec, bool kVecX>
__global__ void gemv_half_kernel(int32_t nc, const __half* __restrict__ H, const float* __restrict__ scale,
                                 const float* __restrict__ x, float* __restrict__ y) {
  const int row = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= nc) return;
  const __half* h = H + (int64_t)row * nc;
  float s = 0.f;
  if constexpr (kVec) {
    const uint4* h8 = reinterpret_cast<const uint4*>(h);
    const int n8 = nc >> 3;
    for (int jb = lane; jb < n8; jb += 32 * kTlIlp) {
      uint4 v[kTlIlp];
#pragma unroll
      for (int u = 0; u < kTlIlp; ++u) v[u] = jb + 32 * u < n8 ? __ldg(h8 + jb + 32 * u) : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
      for (int u = 0; u < kTlIlp; ++u) {
        const int j = jb + 32 * u;
        if (j < n8) {
          float xv[8];
          if constexpr (kVecX) {
            const float4 a = __ldg(reinterpret_cast<const float4*>(x) + 2 * j);
            const float4 b = __ldg(reinterpret_cast<const float4*>(x) + 2 * j + 1);
            xv[0] = a.x; xv[1] = a.y; xv[2] = a.z; xv[3] = a.w;
            xv[4] = b.x; xv[5] = b.y; xv[6] = b.z; xv[7] = b.w;
          } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) xv[k] = __ldg(x + 8 * j + k);
          }
          const __half2* hv = reinterpret_cast<const __half2*>(&v[u]);
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const float2 f = __half22float2(hv[k]);
            s = fmaf(f.x, xv[2 * k], s);
            s = fmaf(f.y, xv[2 * k + 1], s);
          }
        }
      }
    }
  } else {
    for (int j = lane; j < nc; j += 32) s = fmaf(__half2float(h[j]), x[j], s);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[row] = scale[row] * s;
}

inline void launch_gemv_half(int32_t nc, const void* H, const float* scale, const float* x, float* y,
                             cudaStream_t s) {
  const int grid = (nc + kThreads / 32 - 1) / (kThreads / 32);
  const __half* h = static_cast<const __half*>(H);
  const bool vec = (nc & 7) == 0 && ((uintptr_t)H & 15u) == 0;
  const bool vecx = ((uintptr_t)x & 15u) == 0;
  if (vec && vecx) gemv_half_kernel<true, true><<<grid, kThreads, 0, s>>>(nc, h, scale, x, y);
  else if (vec) gemv_half_kernel<true, false><<<grid, kThreads, 0, s>>>(nc, h, scale, x, y);
  else gemv_half_kernel<false, false><<<grid, kThreads, 0, s>>>(nc, h, scale, x, y);
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

// ---- flexible CG with the two-level preconditioner, vector work fused ----
// Scalars live on the device (no host round trip per iteration; slots below
// at fcg_rz_slot).  Dot products reduce per CTA (fixed tree) into part[];
// the kernel that needs the scalar sums part[] in one fixed order in every
// CTA, so every iteration is bitwise repeatable.
constexpr int kFcgThreads = 512;
constexpr int kFcgBlocks = 304;

__device__ __forceinline__ double fcg_block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

__device__ __forceinline__ double fcg_sum_parts(const double* part, int nb) {
  // one warp, lane-strided then a shuffle tree: the same order every call
  double v = 0.0;
  for (int i = threadIdx.x; i < nb; i += 32) v += part[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;  // valid in lane 0
}

// The grid-stride loops below keep four iterations' loads in flight per
// thread and consume them in index order, so every thread's sums are formed
// in the same order as a one-at-a-time loop (the results do not depend on
// the batching).
constexpr int kFcgBatch = 4;

// part[b] = this CTA's share of (a, b)
__global__ void __launch_bounds__(kFcgThreads) fcg_dot_kernel(int64_t n, const double* __restrict__ a,
                                                               const double* __restrict__ b, double* part) {
  __shared__ double red[32];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  double v = 0.0;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i0 < n; i0 += kFcgBatch * stride) {
    double av[kFcgBatch], bv[kFcgBatch];
#pragma unroll
    for (int u = 0; u < kFcgBatch; ++u) {
      const int64_t i = i0 + u * stride;
      av[u] = i < n ? a[i] : 0.0;
      bv[u] = i < n ? b[i] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kFcgBatch; ++u)
      if (i0 + u * stride < n) v = fma(av[u], bv[u], v);
  }
  v = fcg_block_sum(v, red);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

// Scalars of iteration k: rz in sc[0] (k even) or sc[4] (k odd), so that the
// kernel that forms the next rz never overwrites the one its other CTAs are
// reading; alpha in sc[1], beta in sc[2], (p, q) in sc[3].
__device__ __forceinline__ int fcg_rz_slot(int parity) { return parity ? 4 : 0; }

// alpha = rz / (p, q) from the partials of (p, q) (every CTA sums them in
// the same order; 0 when (p, q) <= 0: the iteration then stands still and
// the host's stagnation test takes over), then x += alpha p, r -= alpha q
__global__ void __launch_bounds__(kFcgThreads) fcg_xr_kernel(int64_t n, double* __restrict__ x,
                                                              double* __restrict__ r, const double* __restrict__ p,
                                                              const double* __restrict__ q, const double* part,
                                                              int nb, double* sc, int parity) {
  __shared__ double s_alpha;
  if (threadIdx.x < 32) {
    const double pq = fcg_sum_parts(part, nb);
    if (threadIdx.x == 0) {
      const double al = pq > 0.0 ? sc[fcg_rz_slot(parity)] / pq : 0.0;
      s_alpha = al;
      if (blockIdx.x == 0) {
        sc[1] = al;
        sc[3] = pq;
      }
    }
  }
  __syncthreads();
  const double alpha = s_alpha;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i0 < n; i0 += kFcgBatch * stride) {
    double xv[kFcgBatch], rv[kFcgBatch], pv[kFcgBatch], qv[kFcgBatch];
#pragma unroll
    for (int u = 0; u < kFcgBatch; ++u) {
      const int64_t i = i0 + u * stride;
      const bool ok = i < n;
      xv[u] = ok ? x[i] : 0.0;
      rv[u] = ok ? r[i] : 0.0;
      pv[u] = ok ? p[i] : 0.0;
      qv[u] = ok ? q[i] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kFcgBatch; ++u) {
      const int64_t i = i0 + u * stride;
      if (i < n) {
        x[i] = fma(alpha, pv[u], xv[u]);
        r[i] = fma(-alpha, qv[u], rv[u]);
      }
    }
  }
}

// The application's last step fused with the dot products that follow it:
// z = P (y_c - y_c2) + s, and the CTA's shares of (r, z) into part[b] and of
// (z, q) into part[nb + b] (grid-stride rows, the CTA's fixed tree).
__global__ void __launch_bounds__(kFcgThreads) finish_dot2_kernel(int64_t n, const int32_t* __restrict__ agg,
                                                                   const float* __restrict__ yc,
                                                                   const float* __restrict__ yc2,
                                                                   const float* __restrict__ s1,
                                                                   const double* __restrict__ r,
                                                                   const double* __restrict__ q,
                                                                   double* __restrict__ z, double* part) {
  __shared__ double red[32];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  double a = 0.0, c = 0.0;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i0 < n; i0 += kFcgBatch * stride) {
    int g[kFcgBatch];
    float sv[kFcgBatch];
    double rv[kFcgBatch], qv[kFcgBatch];
#pragma unroll
    for (int u = 0; u < kFcgBatch; ++u) {
      const int64_t i = i0 + u * stride;
      const bool ok = i < n;
      g[u] = ok ? agg[i] : 0;
      sv[u] = ok ? s1[i] : 0.f;
      rv[u] = ok ? r[i] : 0.0;
      qv[u] = ok ? q[i] : 0.0;
    }
    float y1[kFcgBatch], y2[kFcgBatch];
#pragma unroll
    for (int u = 0; u < kFcgBatch; ++u) {
      y1[u] = yc[g[u]];
      y2[u] = yc2[g[u]];
    }
#pragma unroll
    for (int u = 0; u < kFcgBatch; ++u) {
      const int64_t i = i0 + u * stride;
      if (i < n) {
        const double zi = (double)((y1[u] - y2[u]) + sv[u]);
        z[i] = zi;
        a = fma(rv[u], zi, a);
        c = fma(zi, qv[u], c);
      }
    }
  }
  a = fcg_block_sum(a, red);
  c = fcg_block_sum(c, red);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = a;
    part[gridDim.x + blockIdx.x] = c;
  }
}

// Polak-Ribiere beta = max(0, (z, r_new - r_old) / rz_old) with r_new - r_old
// = -alpha q, from the partials of (r, z) and (z, q) (every CTA sums them in
// the same order); rz_new = (r, z) goes to the other rz slot; then
// p = z + beta p
__global__ void __launch_bounds__(kFcgThreads) fcg_p_kernel(int64_t n, double* __restrict__ p,
                                                             const double* __restrict__ z, const double* part,
                                                             int nb, double* sc, int parity) {
  __shared__ double s_beta;
  if (threadIdx.x < 32) {
    const double rzn = fcg_sum_parts(part, nb);
    const double zq = fcg_sum_parts(part + nb, nb);
    if (threadIdx.x == 0) {
      const double rz = sc[fcg_rz_slot(parity)];
      const double b = rz != 0.0 ? -sc[1] * zq / rz : 0.0;
      s_beta = b > 0.0 ? b : 0.0;
      if (blockIdx.x == 0) {
        sc[2] = s_beta;
        sc[fcg_rz_slot(parity ^ 1)] = rzn;
      }
    }
  }
  __syncthreads();
  const double beta = s_beta;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i0 < n; i0 += kFcgBatch * stride) {
    double pv[kFcgBatch], zv[kFcgBatch];
#pragma unroll
    for (int u = 0; u < kFcgBatch; ++u) {
      const int64_t i = i0 + u * stride;
      pv[u] = i < n ? p[i] : 0.0;
      zv[u] = i < n ? z[i] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kFcgBatch; ++u) {
      const int64_t i = i0 + u * stride;
      if (i < n) p[i] = fma(beta, pv[u], zv[u]);
    }
  }
}

// rz of the last iteration back to sc[0] (after an odd number of iterations)
__global__ void fcg_rz_home_kernel(double* sc) { sc[0] = sc[4]; }

// CTAs of the flexible CG's vector kernels: two per SM for large systems,
// fewer for small ones (four rows per thread at least), so that the per-CTA
// partial sums every CTA adds up stay few; a function of n alone, so the
// iteration stays bitwise repeatable.
inline int fcg_blocks(int64_t n) {
  const int64_t want = (n + (int64_t)kFcgThreads * kFcgBatch - 1) / ((int64_t)kFcgThreads * kFcgBatch);
  return (int)(want < 1 ? 1 : (want > kFcgBlocks ? kFcgBlocks : want));
}

// ---- K P (the thin matrix of the coarse space) without a global sort -------
// Row i of K P holds, for each aggregate c among the columns of row i of K,
// the sum of K_ij over those columns j with agg[j] = c: columns in ascending
// aggregate order, each sum taken in the row's CSR order.  One thread per row;
// the aggregates are found by repeated minimum searches over the row (rows
// are short), so no per-row storage is needed.
__global__ void kp_count_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                                const int32_t* __restrict__ agg, int64_t* __restrict__ count) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t k0 = indptr[i], k1 = indptr[i + 1];
  int64_t m = 0;
  int cur = -1;
  for (;;) {
    int nxt = 0x7fffffff;
    for (int64_t k = k0; k < k1; ++k) {
      const int a = agg[idx[k]];
      if (a > cur && a < nxt) nxt = a;
    }
    if (nxt == 0x7fffffff) break;
    ++m;
    cur = nxt;
  }
  count[i] = m;
}

__global__ void kp_fill_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                               const double* __restrict__ val, const int32_t* __restrict__ agg,
                               const int64_t* __restrict__ kp_ptr, int32_t* __restrict__ kp_idx,
                               double* __restrict__ kp_val) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t k0 = indptr[i], k1 = indptr[i + 1];
  int64_t o = kp_ptr[i];
  int cur = -1;
  for (;;) {
    int nxt = 0x7fffffff;
    for (int64_t k = k0; k < k1; ++k) {
      const int a = agg[idx[k]];
      if (a > cur && a < nxt) nxt = a;
    }
    if (nxt == 0x7fffffff) break;
    double s = 0.0;
    for (int64_t k = k0; k < k1; ++k)
      if (agg[idx[k]] == nxt) s += val[k];
    kp_idx[o] = nxt;
    kp_val[o] = s;
    ++o;
    cur = nxt;
  }
}

}  // namespace tl

}  // namespace tmg

// count[i] = aggregates among the columns of row i (fill kp_indptr = exclusive
// scan of it, then call tm_kp_fill)
extern "C" int tm_kp_count(int64_t n, const int64_t* indptr, const int32_t* indices, const int32_t* agg,
                           int64_t* count, void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!indptr || !indices || !agg || !count) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  tmg::tl::kp_count_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, indptr, indices, agg, count);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_kp_fill(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values,
                          const int32_t* agg, const int64_t* kp_indptr, int32_t* kp_indices, double* kp_values,
                          void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!indptr || !indices || !values || !agg || !kp_indptr || !kp_indices || !kp_values) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  tmg::tl::kp_fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, indptr, indices, values, agg, kp_indptr,
                                                                      kp_indices, kp_values);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

// z = M r.  With q_dot and part (the flexible CG), the last step also forms
// the partial sums of (r, z) and (z, q_dot) for fcg_p_kernel.
static int twolevel_apply_impl(const tm_twolevel* t, const double* r, double* z, cudaStream_t s,
                               const double* q_dot = nullptr, double* part = nullptr, int nb = 0) {
  using namespace tmg::tl;
  const int64_t n = t->n;
  const int32_t nc = t->nc;
  // the coarse vectors first, so that the matvec inputs rc and rc2 keep the
  // scratch's alignment (16-byte loads when nc is even)
  float* rc = t->work;
  float* yc = rc + nc;
  float* rc2 = yc + nc;
  float* yc2 = rc2 + nc;
  float* s1 = yc2 + nc;
  float* r2 = s1 + n;
  const int gc = (nc + kThreads / 32 - 1) / (kThreads / 32);
  const int gn = (int)((n + kThreads - 1) / kThreads);
  const bool half = t->kc_half != nullptr;
  const float* rscale = half ? t->kc_scale : nullptr;
  restrict_kernel<double><<<gc, kThreads, 0, s>>>(nc, t->agg_ptr, t->agg_perm, r, rscale, rc);
  if (half) launch_gemv_half(nc, t->kc_half, t->kc_scale, rc, yc, s);
  else launch_gemv(nc, t->kc_inv, rc, yc, s);
  smooth_kernel<<<gn, kThreads, 0, s>>>(n, t->kp_indptr, t->kp_indices, t->kp_values, yc, r, t->sw, s1);
  if (t->k_slice_ptr) {
    const int st = tm_spmv_sell(TM_F32, n, t->k_slice_ptr, t->k_narrow, t->k_scol, t->k_sval, s1, r2, s);
    if (st != TM_OK) return st;
  } else {
    tmg::launch_spmv<float>(n, t->k_nnz, t->k_indptr, t->k_indices, t->k_values, s1, r2, s);
  }
  restrict_kernel<float><<<gc, kThreads, 0, s>>>(nc, t->agg_ptr, t->agg_perm, r2, rscale, rc2);
  if (half) launch_gemv_half(nc, t->kc_half, t->kc_scale, rc2, yc2, s);
  else launch_gemv(nc, t->kc_inv, rc2, yc2, s);
  if (q_dot)
    finish_dot2_kernel<<<nb, kFcgThreads, 0, s>>>(n, t->agg, yc, yc2, s1, r, q_dot, z, part);
  else
    finish_kernel<<<gn, kThreads, 0, s>>>(n, t->agg, yc, yc2, s1, z);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

static bool twolevel_ok(const tm_twolevel* t) {
  return t->n >= 0 && t->nc >= 1 && t->k_nnz >= 0 && t->agg && t->agg_ptr && t->agg_perm && t->kc_inv &&
         t->kp_indptr && t->kp_indices && t->kp_values && t->k_indptr && t->k_indices && t->k_values && t->sw &&
         t->work && (!t->k_slice_ptr || (t->k_scol && t->k_sval)) && (!t->kc_half || t->kc_scale);
}

extern "C" int64_t tm_fcg_workspace_doubles(void) { return 2 * (int64_t)tmg::tl::kFcgBlocks + 8; }

extern "C" int tm_fcg_twolevel_iterations(const tm_twolevel* t, int64_t a_nnz, const int64_t* a_indptr,
                                          const int32_t* a_indices, const double* a_values,
                                          const int64_t* a_slice_ptr, int32_t a_narrow, const void* a_scol,
                                          const double* a_sval, double* x, double* r, double* p, double* q, double* z,
                                          double* sc, double* part, int32_t iters, void* stream) {
  if (!t || !twolevel_ok(t) || iters < 0 || a_nnz < 0) return TM_ERR_INVALID;
  if (!a_indptr || !a_indices || !a_values || !x || !r || !p || !q || !z || !sc || !part) return TM_ERR_INVALID;
  const bool sell = a_slice_ptr != nullptr;
  if (sell && (!a_scol || !a_sval)) return TM_ERR_INVALID;
  using namespace tmg::tl;
  const int64_t n = t->n;
  if (n == 0 || iters == 0) return TM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nb = fcg_blocks(n);
  for (int it = 0; it < iters; ++it) {
    if (sell) {
      const int st = tm_spmv_sell(TM_F64, n, a_slice_ptr, a_narrow, a_scol, a_sval, p, q, stream);
      if (st != TM_OK) return st;
    } else {
      tmg::launch_spmv<double>(n, a_nnz, a_indptr, a_indices, a_values, p, q, s);
    }
    const int parity = it & 1;
    fcg_dot_kernel<<<nb, kFcgThreads, 0, s>>>(n, p, q, part);
    fcg_xr_kernel<<<nb, kFcgThreads, 0, s>>>(n, x, r, p, q, part, nb, sc, parity);
    const int st = twolevel_apply_impl(t, r, z, s, q, part, nb);
    if (st != TM_OK) return st;
    fcg_p_kernel<<<nb, kFcgThreads, 0, s>>>(n, p, z, part, nb, sc, parity);
  }
  if (iters & 1) fcg_rz_home_kernel<<<1, 1, 0, s>>>(sc);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_twolevel_apply(const tm_twolevel* t, const double* r, double* z, void* stream) {
  if (!t || !r || !z) return TM_ERR_INVALID;
  if (t->n < 0 || t->nc < 1 || t->k_nnz < 0) return TM_ERR_INVALID;
  if (t->n == 0) return TM_OK;
  if (!twolevel_ok(t)) return TM_ERR_INVALID;
  return twolevel_apply_impl(t, r, z, static_cast<cudaStream_t>(stream));
}
