// Pieces shared by the persistent PCG kernels (CSR and SELL-32): the solver
// record at the head of the workspace, the bounded grid barrier, the block
// and per-CTA-partial reductions, and the double-float storage pair.
#pragma once
#include "tm_common.cuh"
#include "../../include/tensormesh_gb300.h"

namespace tmg {

struct PcgState {
  unsigned int count;
  unsigned int gen;
  int status;
  int iters;
  double res;   // final recurrence residual norm
  double bnorm;
};

constexpr long long kGridSpinLimit = 1ll << 25;  // ~1 s with the 32 ns back-off

__device__ __forceinline__ bool grid_sync(PcgState* st, unsigned nblocks, unsigned& my_gen,
                                          long long spin_limit = kGridSpinLimit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned g = my_gen;
    __threadfence();
    unsigned arrived = atomicAdd(&st->count, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(&st->count, 0u);
      __threadfence();
      atomicAdd(&st->gen, 1u);
    } else {
      volatile unsigned* gen = &st->gen;
      long long spins = 0;
      while (*gen == g) {
        if (++spins > spin_limit) {
          atomicExch(&st->status, TM_ERR_TIMEOUT);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  ++my_gen;
  __syncthreads();
  return *((volatile int*)&st->status) == TM_OK;
}

template <class T>
__device__ __forceinline__ T block_sum(T v, T* s_red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  T t = 0;
  if (warp == 0) {
    t = lane < (blockDim.x >> 5) ? s_red[lane] : T(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// Sum the per-CTA partials (same order in every CTA).
template <class T>
__device__ __forceinline__ T sum_partials(const T* part, int n, T* s_red) {
  T v = 0;
  if (threadIdx.x < 32) {
    for (int i = threadIdx.x; i < n; i += 32) v += ((volatile T*)part)[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) s_red[0] = v;
  }
  __syncthreads();
  T r = s_red[0];
  __syncthreads();
  return r;
}

// FP64 systems: values and vectors are held as double-float pairs (same bytes
// as double) and every operation runs on the FP32 pipe; GB300's native FP64
// FMA rate (~0.5 T/s) would otherwise bound the SpMV.
struct F2 {
  float hi, lo;
};
TM_D df64 ld2(const F2* a, int64_t i) {
  F2 v = a[i];
  return {v.hi, v.lo};
}
TM_D void st2(F2* a, int64_t i, df64 v) { a[i] = F2{v.hi, v.lo}; }

// Two per-CTA sums at once (one pass of shuffles and one of barriers), for
// CTAs of at most 16 warps (s_red holds 32 doubles); valid in thread 0.
__device__ __forceinline__ void block_sum2(double& a, double& b, double* s_red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    s_red[warp] = a;
    s_red[16 + warp] = b;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    a = lane < nw ? s_red[lane] : 0.0;
    b = lane < nw ? s_red[16 + lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
  }
  __syncthreads();
}

// The sums of two partial arrays (same order in every CTA), in one pass.
__device__ __forceinline__ void sum_partials2(const double* pa, const double* pb, int n, double* s_red, double& a,
                                              double& b) {
  if (threadIdx.x < 32) {
    double va = 0.0, vb = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) {
      va += ((volatile const double*)pa)[i];
      vb += ((volatile const double*)pb)[i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      va += __shfl_down_sync(0xffffffffu, va, o);
      vb += __shfl_down_sync(0xffffffffu, vb, o);
    }
    if (threadIdx.x == 0) {
      s_red[0] = va;
      s_red[1] = vb;
    }
  }
  __syncthreads();
  a = s_red[0];
  b = s_red[1];
  __syncthreads();
}

}  // namespace tmg
