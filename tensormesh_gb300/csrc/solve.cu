// Jacobi-preconditioned CG as one cooperative persistent kernel, plus the
// small CSR kernels around it (diagonal, gathers for static condensation).
//
// Replaces K.solve for SPD systems: the reference's Jacobi preconditioner
// (sparse/solve/torch_solve.py:24-59) inside a CG loop that it runs as one
// PyTorch launch per vector op (torch_solve.py:70-128, 130-248).  Here the
// whole iteration lives in one launch:
//   * rows are split into contiguous ranges, one per CTA;
//   * p is double-buffered, and the SpMV forms p_new = z + beta p_old for the
//     columns it gathers, so an iteration needs two grid barriers (after
//     p.Ap and after r.z);
//   * dot products reduce per CTA, then every CTA sums the per-CTA partials
//     in the same order -- deterministic, no atomics on values;
//   * the grid barrier is a counter + generation word with a bounded wait:
//     after ~1 s it raises TM_ERR_TIMEOUT and every CTA returns.
#include "pcg_common.cuh"

namespace tmg {

constexpr int kPcgThreads = 512;
constexpr int kGroup = 8;  // lanes per CSR row (float32 kernel, first residual)
constexpr int kDfRows = 2; // rows a thread advances together (double-float iteration)
constexpr int kDfIlp = 4;  // CSR entries of each row fetched per round

template <class T>
__global__ void __launch_bounds__(kPcgThreads)
pcg_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
           const T* __restrict__ val, const T* __restrict__ dinv, const T* __restrict__ b, T* __restrict__ x,
           T* r, T* z, T* p0, T* p1, T* q, T* partials, PcgState* st, double rtol, double atol, int maxiter) {
  __shared__ T s_red[32];
  const unsigned nb = gridDim.x;
  unsigned my_gen = 0;
  // my_gen must start at the value of st->gen at launch: the host zeroes it.
  const int64_t rows_per = (n + nb - 1) / nb;
  const int64_t r0 = min(n, (int64_t)blockIdx.x * rows_per), r1 = min(n, r0 + rows_per);
  const int g = threadIdx.x / kGroup, lane = threadIdx.x % kGroup;
  const int ngroups = kPcgThreads / kGroup;
  T* partA = partials;
  T* partB = partials + nb;
  T* partC = partials + 2 * nb;

  // r = b - A x ; z = D^-1 r ; p = z ; partial rz, rr, bb
  T rz_l = 0, rr_l = 0, bb_l = 0;
  // The trip count of every row loop below is uniform across the CTA, so all
  // lanes reach each full-mask shuffle together.
  for (int64_t base = r0; base < r1; base += ngroups) {
    const int64_t row = base + g;
    const bool valid = row < r1;
    T s = 0;
    if (valid)
      for (int64_t k = indptr[row] + lane; k < indptr[row + 1]; k += kGroup) s += val[k] * x[idx[k]];
#pragma unroll
    for (int o = kGroup / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, kGroup);
    if (valid && lane == 0) {
      T rv = b[row] - s;
      T zv = dinv[row] * rv;
      r[row] = rv;
      z[row] = zv;
      p0[row] = zv;
      rz_l += rv * zv;
      rr_l += rv * rv;
      bb_l += b[row] * b[row];
    }
  }
  T t = block_sum(rz_l, s_red);
  if (threadIdx.x == 0) partA[blockIdx.x] = t;
  t = block_sum(rr_l, s_red);
  if (threadIdx.x == 0) partB[blockIdx.x] = t;
  t = block_sum(bb_l, s_red);
  if (threadIdx.x == 0) partC[blockIdx.x] = t;
  if (!grid_sync(st, nb, my_gen)) return;
  T rz = sum_partials(partA, nb, s_red);
  T rr = sum_partials(partB, nb, s_red);
  const T bb = sum_partials(partC, nb, s_red);
  const double bnorm = sqrt((double)bb);
  const double tol = fmax(rtol * bnorm, atol);
  if (blockIdx.x == 0 && threadIdx.x == 0) st->bnorm = bnorm;
  if (!grid_sync(st, nb, my_gen)) return;  // partial buffers are reused below

  T beta = 0;
  T* pold = p0;  // p of the previous iteration (p0 holds z for it=0 with beta=0)
  T* pnew = p1;
  int it = 0;
  int status = TM_ERR_MAXITER;
  for (; it <= maxiter; ++it) {
    if (sqrt((double)rr) <= tol) {
      status = TM_OK;
      break;
    }
    if (it == maxiter) break;
    // q = A p_new, p_new = z + beta p_old formed on the fly; partial p.q.
    // One thread per row, kDfRows rows and kDfIlp entries per round with all
    // loads of the round issued before the first use.
    T pq_l = 0;
    for (int64_t base = r0 + threadIdx.x; base < r1; base += kDfRows * kPcgThreads) {
      int64_t k0[kDfRows], k1[kDfRows];
      T s[kDfRows];
#pragma unroll
      for (int u = 0; u < kDfRows; ++u) {
        const int64_t row = base + (int64_t)u * kPcgThreads;
        const bool ok = row < r1;
        k0[u] = ok ? indptr[row] : 0;
        k1[u] = ok ? indptr[row + 1] : 0;
        s[u] = 0;
      }
      for (int64_t j0 = 0;; j0 += kDfIlp) {
        bool more = false;
#pragma unroll
        for (int u = 0; u < kDfRows; ++u) more |= k0[u] + j0 < k1[u];
        if (!more) break;
        int c[kDfRows][kDfIlp];
        T v[kDfRows][kDfIlp];
#pragma unroll
        for (int u = 0; u < kDfRows; ++u)
#pragma unroll
          for (int j = 0; j < kDfIlp; ++j) {
            const int64_t kk = k0[u] + j0 + j;
            const bool ok = kk < k1[u];
            c[u][j] = ok ? idx[kk] : 0;
            v[u][j] = ok ? val[kk] : T(0);
          }
#pragma unroll
        for (int u = 0; u < kDfRows; ++u)
#pragma unroll
          for (int j = 0; j < kDfIlp; ++j) s[u] += v[u][j] * (z[c[u][j]] + beta * pold[c[u][j]]);
      }
#pragma unroll
      for (int u = 0; u < kDfRows; ++u) {
        const int64_t row = base + (int64_t)u * kPcgThreads;
        if (row < r1) {
          const T pv = z[row] + beta * pold[row];
          q[row] = s[u];
          pq_l += pv * s[u];
        }
      }
    }
    t = block_sum(pq_l, s_red);
    if (threadIdx.x == 0) partA[blockIdx.x] = t;
    if (!grid_sync(st, nb, my_gen)) return;
    const T pq = sum_partials(partA, nb, s_red);
    if (!(pq > T(0))) {
      status = TM_ERR_BREAKDOWN;
      break;
    }
    const T alpha = rz / pq;
    T rz_n = 0, rr_n = 0;
    // every row of p_new is written here by its owner (rows were read as
    // z + beta*pold above, which this CTA's rows still hold in z/pold);
    // kDfRows rows per round, all loads before any store
    for (int64_t base = r0 + threadIdx.x; base < r1; base += kDfRows * kPcgThreads) {
      T zz[kDfRows], po[kDfRows], xx[kDfRows], rr_[kDfRows], qq[kDfRows], di[kDfRows];
#pragma unroll
      for (int u = 0; u < kDfRows; ++u) {
        const int64_t row = base + (int64_t)u * kPcgThreads;
        const bool ok = row < r1;
        zz[u] = ok ? z[row] : T(0);
        po[u] = ok ? pold[row] : T(0);
        xx[u] = ok ? x[row] : T(0);
        rr_[u] = ok ? r[row] : T(0);
        qq[u] = ok ? q[row] : T(0);
        di[u] = ok ? dinv[row] : T(0);
      }
#pragma unroll
      for (int u = 0; u < kDfRows; ++u) {
        const int64_t row = base + (int64_t)u * kPcgThreads;
        if (row < r1) {
          const T pv = zz[u] + beta * po[u];
          const T rv = rr_[u] - alpha * qq[u];
          const T zv = di[u] * rv;
          pnew[row] = pv;
          x[row] = xx[u] + alpha * pv;
          r[row] = rv;
          z[row] = zv;
          rz_n += rv * zv;
          rr_n += rv * rv;
        }
      }
    }
    t = block_sum(rz_n, s_red);
    if (threadIdx.x == 0) partB[blockIdx.x] = t;
    t = block_sum(rr_n, s_red);
    if (threadIdx.x == 0) partC[blockIdx.x] = t;
    if (!grid_sync(st, nb, my_gen)) return;
    const T rzn = sum_partials(partB, nb, s_red);
    rr = sum_partials(partC, nb, s_red);
    beta = rzn / rz;
    rz = rzn;
    T* tmp = pold;
    pold = pnew;
    pnew = tmp;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->iters = it;
    st->res = sqrt((double)rr);
    atomicCAS(&st->status, TM_OK, status);
  }
}


__global__ void split_kernel(int64_t n, const double* __restrict__ src, F2* __restrict__ dst) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    df64 v = tm_from_double(src[i]);
    dst[i] = F2{v.hi, v.lo};
  }
}

__global__ void __launch_bounds__(kPcgThreads, 2)
pcg_df64_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                const F2* __restrict__ val, const double* __restrict__ bd, double* __restrict__ xd, F2* x, F2* r,
                F2* z, F2* p0, F2* p1, F2* q, F2* dinv, double* partials, PcgState* st, double rtol, double atol,
                int maxiter) {
  __shared__ double s_red[32];
  const unsigned nb = gridDim.x;
  unsigned my_gen = 0;
  const int64_t rows_per = (n + nb - 1) / nb;
  const int64_t r0 = min(n, (int64_t)blockIdx.x * rows_per), r1 = min(n, r0 + rows_per);
  const int g = threadIdx.x / kGroup, lane = threadIdx.x % kGroup;
  const int ngroups = kPcgThreads / kGroup;
  double* partA = partials;
  double* partB = partials + nb;
  double* partC = partials + 2 * nb;
  const df64 zero{0.f, 0.f};

  // diag^-1, x = x0, r = b - A x, z = D^-1 r, p = z
  df64 rz_l = zero, rr_l = zero, bb_l = zero;
  for (int64_t base = r0; base < r1; base += ngroups) {
    const int64_t row = base + g;
    const bool valid = row < r1;
    df64 s = zero;
    df64 d = {1.f, 0.f};
    if (valid) {
      for (int64_t k = indptr[row] + lane; k < indptr[row + 1]; k += kGroup) {
        const int c = idx[k];
        const df64 v = ld2(val, k);
        if (c == row) d = v;
        s += v * tm_from_double(xd[c]);
      }
    }
    // the diagonal lives in exactly one lane of the group; find it
    float dh = (d.hi != 1.f || d.lo != 0.f) ? 1.f : 0.f;
#pragma unroll
    for (int o = kGroup / 2; o > 0; o >>= 1) {
      df64 t{__shfl_down_sync(0xffffffffu, s.hi, o, kGroup), __shfl_down_sync(0xffffffffu, s.lo, o, kGroup)};
      s += t;
    }
    // broadcast the diagonal from the lane that saw it (or keep 1)
    unsigned m = __ballot_sync(0xffffffffu, valid && dh != 0.f);
    const unsigned grp_mask = 0xffu << ((threadIdx.x & 31) & ~(kGroup - 1));
    const unsigned hit = m & grp_mask;
    const int src = hit ? __ffs(hit) - 1 : ((threadIdx.x & 31) & ~(kGroup - 1));
    df64 dd{__shfl_sync(0xffffffffu, d.hi, src), __shfl_sync(0xffffffffu, d.lo, src)};
    if (valid && lane == 0) {
      const df64 di = (dd.hi != 0.f) ? df64{1.f, 0.f} / dd : df64{1.f, 0.f};
      const df64 bv = tm_from_double(bd[row]);
      const df64 rv = bv - s;
      const df64 zv = di * rv;
      st2(dinv, row, di);
      st2(x, row, tm_from_double(xd[row]));
      st2(r, row, rv);
      st2(z, row, zv);
      st2(p0, row, zv);
      rz_l += rv * zv;
      rr_l += rv * rv;
      bb_l += bv * bv;
    }
  }
  double t = block_sum(tm_to_double(rz_l), s_red);
  if (threadIdx.x == 0) partA[blockIdx.x] = t;
  t = block_sum(tm_to_double(rr_l), s_red);
  if (threadIdx.x == 0) partB[blockIdx.x] = t;
  t = block_sum(tm_to_double(bb_l), s_red);
  if (threadIdx.x == 0) partC[blockIdx.x] = t;
  if (!grid_sync(st, nb, my_gen)) return;
  double rz = sum_partials(partA, nb, s_red);
  double rr = sum_partials(partB, nb, s_red);
  const double bb = sum_partials(partC, nb, s_red);
  const double bnorm = sqrt(bb);
  const double tol = fmax(rtol * bnorm, atol);
  if (blockIdx.x == 0 && threadIdx.x == 0) st->bnorm = bnorm;
  if (!grid_sync(st, nb, my_gen)) return;

  df64 beta = zero;
  F2* pold = p0;
  F2* pnew = p1;
  int it = 0;
  int status = TM_ERR_MAXITER;
  for (; it <= maxiter; ++it) {
    if (sqrt(rr) <= tol) {
      status = TM_OK;
      break;
    }
    if (it == maxiter) break;
    df64 pq_l = zero;
    // one thread per row, kDfRows rows at a time, kDfIlp entries of each row
    // per round with every load of the round issued before the first use
    // (the gathers of a round are independent, so they overlap in flight)
    for (int64_t base = r0 + threadIdx.x; base < r1; base += kDfRows * kPcgThreads) {
      int64_t k0[kDfRows], k1[kDfRows];
      df64 s[kDfRows];
#pragma unroll
      for (int u = 0; u < kDfRows; ++u) {
        const int64_t row = base + (int64_t)u * kPcgThreads;
        const bool ok = row < r1;
        k0[u] = ok ? indptr[row] : 0;
        k1[u] = ok ? indptr[row + 1] : 0;
        s[u] = zero;
      }
      for (int64_t j0 = 0;; j0 += kDfIlp) {
        bool more = false;
#pragma unroll
        for (int u = 0; u < kDfRows; ++u) more |= k0[u] + j0 < k1[u];
        if (!more) break;
        int c[kDfRows][kDfIlp];
        F2 v[kDfRows][kDfIlp];
#pragma unroll
        for (int u = 0; u < kDfRows; ++u)
#pragma unroll
          for (int j = 0; j < kDfIlp; ++j) {
            const int64_t kk = k0[u] + j0 + j;
            const bool ok = kk < k1[u];
            c[u][j] = ok ? idx[kk] : 0;
            v[u][j] = ok ? val[kk] : F2{0.f, 0.f};
          }
#pragma unroll
        for (int u = 0; u < kDfRows; ++u)
#pragma unroll
          for (int j = 0; j < kDfIlp; ++j)
            s[u] += df64{v[u][j].hi, v[u][j].lo} * (ld2(z, c[u][j]) + beta * ld2(pold, c[u][j]));
      }
#pragma unroll
      for (int u = 0; u < kDfRows; ++u) {
        const int64_t row = base + (int64_t)u * kPcgThreads;
        if (row < r1) {
          const df64 pv = ld2(z, row) + beta * ld2(pold, row);
          st2(q, row, s[u]);
          pq_l += pv * s[u];
        }
      }
    }
    t = block_sum(tm_to_double(pq_l), s_red);
    if (threadIdx.x == 0) partA[blockIdx.x] = t;
    if (!grid_sync(st, nb, my_gen)) return;
    const double pq = sum_partials(partA, nb, s_red);
    if (!(pq > 0.0)) {
      status = TM_ERR_BREAKDOWN;
      break;
    }
    const df64 alpha = tm_from_double(rz / pq);
    df64 rz_n = zero, rr_n = zero;
    // kDfRows rows per round, all loads before any store (the vectors are
    // distinct arrays, which the compiler cannot prove)
    for (int64_t base = r0 + threadIdx.x; base < r1; base += kDfRows * kPcgThreads) {
      F2 zz[kDfRows], po[kDfRows], xx[kDfRows], rr_[kDfRows], qq[kDfRows], di[kDfRows];
#pragma unroll
      for (int u = 0; u < kDfRows; ++u) {
        const int64_t row = base + (int64_t)u * kPcgThreads;
        const bool ok = row < r1;
        const F2 zf{0.f, 0.f};
        zz[u] = ok ? z[row] : zf;
        po[u] = ok ? pold[row] : zf;
        xx[u] = ok ? x[row] : zf;
        rr_[u] = ok ? r[row] : zf;
        qq[u] = ok ? q[row] : zf;
        di[u] = ok ? dinv[row] : zf;
      }
#pragma unroll
      for (int u = 0; u < kDfRows; ++u) {
        const int64_t row = base + (int64_t)u * kPcgThreads;
        if (row < r1) {
          const df64 pv = df64{zz[u].hi, zz[u].lo} + beta * df64{po[u].hi, po[u].lo};
          const df64 rv = df64{rr_[u].hi, rr_[u].lo} - alpha * df64{qq[u].hi, qq[u].lo};
          const df64 zv = df64{di[u].hi, di[u].lo} * rv;
          st2(pnew, row, pv);
          st2(x, row, df64{xx[u].hi, xx[u].lo} + alpha * pv);
          st2(r, row, rv);
          st2(z, row, zv);
          rz_n += rv * zv;
          rr_n += rv * rv;
        }
      }
    }
    t = block_sum(tm_to_double(rz_n), s_red);
    if (threadIdx.x == 0) partB[blockIdx.x] = t;
    t = block_sum(tm_to_double(rr_n), s_red);
    if (threadIdx.x == 0) partC[blockIdx.x] = t;
    if (!grid_sync(st, nb, my_gen)) return;
    const double rzn = sum_partials(partB, nb, s_red);
    rr = sum_partials(partC, nb, s_red);
    beta = tm_from_double(rzn / rz);
    rz = rzn;
    F2* tmp = pold;
    pold = pnew;
    pnew = tmp;
  }
  for (int64_t row = r0 + threadIdx.x; row < r1; row += kPcgThreads) xd[row] = tm_to_double(ld2(x, row));
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->iters = it;
    st->res = sqrt(rr);
    atomicCAS(&st->status, TM_OK, status);
  }
}

template <class T>
__global__ void diag_inv_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                                const T* __restrict__ val, T* __restrict__ dinv) {
  int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= n) return;
  int64_t lo = indptr[row], hi = indptr[row + 1];
  T d = T(1);  // missing diagonal -> 1 (torch_solve.py:24-49, at_least=1)
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    int c = idx[mid];
    if (c == row) {
      d = val[mid];
      break;
    }
    if (c < row) lo = mid + 1; else hi = mid;
  }
  dinv[row] = d != T(0) ? T(1) / d : T(1);
}

template <class T>
__global__ void gather_kernel(int64_t n, const int64_t* __restrict__ map, const T* __restrict__ src, T* __restrict__ dst) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[map[i]];
}

// f_i = rhs[inner_dof[i]] - sum_{k in row i of K_io} K_io[k] * u_o[col[k]]
template <class T>
__global__ void condense_rhs_kernel(int64_t n_inner, const int64_t* __restrict__ inner_dof, const T* __restrict__ rhs,
                                    const int64_t* __restrict__ io_ptr, const int32_t* __restrict__ io_idx,
                                    const T* __restrict__ io_val, const T* __restrict__ u_o, T* __restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n_inner) return;
  T s = 0;
  for (int64_t k = io_ptr[i]; k < io_ptr[i + 1]; ++k) s += io_val[k] * u_o[io_idx[k]];
  out[i] = rhs[inner_dof[i]] - s;
}

template <class T>
__global__ void scatter_kernel(int64_t n, const int64_t* __restrict__ map, const T* __restrict__ src, T* __restrict__ dst) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dst[map[i]] = src[i];
}

}  // namespace tmg

extern "C" int64_t tm_pcg_workspace_bytes(int32_t dtype, int64_t n, int64_t nnz, int32_t max_blocks) {
  if (n < 0 || nnz < 0 || max_blocks < 0 || (dtype != TM_F32 && dtype != TM_F64)) return -TM_ERR_INVALID;
  if (dtype == TM_F64)  // state | 7 df64 vectors | df64 values | double partials
    return 256 + 8 * (7 * n + nnz + 3 * (int64_t)max_blocks);
  // state | dinv r z p0 p1 q (6n) | partials (3 * blocks)
  return 256 + 4 * (6 * n + 3 * (int64_t)max_blocks);
}

extern "C" int tm_pcg_max_blocks(int32_t dtype) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (dtype == TM_F64)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tmg::pcg_df64_kernel, tmg::kPcgThreads, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tmg::pcg_kernel<float>, tmg::kPcgThreads, 0);
  return sms * (per_sm > 2 ? 2 : per_sm);
}

template <class T>
static int launch_pcg(int64_t n, const int64_t* indptr, const int32_t* indices, const T* values, const T* b, T* x,
                      double rtol, double atol, int maxiter, char* w, int nb, cudaStream_t s) {
  tmg::PcgState* st = reinterpret_cast<tmg::PcgState*>(w);
  T* base = reinterpret_cast<T*>(w + 256);
  T* dinv = base;
  T* r = base + n;
  T* z = base + 2 * n;
  T* p0 = base + 3 * n;
  T* p1 = base + 4 * n;
  T* q = base + 5 * n;
  T* partials = base + 6 * n;
  if (cudaMemsetAsync(st, 0, sizeof(tmg::PcgState), s) != cudaSuccess) return TM_ERR_CUDA;
  tmg::diag_inv_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, indptr, indices, values, dinv);
  if (cudaPeekAtLastError() != cudaSuccess) return TM_ERR_CUDA;
  const T* cdinv = dinv;
  void* args[] = {(void*)&n, (void*)&indptr, (void*)&indices, (void*)&values, (void*)&cdinv, (void*)&b, (void*)&x,
                  (void*)&r, (void*)&z, (void*)&p0, (void*)&p1, (void*)&q, (void*)&partials, (void*)&st,
                  (void*)&rtol, (void*)&atol, (void*)&maxiter};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)tmg::pcg_kernel<T>, dim3(nb), dim3(tmg::kPcgThreads), args,
                                              0, s);
  return e == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

static int launch_pcg_df64(int64_t n, const int64_t* indptr, const int32_t* indices, const double* values,
                           const double* b, double* x, double rtol, double atol, int maxiter, char* w, int nb,
                           cudaStream_t s) {
  int64_t nnz = 0;
  if (cudaMemcpyAsync(&nnz, indptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess) return TM_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return TM_ERR_CUDA;
  tmg::PcgState* st = reinterpret_cast<tmg::PcgState*>(w);
  tmg::F2* base = reinterpret_cast<tmg::F2*>(w + 256);
  tmg::F2 *xv = base, *r = base + n, *z = base + 2 * n, *p0 = base + 3 * n, *p1 = base + 4 * n, *q = base + 5 * n,
          *dinv = base + 6 * n, *val = base + 7 * n;
  double* partials = reinterpret_cast<double*>(val + nnz);
  if (cudaMemsetAsync(st, 0, sizeof(tmg::PcgState), s) != cudaSuccess) return TM_ERR_CUDA;
  if (nnz > 0) tmg::split_kernel<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, values, val);
  if (cudaPeekAtLastError() != cudaSuccess) return TM_ERR_CUDA;
  const tmg::F2* cval = val;
  void* args[] = {(void*)&n, (void*)&indptr, (void*)&indices, (void*)&cval, (void*)&b, (void*)&x, (void*)&xv,
                  (void*)&r, (void*)&z, (void*)&p0, (void*)&p1, (void*)&q, (void*)&dinv, (void*)&partials,
                  (void*)&st, (void*)&rtol, (void*)&atol, (void*)&maxiter};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)tmg::pcg_df64_kernel, dim3(nb), dim3(tmg::kPcgThreads),
                                              args, 0, s);
  return e == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_pcg_jacobi(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices,
                             const void* values, const void* b, void* x, double rtol, double atol, int32_t maxiter,
                             void* work, int64_t work_bytes, void* stream) {
  if (n < 0 || maxiter < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!indptr || !indices || !values || !b || !x || !work) return TM_ERR_INVALID;
  const int nb = tm_pcg_max_blocks(dtype);
  if (nb <= 0) return TM_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* w = static_cast<char*>(work);
  if (dtype == TM_F64) {
    int64_t nnz = 0;
    if (cudaMemcpyAsync(&nnz, indptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return TM_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return TM_ERR_CUDA;
    if (work_bytes < tm_pcg_workspace_bytes(dtype, n, nnz, nb)) return TM_ERR_INDEX;
    return launch_pcg_df64(n, indptr, indices, (const double*)values, (const double*)b, (double*)x, rtol, atol,
                           maxiter, w, nb, s);
  }
  if (work_bytes < tm_pcg_workspace_bytes(dtype, n, 0, nb)) return TM_ERR_INDEX;
  if (dtype == TM_F32)
    return launch_pcg<float>(n, indptr, indices, (const float*)values, (const float*)b, (float*)x, rtol, atol,
                             maxiter, w, nb, s);
  return TM_ERR_INVALID;
}

// Reads the solver record written by the last tm_pcg_jacobi on this
// workspace (synchronises the stream).
extern "C" int tm_pcg_result(const void* work, int32_t* iters, double* res, double* bnorm, void* stream) {
  if (!work) return TM_ERR_INVALID;
  tmg::PcgState h;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(&h, work, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return TM_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return TM_ERR_CUDA;
  if (iters) *iters = h.iters;
  if (res) *res = h.res;
  if (bnorm) *bnorm = h.bnorm;
  return h.status;
}

extern "C" int tm_csr_diagonal_inverse(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices,
                                       const void* values, void* out, void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!indptr || !indices || !values || !out) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned grid = (unsigned)((n + 255) / 256);
  if (dtype == TM_F64)
    tmg::diag_inv_kernel<double><<<grid, 256, 0, s>>>(n, indptr, indices, (const double*)values, (double*)out);
  else if (dtype == TM_F32)
    tmg::diag_inv_kernel<float><<<grid, 256, 0, s>>>(n, indptr, indices, (const float*)values, (float*)out);
  else
    return TM_ERR_INVALID;
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_gather(int32_t dtype, int64_t n, const int64_t* map, const void* src, void* dst, void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!map || !src || !dst) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned grid = (unsigned)((n + 255) / 256);
  if (dtype == TM_F64)
    tmg::gather_kernel<double><<<grid, 256, 0, s>>>(n, map, (const double*)src, (double*)dst);
  else if (dtype == TM_F32)
    tmg::gather_kernel<float><<<grid, 256, 0, s>>>(n, map, (const float*)src, (float*)dst);
  else
    return TM_ERR_INVALID;
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_scatter(int32_t dtype, int64_t n, const int64_t* map, const void* src, void* dst, void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!map || !src || !dst) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned grid = (unsigned)((n + 255) / 256);
  if (dtype == TM_F64)
    tmg::scatter_kernel<double><<<grid, 256, 0, s>>>(n, map, (const double*)src, (double*)dst);
  else if (dtype == TM_F32)
    tmg::scatter_kernel<float><<<grid, 256, 0, s>>>(n, map, (const float*)src, (float*)dst);
  else
    return TM_ERR_INVALID;
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_condense_rhs(int32_t dtype, int64_t n_inner, const int64_t* inner_dof, const void* rhs,
                               const int64_t* io_indptr, const int32_t* io_indices, const void* io_values,
                               const void* u_outer, void* out, void* stream) {
  if (n_inner < 0) return TM_ERR_INVALID;
  if (n_inner == 0) return TM_OK;
  if (!inner_dof || !rhs || !io_indptr || !out) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned grid = (unsigned)((n_inner + 255) / 256);
  if (dtype == TM_F64)
    tmg::condense_rhs_kernel<double><<<grid, 256, 0, s>>>(n_inner, inner_dof, (const double*)rhs, io_indptr,
                                                          io_indices, (const double*)io_values,
                                                          (const double*)u_outer, (double*)out);
  else if (dtype == TM_F32)
    tmg::condense_rhs_kernel<float><<<grid, 256, 0, s>>>(n_inner, inner_dof, (const float*)rhs, io_indptr,
                                                         io_indices, (const float*)io_values,
                                                         (const float*)u_outer, (float*)out);
  else
    return TM_ERR_INVALID;
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// Allocation-free float32 Jacobi-PCG.
//
// Some callers cannot allocate device memory at the moment they need a solve:
// a host runtime that plans every device buffer up front and forbids
// allocation afterwards (embedded / real-time deployments), a plugin that
// receives its vectors from a host framework owning the only allocator, or a
// solve issued while that framework's memory pool is exhausted.  For them
// tm_pcg_jacobi_noalloc keeps the solver's scratch (state word, six vectors
// dinv, r, z, p0, p1, q, and the reduction partials) in a fixed array that lives in this library's own
// device memory, so the caller passes only the matrix, b and x.
//
// The array is kTmNoAllocScratchBytes (32 MiB) on every GPU that loads the
// library and stays reserved until the process exits.  It is shared by every
// call: two calls whose kernels overlap on the GPU (different streams, or
// different host threads, on one device) race on it and must be serialised
// by the caller.  The solver state at its start is cleared on every call.
// Limit: n <= kTmNoAllocMaxRows rows (the vectors must fit the array).
// Every call looks up the array's device address on the current device
// (cudaGetSymbolAddress, a host-side query that allocates nothing), so the
// address stays valid across a cudaDeviceReset.  The call synchronises its
// stream to read the result back, so it cannot be issued while that stream
// is being captured into a CUDA graph: a capturing stream is rejected with
// TM_ERR_INVALID before anything is launched.
// ---------------------------------------------------------------------------
constexpr size_t kTmNoAllocScratchBytes = size_t(32) << 20;
constexpr int64_t kTmNoAllocMaxRows = 1000000;
static __device__ __align__(256) unsigned char tm_pcg_noalloc_scratch[kTmNoAllocScratchBytes];

static int noalloc_scratch(void** out) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, tm_pcg_noalloc_scratch) != cudaSuccess || !p) return TM_ERR_CUDA;
  *out = p;
  return TM_OK;
}

extern "C" int tm_pcg_jacobi_noalloc(int64_t n, const int64_t* indptr, const int32_t* indices, const float* values,
                                     const float* b, float* x, double rtol, double atol, int32_t maxiter,
                                     int32_t* out_iters, double* out_res, void* stream) {
  if (out_iters) *out_iters = 0;
  if (out_res) *out_res = 0.0;
  if (n < 0 || maxiter < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!indptr || !indices || !values || !b || !x) return TM_ERR_INVALID;
  if (n > kTmNoAllocMaxRows) return TM_ERR_INDEX;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cap) != cudaSuccess) return TM_ERR_CUDA;
  if (cap != cudaStreamCaptureStatusNone) return TM_ERR_INVALID;
  const int nb = tm_pcg_max_blocks(TM_F32);
  if (nb <= 0) return TM_ERR_CUDA;
  if (tm_pcg_workspace_bytes(TM_F32, n, 0, nb) > (int64_t)kTmNoAllocScratchBytes) return TM_ERR_INDEX;
  void* w = nullptr;
  int st = noalloc_scratch(&w);
  if (st != TM_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  st = launch_pcg<float>(n, indptr, indices, values, b, x, rtol, atol, maxiter, static_cast<char*>(w), nb, s);
  if (st != TM_OK) return st;
  return tm_pcg_result(w, out_iters, out_res, nullptr, stream);
}

// ---------------------------------------------------------------------------
// Self-test of the bounded grid barrier.  A cooperative launch in which CTA 0
// returns without arriving: every other CTA's wait runs out after `spins`
// polls (32 ns apart), the barrier records TM_ERR_TIMEOUT and every CTA
// returns.  Nothing is left waiting, so the context stays usable.
// ---------------------------------------------------------------------------
namespace tmg {
__global__ void barrier_timeout_kernel(PcgState* st, long long spins) {
  unsigned gen = 0;
  if (blockIdx.x == 0) return;  // the CTA that never arrives
  grid_sync(st, gridDim.x, gen, spins);
}
}  // namespace tmg

extern "C" int tm_selftest_barrier_timeout(int32_t n_blocks, int64_t spins, int32_t* out_status, void* work,
                                           void* stream) {
  if (out_status) *out_status = TM_OK;
  if (n_blocks < 2 || spins < 1 || spins > tmg::kGridSpinLimit || !work || !out_status) return TM_ERR_INVALID;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TM_ERR_CUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tmg::barrier_timeout_kernel, 32, 0);
  if (n_blocks > sms * per_sm) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  tmg::PcgState* st = static_cast<tmg::PcgState*>(work);
  if (cudaMemsetAsync(st, 0, sizeof(tmg::PcgState), s) != cudaSuccess) return TM_ERR_CUDA;
  long long sp = spins;
  void* args[] = {(void*)&st, (void*)&sp};
  if (cudaLaunchCooperativeKernel((const void*)tmg::barrier_timeout_kernel, dim3(n_blocks), dim3(32), args, 0, s) !=
      cudaSuccess)
    return TM_ERR_CUDA;
  tmg::PcgState h;
  if (cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return TM_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return TM_ERR_CUDA;
  *out_status = h.status;
  return TM_OK;
}
