// CSR pattern build on the GPU: the unique (row, col) pairs of every element's
// node pairs in canonical order (rows ascending, columns ascending inside a
// row) and the slot map that sends each element entry (e, a, b) to its CSR
// position.  This replaces the reference's from_mesh pattern build
// (assemble/element_assembler.py:838-866: element (row, col) pairs, scipy
// coo -> csr -> coo to deduplicate and sort, then the per-entry `elem_eids`).
//
// Steps (all deterministic: every output is a function of the connectivity
// alone, whatever the order atomics resolve in):
//   1. node -> element incidence: count per node, exclusive scan, fill;
//   2. per row (one warp), the row's columns are the nodes of its incident
//      elements; the warp enumerates them in ascending order by repeated
//      "smallest candidate above the last one" reductions, counting them
//      (pass 1) or writing them (pass 2);
//   3. exclusive scan of the row counts -> indptr;
//   4. slots: each (element, local node a) binary-searches the columns of its
//      own row.
#include <cstdint>
#include <climits>
#include "tm_common.cuh"
#include "../../include/tensormesh_gb300.h"

namespace tmg {

constexpr int kScanThreads = 1024;

__global__ void incidence_count_kernel(const int32_t* __restrict__ el, int64_t n_entries, int32_t* __restrict__ cnt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n_entries) atomicAdd(cnt + el[i], 1);
}

__global__ void incidence_fill_kernel(const int32_t* __restrict__ el, int64_t n_entries, int B,
                                      const int64_t* __restrict__ nptr, int32_t* __restrict__ cursor,
                                      int32_t* __restrict__ nelem) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n_entries) return;
  const int v = el[i];
  const int k = atomicAdd(cursor + v, 1);
  nelem[nptr[v] + k] = (int32_t)(i / B);
}

// Exclusive scan of int32 counts into int64 offsets (out[n] = total), in three
// launches: per-block sums, a scan of those sums in one block, the final pass.
__global__ void scan_block_sums_kernel(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ bsum) {
  __shared__ int64_t s[32];
  const int64_t i = blockIdx.x * (int64_t)kScanThreads + threadIdx.x;
  int64_t v = i < n ? in[i] : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    int64_t t = s[threadIdx.x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) bsum[blockIdx.x] = t;
  }
}

__global__ void scan_sums_kernel(int64_t* __restrict__ bsum, int64_t nb) {
  // one block: each thread scans a contiguous run of the block sums
  __shared__ int64_t s[kScanThreads];
  const int t = threadIdx.x;
  const int64_t per = (nb + kScanThreads - 1) / kScanThreads;
  const int64_t b0 = t * per, b1 = min(nb, b0 + per);
  int64_t run = 0;
  for (int64_t i = b0; i < b1; ++i) run += bsum[i];
  s[t] = run;
  __syncthreads();
  for (int o = 1; o < kScanThreads; o <<= 1) {
    const int64_t add = t >= o ? s[t - o] : 0;
    __syncthreads();
    s[t] += add;
    __syncthreads();
  }
  int64_t acc = s[t] - run;  // exclusive prefix of this thread's run
  for (int64_t i = b0; i < b1; ++i) {
    const int64_t v = bsum[i];
    bsum[i] = acc;
    acc += v;
  }
}

__global__ void scan_final_kernel(const int32_t* __restrict__ in, int64_t n, const int64_t* __restrict__ boff,
                                  int64_t* __restrict__ out) {
  __shared__ int64_t s[32];
  const int64_t i = blockIdx.x * (int64_t)kScanThreads + threadIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t v = i < n ? in[i] : 0;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s[w] = x;
  __syncthreads();
  if (w == 0) {
    int64_t t = s[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    s[lane] = t;
  }
  __syncthreads();
  const int64_t excl = boff[blockIdx.x] + (w > 0 ? s[w - 1] : 0) + x - v;
  if (i < n) out[i] = excl;
  if (i == n - 1) out[n] = excl + v;
}

// The first 32 * kRegCand candidates of a row stay in registers; rows with
// more (high valence) read the rest again on every step.
constexpr int kRegCand = 4;

// Pass over one row's candidate columns with a warp: calls emit(k, col) for
// the k-th distinct column in ascending order; returns the count.
template <class Emit>
__device__ __forceinline__ int row_columns(const int32_t* __restrict__ el, int B, const int32_t* __restrict__ nelem,
                                           int64_t e0, int64_t e1, Emit emit) {
  const int lane = threadIdx.x & 31;
  const int64_t ncand = (e1 - e0) * B;
  auto cand = [&](int64_t c) { return el[(int64_t)nelem[e0 + c / B] * B + (int)(c % B)]; };
  int reg[kRegCand];
#pragma unroll
  for (int k = 0; k < kRegCand; ++k) {
    const int64_t c = lane + 32 * k;
    reg[k] = c < ncand ? cand(c) : INT_MAX;
  }
  int last = INT_MIN, count = 0;
  for (;;) {
    int m = INT_MAX;
#pragma unroll
    for (int k = 0; k < kRegCand; ++k)
      if (reg[k] > last && reg[k] < m) m = reg[k];
    for (int64_t c = 32 * kRegCand + lane; c < ncand; c += 32) {
      const int col = cand(c);
      if (col > last && col < m) m = col;
    }
    m = __reduce_min_sync(0xffffffffu, m);
    if (m == INT_MAX) break;
    emit(count, m);
    ++count;
    last = m;
  }
  return count;
}

__global__ void row_count_kernel(const int32_t* __restrict__ el, int B, int64_t n_points,
                                 const int64_t* __restrict__ nptr, const int32_t* __restrict__ nelem,
                                 int32_t* __restrict__ rcnt) {
  const int64_t r = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= n_points) return;  // whole warps leave together
  const int n = row_columns(el, B, nelem, nptr[r], nptr[r + 1], [](int, int) {});
  if ((threadIdx.x & 31) == 0) rcnt[r] = n;
}

__global__ void row_fill_kernel(const int32_t* __restrict__ el, int B, int64_t n_points,
                                const int64_t* __restrict__ nptr, const int32_t* __restrict__ nelem,
                                const int64_t* __restrict__ indptr, int32_t* __restrict__ indices) {
  const int64_t r = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= n_points) return;
  const int lane = threadIdx.x & 31;
  int32_t* out = indices + indptr[r];
  row_columns(el, B, nelem, nptr[r], nptr[r + 1], [&](int k, int col) {
    if (lane == 0) out[k] = col;
  });
}

__global__ void slot_kernel(const int32_t* __restrict__ el, int64_t n_entries, int B,
                            const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                            int64_t* __restrict__ slots) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // (element, a)
  if (i >= n_entries) return;
  const int64_t e = i / B;
  const int row = el[i];
  const int64_t lo0 = indptr[row], hi0 = indptr[row + 1];
  for (int b = 0; b < B; ++b) {
    const int col = el[e * B + b];
    int64_t lo = lo0, hi = hi0;  // first position with indices >= col
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (indices[mid] < col) lo = mid + 1; else hi = mid;
    }
    slots[i * B + b] = lo;
  }
}

}  // namespace tmg

namespace {
size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
struct PatternWork {
  int32_t* cnt;     // [N] incidence counts, then fill cursors, then row counts
  int64_t* nptr;    // [N + 1]
  int32_t* nelem;   // [E * B]
  int64_t* bsum;    // [ceil(N / kScanThreads)]
};
PatternWork carve(void* work, int64_t E, int B, int64_t N) {
  char* p = static_cast<char*>(work);
  PatternWork w;
  w.cnt = reinterpret_cast<int32_t*>(p);
  p += align256(sizeof(int32_t) * (size_t)N);
  w.nptr = reinterpret_cast<int64_t*>(p);
  p += align256(sizeof(int64_t) * (size_t)(N + 1));
  w.nelem = reinterpret_cast<int32_t*>(p);
  p += align256(sizeof(int32_t) * (size_t)E * B);
  w.bsum = reinterpret_cast<int64_t*>(p);
  return w;
}
int scan(const int32_t* in, int64_t n, int64_t* bsum, int64_t* out, cudaStream_t s) {
  const int64_t nb = (n + tmg::kScanThreads - 1) / tmg::kScanThreads;
  if (nb == 0) return cudaMemsetAsync(out, 0, sizeof(int64_t), s) == cudaSuccess ? TM_OK : TM_ERR_CUDA;
  tmg::scan_block_sums_kernel<<<(unsigned)nb, tmg::kScanThreads, 0, s>>>(in, n, bsum);
  tmg::scan_sums_kernel<<<1, tmg::kScanThreads, 0, s>>>(bsum, nb);
  tmg::scan_final_kernel<<<(unsigned)nb, tmg::kScanThreads, 0, s>>>(in, n, bsum, out);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}
}  // namespace

extern "C" int64_t tm_pattern_workspace_bytes(int64_t n_elements, int32_t n_basis, int64_t n_points) {
  if (n_elements < 0 || n_basis < 1 || n_points < 0) return -1;
  const int64_t nb = (n_points + tmg::kScanThreads - 1) / tmg::kScanThreads + 1;
  return (int64_t)(align256(sizeof(int32_t) * (size_t)n_points) + align256(sizeof(int64_t) * (size_t)(n_points + 1)) +
                   align256(sizeof(int32_t) * (size_t)n_elements * n_basis) + align256(sizeof(int64_t) * (size_t)nb));
}

extern "C" int tm_pattern_count(const int32_t* elements, int64_t n_elements, int32_t n_basis, int64_t n_points,
                                void* work, int64_t* out_indptr, void* stream) {
  if (n_elements < 0 || n_basis < 1 || n_points < 0 || !work || !out_indptr) return TM_ERR_INVALID;
  if (n_elements > 0 && !elements) return TM_ERR_INVALID;
  if (n_elements * n_basis >= (int64_t)INT_MAX) return TM_ERR_INDEX;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n_points == 0) return cudaMemsetAsync(out_indptr, 0, sizeof(int64_t), s) == cudaSuccess ? TM_OK : TM_ERR_CUDA;
  PatternWork w = carve(work, n_elements, n_basis, n_points);
  const int64_t ne = n_elements * n_basis;
  if (cudaMemsetAsync(w.cnt, 0, sizeof(int32_t) * n_points, s) != cudaSuccess) return TM_ERR_CUDA;
  if (ne > 0) tmg::incidence_count_kernel<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(elements, ne, w.cnt);
  int st = scan(w.cnt, n_points, w.bsum, w.nptr, s);
  if (st != TM_OK) return st;
  if (cudaMemsetAsync(w.cnt, 0, sizeof(int32_t) * n_points, s) != cudaSuccess) return TM_ERR_CUDA;
  if (ne > 0)
    tmg::incidence_fill_kernel<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(elements, ne, n_basis, w.nptr, w.cnt,
                                                                         w.nelem);
  const unsigned rb = (unsigned)((n_points + 7) / 8);  // a warp per row, 8 rows per 256-thread block
  tmg::row_count_kernel<<<rb, 256, 0, s>>>(elements, n_basis, n_points, w.nptr, w.nelem, w.cnt);
  st = scan(w.cnt, n_points, w.bsum, out_indptr, s);
  if (st != TM_OK) return st;
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_pattern_fill(const int32_t* elements, int64_t n_elements, int32_t n_basis, int64_t n_points,
                               const void* work, const int64_t* indptr, int32_t* out_indices, int64_t* out_slots,
                               void* stream) {
  if (n_elements < 0 || n_basis < 1 || n_points < 0 || !work || !indptr || !out_indices) return TM_ERR_INVALID;
  if (n_points == 0 || n_elements == 0) return TM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  PatternWork w = carve(const_cast<void*>(work), n_elements, n_basis, n_points);
  const unsigned rb = (unsigned)((n_points + 7) / 8);
  tmg::row_fill_kernel<<<rb, 256, 0, s>>>(elements, n_basis, n_points, w.nptr, w.nelem, indptr, out_indices);
  if (out_slots) {
    const int64_t ne = n_elements * n_basis;
    tmg::slot_kernel<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(elements, ne, n_basis, indptr, out_indices,
                                                                 out_slots);
  }
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

// ---- Morton (Z-order) keys of points, for the spatial partitions ---------
// Point i, coordinate d is quantised to q = rint((x - lo_d) / max(hi_d - lo_d,
// 1e-300) * (2^bits - 1)) (IEEE double, round half to even) and bit b of q
// goes to bit b D + d of the key: the same arithmetic as the torch
// restatement this replaces, so the keys are identical.
namespace tmg {
__global__ void morton_keys_kernel(int64_t n, int dim, const double* __restrict__ x, const double* __restrict__ lo,
                                   const double* __restrict__ hi, int bits, int64_t* __restrict__ keys) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double scale = (double)((1ll << bits) - 1);
  unsigned long long key = 0ull;
  for (int d = 0; d < dim; ++d) {
    const double span = fmax(hi[d] - lo[d], 1e-300);
    const unsigned long long q = (unsigned long long)(long long)rint((x[i * dim + d] - lo[d]) / span * scale);
    for (int b = 0; b < bits; ++b) key |= ((q >> b) & 1ull) << (b * dim + d);
  }
  keys[i] = (int64_t)key;
}
}  // namespace tmg

extern "C" int tm_morton_keys(int64_t n, int32_t dim, const double* coords, const double* lo, const double* hi,
                              int32_t bits, int64_t* keys, void* stream) {
  if (n < 0 || dim < 1 || dim > 3 || bits < 1 || bits * dim > 63) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!coords || !lo || !hi || !keys) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  tmg::morton_keys_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, dim, coords, lo, hi, bits, keys);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}
