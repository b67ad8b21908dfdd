// Batched assemble + Jacobi-PCG of many independent meshes in ONE persistent
// launch (designed to be captured once in a CUDA graph and replayed).
//
// Work decomposition: a thread-block cluster of C CTAs is the unit that owns
// one instance at a time.  Clusters pop instances (largest first) from a
// global counter; for each instance the cluster
//   1. assembles the instance's stiffness matrix and load vector with the
//      patch-assembly device code (patches of the instance round-robin over
//      the C CTAs), writing CSR values / b directly;
//   2. runs Jacobi-PCG on the instance's interior dofs (Dirichlet dofs are
//      masked: x = r = z = p = 0 there, which is CG on K_ii exactly), with
//      the instance's rows split over the C CTAs.  Dot products reduce per
//      CTA and are combined through distributed shared memory in a fixed
//      order after a hardware cluster barrier -- deterministic, and no
//      spin-wait anywhere (cluster barriers are co-scheduled by construction);
//   3. records iterations, recurrence residual and a status per instance.
// Instances never share rows, so clusters never wait on each other.
#include <cooperative_groups.h>

#include "assemble_impl.cuh"

namespace cg = cooperative_groups;

namespace tmg {

struct BatchArgs {
  tm_patch_plan plan;          // union plan; patches of one instance are contiguous
  tm_assemble_args mat;        // matrix form (values -> mat.out)
  tm_assemble_args load;       // load form   (b -> load.out)
  const int32_t* order;        // instances by decreasing size
  const int32_t* inst_pbeg;    // [n_inst+1] patch range of each instance
  const int64_t* inst_rbeg;    // [n_inst+1] row (node) range of each instance
  const int64_t* indptr;       // node-level CSR of the union
  const int32_t* indices;
  const uint8_t* dirichlet;    // [N] 1 = clamped dof (value 0)
  float* x;
  float* r;
  float* z;
  float* p0;
  float* p1;
  float* q;
  float* dinv;
  int32_t* status;             // per instance
  int32_t* iters;
  float* resid;                // recurrence ||r|| / ||b||
  unsigned int* queue;
  int32_t n_inst;
  int32_t maxiter;
  float rtol;
  int32_t chunk;
};

constexpr int kBatchThreads = 512;
constexpr int kRowIlp = 4;  // CSR entries fetched together per row and round
constexpr int kRows = 2;    // rows a thread advances together in the SpMV
constexpr int kVec = 4;     // rows a thread advances together in the vector update

__device__ __forceinline__ double cta_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  __syncthreads();
  return t;  // thread 0
}

// two sums with one pair of barriers; results valid in thread 0
__device__ __forceinline__ void cta_sum2(double& a, double& b, double (*red)[2]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    red[warp][0] = a;
    red[warp][1] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    a = b = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += red[w][0];
      b += red[w][1];
    }
  }
  __syncthreads();
}

// combine one partial per CTA of the cluster, in rank order (same value everywhere)
__device__ __forceinline__ double cluster_combine(cg::cluster_group& cl, double* slot) {
  double s = 0;
  const unsigned n = cl.num_blocks();
  for (unsigned j = 0; j < n; ++j) s += *cl.map_shared_rank(slot, j);
  return s;
}

template <int EL>
__global__ void __launch_bounds__(kBatchThreads, 2) batched_assemble_pcg_kernel(BatchArgs A) {
  cg::cluster_group cl = cg::this_cluster();
  const unsigned rank = cl.block_rank();
  const unsigned C = cl.num_blocks();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  __shared__ double red2[32][2];
  __shared__ double part[2][3];  // [parity][pq, rz, rr]
  __shared__ int task;

  for (;;) {
    if (rank == 0 && threadIdx.x == 0) {
      unsigned t = atomicAdd(A.queue, 1u);
      task = t < (unsigned)A.n_inst ? A.order[t] : -1;
    }
    cl.sync();
    const int k = *cl.map_shared_rank(&task, 0);
    cl.sync();  // every CTA has read rank 0's task before anyone moves on or exits
    if (k < 0) break;

    // ---- 1. assemble the instance (matrix, then load) ----------------------
    const int pb = A.inst_pbeg[k], pe = A.inst_pbeg[k + 1];
    for (int p = pb + (int)rank; p < pe; p += (int)C) {
      assemble_patch<EL, TM_FORM_LAPLACE, 1, float, float>(A.plan, A.mat, p, A.chunk, smem_raw);
      __syncthreads();
      assemble_patch<EL, TM_FORM_LOAD, 1, float, float>(A.plan, A.load, p, A.chunk, smem_raw);
      __syncthreads();
    }
    __threadfence();
    cl.sync();

    // ---- 2. Jacobi-PCG on the interior dofs ----------------------------------
    const int64_t rb = A.inst_rbeg[k], re = A.inst_rbeg[k + 1];
    const int64_t n = re - rb;
    const int64_t per = (n + C - 1) / C;
    const int64_t r0 = rb + min(n, (int64_t)rank * per), r1 = rb + min(n, (int64_t)(rank + 1) * per);
    const float* val = static_cast<const float*>(A.mat.out);
    const float* b = static_cast<const float*>(A.load.out);
    double rz_l = 0, rr_l = 0, bb_l = 0;
    for (int64_t row = r0 + threadIdx.x; row < r1; row += kBatchThreads) {
      const bool fixed = A.dirichlet[row] != 0;
      float d = 1.f;
      for (int64_t kk = A.indptr[row]; kk < A.indptr[row + 1]; ++kk)
        if (A.indices[kk] == row) d = val[kk];
      const float di = (fixed || d == 0.f) ? 0.f : 1.f / d;
      const float rv = fixed ? 0.f : b[row];  // x0 = 0
      const float zv = di * rv;
      A.dinv[row] = di;
      A.x[row] = 0.f;
      A.r[row] = rv;
      A.z[row] = zv;
      A.p0[row] = zv;
      rz_l += (double)rv * zv;
      rr_l += (double)rv * rv;
      bb_l += (double)rv * rv;
    }
    double t0 = cta_sum(rz_l, red), t1 = cta_sum(rr_l, red), t2 = cta_sum(bb_l, red);
    if (threadIdx.x == 0) {
      part[0][0] = t0;
      part[0][1] = t1;
      part[0][2] = t2;
    }
    __threadfence();
    cl.sync();
    double rz = cluster_combine(cl, &part[0][0]);
    double rr = cluster_combine(cl, &part[0][1]);
    const double bb = cluster_combine(cl, &part[0][2]);
    const double tol2 = (double)A.rtol * A.rtol * bb;
    cl.sync();  // part[0] is rewritten below

    float beta = 0.f;
    float* pold = A.p0;
    float* pnew = A.p1;
    int it = 0, st = TM_ERR_MAXITER;
    int par = 1;
    for (; it <= A.maxiter; ++it) {
      if (rr <= tol2) {
        st = TM_OK;
        break;
      }
      if (it == A.maxiter) break;
      double pq_l = 0;
      // one thread per row, kRows rows at a time (rows row, row + T, ...), each
      // row's entries fetched kRowIlp at a time with every load of the round
      // issued before the first use: a warp keeps 32 x kRows x kRowIlp
      // independent gathers in flight instead of one dependent chain per row
      for (int64_t base = r0 + threadIdx.x; base < r1; base += kRows * kBatchThreads) {
        int64_t k0[kRows], k1[kRows];
        float s[kRows];
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
          const int64_t row = base + (int64_t)u * kBatchThreads;
          const bool ok = row < r1;
          k0[u] = ok ? A.indptr[row] : 0;
          k1[u] = ok ? A.indptr[row + 1] : 0;
          s[u] = 0.f;
        }
        for (int64_t j0 = 0;; j0 += kRowIlp) {
          bool more = false;
#pragma unroll
          for (int u = 0; u < kRows; ++u) more |= k0[u] + j0 < k1[u];
          if (!more) break;
          int c[kRows][kRowIlp];
          float v[kRows][kRowIlp];
#pragma unroll
          for (int u = 0; u < kRows; ++u)
#pragma unroll
            for (int j = 0; j < kRowIlp; ++j) {
              const int64_t kk = k0[u] + j0 + j;
              const bool ok = kk < k1[u];
              c[u][j] = ok ? A.indices[kk] : (int)r0;
              v[u][j] = ok ? val[kk] : 0.f;
            }
#pragma unroll
          for (int u = 0; u < kRows; ++u)
#pragma unroll
            for (int j = 0; j < kRowIlp; ++j) s[u] += v[u][j] * (A.z[c[u][j]] + beta * pold[c[u][j]]);
        }
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
          const int64_t row = base + (int64_t)u * kBatchThreads;
          if (row < r1) {
            const bool fixed = A.dirichlet[row] != 0;
            const float pv = A.z[row] + beta * pold[row];
            const float qv = fixed ? 0.f : s[u];
            A.q[row] = qv;
            pq_l += (double)pv * qv;
          }
        }
      }
      t0 = cta_sum(pq_l, red);
      if (threadIdx.x == 0) part[par][0] = t0;
      // the cluster barrier's arrive/wait carry release/acquire semantics at
      // cluster scope: the q rows written above are visible to the other CTAs
      cl.sync();
      const double pq = cluster_combine(cl, &part[par][0]);
      if (!(pq > 0.0)) {
        st = TM_ERR_BREAKDOWN;
        break;
      }
      const float alpha = (float)(rz / pq);
      double rz_n = 0, rr_n = 0;
      // kVec rows per round, every load of the round before any store (the
      // vectors are distinct arrays, but the compiler cannot know that and
      // would otherwise serialise the rows behind one another's stores)
      for (int64_t base = r0 + threadIdx.x; base < r1; base += kVec * kBatchThreads) {
        float zz[kVec], po[kVec], xx[kVec], rr[kVec], qq[kVec], di[kVec];
#pragma unroll
        for (int u = 0; u < kVec; ++u) {
          const int64_t row = base + (int64_t)u * kBatchThreads;
          const bool ok = row < r1;
          zz[u] = ok ? A.z[row] : 0.f;
          po[u] = ok ? pold[row] : 0.f;
          xx[u] = ok ? A.x[row] : 0.f;
          rr[u] = ok ? A.r[row] : 0.f;
          qq[u] = ok ? A.q[row] : 0.f;
          di[u] = ok ? A.dinv[row] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < kVec; ++u) {
          const int64_t row = base + (int64_t)u * kBatchThreads;
          if (row < r1) {
            const float pv = zz[u] + beta * po[u];
            const float rv = rr[u] - alpha * qq[u];
            const float zv = di[u] * rv;
            pnew[row] = pv;
            A.x[row] = xx[u] + alpha * pv;
            A.r[row] = rv;
            A.z[row] = zv;
            rz_n += (double)rv * zv;
            rr_n += (double)rv * rv;
          }
        }
      }
      cta_sum2(rz_n, rr_n, red2);
      if (threadIdx.x == 0) {
        part[par][1] = rz_n;
        part[par][2] = rr_n;
      }
      cl.sync();
      const double rzn = cluster_combine(cl, &part[par][1]);
      rr = cluster_combine(cl, &part[par][2]);
      beta = (float)(rzn / rz);
      rz = rzn;
      float* tmp = pold;
      pold = pnew;
      pnew = tmp;
      par ^= 1;
    }
    if (rank == 0 && threadIdx.x == 0) {
      A.status[k] = st;
      A.iters[k] = it;
      A.resid[k] = (float)sqrt(rr / (bb > 0 ? bb : 1.0));
    }
    cl.sync();  // task / part reuse
  }
}

template <int EL>
int launch_batched(const BatchArgs& A, int cluster, int n_clusters, size_t smem, cudaStream_t s) {
  auto kern = batched_assemble_pcg_kernel<EL>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return TM_ERR_CUDA;
  if (cluster > 8) cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cluster * n_clusters);
  cfg.blockDim = dim3(kBatchThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, kern, A);
  return e == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

}  // namespace tmg

extern "C" int64_t tm_patch_smem_bytes(int32_t element, int32_t form, int32_t n_comp, int32_t dtype,
                                       const tm_patch_plan* plan, int32_t coef_kind, int32_t chunk) {
  if (!plan) return -1;
  const size_t es = dtype == TM_F32 ? 4 : 8;
  // mirrors patch_smem_bytes (element/form generic)
  int D = (element == TM_TRI3 || element == TM_TRI6) ? 2 : 3;
  int B = element == TM_TRI3 ? 3 : element == TM_TRI6 ? 6 : element == TM_TET4 ? 4 : 10;
  int H = form == TM_FORM_ELASTICITY ? D : (form == TM_FORM_LOAD ? n_comp : 1);
  bool load = form == TM_FORM_LOAD;
  size_t SE = load ? (size_t)B * H : (size_t)B * B * H * H;
  size_t HH = load ? H : (size_t)H * H;
  size_t n = tmg::kMaxQuad + tmg::kMaxQuad * B + tmg::kMaxQuad * B * D;
  if (coef_kind == TM_COEF_POINT) n += (size_t)plan->max_vtx * (load ? H : 1);
  n += load ? (size_t)plan->max_rows * H : (size_t)plan->max_slots * HH;
  n += (size_t)chunk * SE;
  return (int64_t)(32 + (size_t)plan->max_vtx * D * 8 + n * es + (size_t)plan->max_rows * sizeof(int) + 16);
}

extern "C" int tm_batched_max_clusters(int32_t element, int32_t cluster, int64_t smem_bytes) {
  if (cluster < 1 || cluster > 16) return -TM_ERR_INVALID;
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(tmg::kBatchThreads);
  cfg.dynamicSmemBytes = (size_t)smem_bytes;
  cfg.gridDim = dim3(cluster);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  cudaError_t e;
  // clusters above the portable size 8 must be allowed before the query
  if (element == TM_TRI3) {
    cudaFuncSetAttribute(tmg::batched_assemble_pcg_kernel<TM_TRI3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem_bytes);
    if (cluster > 8)
      cudaFuncSetAttribute(tmg::batched_assemble_pcg_kernel<TM_TRI3>,
                           cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    e = cudaOccupancyMaxActiveClusters(&n, tmg::batched_assemble_pcg_kernel<TM_TRI3>, &cfg);
  } else if (element == TM_TET4) {
    cudaFuncSetAttribute(tmg::batched_assemble_pcg_kernel<TM_TET4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem_bytes);
    if (cluster > 8)
      cudaFuncSetAttribute(tmg::batched_assemble_pcg_kernel<TM_TET4>,
                           cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    e = cudaOccupancyMaxActiveClusters(&n, tmg::batched_assemble_pcg_kernel<TM_TET4>, &cfg);
  } else {
    return -TM_ERR_UNSUPPORTED;
  }
  return e == cudaSuccess ? n : -TM_ERR_CUDA;
}

extern "C" int tm_batched_assemble_pcg(const tm_batched_args* a, void* stream) {
  if (!a) return TM_ERR_INVALID;
  if (a->element != TM_TRI3 && a->element != TM_TET4) return TM_ERR_UNSUPPORTED;
  if (a->cluster < 1 || a->cluster > 16 || a->n_clusters < 1 || a->n_inst < 0) return TM_ERR_INVALID;
  if (!a->plan || !a->mat || !a->load || !a->order || !a->inst_pbeg || !a->inst_rbeg || !a->dirichlet ||
      !a->work || !a->status || !a->iters || !a->resid || !a->queue)
    return TM_ERR_INVALID;
  if (a->mat->dtype != TM_F32 || a->load->dtype != TM_F32) return TM_ERR_UNSUPPORTED;
  tmg::BatchArgs A;
  A.plan = *a->plan;
  A.mat = *a->mat;
  A.load = *a->load;
  A.order = a->order;
  A.inst_pbeg = a->inst_pbeg;
  A.inst_rbeg = a->inst_rbeg;
  A.indptr = a->plan->indptr;
  A.indices = a->indices;
  A.dirichlet = a->dirichlet;
  const int64_t n = a->n_rows;
  float* w = static_cast<float*>(a->work);
  A.x = a->x;
  A.r = w;
  A.z = w + n;
  A.p0 = w + 2 * n;
  A.p1 = w + 3 * n;
  A.q = w + 4 * n;
  A.dinv = w + 5 * n;
  A.status = a->status;
  A.iters = a->iters;
  A.resid = a->resid;
  A.queue = a->queue;
  A.n_inst = a->n_inst;
  A.maxiter = a->maxiter;
  A.rtol = a->rtol;
  A.chunk = a->chunk;
  cudaStream_t s = static_cast<cudaStream_t>(a->stream ? a->stream : stream);
  if (cudaMemsetAsync(a->queue, 0, sizeof(unsigned int), s) != cudaSuccess) return TM_ERR_CUDA;
  if (a->element == TM_TRI3) return tmg::launch_batched<TM_TRI3>(A, a->cluster, a->n_clusters, a->smem_bytes, s);
  return tmg::launch_batched<TM_TET4>(A, a->cluster, a->n_clusters, a->smem_bytes, s);
}
