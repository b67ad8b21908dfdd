// Specialised FP64 path for the headline case: P1 tetrahedra, Laplace form
// with a per-element (or scalar / interpolated) coefficient, emulated FP64.
//
// Same patch decomposition and deterministic row-owner accumulation as the
// generic kernel (assemble_impl.cuh), with the arithmetic cut to what the
// 1e-12 bar needs:
//   * "lazy" double-float values (hi, lo) whose lo part is not renormalised
//     after every operation (error-free products by FMA, TwoSum only where
//     two leading parts are added);
//   * 1/sqrt(det G) from the MUFU estimate plus one Newton step carried out
//     in double-float, instead of IEEE division and square root;
//   * the 10 unique entries of the symmetric element matrix are staged (not
//     16).
#pragma once
#include "assemble_impl.cuh"

namespace tmg {

// 1/sqrt(x) for x > 0: MUFU estimate, one Newton step in double-float
// (y1 = y0 + y0 (1 - x y0^2) / 2; the residual 1 - x y0^2 is formed with
// error-free products so the step doubles the ~22 correct bits).
TM_D L2 l2_rsqrt(L2 x) {
  x = l2_norm(x);
  const float y0 = rsqrtf(x.h);
  const float y2 = __fmul_rn(y0, y0);
  const float y2e = __fmaf_rn(y0, y0, -y2);           // y0^2 = y2 + y2e exactly
  L2 t = l2_mul(x, L2{y2, y2e});                       // x y0^2
  t = l2_norm(t);
  const float r = __fadd_rn(__fsub_rn(1.0f, t.h), -t.l);  // 1 - x y0^2 (small)
  const float corr = __fmul_rn(__fmul_rn(0.5f, y0), r);
  return l2_norm(L2{y0, corr});
}

// Unique-entry index of (a, b) in the staged upper triangle of a 4x4:
// (0,0)0 (0,1)1 (0,2)2 (0,3)3 (1,1)4 (1,2)5 (1,3)6 (2,2)7 (2,3)8 (3,3)9
TM_D int tri4(int a, int b) {
  const int i = a < b ? a : b, j = a < b ? b : a;
  return i * 4 - (i * (i - 1)) / 2 + (j - i);
}

// Incidence records (see tm_patch_plan): local element, local vertex a and the
// row positions of the off-diagonal columns o_j = (a + 1 + j) mod 4.
template <class W> struct Rec;
template <> struct Rec<uint64_t> {
  static constexpr uint64_t kEnd = ~0ull;  // local element 0xffff: past every chunk
  static TM_D int elem(uint64_t r) { return (int)(r & 0xffff); }
  static TM_D int a(uint64_t r) { return (int)((r >> 16) & 3); }
  static TM_D int pos(uint64_t r, int j) { return (int)((r >> (18 + 8 * j)) & 0xff); }
  static TM_D const uint64_t* ptr(const tm_patch_plan& p) { return p.inc_pack; }
};
template <> struct Rec<uint32_t> {
  static constexpr uint32_t kEnd = ~0u;    // local element 0x7fff: past every chunk
  static TM_D int elem(uint32_t r) { return (int)(r & 0x7fff); }
  static TM_D int a(uint32_t r) { return (int)((r >> 15) & 3); }
  static TM_D int pos(uint32_t r, int j) { return (int)((r >> (17 + 5 * j)) & 31); }
  static TM_D const uint32_t* ptr(const tm_patch_plan& p) { return p.inc_pack32; }
};

// Staged unique-entry index (tri4 order) of the diagonal (nibble 0) and of the
// off-diagonal entries (a, o_j) (nibbles 1-3), 16 bits per local vertex a:
//   a=0: 0 1 2 3   a=1: 4 5 6 1   a=2: 7 8 2 5   a=3: 9 3 6 8
constexpr uint64_t kTet4Stage = 0x8639528716543210ull;

// Arithmetic policies: emulated FP64 (lazy double-float, stored as float2)
// and plain FP32 (the float32 variant of the same kernel).
template <class A> struct Ar;
template <> struct Ar<L2> {
  using S = float2;
  static TM_D L2 ld(S v) { return L2{v.x, v.y}; }
  static TM_D S st(L2 a) { return make_float2(a.h, a.l); }
  static TM_D L2 in(double x) { return l2_from(tm_from_double(x)); }
  static TM_D L2 in(float x) { return L2{x, 0.f}; }
  static TM_D L2 add(L2 a, L2 b) { return l2_add(a, b); }
  static TM_D L2 sub(L2 a, L2 b) { return l2_sub(a, b); }
  static TM_D L2 mul(L2 a, L2 b) { return l2_mul(a, b); }
  static TM_D L2 neg(L2 a) { return l2_neg(a); }
  static TM_D L2 rsqrt(L2 a) { return l2_rsqrt(a); }
  static TM_D L2 zero() { return L2{0.f, 0.f}; }
  static TM_D double out(S v) { return tm_to_double(df64{v.x, v.y}); }
};
template <> struct Ar<float> {
  using S = float;
  static TM_D float ld(S v) { return v; }
  static TM_D S st(float a) { return a; }
  static TM_D float in(double x) { return (float)x; }
  static TM_D float in(float x) { return x; }
  static TM_D float add(float a, float b) { return a + b; }
  static TM_D float sub(float a, float b) { return a - b; }
  static TM_D float mul(float a, float b) { return a * b; }
  static TM_D float neg(float a) { return -a; }
  static TM_D float rsqrt(float a) { return rsqrtf(a); }
  static TM_D float zero() { return 0.f; }
  static TM_D float out(S v) { return v; }
};

template <class T, class A, class RW>
__global__ void __launch_bounds__(kThreads, 4)
p1tet_laplace_fast_kernel(tm_patch_plan plan, tm_assemble_args args, int chunk) {
  using P = Ar<A>;
  using R = Rec<RW>;
  const RW* recs = R::ptr(plan);
  using S = typename P::S;
  const int p = blockIdx.x;
  const int tid = threadIdx.x;
  const int Q = args.n_quad;
  const int vbeg = plan.vptr[p], nv = plan.vptr[p + 1] - vbeg;
  const int ebeg = plan.eptr[p], ne = plan.eptr[p + 1] - ebeg;
  const int rbeg = plan.rptr[p], nr = plan.rptr[p + 1] - rbeg;
  if (nr == 0) return;

  // Accumulators are column-major over the patch's rows: entry k of local row
  // lr sits at s_acc[k * nrp + lr], nrp = max_rows rounded up to 16, so the
  // 16 lanes of a half-warp (consecutive rows) hit 16 distinct bank pairs
  // whatever columns their incidences touch.
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nrp = (plan.max_rows + 15) & ~15;
  S* s_X = reinterpret_cast<S*>(smem_raw);                         // [max_vtx][3]
  S* s_pc = s_X + plan.max_vtx * 3;                                // [max_vtx] point coef
  const int pc_len = args.coef_kind == TM_COEF_POINT ? plan.max_vtx : 0;
  S* s_acc = s_pc + pc_len;                                        // [max_deg][nrp]
  S* s_stage = s_acc + plan.max_deg * nrp;                         // [10][chunk]

  // ---- phase 0: row state (the launcher guarantees nr <= kThreads, so a
  // thread owns at most one row; its incidence cursor and the next packed
  // record stay in registers across chunks), coordinates, coefficients
  const bool owner = tid < nr;
  int cur = 0, end = 0, dpos = 0, deg = 0;
  int64_t o0 = 0;
  RW rec = R::kEnd;
  S* acc = s_acc + tid;  // this thread's row: entry k at acc[k * nrp]
  if (owner) {
    const int r = plan.rows[rbeg + tid];
    o0 = plan.indptr[r];
    deg = (int)(plan.indptr[r + 1] - o0);
    dpos = plan.rdiag[rbeg + tid];
    cur = plan.iptr[rbeg + tid];
    end = plan.iptr[rbeg + tid + 1];
    if (cur < end) rec = recs[cur];
    for (int k = 0; k < deg; ++k) acc[k * nrp] = P::st(P::zero());
  }
  const T* pts = static_cast<const T*>(args.points);
  for (int i = tid; i < nv * 3; i += kThreads) {
    const int v = plan.vtx[vbeg + i / 3];
    s_X[i] = P::st(P::in(pts[(int64_t)v * 3 + i % 3]));
  }
  const T* coef = static_cast<const T*>(args.coef);
  if (args.coef_kind == TM_COEF_POINT) {
    for (int i = tid; i < nv; i += kThreads) s_pc[i] = P::st(P::in(coef[plan.vtx[vbeg + i]]));
  }
  double wsum = 0.0;
  for (int q = 0; q < Q; ++q) wsum += args.tables[q];
  const A W = P::in(wsum);
  const A sc = P::in(args.scal[0]);
  const bool per_elem = args.coef_kind == TM_COEF_ELEMENT;
  // element data of this thread's next element (threads tid < chunk handle
  // element cbeg + tid of every chunk), loaded one chunk ahead
  const bool worker = tid < chunk;
  uint2 cw_next = make_uint2(0u, 0u);
  T c_next = T(0);
  if (worker && tid < ne) {
    cw_next = *reinterpret_cast<const uint2*>(plan.econn + (int64_t)(ebeg + tid) * 4);
    if (per_elem) c_next = coef[plan.elem[ebeg + tid]];
  }
  __syncthreads();

  for (int cbeg = 0; cbeg < ne; cbeg += chunk) {
    const int cend = min(ne, cbeg + chunk);
    // --- phase A -------------------------------------------------------------
    const int le = cbeg + tid;
    if (worker && le < cend) {
      const int pair = ebeg + le;
      const uint2 cw = cw_next;
      const T c_raw = c_next;
      if (le + chunk < ne) {
        cw_next = *reinterpret_cast<const uint2*>(plan.econn + (int64_t)(pair + chunk) * 4);
        if (per_elem) c_next = coef[plan.elem[pair + chunk]];
      }
      const int lv[4] = {(int)(cw.x & 0xffff), (int)(cw.x >> 16), (int)(cw.y & 0xffff), (int)(cw.y >> 16)};
      A X[4][3];
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int d = 0; d < 3; ++d) X[b][d] = P::ld(s_X[lv[b] * 3 + d]);
      A c;
      if (per_elem) {
        c = P::in(c_raw);
      } else if (args.coef_kind == TM_COEF_POINT) {
        // sum_q w_q sum_b N_b(q) c_b / W : P1 -> weighted vertex average
        double cw_ = 0.0;
        for (int q = 0; q < Q; ++q)
          for (int b = 0; b < 4; ++b) cw_ += args.tables[q] * args.tables[Q + q * 4 + b] * P::out(s_pc[lv[b]]);
        c = P::in(cw_ / wsum);
      } else if (args.coef_kind == TM_COEF_QUAD) {
        double cw_ = 0.0;
        for (int q = 0; q < Q; ++q) cw_ += args.tables[q] * (double)coef[(int64_t)plan.elem[pair] * Q + q];
        c = P::in(cw_ / wsum);
      } else {
        c = sc;
      }
      A d[3][3];
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) d[k][dd] = P::sub(X[k + 1][dd], X[0][dd]);
      auto dot3 = [](const A* a, const A* b) {
        return P::add(P::add(P::mul(a[0], b[0]), P::mul(a[1], b[1])), P::mul(a[2], b[2]));
      };
      auto cof = [](A a, A b, A c_, A d_) { return P::sub(P::mul(a, b), P::mul(c_, d_)); };
      const A G00 = dot3(d[0], d[0]), G11 = dot3(d[1], d[1]), G22 = dot3(d[2], d[2]);
      const A G01 = dot3(d[0], d[1]), G02 = dot3(d[0], d[2]), G12 = dot3(d[1], d[2]);
      const A A00 = cof(G11, G22, G12, G12), A11 = cof(G00, G22, G02, G02), A22 = cof(G00, G11, G01, G01);
      const A A01 = cof(G02, G12, G01, G22), A02 = cof(G01, G12, G02, G11), A12 = cof(G01, G02, G00, G12);
      const A detG = P::add(P::add(P::mul(G00, A00), P::mul(G01, A01)), P::mul(G02, A02));
      const A s = P::mul(P::mul(c, W), P::rsqrt(detG));
      const A k11 = P::mul(s, A00), k22 = P::mul(s, A11), k33 = P::mul(s, A22);
      const A k12 = P::mul(s, A01), k13 = P::mul(s, A02), k23 = P::mul(s, A12);
      const A k01 = P::neg(P::add(P::add(k11, k12), k13));
      const A k02 = P::neg(P::add(P::add(k12, k22), k23));
      const A k03 = P::neg(P::add(P::add(k13, k23), k33));
      const A k00 = P::neg(P::add(P::add(k01, k02), k03));
      const int lo = le - cbeg;
      const A vals[10] = {k00, k01, k02, k03, k11, k12, k13, k22, k23, k33};
#pragma unroll
      for (int u = 0; u < 10; ++u) s_stage[u * chunk + lo] = P::st(vals[u]);
    }
    __syncthreads();
    // --- phase B: the row owner adds its incidences of this chunk (fixed
    // order).  The diagonal is summed in registers and added once per chunk;
    // the three off-diagonal contributions of an incidence hit distinct
    // columns, so their read-modify-writes are issued together.  The record
    // that ends the loop is the first one of the next chunk.
    if (owner) {
      A dg = P::zero();
      bool any = false;
      for (;;) {
        const int lel = R::elem(rec);
        if (lel >= cend) break;  // also the end record (its element field is past every chunk)
        const RW next = (cur + 1 < end) ? recs[cur + 1] : R::kEnd;
        const int a = R::a(rec);
        const int lo = lel - cbeg;
        const uint32_t u = (uint32_t)(kTet4Stage >> (16 * a));
        dg = P::add(dg, P::ld(s_stage[(int)(u & 15u) * chunk + lo]));
        int pos[3];
        S v[3], old[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          pos[j] = R::pos(rec, j) * nrp;
          v[j] = s_stage[(int)((u >> (4 * j + 4)) & 15u) * chunk + lo];
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) old[j] = acc[pos[j]];
#pragma unroll
        for (int j = 0; j < 3; ++j) acc[pos[j]] = P::st(P::add(P::ld(old[j]), P::ld(v[j])));
        any = true;
        rec = next;
        ++cur;
      }
      if (any) acc[dpos * nrp] = P::st(P::add(P::ld(acc[dpos * nrp]), dg));
    }
    __syncthreads();
  }
  // --- write the finished row: only its owner ever touched it, so no barrier
  // is needed; consecutive lanes write consecutive rows' k-th entries
  if (owner) {
    T* out = static_cast<T*>(args.out);
    for (int k = 0; k < deg; ++k) out[o0 + k] = (T)P::out(acc[k * nrp]);
  }
}

inline size_t p1tet_smem_bytes(const tm_patch_plan& plan, int coef_kind, int chunk, size_t elem = sizeof(float2)) {
  const size_t nrp = (size_t)((plan.max_rows + 15) & ~15);
  size_t n2 = (size_t)plan.max_vtx * 3 + (coef_kind == TM_COEF_POINT ? plan.max_vtx : 0) +
              (size_t)plan.max_deg * nrp + (size_t)10 * chunk;
  return n2 * elem + 64;
}

// The fast path needs every patch to own at most kThreads rows (one row per
// thread); other plans take the generic patch kernel.
inline bool p1tet_fast_ok(const tm_patch_plan& plan) {
  return plan.inc_pack != nullptr && plan.rdiag != nullptr && plan.max_rows <= kThreads && plan.max_deg > 0;
}

template <class T, class A, class RW>
inline int launch_p1tet_kernel(const tm_patch_plan& plan, const tm_assemble_args& args, cudaStream_t stream) {
  int dev = 0, max_optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  int chunk = kThreads;
  const size_t es = sizeof(typename Ar<A>::S);
  size_t bytes = p1tet_smem_bytes(plan, args.coef_kind, chunk, es);
  while (bytes > (size_t)max_optin && chunk > 32) {
    chunk /= 2;
    bytes = p1tet_smem_bytes(plan, args.coef_kind, chunk, es);
  }
  if (bytes > (size_t)max_optin) return TM_ERR_INDEX;
  auto kern = p1tet_laplace_fast_kernel<T, A, RW>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
    return TM_ERR_CUDA;
  kern<<<plan.n_patches, kThreads, bytes, stream>>>(plan, args, chunk);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

template <class T, class A>
inline int launch_p1tet_laplace_fast(const tm_patch_plan& plan, const tm_assemble_args& args, cudaStream_t stream) {
  if (plan.inc_pack32) return launch_p1tet_kernel<T, A, uint32_t>(plan, args, stream);
  return launch_p1tet_kernel<T, A, uint64_t>(plan, args, stream);
}

}  // namespace tmg
