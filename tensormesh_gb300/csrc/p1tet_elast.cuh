// Specialised path for isotropic linear elasticity on P1 tetrahedra (FP64
// emulated or FP32): same patch decomposition and fixed-order
// row-owner accumulation as the generic kernel, with the element algebra in
// closed form on the patch frame's edge vectors (patch_frame.cuh).  A patch
// with an ill-conditioned element or a modulus outside double-float's range
// is redone in native FP64 by its CTA.
//
// With edge vectors d_k = X_{k+1} - X_0, the cross products C_1 = d_2 x d_3,
// C_2 = d_3 x d_1, C_3 = d_1 x d_2, C_0 = -(C_1 + C_2 + C_3) and
// det = d_1 . C_1, the shape gradients are g_a = C_a / det and the 3x3 block
// of nodes (a, b) is (functional/elasticity.py:132-284, builtin.py:173-179,
// B_a^T C B_b written out)
//     K_ab[i][j] = s (lam C_a[i] C_b[j] + mu C_a[j] C_b[i] + mu delta_ij C_a.C_b),
//     s = c W / |det|,  W = sum of the quadrature weights,
// c the element's coefficient (modulus), lam / mu the Lame constants per unit
// modulus.  Phase A stages per element C (12 values), s lam, s mu and the 10
// dot products C_a.C_b; phase B runs three threads per owned node row, one per
// displacement component i, each adding row i of the incidence's four blocks
// into its accumulators in incidence order.
#pragma once
#include "p1tet_fast.cuh"

namespace tmg {

constexpr int kElastStage = 24;  // staged values per element

// index of the unordered pair (a, b) among the 10 dot products
TM_D int pair4(int a, int b) { return tri4(a, b); }

// One pass over the patch in arithmetic A; with kGuard (double-float) returns
// false on every thread when the patch needs native FP64 (an ill-conditioned
// element or a modulus outside double-float's range).
template <class T, class A, class RW, bool kGuard>
__device__ __forceinline__ bool p1tet_elast_pass(const tm_patch_plan& plan, const tm_assemble_args& args, int chunk,
                                                 unsigned char* smem_raw) {
  using P = Ar<A>;
  using R = Rec<RW>;
  using S = typename P::S;
  const RW* recs = R::ptr(plan);
  const int p = blockIdx.x;
  const int tid = threadIdx.x;
  const int Q = args.n_quad;
  const int vbeg = plan.vptr[p], nv = plan.vptr[p + 1] - vbeg;
  const int ebeg = plan.eptr[p], ne = plan.eptr[p + 1] - ebeg;
  const int rbeg = plan.rptr[p], nr = plan.rptr[p + 1] - rbeg;
  if (nr == 0) return true;

  int64_t* s_out0 = reinterpret_cast<int64_t*>(smem_raw);         // [kThreads/3] first dof value of each row
  uint32_t* s_rd = reinterpret_cast<uint32_t*>(s_out0 + kThreads); // [kThreads/3] acc slot | degree << 24
  unsigned long long* s_red = reinterpret_cast<unsigned long long*>(s_rd + kThreads);  // [3] (4 words reserved)
  long long* s_R = reinterpret_cast<long long*>(s_red + 4);        // [max_vtx][3] integer frame
  S* s_acc = reinterpret_cast<S*>(s_R + plan.max_vtx * 3);         // [max_slots][3][3]
  S* s_stage = s_acc + (int64_t)plan.max_slots * 9;                // [kElastStage][chunk]

  // ---- phase 0: row state; thread t owns component t % 3 of row t / 3
  const int lr = tid / 3, comp = tid - 3 * (tid / 3);
  const bool owner = lr < nr && tid < 3 * (kThreads / 3);
  int cur = 0, end = 0, ro = 0, dpos = 0;
  RW rec = R::kEnd;
  if (owner) {
    const int r = plan.rows[rbeg + lr];
    const int64_t n0 = plan.indptr[r];
    const int deg = (int)(plan.indptr[r + 1] - n0);
    ro = plan.racc[rbeg + lr];
    dpos = plan.rdiag[rbeg + lr];
    cur = plan.iptr[rbeg + lr];
    end = plan.iptr[rbeg + lr + 1];
    if (cur < end) rec = recs[cur];
    if (comp == 0) {
      s_out0[lr] = 9 * n0;
      s_rd[lr] = (uint32_t)ro | ((uint32_t)deg << 24);
    }
    for (int k = 0; k < deg; ++k)
#pragma unroll
      for (int j = 0; j < 3; ++j) s_acc[((ro + k) * 3 + comp) * 3 + j] = P::st(P::zero());
  }
  // the first chunk's element data does not depend on the frame: its loads
  // are issued first, in flight while the frame's gathers and reductions run
  const T* coef = static_cast<const T*>(args.coef);
  const bool per_elem = args.coef_kind == TM_COEF_ELEMENT;
  const bool worker = tid < chunk;
  uint2 cw_next = make_uint2(0u, 0u);
  T c_next = T(0);
  if (worker && tid < ne) {
    cw_next = *reinterpret_cast<const uint2*>(plan.econn + (int64_t)(ebeg + tid) * 4);
    if (per_elem) c_next = coef[plan.elem[ebeg + tid]];
  }
  const T* pts = static_cast<const T*>(args.points);
  const FrameInfo fr = patch_frame<3, T>(pts, plan.vtx + vbeg, nv, s_R, s_red);
  if (fr.bad && kGuard) return false;  // a non-finite coordinate: the native pass writes nan
  bool flag = kGuard && args.coef_kind == TM_COEF_SCALAR && !coef_in_range(args.scal[0]);
  double wsum = 0.0;
  for (int q = 0; q < Q; ++q) wsum += args.tables[q];
  const A W = P::in(wsum);
  const A sc = P::in(args.scal[0]);
  const A lam1 = P::in(args.lam), mu1 = P::in(args.mu);
  __syncthreads();

  for (int cbeg = 0; cbeg < ne; cbeg += chunk) {
    const int cend = min(ne, cbeg + chunk);
    // --- phase A: cross products, scaled Lame constants, dot products --------
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
      const A c = per_elem ? P::in(c_raw) : sc;
      if (kGuard && per_elem && !coef_in_range((double)c_raw)) flag = true;
      // edge vectors in frame units, exact to 2^-48 of themselves
      A dd[3][3];
      if (fr.shortp) {
        const int* r32 = reinterpret_cast<const int*>(s_R);
        const ShortConv conv = short_conv(fr.t + fr.z - 62);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const int r0 = r32[2 * (lv[0] * 3 + d)];
#pragma unroll
          for (int k = 0; k < 3; ++k) dd[k][d] = P::pair(conv(r32[2 * (lv[k + 1] * 3 + d)] - r0), 0.f);
        }
      } else if constexpr (std::is_same<A, double>::value) {
        // native FP64 pass: the full 53 bits of every difference
        const double esc = ldexp(1.0, fr.z - 62);
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int k = 0; k < 3; ++k) dd[k][d] = __ll2double_rn(s_R[lv[k + 1] * 3 + d] - s_R[lv[0] * 3 + d]) * esc;
      } else {
        float eh[3][3], el[3][3];
        const int u = exact_edges<3, 3>(s_R, lv, eh, el);
        if (u < 0 && kGuard) flag = true;
        const float p2 = tm_pow2f(fr.z - (u < 0 ? 0 : u));
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int d = 0; d < 3; ++d) dd[k][d] = P::scale2(P::pair(eh[k][d], el[k][d]), p2);
      }
      auto cross = [](const A* u, const A* v, A* out) {
        out[0] = P::sub(P::mul(u[1], v[2]), P::mul(u[2], v[1]));
        out[1] = P::sub(P::mul(u[2], v[0]), P::mul(u[0], v[2]));
        out[2] = P::sub(P::mul(u[0], v[1]), P::mul(u[1], v[0]));
      };
      A C[4][3];
      cross(dd[1], dd[2], C[1]);
      cross(dd[2], dd[0], C[2]);
      cross(dd[0], dd[1], C[3]);
#pragma unroll
      for (int d = 0; d < 3; ++d) C[0][d] = P::neg(P::add(P::add(C[1][d], C[2][d]), C[3][d]));
      const A det = P::add(P::add(P::mul(dd[0][0], C[1][0]), P::mul(dd[0][1], C[1][1])), P::mul(dd[0][2], C[1][2]));
      if constexpr (kGuard) {
        float trg = 0.f, tra = 0.f;
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            trg = __fmaf_rn(P::hi(dd[k][d]), P::hi(dd[k][d]), trg);
            tra = __fmaf_rn(P::hi(C[k + 1][d]), P::hi(C[k + 1][d]), tra);
          }
        const float dh = P::hi(det);
        if (!(dh * dh >= 1e-30f && trg * tra <= kCondMax * (dh * dh))) flag = true;
      }
      // 1/|det| = (1/sqrt(det^2))
      const A s = P::mul(P::mul(c, W), P::rsqrt(P::mul(det, det)));
      const int lo = le - cbeg;
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) s_stage[(a * 3 + d) * chunk + lo] = P::st(C[a][d]);
      s_stage[12 * chunk + lo] = P::st(P::mul(s, lam1));
      s_stage[13 * chunk + lo] = P::st(P::mul(s, mu1));
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = a; b < 4; ++b) {
          const A dot = P::add(P::add(P::mul(C[a][0], C[b][0]), P::mul(C[a][1], C[b][1])), P::mul(C[a][2], C[b][2]));
          s_stage[(14 + pair4(a, b)) * chunk + lo] = P::st(dot);
        }
    }
    if (__syncthreads_or(kGuard && flag)) return false;
    // --- phase B: component `comp` of the row's blocks, incidence order -----
    if (owner) {
      for (;;) {
        const int lel = R::elem(rec);
        if (lel >= cend) break;  // also the end record
        const RW next = (cur + 1 < end) ? recs[cur + 1] : R::kEnd;
        const int a = R::a(rec);
        const int lo = lel - cbeg;
        const A lw = P::ld(s_stage[12 * chunk + lo]), mw = P::ld(s_stage[13 * chunk + lo]);
        A Ca[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) Ca[d] = P::ld(s_stage[(a * 3 + d) * chunk + lo]);
        const A li = P::mul(lw, Ca[comp]);
        A mj[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) mj[j] = P::mul(mw, Ca[j]);
        // the four blocks (a, b): b = a (diagonal slot dpos) then o_0, o_1, o_2
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int b = (a + t) & 3;
          const int pos = t == 0 ? dpos : R::pos(rec, t - 1);
          A Cb[3];
#pragma unroll
          for (int d = 0; d < 3; ++d) Cb[d] = P::ld(s_stage[(b * 3 + d) * chunk + lo]);
          const A dot = P::ld(s_stage[(14 + pair4(a, b)) * chunk + lo]);
          S* acc = s_acc + ((ro + pos) * 3 + comp) * 3;
          S old[3];
#pragma unroll
          for (int j = 0; j < 3; ++j) old[j] = acc[j];
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            A v = P::add(P::mul(li, Cb[j]), P::mul(mj[j], Cb[comp]));
            if (j == comp) v = P::add(v, P::mul(mw, dot));
            acc[j] = P::st(P::add(P::ld(old[j]), v));
          }
        }
        rec = next;
        ++cur;
      }
    }
    __syncthreads();
  }
  // --- write the finished dof rows: a warp per (node row, component) ----------
  T* out = static_cast<T*>(args.out);
  const int lane = tid & 31, warp = tid >> 5;
  for (int w = warp; w < 3 * nr; w += kThreads / 32) {
    const int r = w / 3, i = w - 3 * (w / 3);
    const uint32_t rd = s_rd[r];
    const int r0 = (int)(rd & 0xffffffu), deg = (int)(rd >> 24);
    const int64_t o0 = s_out0[r] + (int64_t)i * 3 * deg;
    for (int k = lane; k < 3 * deg; k += 32) {
      const int kk = k / 3, j = k - 3 * (k / 3);
      out[o0 + k] = fr.bad ? T(NAN) : (T)tm_scale_pow2(P::out(s_acc[((r0 + kk) * 3 + i) * 3 + j]), fr.k);
    }
  }
  return true;
}

// three CTAs per SM (at most 85 registers): measured at 64^3 with the
// 512-slot plan, 1.37 ms against 1.44 ms for two CTAs per SM at 700 slots
template <class T, class A, class RW>
__global__ void __launch_bounds__(kThreads, 3)
p1tet_elast_kernel(tm_patch_plan plan, tm_assemble_args args, int chunk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr bool kGuard = std::is_same<A, L2>::value;
  if (p1tet_elast_pass<T, A, RW, kGuard>(plan, args, chunk, smem_raw)) return;
  if constexpr (kGuard) {
    __syncthreads();
    p1tet_elast_pass<T, double, RW, false>(plan, args, chunk, smem_raw);
  }
}

inline size_t p1tet_elast_smem_bytes(const tm_patch_plan& plan, int chunk, size_t elem) {
  const size_t n2 = (size_t)plan.max_slots * 9 + (size_t)kElastStage * chunk;
  return (size_t)kThreads * (sizeof(int64_t) + sizeof(uint32_t)) + 32 + (size_t)plan.max_vtx * 3 * 8 + n2 * elem + 64;
}

// three threads per owned node row; node slots addressable in 24 bits
inline bool p1tet_elast_ok(const tm_patch_plan& plan) {
  return plan.inc_pack != nullptr && plan.rdiag != nullptr && 3 * plan.max_rows <= kThreads &&
         (int64_t)plan.max_slots * 9 < (1 << 24);
}

template <class T, class A, class RW>
inline int launch_p1tet_elast_kernel(const tm_patch_plan& plan, const tm_assemble_args& args, cudaStream_t stream) {
  int dev = 0, max_optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t es = sizeof(typename Ar<A>::S);
  int chunk = 128;
  size_t bytes = p1tet_elast_smem_bytes(plan, chunk, es);
  while (bytes > (size_t)max_optin && chunk > 32) {
    chunk /= 2;
    bytes = p1tet_elast_smem_bytes(plan, chunk, es);
  }
  if (bytes > (size_t)max_optin) return TM_ERR_INDEX;
  auto kern = p1tet_elast_kernel<T, A, RW>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
    return TM_ERR_CUDA;
  kern<<<plan.n_patches, kThreads, bytes, stream>>>(plan, args, chunk);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

template <class T, class A>
inline int launch_p1tet_elast(const tm_patch_plan& plan, const tm_assemble_args& args, cudaStream_t stream) {
  if (plan.inc_pack32) return launch_p1tet_elast_kernel<T, A, uint32_t>(plan, args, stream);
  return launch_p1tet_elast_kernel<T, A, uint64_t>(plan, args, stream);
}

}  // namespace tmg
