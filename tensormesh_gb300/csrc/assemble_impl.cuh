// Patch-based deterministic assembly (generic over element, form and
// arithmetic).  One CTA per patch:
//
//   phase 0  gather the patch's vertex coordinates (and point data) into
//            shared memory, converted once to the compute type R;
//   phase A  element-parallel: each thread computes the full element matrix
//            (or load vector) of one element into a shared staging slot --
//            Jacobian, |det J|, physical gradients and the quadrature sum
//            all stay in registers/shared memory;
//   phase B  row-parallel: the thread that owns a CSR row walks that row's
//            incidences (element, local vertex a) in a fixed order and adds
//            stage[e][a][b] into the row's accumulator at the precomputed
//            position of column conn[e][b];
//   write    warp-per-row copy of the finished rows into the canonical CSR
//            value array (each value written exactly once, no atomics).
//
// The accumulation order of every CSR value is fixed by the plan, so the
// result is bitwise reproducible run to run.  This replaces the reference's
// vmap/einsum element integrals (assemble/element_assembler.py:402-464,
// element/element.py:874-968, element/transformation.py:1236-1293) and the
// index_add_ scatter (assemble/projector.py:95-130).
#pragma once
#include "tm_common.cuh"
#include "patch_frame.cuh"
#include "../../include/tensormesh_gb300.h"
#include <type_traits>

namespace tmg {

template <int EL> struct Elem;
template <> struct Elem<TM_TRI3> { static constexpr int D = 2, B = 3; };
template <> struct Elem<TM_TRI6> { static constexpr int D = 2, B = 6; };
template <> struct Elem<TM_TET4> { static constexpr int D = 3, B = 4; };
template <> struct Elem<TM_TET10> { static constexpr int D = 3, B = 10; };

constexpr int kThreads = 256;
constexpr int kMaxQuad = 11;

template <int EL, int FORM, int H>
struct Layout {
  static constexpr int D = Elem<EL>::D, B = Elem<EL>::B;
  static constexpr bool kLoad = FORM == TM_FORM_LOAD;
  // staged entries per element
  static constexpr int SE = kLoad ? B * H : B * B * H * H;
  // accumulator entries per node slot (bilinear) or per owned row (load)
  static constexpr int HH = kLoad ? H : H * H;
};

template <class R>
TM_D R tm_fma_acc(R acc, R a, R b) { return acc + a * b; }

// Inverse-transpose data of one quadrature point: physical gradients and JxW.
template <int D, int B, class R>
TM_D void point_geometry(const R (&X)[B][D], const R* dNq /*[B][D]*/, R wq, R (&g)[B][D], R& jxw) {
  // J[i][j] = sum_b X[b][j] dN[b][i]   (element.py:962, J = dx_j / dxi_i)
  R J[D][D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      R s = Num<R>::zero();
#pragma unroll
      for (int b = 0; b < B; ++b) s = tm_fma_acc(s, X[b][j], dNq[b * D + i]);
      J[i][j] = s;
    }
  R inv[D][D];  // adjugate; divided by det below
  R det;
  if constexpr (D == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    inv[0][0] = J[1][1];
    inv[0][1] = -J[0][1];
    inv[1][0] = -J[1][0];
    inv[1][1] = J[0][0];
  } else {
    inv[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    inv[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    inv[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    inv[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    inv[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    inv[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    inv[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    inv[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    inv[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    det = J[0][0] * inv[0][0] + J[0][1] * inv[1][0] + J[0][2] * inv[2][0];
  }
  R rdet = Num<R>::from_float(1.f) / det;
  // grad[b][j] = sum_i dN[b][i] Jinv[j][i]  (element.py:966)
#pragma unroll
  for (int b = 0; b < B; ++b)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      R s = Num<R>::zero();
#pragma unroll
      for (int i = 0; i < D; ++i) s = tm_fma_acc(s, dNq[b * D + i], inv[j][i]);
      g[b][j] = s * rdet;
    }
  jxw = wq * Num<R>::abs(det);  // transformation.py:1289
}

// Closed-form P1 Laplace element matrix from the edge vectors
// d_k = X_{k+1} - X_0.  The rows of adj(J) (J the matrix of edge columns) are
// C_k = det * grad N_{k+1}: in 3D the cross products d_2 x d_3, d_3 x d_1,
// d_1 x d_2, in 2D the rotated edges (d_1y, -d_1x), (-d_0y, d_0x).  So
//   K_ij = cW C_i . C_j / |det|   (i, j >= 1),   K_0j = -sum_i K_ij,
// where cW = sum_q w_q c(x_q).  For a P1 simplex the gradients are constant,
// so this equals the reference's quadrature sum of c gradu.gradv JxW
// (assemble/builtin.py:62-63, element_assembler.py:211) for every order.  Its
// rounding error grows like the element's aspect ratio (a form through the
// metric tensor G = J^T J grows like its square).
template <int D, class R>
TM_D void p1_laplace_closed_form(const R (&X)[D + 1][D], R cW, Strided<R> Ke) {
  constexpr int B = D + 1;
  R d[D][D];
#pragma unroll
  for (int k = 0; k < D; ++k)
#pragma unroll
    for (int c = 0; c < D; ++c) d[k][c] = X[k + 1][c] - X[0][c];
  R C[D][D];
  R det;
  if constexpr (D == 2) {
    C[0][0] = d[1][1];
    C[0][1] = -d[1][0];
    C[1][0] = -d[0][1];
    C[1][1] = d[0][0];
    det = d[0][0] * d[1][1] - d[0][1] * d[1][0];
  } else {
    auto cross = [](const R* u, const R* v, R* o) {
      o[0] = u[1] * v[2] - u[2] * v[1];
      o[1] = u[2] * v[0] - u[0] * v[2];
      o[2] = u[0] * v[1] - u[1] * v[0];
    };
    cross(d[1], d[2], C[0]);
    cross(d[2], d[0], C[1]);
    cross(d[0], d[1], C[2]);
    det = d[0][0] * C[0][0] + d[0][1] * C[0][1] + d[0][2] * C[0][2];
  }
  const R s = cW / Num<R>::abs(det);
  R k0[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
#pragma unroll
    for (int j = i; j < D; ++j) {
      R dot = C[i][0] * C[j][0];
#pragma unroll
      for (int c = 1; c < D; ++c) dot = dot + C[i][c] * C[j][c];
      const R v = s * dot;
      Ke[(i + 1) * B + (j + 1)] = v;
      Ke[(j + 1) * B + (i + 1)] = v;
    }
  }
#pragma unroll
  for (int j = 0; j < D; ++j) {
    R t = Ke[1 * B + (j + 1)];
#pragma unroll
    for (int i = 1; i < D; ++i) t = t + Ke[(i + 1) * B + (j + 1)];
    k0[j] = -t;
    Ke[j + 1] = k0[j];
    Ke[(j + 1) * B] = k0[j];
  }
  R t = k0[0];
#pragma unroll
  for (int j = 1; j < D; ++j) t = t + k0[j];
  Ke[0] = -t;
}

// A float pair (hi, lo) times 2^e (|e| <= 126, exact) in compute type R.
template <class R> TM_D R frame_value(float h, float l, float p2);
template <> TM_D df64 frame_value<df64>(float h, float l, float p2) { return df64{__fmul_rn(h, p2), __fmul_rn(l, p2)}; }
template <> TM_D double frame_value<double>(float h, float l, float p2) { return ((double)h + (double)l) * (double)p2; }
template <> TM_D float frame_value<float>(float h, float l, float p2) { return __fmul_rn(__fadd_rn(h, l), p2); }

// Frame coordinates of an element's nodes relative to its first node (X[0] =
// 0): exact integer differences of the patch frame, rounded once (see
// patch_frame.cuh).  Returns false for an element whose nodes coincide.
template <int B, int D, class R>
TM_D bool element_frame(const long long* __restrict__ s_R, const FrameInfo& fr, const int (&lv)[B], R (&X)[B][D]) {
#pragma unroll
  for (int c = 0; c < D; ++c) X[0][c] = Num<R>::zero();
  if (fr.shortp) {
    const int* r32 = reinterpret_cast<const int*>(s_R);
    const ShortConv conv = short_conv(fr.t + fr.z - 62);             // difference -> frame units, exactly
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const int r0 = r32[2 * (lv[0] * D + c)];
#pragma unroll
      for (int b = 1; b < B; ++b) X[b][c] = frame_value<R>(conv(r32[2 * (lv[b] * D + c)] - r0), 0.f, 1.f);
    }
    return true;
  }
  if constexpr (std::is_same<R, double>::value) {
    // native FP64: the full 53 bits of every difference (the FP64 pipe's
    // conversion is slow, but this pass runs only for patches handed over)
    const double esc = ldexp(1.0, fr.z - 62);
    bool any = false;
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const long long r0 = s_R[lv[0] * D + c];
#pragma unroll
      for (int b = 1; b < B; ++b) {
        const long long dd = s_R[lv[b] * D + c] - r0;
        any = any || dd != 0;
        X[b][c] = __ll2double_rn(dd) * esc;
      }
    }
    return any;
  }
  float eh[B - 1][D], el[B - 1][D];
  int lvv[B];
#pragma unroll
  for (int b = 0; b < B; ++b) lvv[b] = lv[b];
  const int u = exact_edges<B - 1, D>(s_R, lvv, eh, el);
  if (u < 0) return false;
  const float p2 = tm_pow2f(fr.z - u);
#pragma unroll
  for (int b = 1; b < B; ++b)
#pragma unroll
    for (int c = 0; c < D; ++c) X[b][c] = frame_value<R>(eh[b - 1][c], el[b - 1][c], p2);
  return true;
}

// Conditioning bound of the double-float element algebra, tr(G) tr(adj G) /
// det(G) of the vertex edge vectors (tr(G)^2 / det(G) in 2D); above it (or for
// elements tiny against their patch, whose frame products approach float's
// underflow) a patch is redone in native FP64.  A coefficient whose binary
// exponent leaves +-kCoefExpMax does the same.
constexpr float kGenericCondMax = 1.0e4f;
constexpr int kCoefExpMax = 60;

TM_D bool coef_exp_ok(double c) {
  const int e = (int)(((unsigned long long)__double_as_longlong(c) >> 52) & 0x7ff);
  return c == 0.0 || (e >= 1023 - kCoefExpMax && e <= 1023 + kCoefExpMax);
}

// True when a simplex with vertex edge vectors d (hi parts) is well
// conditioned for double-float.
template <int D>
TM_D bool simplex_well_conditioned(const float (&d)[D][D]) {
  float trg = 0.f;
#pragma unroll
  for (int k = 0; k < D; ++k)
#pragma unroll
    for (int c = 0; c < D; ++c) trg = __fmaf_rn(d[k][c], d[k][c], trg);
  if constexpr (D == 2) {
    const float det = d[0][0] * d[1][1] - d[0][1] * d[1][0];
    return det * det >= 1e-30f && trg * trg <= kGenericCondMax * (det * det);
  } else {
    float C[3][3];
    auto cross = [](const float* u, const float* v, float* o) {
      o[0] = u[1] * v[2] - u[2] * v[1];
      o[1] = u[2] * v[0] - u[0] * v[2];
      o[2] = u[0] * v[1] - u[1] * v[0];
    };
    cross(d[1], d[2], C[0]);
    cross(d[2], d[0], C[1]);
    cross(d[0], d[1], C[2]);
    const float det = d[0][0] * C[0][0] + d[0][1] * C[0][1] + d[0][2] * C[0][2];
    float tra = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) tra = __fmaf_rn(C[k][c], C[k][c], tra);
    return det * det >= 1e-30f && trg * tra <= kGenericCondMax * (det * det);
  }
}

// Power of length of a form's element values (real = frame * 2^(k * p)):
// stiffness (gradients squared times the volume) D - 2, mass and loads D.
template <int D, int FORM>
constexpr int frame_power() { return (FORM == TM_FORM_LAPLACE || FORM == TM_FORM_ELASTICITY) ? D - 2 : D; }

// One pass over the rows owned by patch p in arithmetic R (called by one CTA;
// nthreads = blockDim.x).  With kGuard (double-float), returns false on every
// thread when the patch needs native FP64: an ill-conditioned element or a
// coefficient outside double-float's range.
template <int EL, int FORM, int H, class T, class R, bool kGuard>
__device__ bool assemble_patch_pass(const tm_patch_plan& plan, const tm_assemble_args& args, const int p,
                                    const int chunk, unsigned char* smem_raw) {
  using L = Layout<EL, FORM, H>;
  constexpr int D = L::D, B = L::B, SE = L::SE, HH = L::HH;
  const int tid = threadIdx.x;
  const int kThreads = blockDim.x;
  const int Q = args.n_quad;

  const int vbeg = plan.vptr[p], nv = plan.vptr[p + 1] - vbeg;
  const int ebeg = plan.eptr[p], ne = plan.eptr[p + 1] - ebeg;
  const int rbeg = plan.rptr[p], nr = plan.rptr[p + 1] - rbeg;
  if (nr == 0) return true;

  unsigned long long* s_red = reinterpret_cast<unsigned long long*>(smem_raw);  // [3] (4 words reserved)
  long long* s_R = reinterpret_cast<long long*>(smem_raw + 32);                 // [max_vtx][D] integer frame
  R* s_tab = reinterpret_cast<R*>(s_R + plan.max_vtx * D);    // w, N, dN
  R* s_w = s_tab;
  R* s_N = s_w + kMaxQuad;
  R* s_dN = s_N + kMaxQuad * B;
  R* s_pc = s_dN + kMaxQuad * B * D;                          // [max_vtx][H] point coef
  const int pc_len = (args.coef_kind == TM_COEF_POINT) ? plan.max_vtx * (L::kLoad ? H : 1) : 0;
  R* s_acc = s_pc + pc_len;
  const int acc_len = L::kLoad ? plan.max_rows * H : plan.max_slots * HH;
  R* s_stage = s_acc + acc_len;
  int* s_cur = reinterpret_cast<int*>(s_stage + chunk * SE);

  // --- phase 0: tables, coordinates, point data, zero accumulators -------
  for (int i = tid; i < Q; i += kThreads) s_w[i] = Num<R>::from_double(args.tables[i]);
  for (int i = tid; i < Q * B; i += kThreads) s_N[i] = Num<R>::from_double(args.tables[Q + i]);
  for (int i = tid; i < Q * B * D; i += kThreads) s_dN[i] = Num<R>::from_double(args.tables[Q + Q * B + i]);
  const T* pts = static_cast<const T*>(args.points);
  const FrameInfo fr = patch_frame<D, T>(pts, plan.vtx + vbeg, nv, s_R, s_red);
  if (fr.bad && kGuard) return false;  // a non-finite coordinate: the native pass writes nan
  bool flag = false;                   // (kGuard) the patch needs native FP64
  if (args.coef_kind == TM_COEF_POINT) {
    constexpr int PC = L::kLoad ? H : 1;
    const T* pc = static_cast<const T*>(args.coef);
    for (int i = tid; i < nv * PC; i += kThreads) {
      int v = plan.vtx[vbeg + i / PC];
      const T c = pc[(int64_t)v * PC + i % PC];
      if (kGuard && !coef_exp_ok((double)c)) flag = true;
      s_pc[i] = tm_load<R, T>(c);
    }
  }
  if (kGuard) {
    const int nsc = L::kLoad ? H : 1;
    for (int h = 0; h < nsc; ++h)
      if (args.coef_kind == TM_COEF_SCALAR && !coef_exp_ok(args.scal[h])) flag = true;
  }
  const int nacc = L::kLoad ? nr * H : 0;
  {
    int total = L::kLoad ? nacc : 0;
    if (!L::kLoad) {
      // owned node slots of this patch = racc of last row + its degree
      int lr = rbeg + nr - 1;
      int r = plan.rows[lr];
      total = (plan.racc[lr] + (int)(plan.indptr[r + 1] - plan.indptr[r])) * HH;
    }
    for (int i = tid; i < total; i += kThreads) s_acc[i] = Num<R>::zero();
  }
  for (int i = tid; i < nr; i += kThreads) s_cur[i] = plan.iptr[rbeg + i];
  __syncthreads();

  R scal[3];
#pragma unroll
  for (int h = 0; h < 3; ++h) scal[h] = Num<R>::from_double(args.scal[h]);
  // Lame constants per unit coefficient (functional/elasticity.py:202-284)
  const R lam1 = Num<R>::from_double(args.lam);
  const R mu1 = Num<R>::from_double(args.mu);
  const T* coef = static_cast<const T*>(args.coef);

  for (int cbeg = 0; cbeg < ne; cbeg += chunk) {
    const int cend = min(ne, cbeg + chunk);
    // --- phase A: element matrices into the staging area --------------------
    for (int le = cbeg + tid; le < cend; le += kThreads) {
      const int e = plan.elem[ebeg + le];
      int lv[B];
#pragma unroll
      for (int b = 0; b < B; ++b) lv[b] = plan.econn[(int64_t)(ebeg + le) * B + b];
      // frame coordinates relative to the element's first node (exact integer
      // differences, rounded once)
      R X[B][D];
      if (!element_frame<B, D, R>(s_R, fr, lv, X) && kGuard) flag = true;
      R ce = scal[0];
      if (args.coef_kind == TM_COEF_ELEMENT) {
        const T c = coef[e];
        if (kGuard && !coef_exp_ok((double)c)) flag = true;
        ce = tm_load<R, T>(c);
      }
      if constexpr (kGuard) {
        float dv[D][D];
#pragma unroll
        for (int k = 0; k < D; ++k)
#pragma unroll
          for (int c = 0; c < D; ++c) dv[k][c] = Num<R>::to_float(X[k + 1][c]);
        if (!simplex_well_conditioned<D>(dv)) flag = true;
        if (args.coef_kind == TM_COEF_QUAD)
          for (int q = 0; q < Q * (L::kLoad ? H : 1); ++q)
            if (!coef_exp_ok((double)coef[(int64_t)e * Q * (L::kLoad ? H : 1) + q])) flag = true;
      }
      Strided<R> Ke{s_stage + (le - cbeg), chunk};
      if constexpr (FORM == TM_FORM_LAPLACE && B == D + 1) {
        R cW = Num<R>::zero();
        for (int q = 0; q < Q; ++q) {
          R cq = ce;
          if (args.coef_kind == TM_COEF_POINT) {
            R s = Num<R>::zero();
#pragma unroll
            for (int b = 0; b < B; ++b) s = s + s_pc[lv[b]] * s_N[q * B + b];
            cq = s;
          } else if (args.coef_kind == TM_COEF_QUAD) {
            cq = tm_load<R, T>(coef[(int64_t)e * Q + q]);
          }
          cW = cW + s_w[q] * cq;
        }
        p1_laplace_closed_form<D, R>(X, cW, Ke);
        continue;
      }
      for (int i = 0; i < SE; ++i) Ke[i] = Num<R>::zero();
      for (int q = 0; q < Q; ++q) {
        R g[B][D], jxw;
        point_geometry<D, B, R>(X, s_dN + q * B * D, s_w[q], g, jxw);
        const R* Nq = s_N + q * B;
        if constexpr (FORM == TM_FORM_LOAD) {
          R fq[H];
#pragma unroll
          for (int h = 0; h < H; ++h) {
            if (args.coef_kind == TM_COEF_SCALAR) fq[h] = scal[h];
            else if (args.coef_kind == TM_COEF_ELEMENT) fq[h] = ce;
            else if (args.coef_kind == TM_COEF_QUAD) fq[h] = tm_load<R, T>(coef[((int64_t)e * Q + q) * H + h]);
            else {
              R s = Num<R>::zero();
#pragma unroll
              for (int b = 0; b < B; ++b) s = tm_fma_acc(s, s_pc[lv[b] * H + h], Nq[b]);
              fq[h] = s;
            }
            fq[h] = fq[h] * jxw;
          }
#pragma unroll
          for (int i = 0; i < B; ++i)
#pragma unroll
            for (int h = 0; h < H; ++h) Ke[i * H + h] = tm_fma_acc(Ke[i * H + h], fq[h], Nq[i]);
        } else {
          R cq = ce;
          if (args.coef_kind == TM_COEF_POINT) {
            R s = Num<R>::zero();
#pragma unroll
            for (int b = 0; b < B; ++b) s = tm_fma_acc(s, s_pc[lv[b]], Nq[b]);
            cq = s;
          } else if (args.coef_kind == TM_COEF_QUAD) {
            cq = tm_load<R, T>(coef[(int64_t)e * Q + q]);
          }
          const R cw = cq * jxw;
          if constexpr (FORM == TM_FORM_LAPLACE) {
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
              for (int j = 0; j < B; ++j) {
                R dot = Num<R>::zero();
#pragma unroll
                for (int d = 0; d < D; ++d) dot = tm_fma_acc(dot, g[i][d], g[j][d]);
                Ke[i * B + j] = tm_fma_acc(Ke[i * B + j], cw, dot);
              }
          } else if constexpr (FORM == TM_FORM_MASS) {
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
              for (int j = 0; j < B; ++j) Ke[i * B + j] = tm_fma_acc(Ke[i * B + j], cw, Nq[i] * Nq[j]);
          } else {  // elasticity: lam g_i[a] g_j[b] + mu (delta_ab g_i.g_j + g_i[b] g_j[a])
            const R lw = cw * lam1, mw = cw * mu1;
#pragma unroll
            for (int i = 0; i < B; ++i)
#pragma unroll
              for (int j = 0; j < B; ++j) {
                R dot = Num<R>::zero();
#pragma unroll
                for (int d = 0; d < D; ++d) dot = tm_fma_acc(dot, g[i][d], g[j][d]);
                const int base = (i * B + j) * HH;
#pragma unroll
                for (int a = 0; a < H; ++a)
#pragma unroll
                  for (int b = 0; b < H; ++b) {
                    R v = lw * (g[i][a] * g[j][b]) + mw * (g[i][b] * g[j][a]);
                    if (a == b) v = v + mw * dot;
                    Ke[base + a * H + b] = Ke[base + a * H + b] + v;
                  }
              }
          }
        }
      }
    }
    if (__syncthreads_or(kGuard && flag)) return false;
    // --- phase B: row-owner gather in incidence order ------------------------
    for (int lr = tid; lr < nr; lr += kThreads) {
      int cur = s_cur[lr];
      const int end = plan.iptr[rbeg + lr + 1];
      const int ro = L::kLoad ? lr * H : plan.racc[rbeg + lr] * HH;
      while (cur < end) {
        const int le = plan.inc_elem[cur];
        if (le >= cend) break;
        const int a = plan.inc_a[cur];
        const Strided<R> Ke{s_stage + (le - cbeg), chunk};
        if constexpr (L::kLoad) {
#pragma unroll
          for (int h = 0; h < H; ++h) s_acc[ro + h] = s_acc[ro + h] + Ke[a * H + h];
        } else {
#pragma unroll
          for (int b = 0; b < B; ++b) {
            const int pos = plan.inc_pos[(int64_t)cur * B + b];
            R* dst = s_acc + ro + pos * HH;
            const int src = (a * B + b) * HH;
#pragma unroll
            for (int t = 0; t < HH; ++t) dst[t] = dst[t] + Ke[src + t];
          }
        }
        ++cur;
      }
      s_cur[lr] = cur;
    }
    __syncthreads();
  }

  // --- write the finished rows (frame values scaled back by 2^(k p)) ----------
  T* out = static_cast<T*>(args.out);
  const int ks = fr.k * frame_power<D, FORM>();
  auto put = [&](R v) -> T { return fr.bad ? T(NAN) : (T)tm_scale_pow2(tm_store<T, R>(v), ks); };
  const int lane = tid & 31, warp = tid >> 5;
  for (int lr = warp; lr < nr; lr += kThreads / 32) {
    const int r = plan.rows[rbeg + lr];
    if constexpr (L::kLoad) {
      if (lane < H) out[(int64_t)r * H + lane] = put(s_acc[lr * H + lane]);
    } else {
      const int64_t s0 = plan.indptr[r];
      const int deg = (int)(plan.indptr[r + 1] - s0);
      const int ro = plan.racc[rbeg + lr];
      if constexpr (H == 1) {
        for (int k = lane; k < deg; k += 32) out[s0 + k] = put(s_acc[ro + k]);
      } else {
#pragma unroll
        for (int a = 0; a < H; ++a) {
          const int64_t base = (int64_t)HH * s0 + (int64_t)a * H * deg;
          for (int t = lane; t < deg * H; t += 32) {
            const int k = t / H, b = t - (t / H) * H;
            out[base + t] = put(s_acc[(ro + k) * HH + a * H + b]);
          }
        }
      }
    }
  }
  return true;
}

// Assemble the rows owned by patch p: double-float first, native FP64 when the
// guarded pass hands the patch over (the decision is CTA-uniform).
template <int EL, int FORM, int H, class T, class R>
__device__ void assemble_patch(const tm_patch_plan& plan, const tm_assemble_args& args, const int p, const int chunk,
                               unsigned char* smem_raw) {
  constexpr bool kGuard = std::is_same<R, df64>::value;
  if (assemble_patch_pass<EL, FORM, H, T, R, kGuard>(plan, args, p, chunk, smem_raw)) return;
  if constexpr (kGuard) {
    __syncthreads();
    assemble_patch_pass<EL, FORM, H, T, double, false>(plan, args, p, chunk, smem_raw);
  }
}

template <int EL, int FORM, int H, class T, class R>
__global__ void __launch_bounds__(kThreads)
patch_assemble_kernel(tm_patch_plan plan, tm_assemble_args args, int chunk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  assemble_patch<EL, FORM, H, T, R>(plan, args, blockIdx.x, chunk, smem_raw);
}

// Shared-memory bytes needed by one CTA.
template <int EL, int FORM, int H, class R>
inline size_t patch_smem_bytes(const tm_patch_plan& plan, int coef_kind, int chunk) {
  using L = Layout<EL, FORM, H>;
  constexpr int D = L::D, B = L::B;
  size_t n = kMaxQuad + kMaxQuad * B + kMaxQuad * B * D;
  if (coef_kind == TM_COEF_POINT) n += (size_t)plan.max_vtx * (L::kLoad ? H : 1);
  n += L::kLoad ? (size_t)plan.max_rows * H : (size_t)plan.max_slots * L::HH;
  n += (size_t)chunk * L::SE;
  return 32 + (size_t)plan.max_vtx * D * 8 + n * sizeof(R) + (size_t)plan.max_rows * sizeof(int) + 16;
}

template <int EL, int FORM, int H, class T, class R>
int launch_patch_assemble(const tm_patch_plan& plan, const tm_assemble_args& args, cudaStream_t stream) {
  using L = Layout<EL, FORM, H>;
  int dev = 0;
  cudaGetDevice(&dev);
  int max_optin = 0;
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // staging chunk: as many elements as threads, shrunk to fit shared memory
  int chunk = kThreads;
  size_t bytes = patch_smem_bytes<EL, FORM, H, R>(plan, args.coef_kind, chunk);
  while (bytes > (size_t)max_optin && chunk > 1) {
    chunk = chunk / 2;
    bytes = patch_smem_bytes<EL, FORM, H, R>(plan, args.coef_kind, chunk);
  }
  if (bytes > (size_t)max_optin) return TM_ERR_INDEX;
  auto kern = patch_assemble_kernel<EL, FORM, H, T, R>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
    return TM_ERR_CUDA;
  kern<<<plan.n_patches, kThreads, bytes, stream>>>(plan, args, chunk);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

// Dispatch over form/H for one element type and one arithmetic (T stored,
// R computed in).  The element types instantiate it in their own translation
// units (the heaviest element splits it per arithmetic) so the build
// parallelises.
template <int EL, class T, class R>
int assemble_element_as(const tm_patch_plan& plan, const tm_assemble_args& a, cudaStream_t s) {
  constexpr int D = Elem<EL>::D;
  switch (a.form) {
    case TM_FORM_LAPLACE: return launch_patch_assemble<EL, TM_FORM_LAPLACE, 1, T, R>(plan, a, s);
    case TM_FORM_MASS: return launch_patch_assemble<EL, TM_FORM_MASS, 1, T, R>(plan, a, s);
    case TM_FORM_ELASTICITY: return launch_patch_assemble<EL, TM_FORM_ELASTICITY, D, T, R>(plan, a, s);
    case TM_FORM_LOAD:
      if (a.n_comp == 1) return launch_patch_assemble<EL, TM_FORM_LOAD, 1, T, R>(plan, a, s);
      if (a.n_comp == 2) return launch_patch_assemble<EL, TM_FORM_LOAD, 2, T, R>(plan, a, s);
      if (a.n_comp == 3) return launch_patch_assemble<EL, TM_FORM_LOAD, 3, T, R>(plan, a, s);
      return TM_ERR_UNSUPPORTED;
    default: return TM_ERR_UNSUPPORTED;
  }
}

// float32 in float; float64 in native FP64 (precision "native") or in
// double-float (the default).
template <int EL>
int assemble_element(const tm_patch_plan& plan, const tm_assemble_args& a, cudaStream_t s) {
  if (a.dtype == TM_F32) return assemble_element_as<EL, float, float>(plan, a, s);
  if (a.precision == TM_PREC_NATIVE) return assemble_element_as<EL, double, double>(plan, a, s);
  return assemble_element_as<EL, double, df64>(plan, a, s);
}

}  // namespace tmg
