// Specialised kernel of the headline case: P1 tetrahedra, Laplace form with a
// scalar, per-element, nodal or per-quadrature-point coefficient, float64
// (double-float arithmetic on the FP32 pipe) or float32.
//
// Same patch decomposition and deterministic row-owner accumulation as the
// generic kernel (assemble_impl.cuh); what is specific:
//
//  * the element algebra runs in the patch frame (patch_frame.cuh): the
//    patch's vertices relative to its first vertex, scaled by a power of two,
//    so the result does not depend on where the mesh sits or in which units;
//  * the element matrix comes from the cross products of the edge vectors
//    d_k = X_k - X_0: C_1 = d_2 x d_3, C_2 = d_3 x d_1, C_3 = d_1 x d_2 are
//    det * grad N_1..3, so K_ab = c W C_a . C_b / |det| (a, b >= 1, W the sum
//    of the quadrature weights, c the coefficient averaged over them) and row
//    0 is minus the sum of the others.  Its rounding error grows like the
//    element's aspect ratio (the metric-tensor form G = D^T D grows like its
//    square);
//  * "lazy" double-float values (hi, lo) whose lo part is not renormalised
//    after every operation (error-free products by FMA, TwoSum only where two
//    leading parts are added); 1 / |det| from the MUFU estimate plus one
//    Newton step;
//  * 10 unique values of the symmetric element matrix are staged (one stage
//    of 256 elements: measured on GB300, a double-buffered stage with one
//    barrier per chunk costs more through the lost occupancy than it saves);
//  * 64 registers, so four CTAs share an SM.
//
// The float64 result stays within the 1e-12 bar on every input: a patch with
// an element whose conditioning proxy tr(G) tr(adj G) / det(G) exceeds
// kCondMax (slivers), a coefficient outside the range double-float can hold,
// or a non-finite coordinate, is redone by its CTA in native FP64 from the
// start (the decision is CTA-uniform: __syncthreads_or).
#pragma once
#include "assemble_impl.cuh"
#include "patch_frame.cuh"
#include <type_traits>

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

TM_D float tm_rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// 1/x for x > 0: MUFU estimate y0, then y0 + y0 r with the residual
// r = 1 - x y0 formed from the error-free product x.h y0 = p + pe (1 - p is
// exact: p lies within a few ulps of 1).
TM_D L2 l2_rcp(L2 x) {
  x = l2_norm(x);
  const float y0 = tm_rcp_approx(x.h);
  const float p = __fmul_rn(x.h, y0);
  const float pe = __fmaf_rn(x.h, y0, -p);
  const float r = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, p), pe), __fmul_rn(x.l, y0));
  return l2_norm(L2{y0, __fmul_rn(y0, r)});
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

// Arithmetic policies: emulated FP64 (lazy double-float, stored as float2),
// native FP64 (the fallback) and plain FP32 (the float32 variant).
template <class A> struct Ar;
template <> struct Ar<L2> {
  using S = float2;
  static TM_D L2 pair(float h, float l) { return L2{h, l}; }
  static TM_D L2 scale2(L2 a, float p2) { return L2{__fmul_rn(a.h, p2), __fmul_rn(a.l, p2)}; }
  static TM_D L2 ld(S v) { return L2{v.x, v.y}; }
  static TM_D S st(L2 a) { return make_float2(a.h, a.l); }
  static TM_D L2 in(double x) { return l2_from(tm_from_double(x)); }
  static TM_D L2 in(float x) { return L2{x, 0.f}; }
  static TM_D L2 add(L2 a, L2 b) { return l2_add(a, b); }
  static TM_D L2 sub(L2 a, L2 b) { return l2_sub(a, b); }
  static TM_D L2 mul(L2 a, L2 b) { return l2_mul(a, b); }
  static TM_D L2 neg(L2 a) { return l2_neg(a); }
  static TM_D L2 abs(L2 a) { return a.h < 0.f ? l2_neg(a) : a; }
  static TM_D L2 rsqrt(L2 a) { return l2_rsqrt(a); }
  static TM_D L2 rcp(L2 a) { return l2_rcp(a); }
  static TM_D L2 zero() { return L2{0.f, 0.f}; }
  static TM_D float hi(L2 a) { return a.h; }
  static TM_D double out(S v) { return tm_to_double(df64{v.x, v.y}); }
};
template <> struct Ar<double> {
  using S = double;
  static TM_D double pair(float h, float l) { return (double)h + (double)l; }
  static TM_D double scale2(double a, float p2) { return a * (double)p2; }
  static TM_D double ld(S v) { return v; }
  static TM_D S st(double a) { return a; }
  static TM_D double in(double x) { return x; }
  static TM_D double in(float x) { return (double)x; }
  static TM_D double add(double a, double b) { return a + b; }
  static TM_D double sub(double a, double b) { return a - b; }
  static TM_D double mul(double a, double b) { return a * b; }
  static TM_D double neg(double a) { return -a; }
  static TM_D double abs(double a) { return fabs(a); }
  static TM_D double rsqrt(double a) { return 1.0 / sqrt(a); }
  static TM_D double rcp(double a) { return 1.0 / a; }
  static TM_D double zero() { return 0.0; }
  static TM_D float hi(double a) { return (float)a; }
  static TM_D double out(S v) { return v; }
};
template <> struct Ar<float> {
  using S = float;
  static TM_D float pair(float h, float l) { return __fadd_rn(h, l); }
  static TM_D float scale2(float a, float p2) { return __fmul_rn(a, p2); }
  static TM_D float ld(S v) { return v; }
  static TM_D S st(float a) { return a; }
  static TM_D float in(double x) { return (float)x; }
  static TM_D float in(float x) { return x; }
  static TM_D float add(float a, float b) { return a + b; }
  static TM_D float sub(float a, float b) { return a - b; }
  static TM_D float mul(float a, float b) { return a * b; }
  static TM_D float neg(float a) { return -a; }
  static TM_D float abs(float a) { return fabsf(a); }
  static TM_D float rsqrt(float a) { return rsqrtf(a); }
  static TM_D float rcp(float a) { return 1.0f / a; }
  static TM_D float zero() { return 0.f; }
  static TM_D float hi(float a) { return a; }
  static TM_D float out(S v) { return v; }
};

// Conditioning bound of the double-float element algebra: with frame
// coordinates the cross-product form stays within a few 1e-13 of the element's
// largest entry up to tr(G) tr(adj G) / det(G) = 1e4 (a regular tetrahedron
// has 9, the six Kuhn tetrahedra of a cube 30, aspect ratio ~100 slivers
// ~1e4); elements above it take the native FP64 path.
constexpr float kCondMax = 1.0e4f;
// A coefficient whose binary exponent lies outside +-kCoefExp would push the
// frame element values out of float's exponent range (with room for the lo
// parts); its patch is redone in native FP64.
constexpr int kCoefExp = 60;

TM_D bool coef_in_range(double c) {
  const int e = (int)(((unsigned long long)__double_as_longlong(c) >> 52) & 0x7ff);
  return c == 0.0 || (e >= 1023 - kCoefExp && e <= 1023 + kCoefExp);
}

constexpr int kTetChunk = kThreads;  // elements staged per chunk (one per thread)

// A double in double-float for 2^-74 <= |x| < 2^128: hi = x truncated to 24
// significant bits, lo = the low 29 bits rounded to float (2^-48 of x).  The
// fast pass uses it for coefficients it has checked with coef_in_range (any
// other value sends the patch to the native pass, so its result is unused).
TM_D L2 l2_from_double_in_range(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hw = (unsigned)(b >> 32);
  const unsigned e = (hw >> 20) & 0x7ffu;
  const float h = __uint_as_float((hw & 0x80000000u) | ((e - 896u) << 23) | ((unsigned)(b >> 29) & 0x7fffffu));
  const float l = __fmul_rn(__int2float_rn((int)(b & 0x1fffffffull)), __uint_as_float((e - 948u) << 23));
  return L2{h, (hw & 0x80000000u) ? -l : l};
}

// Shared-memory layout of one CTA.
struct TetSmem {
  unsigned long long* red;  // [3] (4 words reserved)
  long long* R;             // [max_vtx * 3] integer frame coordinates
  unsigned char* pc;        // [max_vtx] point coefficients (TM_COEF_POINT)
  unsigned char* acc;       // [max_deg][nrp] row accumulators
  unsigned char* stage;     // [10][kTetChunk]
};

// Row state of the thread that owns a row (owner == tid < nr).
struct TetRow {
  bool owner;
  int deg, dpos, cur0, end;
  int64_t o0;
};

// One pass over the patch in arithmetic A.  Returns false (on every thread)
// when the patch must be redone in native FP64.
template <class T, class A, class RW, bool kGuard>
__device__ __forceinline__ bool p1tet_laplace_pass(const tm_patch_plan& plan, const tm_assemble_args& args,
                                                   const TetSmem& sm, const TetRow& row, int nrp) {
  using P = Ar<A>;
  using S = typename P::S;
  using R = Rec<RW>;
  const RW* recs = R::ptr(plan);
  const int p = blockIdx.x, tid = threadIdx.x;
  const int Q = args.n_quad;
  const int vbeg = plan.vptr[p], nv = plan.vptr[p + 1] - vbeg;
  const int ebeg = plan.eptr[p], ne = plan.eptr[p + 1] - ebeg;
  const long long* s_R = sm.R;
  S* s_pc = reinterpret_cast<S*>(sm.pc);
  S* s_acc = reinterpret_cast<S*>(sm.acc);
  S* s_stage = reinterpret_cast<S*>(sm.stage);

  // ---- phase 0: frame, point coefficients, zeroed accumulators, cursors.
  // The first chunk's element data and each owner's first record do not
  // depend on the frame: their loads are issued first, so that they are in
  // flight while the frame's coordinate gathers and reductions run.
  const T* coef = static_cast<const T*>(args.coef);
  const bool per_elem = args.coef_kind == TM_COEF_ELEMENT;
  // element data of this thread's next element (thread tid handles element
  // c * kTetChunk + tid of chunk c), loaded one chunk ahead
  uint2 cw_next = make_uint2(0u, 0u);
  T c_next = T(0);
  if (tid < ne) {
    cw_next = *reinterpret_cast<const uint2*>(plan.econn + (int64_t)(ebeg + tid) * 4);
    if (per_elem) c_next = coef[plan.elem[ebeg + tid]];
  }
  int cur = 0;
  RW rec = R::kEnd;
  if (row.owner) {
    cur = row.cur0;
    if (cur < row.end) rec = recs[cur];
  }
  const T* pts = static_cast<const T*>(args.points);
  const FrameInfo fr = patch_frame<3, T>(pts, plan.vtx + vbeg, nv, sm.R, sm.red);
  if (fr.bad) {
    // a coordinate is inf or nan: the guarded pass hands the patch to the
    // native pass, which writes nan to the patch's rows
    if (kGuard) return false;
    if (row.owner) {
      T* out = static_cast<T*>(args.out);
      for (int k = 0; k < row.deg; ++k) out[row.o0 + k] = T(NAN);
    }
    return true;
  }
  const int kf = fr.k;
  const ShortConv sconv = short_conv(fr.t + fr.z - 62);
  const double esc_native = std::is_same<A, double>::value ? ldexp(1.0, fr.z - 62) : 0.0;
  if (args.coef_kind == TM_COEF_POINT)
    for (int i = tid; i < nv; i += kThreads) s_pc[i] = P::st(P::in(coef[plan.vtx[vbeg + i]]));
  S* acc = s_acc + tid;  // this thread's row: entry k at acc[k * nrp]
  if (row.owner)
    for (int k = 0; k < row.deg; ++k) acc[k * nrp] = P::st(P::zero());
  double wsum = 0.0;
  for (int q = 0; q < Q; ++q) wsum += args.tables[q];
  const A W = P::in(wsum);
  const double sc_raw = args.scal[0];
  const A sc = P::in(sc_raw);
  bool flag = kGuard && !coef_in_range((double)sc_raw) && args.coef_kind == TM_COEF_SCALAR;
  __syncthreads();

  // ---- phase A for chunk c: the element of thread tid into stage buffer c & 1
  auto phase_a = [&](int ch) {
    const int le = ch * kTetChunk + tid;
    if (le >= ne) return;
    const int pair = ebeg + le;
    const uint2 cw = cw_next;
    const T c_raw = c_next;
    if (le + kTetChunk < ne) {
      cw_next = *reinterpret_cast<const uint2*>(plan.econn + (int64_t)(pair + kTetChunk) * 4);
      if (per_elem) c_next = coef[plan.elem[pair + kTetChunk]];
    }
    const int lv[4] = {(int)(cw.x & 0xffff), (int)(cw.x >> 16), (int)(cw.y & 0xffff), (int)(cw.y >> 16)};
    double c_dbl = 0.0;  // the coefficient in double where it is formed on the side
    A c;
    if (per_elem) {
      if constexpr (std::is_same<A, L2>::value) c = l2_from_double_in_range((double)c_raw);
      else c = P::in(c_raw);
      c_dbl = (double)c_raw;
    } else if (args.coef_kind == TM_COEF_POINT) {
      // sum_q w_q sum_b N_b(q) c_b / W : the weighted vertex average
      double cw_ = 0.0;
      for (int q = 0; q < Q; ++q)
        for (int b = 0; b < 4; ++b) cw_ += args.tables[q] * args.tables[Q + q * 4 + b] * (double)P::out(s_pc[lv[b]]);
      c_dbl = cw_ / wsum;
      c = P::in(c_dbl);
    } else if (args.coef_kind == TM_COEF_QUAD) {
      double cw_ = 0.0;
      for (int q = 0; q < Q; ++q) cw_ += args.tables[q] * (double)coef[(int64_t)plan.elem[pair] * Q + q];
      c_dbl = cw_ / wsum;
      c = P::in(c_dbl);
    } else {
      c = sc;
      c_dbl = sc_raw;
    }
    if (kGuard && !coef_in_range(c_dbl)) flag = true;
    // edge vectors, exact to 2^-48 of themselves, equal to 2^e_sh times their frame values
    A d[3][3];
    int e_sh;
    if (fr.shortp) {
      // short patch: |difference| < 2^22, converted exactly into frame units
      const int* r32 = reinterpret_cast<const int*>(s_R);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int r0 = r32[2 * (lv[0] * 3 + j)];
#pragma unroll
        for (int k = 0; k < 3; ++k) d[k][j] = P::pair(sconv(r32[2 * (lv[k + 1] * 3 + j)] - r0), 0.f);
      }
      e_sh = 0;
    } else if constexpr (std::is_same<A, double>::value) {
      // native FP64 (patches handed over by the guard): the full 53 bits of
      // every difference, in frame units (a 48-bit split would carry its
      // 2^-48 error through these ill-conditioned elements)
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) d[k][j] = __ll2double_rn(s_R[lv[k + 1] * 3 + j] - s_R[lv[0] * 3 + j]) * esc_native;
      e_sh = 0;
    } else {
      float eh[3][3], el[3][3];
      const int u = exact_edges<3, 3>(s_R, lv, eh, el);
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) d[k][j] = P::pair(eh[k][j], el[k][j]);
      e_sh = u - fr.z;   // u < 0 (a degenerate element) fails the conditioning test below
    }
    auto cross = [](const A* u, const A* v, A* o) {
      o[0] = P::sub(P::mul(u[1], v[2]), P::mul(u[2], v[1]));
      o[1] = P::sub(P::mul(u[2], v[0]), P::mul(u[0], v[2]));
      o[2] = P::sub(P::mul(u[0], v[1]), P::mul(u[1], v[0]));
    };
    auto dot3 = [](const A* u, const A* v) {
      return P::add(P::add(P::mul(u[0], v[0]), P::mul(u[1], v[1])), P::mul(u[2], v[2]));
    };
    A C[3][3];
    cross(d[1], d[2], C[0]);
    cross(d[2], d[0], C[1]);
    cross(d[0], d[1], C[2]);
    const A det = dot3(d[0], C[0]);
    const A D11 = dot3(C[0], C[0]), D22 = dot3(C[1], C[1]), D33 = dot3(C[2], C[2]);
    S* st = s_stage + tid;
    if constexpr (kGuard) {
      float trg = 0.f;
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) trg = __fmaf_rn(P::hi(d[k][j]), P::hi(d[k][j]), trg);
      const float dh = P::hi(det);
      const float tra = P::hi(D11) + P::hi(D22) + P::hi(D33);
      if (!(e_sh >= -100 && e_sh <= 100 && dh * dh >= 1e-30f && trg * tra <= kCondMax * (dh * dh))) {
        // ill-conditioned, degenerate, or tiny against its patch (frame
        // products near float's underflow): the patch goes native
        flag = true;
        return;
      }
    }
    // the edges are 2^e_sh times their frame values and K scales as length^1
    const A s = P::scale2(P::mul(P::mul(c, W), P::rcp(P::abs(det))), tm_pow2f(-e_sh));
    const A k11 = P::mul(s, D11), k22 = P::mul(s, D22), k33 = P::mul(s, D33);
    const A k12 = P::mul(s, dot3(C[0], C[1])), k13 = P::mul(s, dot3(C[0], C[2])), k23 = P::mul(s, dot3(C[1], C[2]));
    const A k01 = P::neg(P::add(P::add(k11, k12), k13));
    const A k02 = P::neg(P::add(P::add(k12, k22), k23));
    const A k03 = P::neg(P::add(P::add(k13, k23), k33));
    const A k00 = P::neg(P::add(P::add(k01, k02), k03));
    const A vals[10] = {k00, k01, k02, k03, k11, k12, k13, k22, k23, k33};
#pragma unroll
    for (int u = 0; u < 10; ++u) st[u * kTetChunk] = P::st(vals[u]);
  };

  // ---- phase B for chunk c: the row owner adds its incidences of the chunk
  // (fixed order).  The diagonal is summed in registers and added once per
  // chunk; the three off-diagonal contributions of an incidence hit distinct
  // columns, so their read-modify-writes are issued together.  The record that
  // ends the loop is the first one of the next chunk.
  auto phase_b = [&](int ch) {
    if (!row.owner) return;
    const int cbeg = ch * kTetChunk, cend = cbeg + kTetChunk;
    const S* stg = s_stage;
    A dg = P::zero();
    bool any = false;
    for (;;) {
      const int lel = R::elem(rec);
      if (lel >= cend) break;  // also the end record (its element field is past every chunk)
      const RW next = (cur + 1 < row.end) ? recs[cur + 1] : R::kEnd;
      const int a = R::a(rec);
      const int lo = lel - cbeg;
      const uint32_t u = (uint32_t)(kTet4Stage >> (16 * a));
      dg = P::add(dg, P::ld(stg[(int)(u & 15u) * kTetChunk + lo]));
      int pos[3];
      S v[3], old[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        pos[j] = R::pos(rec, j) * nrp;
        v[j] = stg[(int)((u >> (4 * j + 4)) & 15u) * kTetChunk + lo];
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) old[j] = acc[pos[j]];
#pragma unroll
      for (int j = 0; j < 3; ++j) acc[pos[j]] = P::st(P::add(P::ld(old[j]), P::ld(v[j])));
      any = true;
      rec = next;
      ++cur;
    }
    if (any) acc[row.dpos * nrp] = P::st(P::add(P::ld(acc[row.dpos * nrp]), dg));
  };

  const int nch = (ne + kTetChunk - 1) / kTetChunk;
  for (int c = 0; c < nch; ++c) {
    phase_a(c);
    if (__syncthreads_or(kGuard && flag)) return false;   // stage c complete (or the patch goes native)
    phase_b(c);
    __syncthreads();                                       // stage free for chunk c + 1
  }
  // ---- write the finished row: only its owner ever touched it, so no
  // barrier is needed; consecutive lanes write consecutive rows' k-th entries
  if (row.owner) {
    T* out = static_cast<T*>(args.out);
    for (int k = 0; k < row.deg; ++k) out[row.o0 + k] = (T)tm_scale_pow2(P::out(acc[k * nrp]), kf);
  }
  return true;
}

template <class T, class A, class RW>
__global__ void __launch_bounds__(kThreads, 4)
p1tet_laplace_fast_kernel(tm_patch_plan plan, tm_assemble_args args) {
  constexpr bool kGuard = std::is_same<A, L2>::value;
  using S = typename Ar<A>::S;
  const int p = blockIdx.x;
  const int tid = threadIdx.x;
  const int rbeg = plan.rptr[p], nr = plan.rptr[p + 1] - rbeg;
  if (nr == 0) return;

  // Accumulators are column-major over the patch's rows: entry k of local row
  // lr sits at acc[k * nrp + lr], nrp = max_rows rounded up to 16, so the
  // 16 lanes of a half-warp (consecutive rows) hit 16 distinct bank pairs
  // whatever columns their incidences touch.
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nrp = (plan.max_rows + 15) & ~15;
  TetSmem sm;
  sm.red = reinterpret_cast<unsigned long long*>(smem_raw);
  sm.R = reinterpret_cast<long long*>(smem_raw + 32);
  unsigned char* q = smem_raw + 32 + (size_t)plan.max_vtx * 3 * 8;
  sm.pc = q;
  if (args.coef_kind == TM_COEF_POINT) q += ((size_t)plan.max_vtx * 8 + 15) & ~size_t(15);
  sm.acc = q;
  q += (size_t)plan.max_deg * nrp * sizeof(S);
  sm.stage = q;

  TetRow row;
  row.owner = tid < nr;
  row.deg = row.dpos = row.cur0 = row.end = 0;
  row.o0 = 0;
  if (row.owner) {
    const int r = plan.rows[rbeg + tid];
    row.o0 = plan.indptr[r];
    row.deg = (int)(plan.indptr[r + 1] - row.o0);
    row.dpos = plan.rdiag[rbeg + tid];
    row.cur0 = plan.iptr[rbeg + tid];
    row.end = plan.iptr[rbeg + tid + 1];
  }
  if (p1tet_laplace_pass<T, A, RW, kGuard>(plan, args, sm, row, nrp)) return;
  if constexpr (kGuard) {
    __syncthreads();  // every thread is done with the double-float pass's shared memory
    p1tet_laplace_pass<T, double, RW, false>(plan, args, sm, row, nrp);
  }
}

inline size_t p1tet_smem_bytes(const tm_patch_plan& plan, int coef_kind, size_t elem) {
  const size_t nrp = (size_t)((plan.max_rows + 15) & ~15);
  size_t b = 32 + (size_t)plan.max_vtx * 3 * 8;
  if (coef_kind == TM_COEF_POINT) b += ((size_t)plan.max_vtx * 8 + 15) & ~size_t(15);
  b += (size_t)plan.max_deg * nrp * elem + (size_t)10 * kTetChunk * elem;
  return b;
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
  const size_t bytes = p1tet_smem_bytes(plan, args.coef_kind, sizeof(typename Ar<A>::S));
  if (bytes > (size_t)max_optin) return TM_ERR_INDEX;
  auto kern = p1tet_laplace_fast_kernel<T, A, RW>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
    return TM_ERR_CUDA;
  kern<<<plan.n_patches, kThreads, bytes, stream>>>(plan, args);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

template <class T, class A>
inline int launch_p1tet_laplace_fast(const tm_patch_plan& plan, const tm_assemble_args& args, cudaStream_t stream) {
  if (plan.inc_pack32) return launch_p1tet_kernel<T, A, uint32_t>(plan, args, stream);
  return launch_p1tet_kernel<T, A, uint64_t>(plan, args, stream);
}

}  // namespace tmg
