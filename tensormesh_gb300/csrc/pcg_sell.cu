// Jacobi-PCG over a SELL-32 copy of the matrix, in two forms: standard
// (Hestenes-Stiefel) PCG with two grid barriers per iteration (the default,
// pcg_sell_hs_kernel), and the pipelined form of Ghysels & Vanroose ("Hiding
// global synchronization latency in the preconditioned Conjugate Gradient
// algorithm", Parallel Computing 40(7), 2014, Algorithm 4) with one barrier
// per iteration (pcg_sell_kernel).  The pipelined recurrences lose accuracy
// faster: in float32 they break down (denominator <= 0) near a 1e-3 relative
// residual on 3D Poisson, and in double-float on ill-conditioned elasticity,
// so they are opt-in.
//
// Same contract as tm_pcg_jacobi (the reference's Jacobi preconditioner,
// sparse/solve/torch_solve.py:24-59, M = diag(A)^-1 with a missing or zero
// diagonal taken as 1, inside its CG loop, torch_solve.py:70-128; stop when
// ||r|| <= max(rtol ||b||, atol) on the recurrence residual), different data
// path:
//
// * SELL-32 layout: rows are grouped in slices of 32 consecutive rows; a
//   slice stores its rows' entries column-major, padded to its longest row
//   (pad entries: column = the row itself, value 0).  Entry j of row
//   32 s + l sits at slice_ptr[s] + 32 j + l, so the 32 lanes of a warp read
//   one contiguous run of column data (128 B of int32 columns, or 64 B of
//   int16 offsets from the row where every offset fits) and one of values
//   (256 B in double-float) per entry.
// * The preconditioner is folded into the stored values: the copy holds
//   A M (column j scaled by M_jj), so the product n = A M w that the
//   pipelined recurrence needs is one gather of w per entry.
// * Pipelined recurrence (u = M r, m = M w and q = M s are formed from r, w
//   and s on the fly) of the opt-in form:
//       gamma = (r, u), delta = (w, u), rho = (r, r)       [reduced at the barrier]
//       n = A m
//       beta = gamma / gamma_old, alpha = gamma / (delta - beta gamma / alpha_old)
//       z = n + beta z;  s = w + beta s;  p = u + beta p
//       x += alpha p;    r -= alpha s;    w -= alpha z
//   The partial sums of the next gamma, delta and rho come out of the same
//   row sweep, and the w that the next product gathers is written to the
//   other half of a double buffer, so a single barrier per iteration orders
//   both.  Partial sums are double-buffered too; every CTA sums all per-CTA
//   partials in the same order, so the scalars are identical everywhere and
//   the solve is bitwise repeatable.
// * FP64 systems iterate in double-float (storage pairs of floats, the
//   FP32 pipe), FP32 systems in float.
#include "pcg_common.cuh"

namespace tmg {

constexpr int kSellThreads = 512;
constexpr int kSellWarps = kSellThreads / 32;
// One slice per warp and round, eight entries of each row fetched per round
// with every load issued before the first use (128^3 Poisson, ms per
// iteration: 2 x 4: 0.135, 1 x 8: 0.127, 2 x 8 and 1 x 12 spill registers)
constexpr int kSellRows = 1;  // slices a warp advances together
constexpr int kSellIlp = 8;   // entries of each row fetched per round

template <class S> struct SellT;
template <> struct SellT<float> {
  using A = float;   // arithmetic
  using V = float;   // user vectors and CSR values
  static TM_D A ld(const float* p, int64_t i) { return p[i]; }
  static TM_D void st(float* p, int64_t i, A v) { p[i] = v; }
  static TM_D A mk(float v) { return v; }
  static TM_D float pack(A v) { return v; }
  static TM_D A in(V v) { return v; }
  static TM_D V out(A v) { return v; }
  static TM_D A from_double(double d) { return (float)d; }
  static TM_D double to_double(A v) { return (double)v; }
  static TM_D A zero() { return 0.f; }
};
template <> struct SellT<double> {  // native FP64 (plain products, no iteration)
  using A = double;
  using V = double;
  static TM_D A ld(const double* p, int64_t i) { return p[i]; }
  static TM_D void st(double* p, int64_t i, A v) { p[i] = v; }
  static TM_D A mk(double v) { return v; }
  static TM_D double pack(A v) { return v; }
  static TM_D A in(V v) { return v; }
  static TM_D V out(A v) { return v; }
  static TM_D A from_double(double d) { return d; }
  static TM_D double to_double(A v) { return v; }
  static TM_D A zero() { return 0.0; }
};
template <> struct SellT<F2> {
  using A = df64;
  using V = double;
  static TM_D A ld(const F2* p, int64_t i) { return ld2(p, i); }
  static TM_D void st(F2* p, int64_t i, A v) { st2(p, i, v); }
  static TM_D A mk(F2 v) { return {v.hi, v.lo}; }
  static TM_D F2 pack(A v) { return F2{v.hi, v.lo}; }
  static TM_D A in(V v) { return tm_from_double(v); }
  static TM_D V out(A v) { return tm_to_double(v); }
  static TM_D A from_double(double d) { return tm_from_double(d); }
  static TM_D double to_double(A v) { return tm_to_double(v); }
  static TM_D A zero() { return {0.f, 0.f}; }
};

// Column of a stored entry: absolute (int32) or relative to the row (int16,
// for matrices whose every |column - row| fits; FEM orderings keep the
// coupling bandwidth small), the latter saving 2 of the 12 bytes an entry
// streams per iteration.
TM_D int col_of(const int32_t* scol, int64_t k, int64_t) { return __ldg(scol + k); }
TM_D int col_of(const int16_t* scol, int64_t k, int64_t row) { return (int)row + (int)__ldg(scol + k); }

// Largest |column - row| of the matrix (atomic max into *span).
__global__ void sell_span_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                                 unsigned long long* span) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  unsigned long long m = 0ull;
  if (row < n)
    for (int64_t k = indptr[row]; k < indptr[row + 1]; ++k) {
      const long long d = (long long)idx[k] - row;
      m = max(m, (unsigned long long)(d < 0 ? -d : d));
    }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m) atomicMax(span, m);
}

// Slice widths (32 x the longest row of each slice) into sptr[1..n_slices].
__global__ void sell_width_kernel(int64_t n, const int64_t* __restrict__ indptr, int64_t* __restrict__ sptr) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t n_slices = (n + 31) >> 5;
  if ((row >> 5) >= n_slices) return;
  int64_t len = row < n ? indptr[row + 1] - indptr[row] : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) len = max(len, (int64_t)__shfl_xor_sync(0xffffffffu, len, o));
  if ((threadIdx.x & 31) == 0) sptr[(row >> 5) + 1] = len * 32;
}

// In-place inclusive scan of sptr[1..m] with sptr[0] = 0, one CTA: each
// thread scans a contiguous run, the run totals are scanned in shared memory.
__global__ void __launch_bounds__(1024) sell_scan_kernel(int64_t m, int64_t* __restrict__ sptr) {
  __shared__ int64_t s_tot[1024];
  const int t = threadIdx.x;
  const int64_t per = (m + 1023) / 1024;
  const int64_t a = min(m, t * per), b = min(m, a + per);
  int64_t sum = 0;
  for (int64_t i = a; i < b; ++i) sum += sptr[i + 1];
  s_tot[t] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int64_t v = t >= o ? s_tot[t - o] : 0;
    __syncthreads();
    s_tot[t] += v;
    __syncthreads();
  }
  int64_t run = s_tot[t] - sum;
  for (int64_t i = a; i < b; ++i) {
    run += sptr[i + 1];
    sptr[i + 1] = run;
  }
  if (t == 0) sptr[0] = 0;
}

// M = diag(A)^-1 (a missing or zero diagonal counts as 1), computed in
// double and stored in the iteration's type.
template <class S>
__global__ void sell_dinv_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                                 const typename SellT<S>::V* __restrict__ val, S* __restrict__ dinv) {
  using Tr = SellT<S>;
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= n) return;
  int64_t lo = indptr[row], hi = indptr[row + 1];
  double d = 1.0;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    const int c = idx[mid];
    if (c == row) {
      d = (double)val[mid];
      break;
    }
    if (c < row) lo = mid + 1; else hi = mid;
  }
  Tr::st(dinv, row, Tr::from_double(d != 0.0 ? 1.0 / d : 1.0));
}

// The SELL-32 copy of A M, and y = M^-1 x0 (so that A x0 = (A M) y).  One
// warp per slice, lane l on row 32 s + l.  A slice plan that does not cover
// its rows (width < 32 x row length, or a range outside [0, n_pad]) raises
// TM_ERR_INDEX in the solver record instead of writing.
template <class S, class CT>
__global__ void sell_fill_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                                 const typename SellT<S>::V* __restrict__ val, const int64_t* __restrict__ sptr,
                                 int64_t n_pad, const S* __restrict__ dinv, const typename SellT<S>::V* __restrict__ x0,
                                 CT* __restrict__ scol, S* __restrict__ sval, S* __restrict__ y,
                                 PcgState* st) {
  constexpr bool kRel = sizeof(CT) == 2;
  using Tr = SellT<S>;
  using A = typename Tr::A;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t n_slices = (n + 31) >> 5;
  if (gw >= n_slices) return;
  const int64_t row = gw * 32 + lane;
  const int64_t s0 = sptr[gw], s1 = sptr[gw + 1];
  const int64_t width = s1 - s0;
  const int64_t len = row < n ? indptr[row + 1] - indptr[row] : 0;
  const bool bad = s0 < 0 || s1 > n_pad || width < 0 || (width & 31) != 0 || len > (width >> 5);
  if (__any_sync(0xffffffffu, bad)) {
    if (lane == 0) atomicExch(&st->status, TM_ERR_INDEX);
    return;
  }
  const int L = (int)(width >> 5);
  const int64_t base = row < n ? indptr[row] : 0;
  // pad entries gather a valid column: the row itself, or the last row for
  // the lanes past n of the last slice
  const int32_t pad_col = row < n ? (int32_t)row : (int32_t)(n - 1);
  bool wide = false;  // a column outside [0, n), or an offset that does not fit 16 bits
  for (int j = 0; j < L; ++j) {
    const int64_t k = s0 + (int64_t)j * 32 + lane;
    int32_t c = pad_col;
    A v = Tr::zero();
    if (j < len) {
      const int32_t cj = idx[base + j];
      if (cj < 0 || cj >= n) {
        wide = true;  // stored as the pad entry; the solve stops with TM_ERR_INDEX
      } else {
        c = cj;
        v = Tr::in(val[base + j]) * Tr::ld(dinv, c);
      }
    }
    if constexpr (kRel) {
      const long long d = (long long)c - row;
      wide = wide || d < -32768 || d > 32767;
      scol[k] = (CT)d;
    } else {
      scol[k] = c;
    }
    sval[k] = Tr::pack(v);
  }
  if (__any_sync(0xffffffffu, wide) && lane == 0) atomicExch(&st->status, TM_ERR_INDEX);
  if (row < n) Tr::st(y, row, Tr::in(x0[row]) / Tr::ld(dinv, row));
}

// acc[u] = sum_j sval[.] * g(scol[.]) over the rows of slices sl + u * kSellWarps
// (u < kSellRows) of [sl, s_hi), for the calling lane's row.  g gathers the
// operand's column value (one vector, or a combination of two).
template <class S, class CT, class G>
TM_D void sell_rows(const int64_t* __restrict__ sptr, const CT* __restrict__ scol, const S* __restrict__ sval,
                    const G& g, int64_t sl, int64_t s_hi, typename SellT<S>::A (&acc)[kSellRows]) {
  using Tr = SellT<S>;
  const int lane = threadIdx.x & 31;
  int64_t off[kSellRows];
  int len[kSellRows];
  int lmax = 0;
#pragma unroll
  for (int u = 0; u < kSellRows; ++u) {
    const int64_t s = sl + (int64_t)u * kSellWarps;
    const bool ok = s < s_hi;
    off[u] = ok ? sptr[s] + lane : 0;
    len[u] = ok ? (int)((sptr[s + 1] - sptr[s]) >> 5) : 0;
    lmax = max(lmax, len[u]);
    acc[u] = Tr::zero();
  }
  for (int j0 = 0; j0 < lmax; j0 += kSellIlp) {
    int c[kSellRows][kSellIlp];
    S v[kSellRows][kSellIlp];
#pragma unroll
    for (int u = 0; u < kSellRows; ++u)
#pragma unroll
      for (int j = 0; j < kSellIlp; ++j) {
        const bool ok = j0 + j < len[u];
        const int64_t k = off[u] + (int64_t)(j0 + j) * 32;
        c[u][j] = ok ? col_of(scol, k, (sl + (int64_t)u * kSellWarps) * 32 + lane) : 0;
        v[u][j] = ok ? sval[k] : S{};
      }
#pragma unroll
    for (int u = 0; u < kSellRows; ++u)
#pragma unroll
      for (int j = 0; j < kSellIlp; ++j) acc[u] += Tr::mk(v[u][j]) * g(c[u][j]);
  }
}

// Standard (Hestenes-Stiefel) Jacobi-PCG over the SELL-32 copy of A M, two
// grid barriers per iteration.  With pt = M^-1 p (so that A p = (A M) pt and
// pt_new = r + beta pt_old), an iteration is
//   sweep 1: q = (A M)(r + beta pt_old), gathering r and pt_old and forming
//            the combination per column; pt_new (own rows) to the other half
//            of a double buffer; partial (p, q) = sum M pt q       [barrier]
//   sweep 2: alpha = rz / (p, q); x += alpha M pt; r -= alpha q; partial
//            rz = sum M r^2 and rr = sum r^2                        [barrier]
// The iterates are those of tm_pcg_jacobi's recurrence (z = M r, p = z +
// beta p), so its rounding behaviour is that of standard PCG.
template <class S, class CT>
__global__ void __launch_bounds__(kSellThreads, 2)
pcg_sell_hs_kernel(int64_t n, const int64_t* __restrict__ sptr, const CT* __restrict__ scol,
                   const S* __restrict__ sval, const S* __restrict__ dinv, const typename SellT<S>::V* __restrict__ bv,
                   typename SellT<S>::V* __restrict__ xv, S* x, S* r, S* q, S* pt0, S* pt1, const S* y,
                   double* partials, PcgState* st, double rtol, double atol, int maxiter) {
  using Tr = SellT<S>;
  using A = typename Tr::A;
  __shared__ double s_red[32];
  const unsigned nb = gridDim.x;
  unsigned my_gen = 0;  // the host zeroes st->gen before the launch
  if (*((volatile int*)&st->status) != TM_OK) return;  // slice plan rejected by the fill kernel
  const int64_t n_slices = (n + 31) >> 5;
  const int64_t per = (n_slices + nb - 1) / nb;
  const int64_t s_lo = min(n_slices, (int64_t)blockIdx.x * per), s_hi = min(n_slices, s_lo + per);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* pA = partials;
  double* pB = partials + nb;
  double* pC = partials + 2 * (int64_t)nb;
  auto row_of = [&](int64_t sl, int u) { return (sl + (int64_t)u * kSellWarps) * 32 + lane; };
  auto valid = [&](int64_t sl, int u) { return sl + (int64_t)u * kSellWarps < s_hi && row_of(sl, u) < n; };
  auto publish2 = [&](double* da, A va, double* db, A vb) {
    double a = Tr::to_double(va), b = Tr::to_double(vb);
    block_sum2(a, b, s_red);
    if (threadIdx.x == 0) {
      da[blockIdx.x] = a;
      db[blockIdx.x] = b;
    }
  };

  // ---- r = b - (A M) y, x = x0, pt_old = 0; rz, rr, bb
  {
    A rz_l = Tr::zero(), rr_l = Tr::zero(), bb_l = Tr::zero();
    for (int64_t sl = s_lo + warp; sl < s_hi; sl += (int64_t)kSellRows * kSellWarps) {
      A acc[kSellRows];
      sell_rows<S, CT>(sptr, scol, sval, [&](int c) { return Tr::ld(y, c); }, sl, s_hi, acc);
#pragma unroll
      for (int u = 0; u < kSellRows; ++u) {
        if (!valid(sl, u)) continue;
        const int64_t row = row_of(sl, u);
        const A b = Tr::in(bv[row]);
        const A rv = b - acc[u];
        Tr::st(r, row, rv);
        Tr::st(x, row, Tr::in(xv[row]));
        Tr::st(pt0, row, Tr::zero());
        rz_l += Tr::ld(dinv, row) * rv * rv;
        rr_l += rv * rv;
        bb_l += b * b;
      }
    }
    publish2(pA, rz_l, pB, rr_l);
    const double t = block_sum(Tr::to_double(bb_l), s_red);
    if (threadIdx.x == 0) pC[blockIdx.x] = t;
  }
  if (!grid_sync(st, nb, my_gen)) return;
  double rz, rr;
  sum_partials2(pA, pB, nb, s_red, rz, rr);
  const double bnorm = sqrt(sum_partials(pC, nb, s_red));
  const double tol = fmax(rtol * bnorm, atol);
  if (blockIdx.x == 0 && threadIdx.x == 0) st->bnorm = bnorm;
  if (!grid_sync(st, nb, my_gen)) return;  // the partial buffers are reused below

  A beta = Tr::zero();
  S* pold = pt0;
  S* pnew = pt1;
  int it = 0;
  int status = TM_ERR_MAXITER;
  for (;; ++it) {
    if (sqrt(rr) <= tol) {
      status = TM_OK;
      break;
    }
    if (it == maxiter) break;
    // sweep 1
    A pq_l = Tr::zero();
    const S* cpold = pold;
    for (int64_t sl = s_lo + warp; sl < s_hi; sl += (int64_t)kSellRows * kSellWarps) {
      A acc[kSellRows];
      sell_rows<S, CT>(sptr, scol, sval, [&](int c) { return Tr::ld(r, c) + beta * Tr::ld(cpold, c); }, sl,
                       s_hi, acc);
#pragma unroll
      for (int u = 0; u < kSellRows; ++u) {
        if (!valid(sl, u)) continue;
        const int64_t row = row_of(sl, u);
        const A pv = Tr::ld(r, row) + beta * Tr::ld(cpold, row);
        Tr::st(pnew, row, pv);
        Tr::st(q, row, acc[u]);
        pq_l += Tr::ld(dinv, row) * pv * acc[u];
      }
    }
    {
      const double t = block_sum(Tr::to_double(pq_l), s_red);
      if (threadIdx.x == 0) pA[blockIdx.x] = t;
    }
    if (!grid_sync(st, nb, my_gen)) return;
    const double pq = sum_partials(pA, nb, s_red);
    if (!(pq > 0.0)) {
      status = TM_ERR_BREAKDOWN;
      break;
    }
    const A alpha = Tr::from_double(rz / pq);
    // sweep 2
    A rz_l = Tr::zero(), rr_l = Tr::zero();
    for (int64_t sl = s_lo + warp; sl < s_hi; sl += kSellWarps) {
      const int64_t row = sl * 32 + lane;
      if (row >= n) continue;
      const A di = Tr::ld(dinv, row), pv = Tr::ld(pnew, row), qv = Tr::ld(q, row);
      const A xo = Tr::ld(x, row), ro = Tr::ld(r, row);
      const A rn = ro - alpha * qv;
      Tr::st(x, row, xo + alpha * (di * pv));
      Tr::st(r, row, rn);
      rz_l += di * rn * rn;
      rr_l += rn * rn;
    }
    publish2(pB, rz_l, pC, rr_l);
    if (!grid_sync(st, nb, my_gen)) return;
    double rzn;
    sum_partials2(pB, pC, nb, s_red, rzn, rr);
    beta = Tr::from_double(rzn / rz);
    rz = rzn;
    S* t = pold;
    pold = pnew;
    pnew = t;
  }
  for (int64_t sl = s_lo + warp; sl < s_hi; sl += kSellWarps) {
    const int64_t row = sl * 32 + lane;
    if (row < n) xv[row] = Tr::out(Tr::ld(x, row));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->iters = it;
    st->res = sqrt(rr);
    atomicCAS(&st->status, TM_OK, status);
  }
}

template <class S, class CT>
__global__ void __launch_bounds__(kSellThreads, 2)
pcg_sell_kernel(int64_t n, const int64_t* __restrict__ sptr, const CT* __restrict__ scol,
                const S* __restrict__ sval, const S* __restrict__ dinv, const typename SellT<S>::V* __restrict__ bv,
                typename SellT<S>::V* __restrict__ xv, S* x, S* r, S* p, S* s, S* z, S* w0, S* w1,
                double* partials, PcgState* st, double rtol, double atol, int maxiter) {
  using Tr = SellT<S>;
  using A = typename Tr::A;
  __shared__ double s_red[32];
  const unsigned nb = gridDim.x;
  unsigned my_gen = 0;  // the host zeroes st->gen before the launch
  // a slice plan rejected by the fill kernel: nothing to iterate
  if (*((volatile int*)&st->status) != TM_OK) return;
  const int64_t n_slices = (n + 31) >> 5;
  const int64_t per = (n_slices + nb - 1) / nb;
  const int64_t s_lo = min(n_slices, (int64_t)blockIdx.x * per), s_hi = min(n_slices, s_lo + per);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* pb = partials + 6 * (int64_t)nb;  // ||b||^2 partials
  auto row_of = [&](int64_t sl, int u) { return (sl + (int64_t)u * kSellWarps) * 32 + lane; };
  auto valid = [&](int64_t sl, int u) { return sl + (int64_t)u * kSellWarps < s_hi && row_of(sl, u) < n; };
  auto publish = [&](double* dst, A g, A d, A rr) {
    double t = block_sum(Tr::to_double(g), s_red);
    if (threadIdx.x == 0) dst[blockIdx.x] = t;
    t = block_sum(Tr::to_double(d), s_red);
    if (threadIdx.x == 0) dst[nb + blockIdx.x] = t;
    t = block_sum(Tr::to_double(rr), s_red);
    if (threadIdx.x == 0) dst[2 * nb + blockIdx.x] = t;
  };

  // ---- r = b - (A M) y, x = x0, p = s = 0 (p and s of "iteration -1", scaled by beta = 0)
  A bb_l = Tr::zero();
  for (int64_t sl = s_lo + warp; sl < s_hi; sl += (int64_t)kSellRows * kSellWarps) {
    A acc[kSellRows];
    sell_rows<S, CT>(sptr, scol, sval, [&](int c) { return Tr::ld(z, c); }, sl, s_hi, acc);
#pragma unroll
    for (int u = 0; u < kSellRows; ++u) {
      if (!valid(sl, u)) continue;
      const int64_t row = row_of(sl, u);
      const A b = Tr::in(bv[row]);
      const A rv = b - acc[u];
      Tr::st(r, row, rv);
      Tr::st(x, row, Tr::in(xv[row]));
      Tr::st(p, row, Tr::zero());
      Tr::st(s, row, Tr::zero());
      bb_l += b * b;
    }
  }
  {
    const double t = block_sum(Tr::to_double(bb_l), s_red);
    if (threadIdx.x == 0) pb[blockIdx.x] = t;
  }
  if (!grid_sync(st, nb, my_gen)) return;
  const double bnorm = sqrt(sum_partials(pb, nb, s_red));
  const double tol = fmax(rtol * bnorm, atol);
  if (blockIdx.x == 0 && threadIdx.x == 0) st->bnorm = bnorm;

  // ---- w = A u = (A M) r; gamma, delta, rho of iteration 0; z = 0
  {
    A g_l = Tr::zero(), d_l = Tr::zero(), r_l = Tr::zero();
    for (int64_t sl = s_lo + warp; sl < s_hi; sl += (int64_t)kSellRows * kSellWarps) {
      A acc[kSellRows];
      sell_rows<S, CT>(sptr, scol, sval, [&](int c) { return Tr::ld(r, c); }, sl, s_hi, acc);
#pragma unroll
      for (int u = 0; u < kSellRows; ++u) {
        if (!valid(sl, u)) continue;
        const int64_t row = row_of(sl, u);
        const A rv = Tr::ld(r, row);
        const A uv = Tr::ld(dinv, row) * rv;
        Tr::st(w0, row, acc[u]);
        Tr::st(z, row, Tr::zero());
        g_l += rv * uv;
        d_l += acc[u] * uv;
        r_l += rv * rv;
      }
    }
    publish(partials, g_l, d_l, r_l);
  }
  if (!grid_sync(st, nb, my_gen)) return;

  int it = 0;
  int status = TM_ERR_MAXITER;
  double gamma_old = 1.0, alpha_old = 1.0, rho = 0.0;
  for (;; ++it) {
    const double* P = partials + (it & 1) * 3 * (int64_t)nb;
    const double gamma = sum_partials(P, nb, s_red);
    const double delta = sum_partials(P + nb, nb, s_red);
    rho = sum_partials(P + 2 * nb, nb, s_red);
    if (sqrt(rho) <= tol) {
      status = TM_OK;
      break;
    }
    if (it == maxiter) break;
    const double beta_d = it == 0 ? 0.0 : gamma / gamma_old;
    const double denom = it == 0 ? delta : delta - beta_d * gamma / alpha_old;  // = (p, A p)
    if (!(denom > 0.0)) {
      status = TM_ERR_BREAKDOWN;
      break;
    }
    const double alpha_d = gamma / denom;
    const A beta = Tr::from_double(beta_d), alpha = Tr::from_double(alpha_d);
    const S* wc = (it & 1) ? w1 : w0;
    S* wn = (it & 1) ? w0 : w1;
    A g_l = Tr::zero(), d_l = Tr::zero(), r_l = Tr::zero();
    for (int64_t sl = s_lo + warp; sl < s_hi; sl += (int64_t)kSellRows * kSellWarps) {
      A acc[kSellRows];
      sell_rows<S, CT>(sptr, scol, sval, [&](int c) { return Tr::ld(wc, c); }, sl, s_hi, acc);
#pragma unroll
      for (int u = 0; u < kSellRows; ++u) {
        if (!valid(sl, u)) continue;
        const int64_t row = row_of(sl, u);
        const A di = Tr::ld(dinv, row), rv = Tr::ld(r, row), wv = Tr::ld(wc, row);
        const A zo = Tr::ld(z, row), so = Tr::ld(s, row), po = Tr::ld(p, row), xo = Tr::ld(x, row);
        const A zv = acc[u] + beta * zo;
        const A sv = wv + beta * so;
        const A pv = di * rv + beta * po;
        const A rn = rv - alpha * sv;
        const A wnv = wv - alpha * zv;
        Tr::st(z, row, zv);
        Tr::st(s, row, sv);
        Tr::st(p, row, pv);
        Tr::st(x, row, xo + alpha * pv);
        Tr::st(r, row, rn);
        Tr::st(wn, row, wnv);
        const A un = di * rn;
        g_l += rn * un;
        d_l += wnv * un;
        r_l += rn * rn;
      }
    }
    publish(partials + ((it + 1) & 1) * 3 * (int64_t)nb, g_l, d_l, r_l);
    if (!grid_sync(st, nb, my_gen)) return;
    gamma_old = gamma;
    alpha_old = alpha_d;
  }
  for (int64_t sl = s_lo + warp; sl < s_hi; sl += kSellWarps) {
    const int64_t row = sl * 32 + lane;
    if (row < n) xv[row] = Tr::out(Tr::ld(x, row));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->iters = it;
    st->res = sqrt(rho);
    atomicCAS(&st->status, TM_OK, status);
  }
}

// ---- plain SELL-32 copies and products (y = A x), for solvers that apply A
// many times outside the PCG kernels (the two-level flexible CG)
template <class S, class CT>
__global__ void sell_copy_kernel(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                                 const typename SellT<S>::V* __restrict__ val, const int64_t* __restrict__ sptr,
                                 int64_t n_pad, CT* __restrict__ scol, S* __restrict__ sval, int* bad) {
  constexpr bool kRel = sizeof(CT) == 2;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t n_slices = (n + 31) >> 5;
  if (gw >= n_slices) return;
  const int64_t row = gw * 32 + lane;
  const int64_t s0 = sptr[gw], s1 = sptr[gw + 1];
  const int64_t width = s1 - s0;
  const int64_t len = row < n ? indptr[row + 1] - indptr[row] : 0;
  bool wrong = s0 < 0 || s1 > n_pad || width < 0 || (width & 31) != 0 || len > (width >> 5);
  if (__any_sync(0xffffffffu, wrong)) {
    if (lane == 0) atomicExch(bad, 1);
    return;
  }
  const int L = (int)(width >> 5);
  const int64_t base = row < n ? indptr[row] : 0;
  const int32_t pad_col = row < n ? (int32_t)row : (int32_t)(n - 1);
  for (int j = 0; j < L; ++j) {
    const int64_t k = s0 + (int64_t)j * 32 + lane;
    int32_t c = pad_col;
    S v = S(0);
    if (j < len) {
      const int32_t cj = idx[base + j];
      if (cj < 0 || cj >= n) {
        wrong = true;
      } else {
        c = cj;
        v = (S)val[base + j];
      }
    }
    if constexpr (kRel) {
      const long long d = (long long)c - row;
      wrong = wrong || d < -32768 || d > 32767;
      scol[k] = (CT)d;
    } else {
      scol[k] = c;
    }
    sval[k] = v;
  }
  if (__any_sync(0xffffffffu, wrong) && lane == 0) atomicExch(bad, 1);
}

template <class S, class CT>
__global__ void __launch_bounds__(256) sell_spmv_kernel(int64_t n, const int64_t* __restrict__ sptr,
                                                         const CT* __restrict__ scol, const S* __restrict__ sval,
                                                         const S* __restrict__ x, S* __restrict__ y) {
  using Tr = SellT<S>;
  using A = typename Tr::A;
  const int64_t sl = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t n_slices = (n + 31) >> 5;
  if (sl >= n_slices) return;  // whole warps leave together
  A acc[kSellRows];
  // sell_rows advances slices sl + u * kSellWarps; with kSellRows = 1 only sl
  sell_rows<S, CT>(sptr, scol, sval, [&](int c) { return Tr::ld(x, c); }, sl, sl + 1, acc);
  const int64_t row = sl * 32 + (threadIdx.x & 31);
  if (row < n) Tr::st(y, row, acc[0]);
}

inline int64_t align256(int64_t b) { return (b + 255) & ~int64_t(255); }

constexpr int kSellMaxBlocks = 4096;

// Cooperative grid: two CTAs per SM when each gets at least kSlicesPerCta
// slices, else one.  Small systems are bound by the two grid barriers and
// the partial-sum reads per iteration, which cost more with more CTAs
// (us per iteration, 304 / 152 CTAs: 2D 65k rows 23.2 / 16.3, 3D 64^3 31.2 /
// 27.3, 96^3 64.4 / 80.1, 128^3 127 / 172).
constexpr int kSlicesPerCta = 48;

template <class K>
int sell_blocks(K kern, int64_t n_slices) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSellThreads, 0);
  int nb = sms * min(per_sm, 2);
  if (n_slices < (int64_t)kSlicesPerCta * nb) nb = min(nb, sms);
  return min(kSellMaxBlocks, nb);
}

template <class S, class CT>
int launch_pcg_sell(int64_t n, const int64_t* indptr, const int32_t* indices, const typename SellT<S>::V* values,
                    const int64_t* sptr, int64_t n_pad, const typename SellT<S>::V* b, typename SellT<S>::V* x,
                    double rtol, double atol, int maxiter, bool pipe, char* w, cudaStream_t s) {
  const int64_t n_slices_all = (n + 31) >> 5;
  const int nb = pipe ? sell_blocks(pcg_sell_kernel<S, CT>, n_slices_all)
                      : sell_blocks(pcg_sell_hs_kernel<S, CT>, n_slices_all);
  if (nb <= 0) return TM_ERR_CUDA;
  PcgState* st = reinterpret_cast<PcgState*>(w);
  char* q = w + 256;
  double* partials = reinterpret_cast<double*>(q);
  q += align256(7 * (int64_t)kSellMaxBlocks * 8);
  S* vec[9];
  for (int i = 0; i < 9; ++i) {
    vec[i] = reinterpret_cast<S*>(q);
    q += align256(n * (int64_t)sizeof(S));
  }
  S* sval = reinterpret_cast<S*>(q);
  q += align256(n_pad * (int64_t)sizeof(S));
  CT* scol = reinterpret_cast<CT*>(q);
  S* dinv = vec[0];
  S* y = vec[5];  // M^-1 x0, read by the first sweep only
  if (cudaMemsetAsync(st, 0, sizeof(PcgState), s) != cudaSuccess) return TM_ERR_CUDA;
  sell_dinv_kernel<S><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, indptr, indices, values, dinv);
  const int64_t n_slices = (n + 31) >> 5;
  sell_fill_kernel<S, CT><<<(unsigned)((n_slices * 32 + 255) / 256), 256, 0, s>>>(n, indptr, indices, values, sptr,
                                                                                  n_pad, dinv, x, scol, sval, y, st);
  if (cudaPeekAtLastError() != cudaSuccess) return TM_ERR_CUDA;
  const CT* cscol = scol;
  const S* csval = sval;
  const S* cdinv = dinv;
  cudaError_t e;
  if (pipe) {
    S *xs = vec[1], *r = vec[2], *p = vec[3], *sv = vec[4], *z = vec[5], *w0 = vec[6], *w1 = vec[7];
    void* args[] = {(void*)&n, (void*)&sptr, (void*)&cscol, (void*)&csval, (void*)&cdinv, (void*)&b, (void*)&x,
                    (void*)&xs, (void*)&r, (void*)&p, (void*)&sv, (void*)&z, (void*)&w0, (void*)&w1,
                    (void*)&partials, (void*)&st, (void*)&rtol, (void*)&atol, (void*)&maxiter};
    e = cudaLaunchCooperativeKernel((const void*)pcg_sell_kernel<S, CT>, dim3(nb), dim3(kSellThreads), args, 0, s);
  } else {
    S *xs = vec[1], *r = vec[2], *qv = vec[3], *pt0 = vec[4], *pt1 = vec[6];
    const S* cy = y;
    void* args[] = {(void*)&n, (void*)&sptr, (void*)&cscol, (void*)&csval, (void*)&cdinv, (void*)&b, (void*)&x,
                    (void*)&xs, (void*)&r, (void*)&qv, (void*)&pt0, (void*)&pt1, (void*)&cy,
                    (void*)&partials, (void*)&st, (void*)&rtol, (void*)&atol, (void*)&maxiter};
    e = cudaLaunchCooperativeKernel((const void*)pcg_sell_hs_kernel<S, CT>, dim3(nb), dim3(kSellThreads), args, 0,
                                    s);
  }
  return e == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

template <class S>
int launch_pcg_sell_any(int64_t n, const int64_t* indptr, const int32_t* indices, const typename SellT<S>::V* values,
                        const int64_t* sptr, int64_t n_pad, const typename SellT<S>::V* b, typename SellT<S>::V* x,
                        double rtol, double atol, int maxiter, int method, char* w, cudaStream_t s) {
  const bool pipe = (method & 1) == TM_PCG_PIPELINED;
  if (method & TM_PCG_NARROW)
    return launch_pcg_sell<S, int16_t>(n, indptr, indices, values, sptr, n_pad, b, x, rtol, atol, maxiter, pipe, w, s);
  return launch_pcg_sell<S, int32_t>(n, indptr, indices, values, sptr, n_pad, b, x, rtol, atol, maxiter, pipe, w, s);
}

}  // namespace tmg

extern "C" int64_t tm_sell_plan(int64_t n, const int64_t* indptr, const int32_t* indices, int64_t* slice_ptr,
                                int32_t* out_narrow, void* stream) {
  if (n < 0) return -TM_ERR_INVALID;
  if (!slice_ptr || (n > 0 && (!indptr || !indices))) return -TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t n_slices = (n + 31) >> 5;
  if (out_narrow) *out_narrow = 1;
  if (n_slices == 0) {
    const int64_t zero = 0;
    if (cudaMemcpyAsync(slice_ptr, &zero, sizeof(zero), cudaMemcpyHostToDevice, s) != cudaSuccess) return -TM_ERR_CUDA;
    return cudaStreamSynchronize(s) == cudaSuccess ? 0 : -TM_ERR_CUDA;
  }
  // slice_ptr[0] first collects the largest |column - row| (the scan then sets it to 0)
  if (cudaMemsetAsync(slice_ptr, 0, sizeof(int64_t), s) != cudaSuccess) return -TM_ERR_CUDA;
  tmg::sell_width_kernel<<<(unsigned)((n_slices * 32 + 255) / 256), 256, 0, s>>>(n, indptr, slice_ptr);
  tmg::sell_span_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, indptr, indices,
                                                                   reinterpret_cast<unsigned long long*>(slice_ptr));
  int64_t span = 0;
  if (cudaMemcpyAsync(&span, slice_ptr, sizeof(span), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -TM_ERR_CUDA;
  tmg::sell_scan_kernel<<<1, 1024, 0, s>>>(n_slices, slice_ptr);
  if (cudaPeekAtLastError() != cudaSuccess) return -TM_ERR_CUDA;
  int64_t total = 0;
  if (cudaMemcpyAsync(&total, slice_ptr + n_slices, sizeof(total), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return -TM_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return -TM_ERR_CUDA;
  if (out_narrow) *out_narrow = span <= 32767 ? 1 : 0;
  if (total >= (int64_t(1) << 40)) return -TM_ERR_INDEX;
  return total;
}

extern "C" int64_t tm_pcg_sell_workspace_bytes(int32_t dtype, int64_t n, int64_t n_pad) {
  if (n < 0 || n_pad < 0 || (dtype != TM_F32 && dtype != TM_F64)) return -TM_ERR_INVALID;
  const int64_t es = dtype == TM_F64 ? 8 : 4;
  return 256 + tmg::align256(7 * (int64_t)tmg::kSellMaxBlocks * 8) + 9 * tmg::align256(n * es) +
         tmg::align256(n_pad * es) + tmg::align256(n_pad * 4);
}

extern "C" int tm_pcg_jacobi_sell(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices,
                                  const void* values, const int64_t* slice_ptr, int64_t n_pad, const void* b, void* x,
                                  double rtol, double atol, int32_t maxiter, int32_t method, void* work,
                                  int64_t work_bytes, void* stream) {
  if (n < 0 || n_pad < 0 || maxiter < 0) return TM_ERR_INVALID;
  if (method < 0 || method > (TM_PCG_PIPELINED | TM_PCG_NARROW)) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!indptr || !indices || !values || !slice_ptr || !b || !x || !work) return TM_ERR_INVALID;
  if (dtype != TM_F32 && dtype != TM_F64) return TM_ERR_INVALID;
  if (n >= (int64_t(1) << 31) || n_pad < n) return TM_ERR_INDEX;
  if (work_bytes < tm_pcg_sell_workspace_bytes(dtype, n, n_pad)) return TM_ERR_INDEX;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* w = static_cast<char*>(work);
  if (dtype == TM_F64)
    return tmg::launch_pcg_sell_any<tmg::F2>(n, indptr, indices, (const double*)values, slice_ptr, n_pad,
                                         (const double*)b, (double*)x, rtol, atol, maxiter, method, w, s);
  return tmg::launch_pcg_sell_any<float>(n, indptr, indices, (const float*)values, slice_ptr, n_pad, (const float*)b,
                                     (float*)x, rtol, atol, maxiter, method, w, s);
}

// A plain SELL-32 copy of a CSR matrix (values as given) on a tm_sell_plan
// slice plan; scol holds int16 offsets when narrow, else int32 columns.
extern "C" int tm_sell_fill(int32_t dtype, int64_t n, const int64_t* indptr, const int32_t* indices,
                            const void* values, const int64_t* slice_ptr, int64_t n_pad, int32_t narrow, void* scol,
                            void* sval, int32_t* bad_flag, void* stream) {
  if (n < 0 || n_pad < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!indptr || !indices || !values || !slice_ptr || !scol || !sval || !bad_flag) return TM_ERR_INVALID;
  if (dtype != TM_F32 && dtype != TM_F64) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t n_slices = (n + 31) >> 5;
  const unsigned grid = (unsigned)((n_slices * 32 + 255) / 256);
  if (cudaMemsetAsync(bad_flag, 0, sizeof(int32_t), s) != cudaSuccess) return TM_ERR_CUDA;
  if (dtype == TM_F64) {
    if (narrow)
      tmg::sell_copy_kernel<double, int16_t><<<grid, 256, 0, s>>>(n, indptr, indices, (const double*)values, slice_ptr,
                                                                   n_pad, (int16_t*)scol, (double*)sval, bad_flag);
    else
      tmg::sell_copy_kernel<double, int32_t><<<grid, 256, 0, s>>>(n, indptr, indices, (const double*)values, slice_ptr,
                                                                   n_pad, (int32_t*)scol, (double*)sval, bad_flag);
  } else {
    if (narrow)
      tmg::sell_copy_kernel<float, int16_t><<<grid, 256, 0, s>>>(n, indptr, indices, (const float*)values, slice_ptr,
                                                                  n_pad, (int16_t*)scol, (float*)sval, bad_flag);
    else
      tmg::sell_copy_kernel<float, int32_t><<<grid, 256, 0, s>>>(n, indptr, indices, (const float*)values, slice_ptr,
                                                                  n_pad, (int32_t*)scol, (float*)sval, bad_flag);
  }
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

// y = A x on a tm_sell_fill copy (dtype of values, x and y; FP64 in native
// double): one warp per slice, eight entries of each row in flight.
extern "C" int tm_spmv_sell(int32_t dtype, int64_t n, const int64_t* slice_ptr, int32_t narrow, const void* scol,
                            const void* sval, const void* x, void* y, void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!slice_ptr || !scol || !sval || !x || !y) return TM_ERR_INVALID;
  if (dtype != TM_F32 && dtype != TM_F64) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t n_slices = (n + 31) >> 5;
  const unsigned grid = (unsigned)((n_slices * 32 + 255) / 256);
  if (dtype == TM_F64) {
    if (narrow)
      tmg::sell_spmv_kernel<double, int16_t><<<grid, 256, 0, s>>>(n, slice_ptr, (const int16_t*)scol,
                                                                   (const double*)sval, (const double*)x, (double*)y);
    else
      tmg::sell_spmv_kernel<double, int32_t><<<grid, 256, 0, s>>>(n, slice_ptr, (const int32_t*)scol,
                                                                   (const double*)sval, (const double*)x, (double*)y);
  } else {
    if (narrow)
      tmg::sell_spmv_kernel<float, int16_t><<<grid, 256, 0, s>>>(n, slice_ptr, (const int16_t*)scol,
                                                                  (const float*)sval, (const float*)x, (float*)y);
    else
      tmg::sell_spmv_kernel<float, int32_t><<<grid, 256, 0, s>>>(n, slice_ptr, (const int32_t*)scol,
                                                                  (const float*)sval, (const float*)x, (float*)y);
  }
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}
