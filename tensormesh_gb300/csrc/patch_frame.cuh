// Patch frame: the coordinates a patch kernel computes with.
//
// A patch's element algebra runs on the coordinates of its local vertices
// relative to the patch's first local vertex, scaled by a power of two so the
// largest relative coordinate lies in [1, 2) (frame edge vectors are formed
// exactly from integer coordinates, see below):
//
//   frame(x) = (x - x_origin) * 2^-k,   real = frame * 2^k.
//
// The differences are taken exactly: every coordinate of the patch is written
// as a 64-bit integer on the grid 2^(Ep - bias - 59) (Ep the largest biased
// exponent in the patch; |integer| < 2^60, exact for every coordinate within
// 2^7 of the largest and truncated below 2^-59 of it otherwise), the origin is
// subtracted in integer arithmetic, and each element's edge vectors are
// exact integer differences rounded once into the kernel's number format.
// This removes the two failure modes of converting raw coordinates:
//   * precision: a double-float holds a raw coordinate to 2^-49 of |x|, so
//     edge vectors of small elements far from the origin lose |x| / h of that;
//     frame edge vectors carry 48 bits of their own length;
//   * range: products of edge vectors (h^2, h^3, ...) of a mesh in metres at
//     micrometre or continental scale leave float's exponent range; frame
//     edge vectors are O(1/8) whatever the mesh's units.
// Element matrices computed in the frame are scaled back with
// tm_scale_pow2(value, k * p), p the power of length of the form (D - 2 for
// stiffness, D for mass and loads); that scaling is an exponent add.
#pragma once
#include "tm_common.cuh"

namespace tmg {

template <class T> struct FBits;
template <> struct FBits<double> {
  using U = unsigned long long;
  static constexpr int kMant = 52, kBias = 1023, kMaxE = 2047;
  static TM_D U bits(double x) { return (U)__double_as_longlong(x); }
};
template <> struct FBits<float> {
  using U = unsigned int;
  static constexpr int kMant = 23, kBias = 127, kMaxE = 255;
  static TM_D U bits(float x) { return __float_as_uint(x); }
};

// Biased exponent of x, with zero and subnormals counted as 1.
template <class T>
TM_D int tm_bexp(T x) {
  using F = FBits<T>;
  const int e = (int)((F::bits(x) >> F::kMant) & (typename F::U)F::kMaxE);
  return e > 0 ? e : 1;
}

// x on the integer grid 2^(Ep - bias - 59), truncated toward zero (Ep >= the
// biased exponent of x, so |result| < 2^60; differences of differences stay
// below 2^62).
template <class T>
TM_D long long tm_fixed(T x, int Ep) {
  using F = FBits<T>;
  const typename F::U b = F::bits(x);
  int e = (int)((b >> F::kMant) & (typename F::U)F::kMaxE);
  unsigned long long m = (unsigned long long)(b & ((typename F::U(1) << F::kMant) - 1));
  if (e) m |= 1ull << F::kMant; else e = 1;
  const int s = e - Ep + 59 - F::kMant;
  const unsigned long long v = s >= 0 ? (m << s) : (s > -64 ? (m >> -s) : 0ull);
  const bool neg = (b >> (8 * sizeof(T) - 1)) & 1;
  return neg ? -(long long)v : (long long)v;
}

// Frame edge vectors.  The patch's integer coordinates R (relative to its
// first local vertex) stay in shared memory; an edge vector component is the
// exact integer difference d = R_k - R_0.  Frame units: frame = R * 2^(z - 62)
// with z = clz(max |R|) - 1 (the largest |frame coordinate| lies in [1, 2)),
// and real = frame * 2^k.
//
// Two ways to turn d into a float pair, both exact to 2^-48 of the edge:
//  * short patches -- every R has at most 21 significant bits above a common
//    trailing-zero count t (true of grid-like meshes, whose coordinates are
//    short binary fractions): shared memory holds R >> t, and a difference of
//    two such values (|d| < 2^22) becomes its frame value exactly by a
//    magic-number conversion (one integer add, one float subtract);
//  * general patches: the element's differences are shifted left together so
//    the largest has 62 significant bits, and the top 48 bits of each are
//    converted as two exact 24-bit halves; the element's shift is carried as a
//    power of two on its matrix.
// (64-bit integer <-> float conversions run on GB300's FP64 pipe at ~1/60 of
// the FP32 rate, so the kernels use only 32-bit ones.)
struct FrameInfo {
  int k;       // real = frame * 2^k
  int z;       // frame = R * 2^(z - 62)
  int t;       // short patches hold R >> t
  bool shortp; // every |R >> t| is below 2^21
  bool bad;    // a coordinate is not finite
};

// 2^e as a float for -126 <= e <= 127.
TM_D float tm_pow2f(int e) { return __uint_as_float((unsigned)(e + 127) << 23); }

// Exact frame edge vectors of one element with NE edges (d[j][c] = R[lv[j+1]]
// - R[lv[0]] in component c), general patches.  Writes (hi, lo) pairs in units
// of 2^(-62 + u) of the integer grid and returns u; the frame values are
// those times 2^(z - u).  Returns -1 when every difference is zero.
template <int NE, int D>
TM_D int exact_edges(const long long* __restrict__ s_R, const int* lv, float (&h)[NE][D], float (&l)[NE][D]) {
  long long dd[NE][D];
  unsigned long long m = 0ull;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const long long r0 = s_R[lv[0] * D + c];
#pragma unroll
    for (int j = 0; j < NE; ++j) {
      const long long v = s_R[lv[j + 1] * D + c] - r0;
      dd[j][c] = v;
      m |= (unsigned long long)(v ^ (v >> 63));   // |v| up to one: enough for the leading bit
    }
  }
  if (m == 0ull) return -1;
  const int u = __clzll((long long)m) - 2;          // the largest |v << u| lies in [2^61, 2^62)
#pragma unroll
  for (int j = 0; j < NE; ++j)
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const long long v = (long long)((unsigned long long)dd[j][c] << u);
      const int top = (int)(v >> 38);                                  // signed, |top| < 2^24
      const int mid = (int)((unsigned long long)(v >> 14) & 0xffffffull);  // 24 bits
      const float fh = __fmul_rn(__int2float_rn(top), 0x1p-24f);      // v 2^-62 = top 2^-24 + mid 2^-48
      const float fl = __fmul_rn(__int2float_rn(mid), 0x1p-48f);
      const float s = __fadd_rn(fh, fl);                               // Fast2Sum: |fh| >= 2^-24 > fl or fh = 0
      h[j][c] = s;
      l[j][c] = __fsub_rn(fl, __fsub_rn(s, fh));
    }
  return u;
}

// d 2^e for an integer |d| < 2^22, exactly (e + 23 within float's normal
// exponent range): the magic constant 1.5 2^(e + 23) has ulp 2^e, so its bit
// pattern plus d reads back as the constant plus d 2^e (one integer add, one
// float subtract).  Short patches use e = t + z - 62, which gives the
// difference directly in frame units.
struct ShortConv {
  int bits;
  float value;
  TM_D float operator()(int d) const { return __fsub_rn(__int_as_float(bits + d), value); }
};
TM_D ShortConv short_conv(int e) {
  const int bits = ((e + 23 + 127) << 23) | 0x400000;
  return ShortConv{bits, __int_as_float(bits)};
}

// Builds the frame of one patch in shared memory: s_R[i] for i = v * D + d
// (nv * D of them; R >> t on short patches).  Called by every thread of the
// CTA; `s_red` is three 8-byte shared words of scratch.  The returned
// FrameInfo is the same on every thread; when `bad` is set the frame is not
// written.  Ends without a barrier: the caller synchronises before reading.
template <int D, class T>
TM_D FrameInfo patch_frame(const T* __restrict__ pts, const int32_t* __restrict__ vtx, int nv, long long* s_R,
                           unsigned long long* s_red) {
  using F = FBits<T>;
  const int tid = threadIdx.x, nth = blockDim.x;
  FrameInfo fi{0, 0, 0, false, false};
  if (tid < 3) s_red[tid] = 0ull;
  __syncthreads();
  // pass 1: the largest biased exponent of the patch's coordinates (four
  // index loads, then four coordinate loads, in flight per round)
  int emax = 1;
  for (int i0 = tid; i0 < nv * D; i0 += 4 * nth) {
    int64_t at[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * nth;
      at[u] = i < nv * D ? (int64_t)vtx[i / D] * D + i % D : -1;
    }
    T x[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) x[u] = at[u] >= 0 ? pts[at[u]] : T(0);
#pragma unroll
    for (int u = 0; u < 4; ++u) emax = max(emax, tm_bexp(x[u]));
  }
  if (emax > 1) atomicMax(reinterpret_cast<unsigned long long*>(s_red), (unsigned long long)emax);
  __syncthreads();
  const int Ep = (int)s_red[0] > 1 ? (int)s_red[0] : 1;
  fi.bad = Ep >= F::kMaxE;
  if (fi.bad) return fi;
  // pass 2: integer coordinates relative to the first local vertex, their
  // largest magnitude and the union of their bits (for the trailing zeros)
  long long O[D];
  const int64_t v0 = vtx[0];
#pragma unroll
  for (int d = 0; d < D; ++d) O[d] = tm_fixed(pts[v0 * D + d], Ep);
  unsigned long long amax = 0ull, bits = 0ull;
  for (int i0 = tid; i0 < nv * D; i0 += 4 * nth) {
    int64_t at[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * nth;
      at[u] = i < nv * D ? (int64_t)vtx[i / D] * D + i % D : -1;
    }
    T x[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) x[u] = at[u] >= 0 ? pts[at[u]] : T(0);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * nth;
      if (i >= nv * D) break;
      const long long r = tm_fixed(x[u], Ep) - O[i % D];
      s_R[i] = r;
      const unsigned long long a = (unsigned long long)(r < 0 ? -r : r);
      amax = a > amax ? a : amax;
      bits |= a;
    }
  }
  if (amax) atomicMax(s_red + 1, amax);
  if (bits) atomicOr(s_red + 2, bits);
  __syncthreads();
  const unsigned long long M = s_red[1], B = s_red[2];
  fi.z = M ? __clzll((long long)M) - 1 : 0;
  fi.k = Ep - F::kBias + 3 - fi.z;
  fi.t = B ? __ffsll((long long)B) - 1 : 0;
  fi.shortp = (M >> fi.t) < (1ull << 21);
  if (fi.shortp && fi.t > 0)
    for (int i = tid; i < nv * D; i += nth) s_R[i] >>= fi.t;   // exact: the low t bits are zero
  return fi;
}

// v * 2^k.  An exponent add when v and the result are normal; the rare
// remaining cases (zero, inf / nan, subnormal input or result) go through
// scalbn.
TM_D double tm_scale_pow2(double v, int k) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  const int ne = e + k;
  if (e != 0 && e != 2047 && ne > 0 && ne < 2047) return __longlong_as_double((long long)b + (long long)k * (1ll << 52));
  if (v == 0.0 || e == 2047) return v;
  return scalbn(v, k);
}
TM_D float tm_scale_pow2(float v, int k) {
  const unsigned b = __float_as_uint(v);
  const int e = (int)((b >> 23) & 0xff);
  const int ne = e + k;
  if (e != 0 && e != 255 && ne > 0 && ne < 255) return __uint_as_float((unsigned)((int)b + k * (1 << 23)));
  if (v == 0.f || e == 255) return v;
  return scalbnf(v, k);
}

}  // namespace tmg
