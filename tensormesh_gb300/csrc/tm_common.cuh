// Shared device helpers for the tensormesh_gb300 kernels (sm_103a).
//
// df64: an unevaluated sum hi + lo of two floats (~48-bit significand).
// GB300 executes native FP64 FMA at ~1/73 of the FP32 FMA rate (measured
// 0.50 T DFMA/s vs 36.8 T FFMA/s on this part), so the FP64 entry points do
// their arithmetic in df64 on the FP32 pipe and convert to/from double only at
// the boundary.  The algorithms are the classic error-free transformations:
// Knuth's TwoSum, Dekker's Fast2Sum, and the FMA-based exact product
// (Ogita, Rump & Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput.
// 26(6), 2005), with the "sloppy" double-float add/mul/div/sqrt of Hida, Li &
// Bailey ("Library for double-double and quad-double arithmetic", 2007),
// transposed to float pairs.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define TM_HD __host__ __device__ __forceinline__
#define TM_D __device__ __forceinline__

struct df64 {
  float hi, lo;
};

TM_D df64 tm_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
TM_D df64 tm_fast_two_sum(float a, float b) {  // requires |a| >= |b| (or a == 0)
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}
TM_D df64 operator+(df64 a, df64 b) {
  df64 s = tm_two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return tm_fast_two_sum(s.hi, s.lo);
}
TM_D df64 operator-(df64 a) { return {-a.hi, -a.lo}; }
TM_D df64 operator-(df64 a, df64 b) { return a + (-b); }
TM_D df64 operator*(df64 a, df64 b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return tm_fast_two_sum(p, e);
}
TM_D df64 operator/(df64 a, df64 b) {
  float q1 = __fdiv_rn(a.hi, b.hi);
  df64 r = a - df64{q1, 0.f} * b;
  float q2 = __fdiv_rn(r.hi, b.hi);
  return tm_fast_two_sum(q1, q2);
}
TM_D df64& operator+=(df64& a, df64 b) { a = a + b; return a; }
TM_D df64& operator-=(df64& a, df64 b) { a = a - b; return a; }
TM_D df64& operator*=(df64& a, df64 b) { a = a * b; return a; }
TM_D df64 tm_sqrt(df64 a) {
  if (a.hi <= 0.f) return {0.f, 0.f};
  float s = __fsqrt_rn(a.hi);
  // residual a - s*s, exact in its leading part thanks to the FMA
  float r = __fadd_rn(__fmaf_rn(-s, s, a.hi), a.lo);
  return tm_fast_two_sum(s, __fdiv_rn(r, __fadd_rn(s, s)));
}
TM_D df64 tm_abs(df64 a) { return a.hi < 0.f ? -a : a; }
TM_D float tm_approx(df64 a) { return a.hi; }

// double <-> df64.  float<->double conversions and FP64 adds run on the
// FP64 pipe (measured on GB300: ~0.6 T/s for the whole GPU), so both
// directions work on the bit patterns with integer and FP32 operations only.

// x = h + l with h = x rounded to 24 significant bits (round half up) and
// l = the remainder rounded to float: |l| <= ulp(h)/2, |x - h - l| <= 2^-49 |x|
// while l is a normal float.  The 52-bit fraction of x splits into its top 23
// bits (h, with bit 28 as the rounding bit) and the low 29 bits r, whose
// weight is 2^(E - 1075) for the biased exponent E.  Values whose r weight is
// not a normal float are scaled by 2^+-100 first (exact) and the pair is
// scaled back (rounding like float where it under- or overflows); zero and
// doubles below 2^-174 give 0, inf / nan map to float inf / nan.  Written
// with selects rather than branches (branches here cost the calling kernels
// dozens of registers).
TM_D df64 tm_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((b >> 52) & 0x7ff);
  const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
  const bool big = E > 1149, small = E < 949;
  const int shift = big ? -100 : (small ? 100 : 0);
  const unsigned long long bs = b + ((unsigned long long)(long long)shift << 52);
  const int Es = E + shift;
  const unsigned rb = (unsigned)(bs >> 28) & 1u;
  float h = __uint_as_float((sgn | ((unsigned)(Es - 896) << 23) | (unsigned)((bs >> 29) & 0x7fffffu)) + rb);
  const int r = (int)(bs & 0x1fffffffu) - (int)(rb << 29);
  float l = __uint_as_float(__float_as_uint(__int2float_rn(r) * __uint_as_float((unsigned)(Es - 948) << 23)) ^ sgn);
  const float post = big ? 0x1p100f : (small ? 0x1p-100f : 1.f);
  h = __fmul_rn(h, post);
  l = __fmul_rn(l, post);
  const bool zero = E < 849, inf = E > 1150;
  const unsigned hs = sgn | (inf ? (0x7f800000u | ((E == 2047 && (b << 12)) ? 0x400000u : 0u)) : 0u);
  h = (zero || inf) ? __uint_as_float(hs) : h;
  l = (zero || inf) ? 0.f : l;
  return {h, l};
}

// The double nearest to a.hi + a.lo (the same value as (double)hi + (double)lo).
// (s, e) = TwoSum(hi, lo) is exact; s is written as a double, and e is added
// as k units in the last place of that double, k = RN(e / ulp), ulp being the
// spacing just below |s| when s is a power of two and e points towards zero.
// Small s (and e) are scaled by 2^100 first and the exponent field corrected;
// zero, inf and nan are selected at the end.
TM_D double tm_to_double(df64 a) {
  const float s0 = __fadd_rn(a.hi, a.lo);
  const float bb = __fsub_rn(s0, a.hi);
  const float e0 = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s0, bb)), __fsub_rn(a.lo, bb));
  const bool small = ((__float_as_uint(s0) >> 23) & 0xffu) < 53u;
  const float sc = small ? 0x1p100f : 1.f;
  const float s = __fmul_rn(s0, sc), e = __fmul_rn(e0, sc);
  const unsigned fs = __float_as_uint(s);
  const unsigned es = (fs >> 23) & 0xffu;
  const unsigned ss = fs >> 31;
  const unsigned long long top = ((unsigned long long)ss << 63) | ((unsigned long long)(fs & 0x7fffffu) << 29);
  const unsigned long long d = top | ((unsigned long long)(es + 896u - (small ? 100u : 0u)) << 52);
  const unsigned down = ((fs & 0x7fffffu) == 0u && e != 0.f && (__float_as_uint(e) >> 31) != ss) ? 1u : 0u;
  const int sh = 179 - (int)es + (int)down;  // ulp of the scaled d is 2^-sh
  const int k = __float2int_rn(__fmul_rn(e, __uint_as_float((unsigned)(sh + 127) << 23)));
  long long bits = (long long)d + (ss ? -(long long)k : (long long)k);
  bits = es == 255u ? (long long)(top | (0x7ffull << 52)) : bits;
  bits = s0 == 0.f ? (long long)((unsigned long long)ss << 63) : bits;
  return __longlong_as_double(bits);
}

// Uniform scalar interface so kernels can be written once over
// R in {float, double, df64}.
template <class R> struct Num;
template <> struct Num<float> {
  static TM_D float from_double(double x) { return (float)x; }
  static TM_D float from_float(float x) { return x; }
  static TM_D float zero() { return 0.f; }
  static TM_D float abs(float x) { return fabsf(x); }
  static TM_D float sqrt(float x) { return sqrtf(x); }
  static TM_D bool neg(float x) { return x < 0.f; }
  static TM_D double to_double(float x) { return (double)x; }
  static TM_D float to_float(float x) { return x; }
};
template <> struct Num<double> {
  static TM_D double from_double(double x) { return x; }
  static TM_D double from_float(float x) { return (double)x; }
  static TM_D double zero() { return 0.0; }
  static TM_D double abs(double x) { return fabs(x); }
  static TM_D double sqrt(double x) { return ::sqrt(x); }
  static TM_D bool neg(double x) { return x < 0.0; }
  static TM_D double to_double(double x) { return x; }
  static TM_D float to_float(double x) { return (float)x; }
};
template <> struct Num<df64> {
  static TM_D df64 from_double(double x) { return tm_from_double(x); }
  static TM_D df64 from_float(float x) { return {x, 0.f}; }
  static TM_D df64 zero() { return {0.f, 0.f}; }
  static TM_D df64 abs(df64 x) { return tm_abs(x); }
  static TM_D df64 sqrt(df64 x) { return tm_sqrt(x); }
  static TM_D bool neg(df64 x) { return x.hi < 0.f; }
  static TM_D double to_double(df64 x) { return tm_to_double(x); }
  static TM_D float to_float(df64 x) { return x.hi + x.lo; }
};

// Load an input value of storage type T into compute type R.
template <class R, class T> TM_D R tm_load(T v);
template <> TM_D float tm_load<float, float>(float v) { return v; }
template <> TM_D double tm_load<double, double>(double v) { return v; }
template <> TM_D df64 tm_load<df64, double>(double v) { return tm_from_double(v); }
template <> TM_D float tm_load<float, double>(double v) { return (float)v; }

template <class T, class R> TM_D T tm_store(R v);
template <> TM_D float tm_store<float, float>(float v) { return v; }
template <> TM_D double tm_store<double, double>(double v) { return v; }
template <> TM_D double tm_store<double, df64>(df64 v) { return tm_to_double(v); }

// Strided view of a staging slot: element-major slots are laid out
// structure-of-arrays ([entry][element]) so that the threads of a warp, each
// working on its own element, touch consecutive shared-memory words.
template <class R>
struct Strided {
  R* p;
  int s;
  TM_D R& operator[](int i) const { return p[i * s]; }
};

// Lazy double-float: value = h + l with |l| << |h| but not renormalised after
// every operation (error-free products by FMA; TwoSum only where two leading
// parts are added).  Used on the hot paths where full df64 normalisation
// would double the instruction count.
struct L2 {
  float h, l;
};

TM_D L2 l2_from(df64 a) { return {a.hi, a.lo}; }
TM_D L2 l2_sub(L2 a, L2 b) {
  const float s = __fsub_rn(a.h, b.h);
  const float bb = __fsub_rn(s, a.h);
  const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(-b.h, bb));
  return {s, __fadd_rn(e, __fsub_rn(a.l, b.l))};
}
TM_D L2 l2_add(L2 a, L2 b) {
  const float s = __fadd_rn(a.h, b.h);
  const float bb = __fsub_rn(s, a.h);
  const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
  return {s, __fadd_rn(e, __fadd_rn(a.l, b.l))};
}
TM_D L2 l2_mul(L2 a, L2 b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return {p, e};
}
TM_D L2 l2_neg(L2 a) { return {-a.h, -a.l}; }
TM_D L2 l2_norm(L2 a) {
  const float s = __fadd_rn(a.h, a.l);
  return {s, __fsub_rn(a.l, __fsub_rn(s, a.h))};
}
// dot of two 3-vectors
TM_D L2 l2_dot3(const L2* a, const L2* b) {
  return l2_add(l2_add(l2_mul(a[0], b[0]), l2_mul(a[1], b[1])), l2_mul(a[2], b[2]));
}
// a*b - c*d
TM_D L2 l2_cof(L2 a, L2 b, L2 c, L2 d) { return l2_sub(l2_mul(a, b), l2_mul(c, d)); }

