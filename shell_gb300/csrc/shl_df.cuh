// shl_df.cuh -- double-float ("df") arithmetic for the FP64-class element path.
//
// GB300 issues 64 FP32 operations per FP64 operation.  A value carried as an
// unevaluated pair hi + lo of floats holds about 48 significant bits; its
// operations are short sequences of FP32 instructions built from the
// error-free transformations of Knuth (TwoSum) and Dekker (TwoProd, here with
// the fused multiply-add), as in the published double-float / double-double
// methods (T. J. Dekker, "A floating-point technique for extending the
// available precision", Numer. Math. 18, 1971; Y. Hida, X. S. Li, D. H.
// Bailey, "Algorithms for quad-double precision floating point arithmetic",
// 2001).  Additions use the "sloppy" form (one TwoSum of the heads): its error
// is relative to |x| + |y|, which is all the element path needs, since it is
// written without subtracting nearly equal quantities.  The intrinsics keep
// the compiler from re-associating or fusing the error terms.
#ifndef SHL_DF_CUH_
#define SHL_DF_CUH_

#include <cuda_runtime.h>

namespace shl {

struct df2 {
  float h, l;
};

__device__ __forceinline__ df2 dfv(float a) { return {a, 0.f}; }

__device__ __forceinline__ df2 df_from_double(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}

__device__ __forceinline__ double df_to_double(df2 x) { return (double)x.h + (double)x.l; }

// s + e = a + b exactly, |a| >= |b| not required (Knuth)
__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// s + e = a + b exactly for |a| >= |b|
__device__ __forceinline__ void df_quick_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ df2 operator+(df2 x, df2 y) {
  float s, e;
  df_two_sum(x.h, y.h, s, e);
  e = __fadd_rn(e, __fadd_rn(x.l, y.l));
  df2 r;
  df_quick_two_sum(s, e, r.h, r.l);
  return r;
}

__device__ __forceinline__ df2 operator-(df2 x) { return {-x.h, -x.l}; }
__device__ __forceinline__ df2 operator-(df2 x, df2 y) { return x + (-y); }

__device__ __forceinline__ df2 operator*(df2 x, df2 y) {
  const float p = __fmul_rn(x.h, y.h);
  float e = __fmaf_rn(x.h, y.h, -p);
  e = __fmaf_rn(x.h, y.l, e);
  e = __fmaf_rn(x.l, y.h, e);
  df2 r;
  df_quick_two_sum(p, e, r.h, r.l);
  return r;
}

__device__ __forceinline__ df2 operator*(float a, df2 y) {
  const float p = __fmul_rn(a, y.h);
  float e = __fmaf_rn(a, y.h, -p);
  e = __fmaf_rn(a, y.l, e);
  df2 r;
  df_quick_two_sum(p, e, r.h, r.l);
  return r;
}
__device__ __forceinline__ df2 operator*(df2 x, float a) { return a * x; }

__device__ __forceinline__ df2& operator+=(df2& x, df2 y) { return x = x + y; }

// x * y + z
__device__ __forceinline__ df2 df_fma(df2 x, df2 y, df2 z) { return x * y + z; }

// sqrt by one Newton step on the float root: r = s + (x - s^2) / (2 s)
__device__ __forceinline__ df2 df_sqrt(df2 x) {
  if (!(x.h > 0.f)) return {sqrtf(x.h), 0.f};
  const float s = sqrtf(x.h);
  const df2 s2 = dfv(s) * dfv(s);
  const df2 d = x - s2;
  const float corr = __fdiv_rn(d.h, __fmul_rn(2.f, s));
  df2 r;
  df_quick_two_sum(s, corr, r.h, r.l);
  return r;
}

// 1 / x by one Newton step on the float reciprocal: q + q (1 - x q)
__device__ __forceinline__ df2 df_recip(df2 x) {
  const float q = __frcp_rn(x.h);
  const df2 rres = dfv(1.f) - x * dfv(q);
  const float corr = __fmul_rn(q, rres.h);
  df2 r;
  df_quick_two_sum(q, corr, r.h, r.l);
  return r;
}

__device__ __forceinline__ df2 dot3df(const df2* a, const df2* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

__device__ __forceinline__ void cross3df(const df2* a, const df2* b, df2* r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

}  // namespace shl

#endif  // SHL_DF_CUH_
