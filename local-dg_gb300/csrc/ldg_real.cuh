// Arithmetic types of the LDG kernels.
//
// double : the FP64 path (every operation in FP64).
// dd     : a pair of FP32 numbers (h + l, |l| <= ulp(h)/2), the "double-word"
//          representation with a 48-bit significand.  On GB300 the FP32 pipe
//          issues 64x more operations per cycle than the FP64 pipe, so the
//          mixed-precision path evaluates the right-hand side in dd and keeps
//          FP64 only for the conserved state, the RK4 accumulation and the
//          reductions.  Relative error per operation ~2^-44..2^-47 (vs 2^-53
//          in FP64), far below the mixed path's 1e-9 bar.
//
// The dd operations are written from the published error-free
// transformations: TwoSum (Knuth, TAOCP vol. 2), Fast2Sum (Dekker 1971),
// TwoProd with FMA, and the double-word algorithms of Joldes, Muller and
// Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44(2), 2017: SloppyDWPlusDW (Alg. 5),
// DWTimesDW3 (Alg. 12), and a Newton step for the reciprocal and square
// root.  Rounded intrinsics (__fadd_rn etc.) keep the compiler from
// contracting or reassociating the error terms.
//
// Storage: intermediates (gradient, traces) are stored as `double` on the
// FP64 path and as float2 (h, l) on the dd path -- 8 bytes either way.
#pragma once
#include <cuda_runtime.h>

namespace ldg {

struct dd {
  float h, l;
};

__device__ __forceinline__ dd dd_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dd dd_two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ dd operator+(dd x, dd y) {  // SloppyDWPlusDW
  dd s = dd_two_sum(x.h, y.h);
  float v = __fadd_rn(x.l, y.l);
  float w = __fadd_rn(s.l, v);
  return dd_fast_two_sum(s.h, w);
}
__device__ __forceinline__ dd operator-(dd x) { return {-x.h, -x.l}; }
__device__ __forceinline__ dd operator-(dd x, dd y) { return x + (-y); }
__device__ __forceinline__ dd operator*(dd x, dd y) {  // DWTimesDW3
  dd c = dd_two_prod(x.h, y.h);
  float t0 = __fmul_rn(x.l, y.l);
  float t1 = __fmaf_rn(x.h, y.l, t0);
  float c2 = __fmaf_rn(x.l, y.h, t1);
  float c3 = __fadd_rn(c.l, c2);
  return dd_fast_two_sum(c.h, c3);
}
__device__ __forceinline__ dd& operator+=(dd& x, dd y) { return x = x + y; }
__device__ __forceinline__ dd& operator-=(dd& x, dd y) { return x = x - y; }

// a*b + c with one renormalisation (the product's error terms are folded
// into the low part before the final Fast2Sum).
__device__ __forceinline__ dd fma(dd a, dd b, dd c) {
  dd p = dd_two_prod(a.h, b.h);
  float e = __fmaf_rn(a.h, b.l, p.l);
  e = __fmaf_rn(a.l, b.h, e);
  dd s = dd_two_sum(p.h, c.h);
  float t = __fadd_rn(__fadd_rn(s.l, e), c.l);
  return dd_fast_two_sum(s.h, t);
}

// 1/y: FP32 reciprocal refined by one Newton step in double-word.
__device__ __forceinline__ dd rcp(dd y) {
  float r = __frcp_rn(y.h);
  float e = __fmaf_rn(-y.h, r, 1.0f);
  e = __fmaf_rn(-y.l, r, e);
  return dd_fast_two_sum(r, __fmul_rn(r, e));
}

// sqrt(x): FP32 square root refined by one Newton step.
__device__ __forceinline__ dd sqrt(dd x) {
  float s = __fsqrt_rn(x.h);
  dd p = dd_two_prod(s, s);
  float r = __fadd_rn(__fsub_rn(__fsub_rn(x.h, p.h), p.l), x.l);
  return dd_fast_two_sum(s, __fmul_rn(r, __fdiv_rn(0.5f, s)));
}

__device__ __forceinline__ dd fabs(dd x) { return x.h < 0.0f ? -x : x; }

// Scaling by a power of two is exact.
__device__ __forceinline__ dd scale2(dd x, float p2) { return {x.h * p2, x.l * p2}; }

// Dot-product accumulators: sum_k a_k b_k + c term by term.
// Acc<double> is the FMA chain of the FP64 path (bit for bit the loops it
// replaces).  Acc<dd> follows the "Dot2" scheme of Ogita, Rump and Oishi,
// "Accurate sum and dot product", SIAM J. Sci. Comput. 26(6), 2005: the
// high parts' products are split exactly (TwoProd with FMA) and summed with
// TwoSum, and every error term and low-part product goes into one FP32
// accumulator; the pair is renormalised once at the end.  About 12 FP32
// operations per term against 15 for a renormalising pair FMA, with shorter
// dependency chains; the result is as accurate as if computed in twice the
// working precision (error ~ K u^2 sum |a_k b_k|, u = 2^-24).
template <class T>
struct Acc;

template <>
struct Acc<double> {
  double v;
  __device__ __forceinline__ explicit Acc(double c = 0.0) : v(c) {}
  __device__ __forceinline__ void add(double a, double b) { v = ::fma(a, b, v); }
  __device__ __forceinline__ double get() const { return v; }
};

template <>
struct Acc<dd> {
  float s, c;
  __device__ __forceinline__ explicit Acc(dd x = dd{0.0f, 0.0f}) : s(x.h), c(x.l) {}
  __device__ __forceinline__ void add(dd a, dd b) {
    const float p = __fmul_rn(a.h, b.h);
    const float e = __fmaf_rn(a.h, b.h, -p);
    const dd t = dd_two_sum(s, p);
    s = t.h;
    c = __fmaf_rn(a.h, b.l, c);
    c = __fmaf_rn(a.l, b.h, c);
    c = __fadd_rn(c, __fadd_rn(t.l, e));
  }
  __device__ __forceinline__ dd get() const { return dd_two_sum(s, c); }
};

// ----------------------------------------------------------------- traits
template <class T>
struct Real;

template <>
struct Real<double> {
  using S = double;
  static __device__ __forceinline__ double ld(const S* p) { return *p; }
  static __device__ __forceinline__ void st(S* p, double v) { *p = v; }
  static __device__ __forceinline__ double from_f64(double x) { return x; }
  static __device__ __forceinline__ double to_f64(double x) { return x; }
  static __host__ __device__ constexpr double cst(double v) { return v; }
};

template <>
struct Real<dd> {
  using S = float2;
  static __device__ __forceinline__ dd ld(const S* p) {
    float2 v = *p;
    return {v.x, v.y};
  }
  static __device__ __forceinline__ void st(S* p, dd v) { *p = make_float2(v.h, v.l); }
  static __device__ __forceinline__ dd from_f64(double x) {
    float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};
  }
  static __device__ __forceinline__ double to_f64(dd x) { return (double)x.h + (double)x.l; }
  static __host__ __device__ constexpr dd cst(double v) {
    return {(float)v, (float)(v - (double)(float)v)};
  }
};

// Host-side split of a double into a dd pair.
inline dd dd_from_host(double v) {
  float h = (float)v;
  return {h, (float)(v - (double)h)};
}

}  // namespace ldg
