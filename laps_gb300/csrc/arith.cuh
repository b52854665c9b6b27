// Arithmetic types of the engine: native FP64 (`double`), float-float (`dd`, an unevaluated
// sum hi + lo of two FP32 values, ~48-bit significand, executed on the FP32 pipes), and FP32.
//
// On GB300 the FP64 pipe issues about 1.6 instructions/clock/SM against about 117 for FP32
// FMA, so an FFT-based right-hand side in native FP64 is bound by the FP64 ALU, not by HBM.
// `dd` trades ~10 FP32 instructions per FP64-equivalent operation for a 72x faster pipe.
//
// The float-float algorithms are the classical error-free transformations:
//   two_sum (Knuth, TAOCP vol. 2, 4.2.2), fast_two_sum (Dekker 1971), two_prod via FMA,
// assembled as in Hida, Li & Bailey, "Library for double-double and quad-double arithmetic"
// (2007) ("sloppy" addition: its error is bounded relative to |a|+|b|, the norm-wise bound
// FFT error analysis uses).  Every FP32 add here is an `__fadd_rn`/`__fsub_rn` intrinsic so
// that the compiler cannot contract it into an FMA, which would break the error terms.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace laps {

// ------------------------------------------------------------------------------ float-float
struct dd {
  float hi, lo;
};

__device__ __forceinline__ dd dd_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {  // requires |a| >= |b| or a == 0
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}
__device__ __forceinline__ dd operator+(dd a, dd b) {
  dd s = dd_two_sum(a.hi, b.hi);
  float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return dd_fast_two_sum(s.hi, e);
}
__device__ __forceinline__ dd operator-(dd a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__device__ __forceinline__ dd operator*(dd a, dd b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return dd_fast_two_sum(p, e);
}
__device__ __forceinline__ dd dd_mul_f(dd a, float b) {
  float p = __fmul_rn(a.hi, b);
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return dd_fast_two_sum(p, e);
}
// exact scaling by a power of two
__device__ __forceinline__ dd dd_ldexp(dd a, int e) {  // -127 < e < 128 (the transforms' normalisations)
  const float s = __int_as_float((127 + e) << 23);
  return {a.hi * s, a.lo * s};
}
__device__ __forceinline__ dd operator/(dd a, dd b) {
  float q1 = __fdiv_rn(a.hi, b.hi);
  dd r = a - dd_mul_f(b, q1);
  float q2 = __fdiv_rn(r.hi, b.hi);
  r = r - dd_mul_f(b, q2);
  float q3 = __fdiv_rn(r.hi, b.hi);
  dd q = dd_fast_two_sum(q1, q2);
  return q + dd{q3, 0.f};
}
// 1 / b: the nearest float r0 of 1 / b.hi, then one Newton step r0 + r0 (1 - b r0) with the
// residual 1 - b r0 formed in float-float (its error is of order (1 - b r0)^2 ~ 2^-48, the
// float-float precision); a quarter of the instructions of operator/ with three quotient terms
__device__ __forceinline__ dd dd_recip(dd b) {
  const float r0 = __frcp_rn(b.hi);
  const dd e = dd{1.f, 0.f} - dd_mul_f(b, r0);
  return dd_fast_two_sum(r0, __fmul_rn(r0, e.hi));
}
__device__ __forceinline__ dd dd_sqrt(dd a) {
  if (!(a.hi > 0.f)) return {sqrtf(a.hi), 0.f};  // 0, negative (NaN) or NaN propagate
  float s = __fsqrt_rn(a.hi);
  // one Newton step in dd: s + (a - s^2) / (2 s)
  float p = __fmul_rn(s, s);
  float e = fmaf(s, s, -p);
  dd sq = dd_fast_two_sum(p, e);
  dd r = a - sq;
  float c = __fdiv_rn(r.hi, __fmul_rn(2.f, s));
  return dd_fast_two_sum(s, c);
}
__device__ __forceinline__ bool operator<(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dd a, dd b) { return b < a; }
__device__ __forceinline__ dd dd_abs(dd a) { return (a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f)) ? -a : a; }

// Host and device split of a double into a float-float (hi = nearest float, lo = rest).
__host__ __device__ __forceinline__ dd dd_from_double(double d) {
  float h = (float)d;
  float l = (float)(d - (double)h);
  return {h, l};
}
__host__ __device__ __forceinline__ double dd_to_double(dd a) { return (double)a.hi + (double)a.lo; }

// ------------------------------------------------------------------------------ traits
// LAPS_DD_RECIP: float-float reciprocals by dd_recip (1 / rho of the fluxes, the implicit
// diffusion factor); 0 restores the float-float division
#ifndef LAPS_DD_RECIP
#define LAPS_DD_RECIP 1
#endif
// Real<T>: scalar ops used by generic code.  `cst(x)` turns a compile-time double into T.
template <class T> struct Real;
template <> struct Real<double> {
  __device__ __forceinline__ static double cst(double x) { return x; }
  __device__ __forceinline__ static double from_d(double x) { return x; }
  __device__ __forceinline__ static double to_d(double x) { return x; }
  __device__ __forceinline__ static double sqrt_(double x) { return sqrt(x); }
  __device__ __forceinline__ static double abs_(double x) { return fabs(x); }
  __device__ __forceinline__ static double max_(double a, double b) { return (a > b || a != a) ? a : b; }
  // a * 2^e for the transforms' normalisations (-1022 < e < 1024): one multiplication by the
  // exact power of two built from its exponent field
  __device__ __forceinline__ static double mul_pow2(double a, int e) {
    return a * __longlong_as_double((long long)(1023 + e) << 52);
  }
  __device__ __forceinline__ static float lead(double x) { return (float)x; }
  __device__ __forceinline__ static bool isnan_(double x) { return x != x; }
  __device__ __forceinline__ static double min_(double a, double b) { return b < a ? b : a; }
  __device__ __forceinline__ static double inf() { return __longlong_as_double(0x7FF0000000000000ll); }
  __device__ __forceinline__ static double recip(double x) { return 1.0 / x; }
};
template <> struct Real<dd> {
  __device__ __forceinline__ static dd cst(double x) { return dd_from_double(x); }
  __device__ __forceinline__ static dd from_d(double x) { return dd_from_double(x); }
  __device__ __forceinline__ static double to_d(dd x) { return dd_to_double(x); }
  __device__ __forceinline__ static dd sqrt_(dd x) { return dd_sqrt(x); }
  __device__ __forceinline__ static dd abs_(dd x) { return dd_abs(x); }
  __device__ __forceinline__ static dd max_(dd a, dd b) { return (a > b || a.hi != a.hi) ? a : b; }
  __device__ __forceinline__ static dd mul_pow2(dd a, int e) { return dd_ldexp(a, e); }
  __device__ __forceinline__ static float lead(dd x) { return x.hi; }
  __device__ __forceinline__ static bool isnan_(dd x) { return x.hi != x.hi; }
  __device__ __forceinline__ static dd min_(dd a, dd b) { return b < a ? b : a; }
  __device__ __forceinline__ static dd inf() { return {__int_as_float(0x7f800000), 0.f}; }
  __device__ __forceinline__ static dd recip(dd x) { return LAPS_DD_RECIP ? dd_recip(x) : dd{1.f, 0.f} / x; }
};
template <> struct Real<float> {
  __device__ __forceinline__ static float cst(double x) { return (float)x; }
  __device__ __forceinline__ static float from_d(double x) { return (float)x; }
  __device__ __forceinline__ static double to_d(float x) { return (double)x; }
  __device__ __forceinline__ static float sqrt_(float x) { return sqrtf(x); }
  __device__ __forceinline__ static float abs_(float x) { return fabsf(x); }
  __device__ __forceinline__ static float max_(float a, float b) { return (a > b || a != a) ? a : b; }
  // a * 2^e for |e| < 126 (transform scale factors): one exact multiply
  __device__ __forceinline__ static float mul_pow2(float a, int e) { return a * __int_as_float((127 + e) << 23); }
  __device__ __forceinline__ static float lead(float x) { return x; }
  __device__ __forceinline__ static bool isnan_(float x) { return x != x; }
  __device__ __forceinline__ static float min_(float a, float b) { return b < a ? b : a; }
  __device__ __forceinline__ static float inf() { return __int_as_float(0x7f800000); }
  __device__ __forceinline__ static float recip(float x) { return 1.0f / x; }
};

// Division and square root policies of the CFL bound: exact in the arithmetic type, or the
// approximate FP32 instructions (relative error ~1e-7) for the FP32 screen of pass C.
template <class T> struct MathExact {
  __device__ __forceinline__ static T div(T a, T b) { return a / b; }
  __device__ __forceinline__ static T sqrt(T x) { return Real<T>::sqrt_(x); }
};
struct MathFastF {
  __device__ __forceinline__ static float div(float a, float b) { return __fdividef(a, b); }
  __device__ __forceinline__ static float sqrt(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
};

// ------------------------------------------------------------------------------ complex
template <class T> struct cx {
  T re, im;
};
template <class T> __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <class T> __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <class T> __device__ __forceinline__ cx<T> operator-(cx<T> a) { return {-a.re, -a.im}; }
template <class T> __device__ __forceinline__ cx<T> operator*(cx<T> a, cx<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class T> __device__ __forceinline__ cx<T> operator*(cx<T> a, T s) { return {a.re * s, a.im * s}; }
template <class T> __device__ __forceinline__ cx<T> conj(cx<T> a) { return {a.re, -a.im}; }
// multiply by i * s  (the spectral derivative with real wave number s)
template <class T> __device__ __forceinline__ cx<T> mul_i(cx<T> a, T s) { return {-(a.im * s), a.re * s}; }
// multiply by +i or -i
template <class T> __device__ __forceinline__ cx<T> times_i(cx<T> a) { return {-a.im, a.re}; }
template <class T> __device__ __forceinline__ cx<T> times_mi(cx<T> a) { return {a.im, -a.re}; }
template <class T> __device__ __forceinline__ cx<T> cx_zero() { return {Real<T>::cst(0.0), Real<T>::cst(0.0)}; }

// ------------------------------------------------------- packed float-float complex values
// Blackwell issues an FP32 add, multiply or fused multiply-add on the two lanes of a 64-bit
// register pair as one instruction (__fadd2_rn, __fmul2_rn, __ffma2_rn, sub.rn.f32x2).  A
// complex float-float value maps onto them with its real part in lane x and its imaginary part
// in lane y: h = (re.hi, im.hi), l = (re.lo, im.lo).  Each lane runs the scalar algorithm above
// step for step with the same round-to-nearest operations, so every result is bit-identical to
// the scalar form, in half the arithmetic instructions.
#ifndef LAPS_PACKED_DD
#define LAPS_PACKED_DD 1
#endif
struct pdd {
  float2 h, l;
};
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ pdd pk(cx<dd> a) { return {make_float2(a.re.hi, a.im.hi), make_float2(a.re.lo, a.im.lo)}; }
__device__ __forceinline__ cx<dd> upk(pdd a) { return {{a.h.x, a.l.x}, {a.h.y, a.l.y}}; }
__device__ __forceinline__ pdd pbcast(dd s) { return {make_float2(s.hi, s.hi), make_float2(s.lo, s.lo)}; }
// dd_two_sum / dd_fast_two_sum per lane: s in .h, error in .l
__device__ __forceinline__ pdd p_two_sum(float2 a, float2 b) {
  const float2 s = f2add(a, b);
  const float2 bb = f2sub(s, a);
  return {s, f2add(f2sub(a, f2sub(s, bb)), f2sub(b, bb))};
}
__device__ __forceinline__ pdd p_fast_two_sum(float2 a, float2 b) {
  const float2 s = f2add(a, b);
  return {s, f2sub(b, f2sub(s, a))};
}
// a + b and a - b per lane (operator+ of dd; a - b as a + (-b), whose roundings are those of
// the subtractions written here: RN(-x - y) = -RN(x + y))
__device__ __forceinline__ pdd padd(pdd a, pdd b) {
  const pdd s = p_two_sum(a.h, b.h);
  return p_fast_two_sum(s.h, f2add(s.l, f2add(a.l, b.l)));
}
__device__ __forceinline__ pdd psub(pdd a, pdd b) {
  const float2 s = f2sub(a.h, b.h);
  const float2 bb = f2sub(s, a.h);
  const float2 e = f2sub(f2sub(a.h, f2sub(s, bb)), f2add(b.h, bb));
  return p_fast_two_sum(s, f2add(e, f2sub(a.l, b.l)));
}
// a * m per lane (operator* of dd), m one multiplier per lane
__device__ __forceinline__ pdd pmul(pdd a, pdd m) {
  const float2 p = f2mul(a.h, m.h);
  float2 e = f2fma(a.h, m.h, f2neg(p));
  e = f2fma(a.h, m.l, e);
  e = f2fma(a.l, m.h, e);
  return p_fast_two_sum(p, e);
}

// FP32 complex sums and differences as one two-lane instruction each
#ifndef LAPS_PACKED_F32
#define LAPS_PACKED_F32 1
#endif
#if LAPS_PACKED_F32
__device__ __forceinline__ cx<float> operator+(cx<float> a, cx<float> b) {
  const float2 r = f2add(make_float2(a.re, a.im), make_float2(b.re, b.im));
  return {r.x, r.y};
}
__device__ __forceinline__ cx<float> operator-(cx<float> a, cx<float> b) {
  const float2 r = f2sub(make_float2(a.re, a.im), make_float2(b.re, b.im));
  return {r.x, r.y};
}
#endif

#if LAPS_PACKED_DD
__device__ __forceinline__ cx<dd> operator+(cx<dd> a, cx<dd> b) { return upk(padd(pk(a), pk(b))); }
__device__ __forceinline__ cx<dd> operator-(cx<dd> a, cx<dd> b) { return upk(psub(pk(a), pk(b))); }
__device__ __forceinline__ cx<dd> operator*(cx<dd> a, dd s) { return upk(pmul(pk(a), pbcast(s))); }
// The complex product below, lane x the real part and lane y the imaginary part of each step.
__device__ __forceinline__ cx<dd> operator*(cx<dd> a, cx<dd> b) {
  const float2 arh = make_float2(a.re.hi, a.re.hi), arl = make_float2(a.re.lo, a.re.lo);
  const float2 aih = make_float2(-a.im.hi, a.im.hi), ail = make_float2(-a.im.lo, a.im.lo);
  const float2 bh = make_float2(b.re.hi, b.im.hi), bl = make_float2(b.re.lo, b.im.lo);
  const float2 bhs = make_float2(b.im.hi, b.re.hi), bls = make_float2(b.im.lo, b.re.lo);
  const float2 p = f2mul(arh, bh), q = f2mul(aih, bhs);  // (p1, q1), (-p2, q2)
  const float2 e1 = f2fma(arh, bh, f2neg(p)), e2 = f2fma(aih, bhs, f2neg(q));
  const pdd s = p_two_sum(p, q);
  float2 e = f2add(s.l, f2add(e1, e2));
  e = f2fma(arh, bl, e);
  e = f2fma(arl, bh, e);
  e = f2fma(aih, bls, e);
  e = f2fma(ail, bhs, e);
  return upk(p_fast_two_sum(s.h, e));
}
#else
// Complex float-float product with shared error terms (~36 FP32 instructions instead of 50).
__device__ __forceinline__ cx<dd> operator*(cx<dd> a, cx<dd> b) {
  // re = a.re*b.re - a.im*b.im ; im = a.re*b.im + a.im*b.re
  float p1 = __fmul_rn(a.re.hi, b.re.hi), p2 = __fmul_rn(a.im.hi, b.im.hi);
  float e1 = fmaf(a.re.hi, b.re.hi, -p1), e2 = fmaf(a.im.hi, b.im.hi, -p2);
  dd s = dd_two_sum(p1, -p2);
  float e = __fadd_rn(s.lo, __fsub_rn(e1, e2));
  e = fmaf(a.re.hi, b.re.lo, e);
  e = fmaf(a.re.lo, b.re.hi, e);
  e = fmaf(-a.im.hi, b.im.lo, e);
  e = fmaf(-a.im.lo, b.im.hi, e);
  dd re = dd_fast_two_sum(s.hi, e);
  float q1 = __fmul_rn(a.re.hi, b.im.hi), q2 = __fmul_rn(a.im.hi, b.re.hi);
  float f1 = fmaf(a.re.hi, b.im.hi, -q1), f2 = fmaf(a.im.hi, b.re.hi, -q2);
  dd t = dd_two_sum(q1, q2);
  float f = __fadd_rn(t.lo, __fadd_rn(f1, f2));
  f = fmaf(a.re.hi, b.im.lo, f);
  f = fmaf(a.re.lo, b.im.hi, f);
  f = fmaf(a.im.hi, b.re.lo, f);
  f = fmaf(a.im.lo, b.re.hi, f);
  dd im = dd_fast_two_sum(t.hi, f);
  return {re, im};
}
#endif

// ------------------------------------------------------------------------------ storage
// How a value of type T lives in memory.  Complex values are one 16-byte (FP64, dd) or
// 8-byte (FP32) vector so that a quarter-warp moves one 128-byte row per instruction.
template <class T> struct Store;
template <> struct Store<double> {
  using R = double;
  using C = double2;
  __device__ __forceinline__ static double ld(const R* p) { return *p; }
  __device__ __forceinline__ static void st(R* p, double v) { *p = v; }
  __device__ __forceinline__ static cx<double> ldc(const C* p) { C v = *p; return {v.x, v.y}; }
  __device__ __forceinline__ static cx<double> ldg(const C* p) { C v = __ldg(p); return {v.x, v.y}; }
  __device__ __forceinline__ static void stc(C* p, cx<double> v) { *p = make_double2(v.re, v.im); }
};
template <> struct Store<dd> {
  using R = float2;
  using C = float4;
  __device__ __forceinline__ static dd ld(const R* p) { R v = *p; return {v.x, v.y}; }
  __device__ __forceinline__ static void st(R* p, dd v) { *p = make_float2(v.hi, v.lo); }
  __device__ __forceinline__ static cx<dd> ldc(const C* p) { C v = *p; return {{v.x, v.y}, {v.z, v.w}}; }
  __device__ __forceinline__ static cx<dd> ldg(const C* p) { C v = __ldg(p); return {{v.x, v.y}, {v.z, v.w}}; }
  __device__ __forceinline__ static void stc(C* p, cx<dd> v) { *p = make_float4(v.re.hi, v.re.lo, v.im.hi, v.im.lo); }
};
template <> struct Store<float> {
  using R = float;
  using C = float2;
  __device__ __forceinline__ static float ld(const R* p) { return *p; }
  __device__ __forceinline__ static void st(R* p, float v) { *p = v; }
  __device__ __forceinline__ static cx<float> ldc(const C* p) { C v = *p; return {v.x, v.y}; }
  __device__ __forceinline__ static cx<float> ldg(const C* p) { C v = __ldg(p); return {v.x, v.y}; }
  __device__ __forceinline__ static void stc(C* p, cx<float> v) { *p = make_float2(v.re, v.im); }
};

// ------------------------------------------------------------------------------ conversions
// between the compute type of the transforms and the storage type of the state
template <class D, class S> struct Cvt;
template <class T> struct Cvt<T, T> {
  __device__ __forceinline__ static T r(T x) { return x; }
};
template <> struct Cvt<float, dd> {  // nearest float of hi + lo
  __device__ __forceinline__ static float r(dd x) { return __fadd_rn(x.hi, x.lo); }
};
template <> struct Cvt<dd, float> {
  __device__ __forceinline__ static dd r(float x) { return {x, 0.f}; }
};
template <> struct Cvt<float, double> {
  __device__ __forceinline__ static float r(double x) { return __double2float_rn(x); }
};
template <> struct Cvt<double, float> {
  __device__ __forceinline__ static double r(float x) { return (double)x; }
};
template <class D, class S> __device__ __forceinline__ cx<D> cvtc(cx<S> v) { return {Cvt<D, S>::r(v.re), Cvt<D, S>::r(v.im)}; }

// ------------------------------------------------------- FP32 <-> FP64 on the integer pipes
// Conversions written on the IEEE 754 bit fields with integer instructions, for kernels whose
// FP64 pipe is the bottleneck (on GB300 a conversion to or from binary64 issues at the FP64
// pipe's rate, ~1/70 of FP32).  f32_to_f64_bits is exact for normal numbers, zeros,
// infinities and NaN (a subnormal float becomes a signed zero).  f64_to_f32_rn rounds to the
// nearest float, ties to even (the carry of the rounding increment runs into the exponent and
// on to infinity), flushes magnitudes below the FP32 normal range to a signed zero, maps
// larger ones to infinity and keeps NaN a NaN.
__host__ __device__ __forceinline__ uint64_t f64_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  __builtin_memcpy(&b, &x, 8);
  return b;
#endif
}
__host__ __device__ __forceinline__ double f64_from_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  __builtin_memcpy(&x, &b, 8);
  return x;
#endif
}
__host__ __device__ __forceinline__ uint32_t f32_bits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t b;
  __builtin_memcpy(&b, &x, 4);
  return b;
#endif
}
__host__ __device__ __forceinline__ float f32_from_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  __builtin_memcpy(&x, &b, 4);
  return x;
#endif
}
__host__ __device__ __forceinline__ double f32_to_f64_bits(float x) {
  const uint32_t b = f32_bits(x);
  const uint32_t sign = b & 0x80000000u, e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  const uint32_t de = e == 0xffu ? 0x7ffu : e + 896u;  // rebias 127 -> 1023
  const uint32_t hi = e == 0 ? sign : (sign | (de << 20) | (m >> 3));
  const uint32_t lo = e == 0 ? 0u : (m << 29);
  return f64_from_bits(((uint64_t)hi << 32) | lo);
}
__host__ __device__ __forceinline__ float f64_to_f32_rn(double x) {
  const uint64_t d = f64_bits(x);
  const uint32_t hi = (uint32_t)(d >> 32), lo = (uint32_t)d;
  const uint32_t sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu), fe = e - 896;  // rebias 1023 -> 127
  const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // the 23 kept significand bits
  const uint32_t rem = lo & 0x1fffffffu;                    // the 29 dropped ones
  uint32_t b;
  if (e == 0x7ff) b = sign | 0x7f800000u | ((((hi & 0xfffffu) | lo) != 0u) ? 0x400000u : 0u);
  else if (fe <= 0) b = sign;
  else if (fe >= 255) b = sign | 0x7f800000u;
  else b = (sign | ((uint32_t)fe << 23) | m) + ((rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u);
  return f32_from_bits(b);
}

// An FP32 view of a state-type value and a state-type value of an FP32 increment, as the
// FP32-increment RK update needs them (binary64: through the bit fields above).
template <class T> struct IncCvt {
  __device__ __forceinline__ static cx<float> to_f32(cx<T> v) { return cvtc<float>(v); }
  __device__ __forceinline__ static cx<T> from_f32(cx<float> v) { return cvtc<T>(v); }
};
template <> struct IncCvt<double> {
  __device__ __forceinline__ static cx<float> to_f32(cx<double> v) { return {f64_to_f32_rn(v.re), f64_to_f32_rn(v.im)}; }
  __device__ __forceinline__ static cx<double> from_f32(cx<float> v) { return {f32_to_f64_bits(v.re), f32_to_f64_bits(v.im)}; }
};

}  // namespace laps
