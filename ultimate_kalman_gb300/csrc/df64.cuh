/*
 * df64.cuh -- FP64 <-> FP32 conversions by integer bit operations, and
 * double-float ("df") arithmetic: a value is the unevaluated sum hi + lo of two
 * FP32 numbers with |lo| <= ulp(hi), about 47 significant bits.
 *
 * Why: on GB300 the FP64 pipe issues about 1/70 of the FP32 rate, and the
 * cvt.f32.f64 / cvt.f64.f32 conversions run on that same pipe (measured:
 * ~0.5 T conversions/s against ~37 T FP32 FMA/s on one GPU).  Kernels whose
 * arithmetic is FP32 but whose inputs and outputs are FP64 therefore convert
 * with integer instructions here, and the refinement residual, which needs
 * more than FP32 precision, runs in df arithmetic on the FP32 pipe.
 *
 * The df algorithms are the classical error-free transformations: Knuth's
 * TwoSum and Dekker's FastTwoSum (exact sums), the FMA form of Dekker's
 * TwoProduct (exact products), and one Newton step in df for the square root
 * and the reciprocal (Dekker 1971, "A floating-point technique for extending
 * the available precision"; the same steps as the double-double library of
 * Hida, Li and Bailey).  Magnitudes must stay inside FP32's normal range
 * (about 1.2e-38 .. 3.4e38): values below it become zero.
 */
#pragma once
#include <cstdint>

namespace ukg_df {

/* FP64 -> FP32, rounded to nearest (ties away from zero); inputs below FP32's
 * normal range become signed zero, inputs above it infinity, NaN stays NaN. */
__device__ __forceinline__ float f64_to_f32(double x)
{
  const uint32_t h = (uint32_t)__double2hiint(x), l = (uint32_t)__double2loint(x);
  const uint32_t s = h & 0x80000000u, e = (h >> 20) & 0x7ffu;
  uint32_t r = s | ((((e - 896u) << 23) | ((h & 0xfffffu) << 3) | (l >> 29)) + ((l >> 28) & 1u));
  if (e - 897u > 253u) /* biased FP32 exponent outside [1, 254] */
    r = e < 897u ? s : (e == 2047u && ((h & 0xfffffu) | l) ? (s | 0x7fc00000u) : (s | 0x7f800000u));
  return __uint_as_float(r);
}

/* FP32 -> FP64, exact; FP32 subnormals become signed zero. */
__device__ __forceinline__ double f32_to_f64(float f)
{
  const uint32_t b = __float_as_uint(f);
  const uint32_t s = b & 0x80000000u, e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  uint32_t hi = s | ((e + 896u) << 20) | (m >> 3), lo = m << 29;
  if (e == 0u) hi = s, lo = 0u;
  if (e == 255u) hi = s | 0x7ff00000u | (m >> 3);
  return __hiloint2double((int)hi, (int)lo);
}

template <typename T>
__device__ __forceinline__ T narrow(double x) { return x; }
template <>
__device__ __forceinline__ float narrow<float>(double x) { return f64_to_f32(x); }
__device__ __forceinline__ double widen(double x) { return x; }
__device__ __forceinline__ double widen(float x) { return f32_to_f64(x); }

struct df {
  float hi, lo;
};

/* Exact split of an FP64 value: hi = its leading 24 bits, lo = the next 23
 * (the last 6 bits are dropped).  Outside 2^-103 <= |x| < 2^128, lo is 0 and hi
 * the rounded FP32 value.  In range, hi's exponent field is the FP64 one's low
 * eight bits with the top bit flipped (e - 896 = e - 128 mod 256), so hi comes
 * from one funnel shift; lo = (bits 28..6 of the low word) * 2^(e-1069) is
 * built as 2^E0 (1 + f) - 2^E0 with E0 = e - 1046 (an exact subtraction). */
__device__ __forceinline__ df split(double x)
{
  const uint32_t h = (uint32_t)__double2hiint(x), l = (uint32_t)__double2loint(x);
  const uint32_t e = (h >> 20) & 0x7ffu;
  df r;
  if (e - 920u <= 230u) {
    const uint32_t t = __funnelshift_l(l, h, 3) ^ 0x40000000u;
    const uint32_t hb = (t & 0x7fffffffu) | (h & 0x80000000u);
    const uint32_t E = (hb & 0xff800000u) - (23u << 23);
    r.hi = __uint_as_float(hb);
    r.lo = __uint_as_float(E | ((l >> 6) & 0x7fffffu)) - __uint_as_float(E);
  } else {
    r.hi = f64_to_f32(x);
    r.lo = 0.0f;
  }
  return r;
}

__device__ __forceinline__ double join(df a) { return f32_to_f64(a.hi) + f32_to_f64(a.lo); }
__device__ __forceinline__ float round_df(df a) { return a.hi + a.lo; }

__device__ __forceinline__ df make(float hi) { return df{hi, 0.0f}; }
__device__ __forceinline__ df neg(df a) { return df{-a.hi, -a.lo}; }

/* FastTwoSum, |a| >= |b| or a == 0 */
__device__ __forceinline__ df fast_two_sum(float a, float b)
{
  const float s = __fadd_rn(a, b);
  return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}

/* TwoSum: s + e == a + b exactly */
__device__ __forceinline__ df two_sum(float a, float b)
{
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df{s, e};
}

__device__ __forceinline__ df add(df a, df b)
{
  const df s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}

__device__ __forceinline__ df sub(df a, df b) { return add(a, neg(b)); }

/* a * b, with the lo*lo term (below 2^-46 relative) left out */
__device__ __forceinline__ df mul(df a, df b)
{
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

/* acc + a * b */
__device__ __forceinline__ df fma(df a, df b, df acc)
{
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const df s = two_sum(acc.hi, p);
  return fast_two_sum(s.hi, s.lo + (acc.lo + e));
}

/* Unnormalized accumulator for a sum of products (the compensated dot
 * product "Dot2" of Ogita, Rump and Oishi, 2005, with double-float operands):
 * hi is the running FP32 sum, made exact by TwoSum, and lo collects its
 * rounding errors and the products' low parts; finish() normalizes once.    */
struct acc {
  float hi, lo;
};
__device__ __forceinline__ acc start(df a) { return acc{a.hi, a.lo}; }
__device__ __forceinline__ void add_prod(acc& s, df a, df b)
{
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const df t = two_sum(s.hi, p);
  s.hi = t.hi;
  s.lo = __fadd_rn(s.lo, __fadd_rn(t.lo, e));
}
__device__ __forceinline__ df finish(acc s) { return two_sum(s.hi, s.lo); }

/* 1 / d by one Newton step on the FP32 reciprocal: r0 (1 + (1 - d r0)) */
__device__ __forceinline__ df rcp(df d)
{
  const float r0 = __frcp_rn(d.hi);
  const float p = __fmul_rn(d.hi, r0);
  const float pe = __fmaf_rn(d.hi, r0, -p);
  const float res = __fsub_rn(__fsub_rn(1.0f - p, pe), __fmul_rn(d.lo, r0)); /* 1 - d r0 */
  return fast_two_sum(r0, __fmul_rn(r0, res));
}

/* sqrt(a), a > 0, by one Newton step on the FP32 root: s0 + (a - s0^2)/(2 s0) */
__device__ __forceinline__ df sqrt(df a)
{
  const float s0 = __fsqrt_rn(a.hi);
  const float p = __fmul_rn(s0, s0);
  const float pe = __fmaf_rn(s0, s0, -p);
  const float res = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo); /* a - s0^2 */
  return fast_two_sum(s0, __fmul_rn(res, __fdividef(0.5f, s0)));
}

/* ---------------------------------------------------------------------------
 * dd: a double-float number as a value type, so that kernels written for a
 * scalar type T (fma, sqrt, copysign, T(0), T(1) / x, comparisons) compile
 * unchanged with T = dd and run their FP64 algorithm on the FP32 pipe with
 * about 47 significant bits.  8 bytes, 8-byte aligned: the same footprint as
 * FP64 in every array and shared-memory slice.  Values stay normalized
 * (|lo| <= ulp(hi) / 2), so equality with zero is a test of hi.
 * ------------------------------------------------------------------------ */
struct __align__(8) dd {
  float hi, lo;
  dd() = default;
  __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr dd(int v) : hi((float)v), lo(0.0f) {}
  __host__ __device__ constexpr dd(float v) : hi(v), lo(0.0f) {}
  __device__ __forceinline__ dd(df a) : hi(a.hi), lo(a.lo) {}
  __device__ __forceinline__ dd(double x) : dd(split(x)) {} /* the exact leading 47 bits */
  __device__ __forceinline__ operator df() const { return df{hi, lo}; }
};

__device__ __forceinline__ dd operator+(dd a, dd b) { return add(a, b); }
__device__ __forceinline__ dd operator-(dd a, dd b) { return add(a, neg(b)); }
__device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }
__device__ __forceinline__ dd operator*(dd a, dd b) { return mul(a, b); }
/* a / b = a * (1 / b), the reciprocal by one Newton step (rcp above)        */
__device__ __forceinline__ dd operator/(dd a, dd b) { return mul(a, rcp(b)); }
__device__ __forceinline__ dd& operator+=(dd& a, dd b) { return a = a + b; }
__device__ __forceinline__ dd& operator-=(dd& a, dd b) { return a = a - b; }
__device__ __forceinline__ dd& operator*=(dd& a, dd b) { return a = a * b; }
__device__ __forceinline__ dd& operator/=(dd& a, dd b) { return a = a / b; }
__device__ __forceinline__ bool operator==(dd a, dd b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(dd a, dd b) { return !(a == b); }
__device__ __forceinline__ bool operator<(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dd a, dd b) { return b < a; }
__device__ __forceinline__ bool operator<=(dd a, dd b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(dd a, dd b) { return !(a < b); }
__device__ __forceinline__ dd fma(dd a, dd b, dd c) { return fma(df(a), df(b), df(c)); }
__device__ __forceinline__ dd fabs(dd a) { return a.hi < 0.0f ? -a : a; }
__device__ __forceinline__ dd copysign(dd a, dd b)
{
  return (signbit(a.hi) != signbit(b.hi)) ? -a : a;
}
/* the Newton step needs a positive argument; 0 (and negative or NaN
 * arguments) take the FP32 square root's value                             */
__device__ __forceinline__ dd sqrt(dd a) { return a.hi > 0.0f ? dd(sqrt(df(a))) : dd(sqrtf(a.hi), 0.0f); }

/* warp shuffle of both parts (found by argument-dependent lookup where
 * kernels shuffle a T)                                                      */
__device__ __forceinline__ dd __shfl_xor_sync(unsigned mask, dd v, int lane_mask)
{
  return dd(::__shfl_xor_sync(mask, v.hi, lane_mask), ::__shfl_xor_sync(mask, v.lo, lane_mask));
}

template <>
__device__ __forceinline__ dd narrow<dd>(double x) { return dd(split(x)); }
__device__ __forceinline__ double widen(dd x) { return join(df(x)); }
/* an output value as FP64: the plain conversion for float and double, the
 * sum of the parts for dd                                                   */
template <typename T>
__device__ __forceinline__ double to_f64(T x) { return (double)x; }
__device__ __forceinline__ double to_f64(dd x) { return join(df(x)); }

} /* namespace ukg_df */
