// dfloat.cuh — double-float arithmetic: a value is an unevaluated sum
// hi + lo of two floats (|lo| <= ulp(hi)/2), about 44-48 significant bits,
// computed on the FP32 pipe. On GB300 the FP64 pipe issues at about 1/64 of
// the FP32 rate, so element math that needs more than FP32 accuracy but not
// bit-exact FP64 (the MIXED Newton residual) runs faster this way.
//
// Published error-free transformations: Knuth's TwoSum (The Art of Computer
// Programming, vol. 2, 4.2.2), Dekker's Fast-TwoSum (Numer. Math. 18, 1971)
// and TwoProduct with a fused multiply-add; the accurate addition and the
// multiplication follow the double-double scheme of Hida, Li and Bailey
// (ARITH-15, 2001). Every step uses the _rn intrinsics so that the compiler
// cannot contract a product and a sum into one FMA, which would break the
// transformations.
#pragma once

#include "common.cuh"

namespace gbfem
{

struct DF
{
  float hi, lo;
};

// Compile-time split of a double constant (for reference tables).
__host__ __device__ constexpr DF dfConst(double d)
{
  const float h = static_cast<float>(d);
  return {h, static_cast<float>(d - static_cast<double>(h))};
}

__device__ __forceinline__ DF dfTwoSum(float a, float b)
{
  const float s  = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e  = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// Fast-TwoSum, valid when |a| >= |b| (or a == 0)
__device__ __forceinline__ DF dfQuickTwoSum(float a, float b)
{
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ DF operator+(DF x, DF y)
{
  DF s = dfTwoSum(x.hi, y.hi);
  DF t = dfTwoSum(x.lo, y.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s    = dfQuickTwoSum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return dfQuickTwoSum(s.hi, s.lo);
}

__device__ __forceinline__ DF operator-(DF x)
{
  return {-x.hi, -x.lo};
}

__device__ __forceinline__ DF operator-(DF x, DF y)
{
  return x + (-y);
}

__device__ __forceinline__ DF operator*(DF x, DF y)
{
  const float p = __fmul_rn(x.hi, y.hi);
  float       e = __fmaf_rn(x.hi, y.hi, -p);
  e             = __fmaf_rn(x.hi, y.lo, e);
  e             = __fmaf_rn(x.lo, y.hi, e);
  return dfQuickTwoSum(p, e);
}

__device__ __forceinline__ DF& operator+=(DF& x, DF y)
{
  return x = x + y;
}

__device__ __forceinline__ DF& operator-=(DF& x, DF y)
{
  return x = x - y;
}

// acc + x*y for dot products (the Dot2 scheme of Ogita, Rump and Oishi,
// SIAM J. Sci. Comput. 26, 2005): the leading product is split exactly
// (TwoProduct) and added with TwoSum; both error terms and the cross
// products go into acc.lo, which is left unnormalised until dfNorm.
__device__ __forceinline__ DF dfFma(DF x, DF y, DF acc)
{
  const float p  = __fmul_rn(x.hi, y.hi);
  const float pe = __fmaf_rn(x.hi, y.hi, -p);
  const DF    s  = dfTwoSum(acc.hi, p);
  float       lo = __fadd_rn(acc.lo, __fadd_rn(s.lo, pe));
  lo             = __fmaf_rn(x.hi, y.lo, lo);
  lo             = __fmaf_rn(x.lo, y.hi, lo);
  return {s.hi, lo};
}

__device__ __forceinline__ DF dfNorm(DF x)
{
  return dfTwoSum(x.hi, x.lo);
}

// Runtime conversions: the split costs one FP64 subtraction, the
// recombination one FP64 addition; the float <-> double steps are the
// integer-pipe conversions of common.cuh.
__device__ __forceinline__ DF dfFromF64(double d)
{
  const float h = f64ToF32(d);
  return {h, f64ToF32(d - f32ToF64(h))};
}

__device__ __forceinline__ double dfToF64(DF x)
{
  return f32ToF64(x.hi) + f32ToF64(x.lo);
}

// A double-float value with arithmetic operators, so that element code
// written once for float and double (thBlock<T>) runs in double-float: the
// FP64-accurate Taylor-Hood Jacobian on the FP32 pipe. Multiplication is
// TwoProduct with the cross terms (Dekker with an FMA), addition the "sloppy"
// double-double sum of Hida, Li and Bailey (TwoSum of the leading parts, the
// trailing parts added, renormalised): its error is bounded relative to
// |a| + |b| rather than |a + b|, which is what element sums need (every
// result is compared with the size of its terms). About 2^-46 relative per
// operation.
struct Dd
{
  float hi, lo;
  Dd() = default;
  __host__ __device__ constexpr Dd(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr Dd(int v) : hi(static_cast<float>(v)), lo(0.0f) {}
  // compile-time split of a double constant
  __host__ __device__ constexpr explicit Dd(double d)
    : hi(static_cast<float>(d)),
      lo(static_cast<float>(d - static_cast<double>(static_cast<float>(d))))
  {
  }
};

__device__ __forceinline__ Dd ddQuick(float a, float b) // |a| >= |b|
{
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ Dd operator+(Dd a, Dd b)
{
  const float s  = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e  = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return ddQuick(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ Dd operator-(Dd a)
{
  return {-a.hi, -a.lo};
}

__device__ __forceinline__ Dd operator-(Dd a, Dd b)
{
  return a + (-b);
}

__device__ __forceinline__ Dd operator*(Dd a, Dd b)
{
  const float p = __fmul_rn(a.hi, b.hi);
  float       e = __fmaf_rn(a.hi, b.hi, -p);
  e             = __fmaf_rn(a.hi, b.lo, e);
  e             = __fmaf_rn(a.lo, b.hi, e);
  return ddQuick(p, e);
}

// Long division of double-double arithmetic: three quotient digits, each a
// float division of the running remainder's leading part.
__device__ __forceinline__ Dd operator/(Dd a, Dd b)
{
  const float q1 = __fdiv_rn(a.hi, b.hi);
  Dd          r  = a - Dd(q1, 0.0f) * b;
  const float q2 = __fdiv_rn(r.hi, b.hi);
  r              = r - Dd(q2, 0.0f) * b;
  const float q3 = __fdiv_rn(r.hi, b.hi);
  const Dd    q  = ddQuick(q1, q2);
  return q + Dd(q3, 0.0f);
}

__device__ __forceinline__ Dd& operator+=(Dd& a, Dd b)
{
  return a = a + b;
}

__device__ __forceinline__ Dd& operator-=(Dd& a, Dd b)
{
  return a = a - b;
}

__device__ __forceinline__ bool operator<(Dd a, Dd b)
{
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}

__device__ __forceinline__ bool operator>=(Dd a, Dd b)
{
  return !(a < b);
}

template <>
__device__ __forceinline__ Dd fromF64<Dd>(double d)
{
  const float h = f64ToF32(d);
  return {h, f64ToF32(d - f32ToF64(h))};
}

__device__ __forceinline__ double toF64(Dd x)
{
  return f32ToF64(x.hi) + f32ToF64(x.lo);
}

__device__ __forceinline__ double toF64Ftz(Dd x)
{
  return toF64(x);
}

} // namespace gbfem
