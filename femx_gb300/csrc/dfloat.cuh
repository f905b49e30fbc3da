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


// double -> double-float entirely on the integer and FP32 pipes (no FP64
// instruction, no hardware conversion): hi takes the leading 24 significant
// bits of x (truncated), lo the next 23. The remaining 6 bits are dropped,
// so hi + lo is within 2^-46 |x| of x. lo is built without normalising: the
// 23 bits are placed under an implicit leading one of weight 2^(E-23) (E the
// exponent of x) and that one is subtracted again in FP32, exactly
// (Sterbenz). Finite x with 2^-126 <= |x| < 2^127 are split (below 2^-103
// lo is 0); smaller magnitudes become 0; larger ones take the FP64 path.
__device__ __forceinline__ Dd ddSplitInt(double x)
{
  const unsigned hi32 = static_cast<unsigned>(__double2hiint(x));
  const unsigned lo32 = static_cast<unsigned>(__double2loint(x));
  const unsigned sgn  = hi32 & 0x80000000u;
  const unsigned ax   = hi32 & 0x7fffffffu;
  const unsigned e    = ax >> 20; // biased FP64 exponent
  if (e >= 1150u)
  {
    return fromF64<Dd>(x);
  }
  // (e - 896) << 23 | 23 leading fraction bits: the float with x's sign
  const unsigned hb = sgn | __funnelshift_l(lo32, ax - 0x38000000u, 3);
  const unsigned eb = (e - 919u) << 23; // weight 2^(E-23) as a float exponent
  const unsigned lb = sgn | eb | ((lo32 >> 6) & 0x7fffffu);
  const float    lo = __fsub_rn(__uint_as_float(lb), __uint_as_float(sgn | eb));
  return Dd(e > 896u ? __uint_as_float(hb) : 0.0f, e >= 920u ? lo : 0.0f);
}

// double-float -> double, for a normalised pair (|lo| <= ulp(hi)/2, as
// every Dd operation leaves it), with no FP64 instruction and no branch. hi
// is widened exactly into the FP64 bit pattern on the integer pipe; lo times
// sign(hi) is scaled by a power of two into units of the last FP64 place of
// hi, exactly, truncated to an integer (|t| < 2^30) by one float-to-integer
// conversion and added to that pattern as a 64-bit integer. hi + lo stays
// inside hi's binade except when hi is a power of two and lo has the other
// sign: the result then lies in the binade below, whose unit is half as
// large, and the scale counts lo in those units. Faithful (between hi + lo
// and hi, within one unit of the last FP64 place of hi + lo) for 2^-74 <=
// |hi| < 2^128; for smaller normal hi the scale is capped at 2^127, so lo
// counts less than its value (an error below |lo| <= 2^-98). Zero and
// subnormal hi give a zero of hi's sign; an infinite or NaN hi is widened
// as it is (lo ignored).
__device__ __forceinline__ double ddJoinInt(Dd v)
{
  const unsigned hb = __float_as_uint(v.hi);
  const unsigned ha = hb & 0x7fffffffu;
  const unsigned eh = ha >> 23; // biased exponent of hi
  const unsigned sg = hb & 0x80000000u;
  const unsigned dn =
      ((ha & 0x7fffffu) == 0u && ((hb ^ __float_as_uint(v.lo)) & 0x80000000u) != 0u) ? 1u : 0u;
  const bool sp = eh == 0u || eh == 0xffu;
  // 2^(52 - E + dn) sign(hi), E = eh - 127 the exponent of hi
  const unsigned se    = min(306u + dn - eh, 254u);
  const float    scale = __uint_as_float((se << 23) | sg);
  const int      t     = sp ? 0 : __float2int_rz(__fmul_rn(v.lo, scale));
  // float exponent bias 127 -> FP64 bias 1023 (896 << 20); all ones stays all ones
  const unsigned off = eh == 0u ? 0u : (eh == 0xffu ? 0x70000000u : 0x38000000u);
  const unsigned hx  = eh == 0u ? 0u : ha;
  const unsigned long long w =
      (static_cast<unsigned long long>((hx >> 3) + off) << 32) | (hx << 29);
  const unsigned long long m = w + static_cast<unsigned long long>(static_cast<long long>(t));
  return __longlong_as_double(
      static_cast<long long>(m | (static_cast<unsigned long long>(sg) << 32)));
}

// 1/x in double-float: a float reciprocal refined by one Newton step,
// y = y0 + y0 (1 - x y0), with x y0 formed exactly (TwoProduct) so that the
// residual 1 - x y0 carries x's low part; relative error about 2^-46.
__device__ __forceinline__ Dd ddRcp(Dd x)
{
  const float y0 = __frcp_rn(x.hi);
  const float p  = __fmul_rn(x.hi, y0);
  const float pe = __fmaf_rn(x.hi, y0, -p);
  // 1 - x y0 = (1 - p) - pe - x.lo y0; 1 - p is exact (p is within an ulp of 1)
  const float r = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, p), pe), __fmul_rn(x.lo, y0));
  return ddQuick(y0, __fmul_rn(y0, r));
}

} // namespace gbfem
