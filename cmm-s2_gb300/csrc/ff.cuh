// Float-float ("double-single") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum h + l of two floats (|l| below one ulp of
// h), which carries ~48 significand bits (relative rounding ~2^-47 against
// FP64's 2^-53): enough for quantities that need
// FP64-level accuracy but not IEEE FP64 itself, on a part whose FP64 rate
// is 1/64 of its FP32 rate.  The building blocks are the published
// error-free transformations:
//   * Knuth's TwoSum (The Art of Computer Programming, vol. 2, 4.2.2):
//     s = fl(a + b) and the exact error e with a + b = s + e, six additions;
//   * Dekker's exact product (Dekker 1971, "A floating-point technique for
//     extending the available precision") in its FMA form:
//     p = fl(a b), e = fma(a, b, -p), a b = p + e exactly.
// Every operation is written as an _rn intrinsic or an explicit fmaf, which
// the compiler neither contracts nor reassociates: each kernel that
// inlines these functions computes bitwise the same values, whatever code
// surrounds them (a plain a * b + c may or may not become an FMA,
// depending on the instruction schedule of each instantiation).
#pragma once
#include <cuda_runtime.h>

namespace cmm {
namespace dev {

struct ff {
  float h, l;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ff{s, e};
}

// the double x as h + l: h = x truncated to a float, l = the remaining 29
// significand bits (truncated to 24), both from x's bit pattern on the
// integer pipe (a rounding conversion would occupy the FP64 pipe).  h + l
// equals x to within 2^-47 |x| (the two floats hold 48 of x's 53
// significand bits) for 2^-74 <= |x| < 2^128; below 2^-74 the low
// part is dropped (x is then negligible beside the O(1) quantities it is
// combined with); |x| >= 2^128, infinities and NaNs give an infinite or NaN
// h and l = 0.
__device__ __forceinline__ ff ff_of(double x) {
  const long long b = __double_as_longlong(x);
  const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  const unsigned mag = hw & 0x7fffffffu, sgn = hw & 0x80000000u;
  const unsigned e = mag >> 20;                       // biased FP64 exponent
  unsigned fh = e < 897u ? 0u : (((mag - (896u << 20)) << 3) | (lw >> 29));
  const unsigned r = lw & 0x1fffffffu;                // x - h = r * 2^(e - 1075)
  float lo = 0.f;
  if (e > 1150u) {
    const bool nan_x = e == 2047u && ((mag & 0xfffffu) | lw) != 0u;
    fh = nan_x ? 0x7fc00000u : 0x7f800000u;
  } else if (r != 0u && e >= 950u) {
    lo = __fmul_rn(__uint2float_rz(r), __uint_as_float((e - 948u) << 23));
  }
  return ff{__uint_as_float(sgn | fh), sgn ? -lo : lo};
}

// The high float of ff_of(x) alone (the same bits): x truncated to 24
// significand bits, from its bit pattern.
__device__ __forceinline__ float ff_hi(double x) {
  const long long b = __double_as_longlong(x);
  const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  const unsigned mag = hw & 0x7fffffffu, sgn = hw & 0x80000000u;
  const unsigned e = mag >> 20;
  unsigned fh = e < 897u ? 0u : (((mag - (896u << 20)) << 3) | (lw >> 29));
  if (e > 1150u) fh = (e == 2047u && ((mag & 0xfffffu) | lw) != 0u) ? 0x7fc00000u : 0x7f800000u;
  return __uint_as_float(sgn | fh);
}

// h + l rounded to a double (one FP64 addition; the conversions are exact)
__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.h + (double)a.l; }

__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.h, -a.l}; }

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = two_sum(a.h, b.h);
  const ff t = two_sum(a.l, b.l);
  return two_sum(s.h, __fadd_rn(__fadd_rn(s.l, t.h), t.l));
}

__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.h, b.h);
  // the exact error of the leading product, then the cross terms by FMA
  const float e = fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -p)));
  return two_sum(p, e);
}

// a0 b0 + a1 b1 + a2 b2: the three leading products summed by TwoSum, every
// rounding error and cross term collected in one float correction (the
// products' exact errors summed, then the cross terms by FMA).
__device__ __forceinline__ ff ff_dot3(ff a0, ff b0, ff a1, ff b1, ff a2, ff b2) {
  const float p0 = __fmul_rn(a0.h, b0.h), p1 = __fmul_rn(a1.h, b1.h), p2 = __fmul_rn(a2.h, b2.h);
  float e = __fadd_rn(__fadd_rn(fmaf(a0.h, b0.h, -p0), fmaf(a1.h, b1.h, -p1)), fmaf(a2.h, b2.h, -p2));
  e = fmaf(a0.h, b0.l, e);
  e = fmaf(a0.l, b0.h, e);
  e = fmaf(a1.h, b1.l, e);
  e = fmaf(a1.l, b1.h, e);
  e = fmaf(a2.h, b2.l, e);
  e = fmaf(a2.l, b2.h, e);
  const ff s = two_sum(p0, p1);
  const ff t = two_sum(s.h, p2);
  return two_sum(t.h, __fadd_rn(__fadd_rn(e, s.l), t.l));
}

// a0 b0 + a1 b1, as ff_dot3
__device__ __forceinline__ ff ff_dot2(ff a0, ff b0, ff a1, ff b1) {
  const float p0 = __fmul_rn(a0.h, b0.h), p1 = __fmul_rn(a1.h, b1.h);
  float e = __fadd_rn(fmaf(a0.h, b0.h, -p0), fmaf(a1.h, b1.h, -p1));
  e = fmaf(a0.h, b0.l, e);
  e = fmaf(a0.l, b0.h, e);
  e = fmaf(a1.h, b1.l, e);
  e = fmaf(a1.l, b1.h, e);
  const ff s = two_sum(p0, p1);
  return two_sum(s.h, __fadd_rn(e, s.l));
}

// 1/sqrt(a) for a > 0: the FP32 value 1/sqrt(a.h) (relative error below
// 2^-23) refined by two Newton steps r += r (1 - a r^2) / 2 whose residual
// is formed in float-float; the first leaves ~1.5 * 2^-46, the second the
// float-float rounding level.
__device__ __forceinline__ ff ff_rsqrt(ff a) {
  ff r{__frcp_rn(__fsqrt_rn(a.h)), 0.f};
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const ff res = ff_sub(ff{1.f, 0.f}, ff_mul(a, ff_mul(r, r)));
    r = ff_add(r, ff{__fmul_rn(__fmul_rn(0.5f, r.h), __fadd_rn(res.h, res.l)), 0.f});
  }
  return r;
}

}  // namespace dev
}  // namespace cmm
