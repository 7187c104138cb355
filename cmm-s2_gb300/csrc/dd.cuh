// Double-double arithmetic on the FP64 pipe, for set-up work that must be
// exact beyond FP64 (the quadratic-form assembly of the map records).
//
// A value is the unevaluated sum h + l of two doubles (~106 significand
// bits), built from the published error-free transformations: Knuth's
// TwoSum (The Art of Computer Programming, vol. 2, 4.2.2), Dekker's
// FastTwoSum for |a| >= |b|, and the FMA form of Dekker's exact product
// (p = fl(a b), e = fma(a, b, -p)).  The rounding steps use the _rn
// intrinsics, which the compiler neither contracts nor reassociates.
#pragma once
#include <cuda_runtime.h>

namespace cmm {
namespace dev {

struct dd {
  double h, l;
};

__device__ __forceinline__ dd dd_two_sum(double a, double b) {
  const double s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  const double e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
  return dd{s, e};
}

__device__ __forceinline__ dd dd_fast_two_sum(double a, double b) {
  const double s = __dadd_rn(a, b);
  return dd{s, __dsub_rn(b, __dsub_rn(s, a))};
}

__device__ __forceinline__ dd dd_two_prod(double a, double b) {
  const double p = __dmul_rn(a, b);
  return dd{p, __fma_rn(a, b, -p)};
}

// a + b with both error terms carried (the accurate double-double sum)
__device__ __forceinline__ dd dd_add(dd a, dd b) {
  dd s = dd_two_sum(a.h, b.h);
  const dd t = dd_two_sum(a.l, b.l);
  s.l = __dadd_rn(s.l, t.h);
  s = dd_fast_two_sum(s.h, s.l);
  s.l = __dadd_rn(s.l, t.l);
  return dd_fast_two_sum(s.h, s.l);
}

__device__ __forceinline__ dd dd_mul_d(dd a, double b) {
  dd p = dd_two_prod(a.h, b);
  p.l = __fma_rn(a.l, b, p.l);
  return dd_fast_two_sum(p.h, p.l);
}

__device__ __forceinline__ dd dd_mul(dd a, dd b) {
  dd p = dd_two_prod(a.h, b.h);
  p.l = __fma_rn(a.h, b.l, __fma_rn(a.l, b.h, p.l));
  return dd_fast_two_sum(p.h, p.l);
}

__device__ __forceinline__ double dd_round(dd a) { return __dadd_rn(a.h, a.l); }

// a + b with the low parts added in FP64 (Dekker's sum): error ~2^-105 of
// |a| + |b|, enough where the cancellation is far below 2^52
__device__ __forceinline__ dd dd_add_fast(dd a, dd b) {
  const dd s = dd_two_sum(a.h, b.h);
  return dd_fast_two_sum(s.h, __dadd_rn(s.l, __dadd_rn(a.l, b.l)));
}

// sum_k x_k m_k for six double-double x_k and doubles m_k, rounded once:
// exact products of the high parts, their sum by a TwoSum cascade, every
// error term and the low parts' products collected in one FP64
// correction (relative error ~2^-104 of sum |x_k m_k|)
__device__ __forceinline__ double dd_dot_d(const dd* x, const double* m) {
  dd p = dd_two_prod(x[0].h, m[0]);
  double err = __fma_rn(x[0].l, m[0], p.l);
  double s = p.h;
#pragma unroll
  for (int k = 1; k < 6; ++k) {
    const dd q = dd_two_prod(x[k].h, m[k]);
    const dd t = dd_two_sum(s, q.h);
    s = t.h;
    err = __dadd_rn(err, __dadd_rn(t.l, __fma_rn(x[k].l, m[k], q.l)));
  }
  return __dadd_rn(s, err);
}

}  // namespace dev
}  // namespace cmm
