// Double-float ("dd") arithmetic on FP32 units: a value is an unevaluated
// sum hi + lo of two floats with |lo| <= ulp(hi)/2, about 48 significant
// bits.  Built from error-free transformations:
//   TwoSum  (Knuth, TAOCP vol. 2, 4.2.2): s + e == a + b exactly;
//   FastTwoSum (Dekker 1971), valid for |a| >= |b|;
//   TwoProd via one fused multiply-add (p = a*b, e = fma(a, b, -p)).
// GB300 runs FP64 at a small fraction of its FP32 rate, so the batched
// solver keeps its Krylov vectors in this format and does the arithmetic
// that needs more than FP32 (the curl-curl product, the vector updates) in
// it, at FP32 speed.
#pragma once

#include <cuda_runtime.h>

namespace efg_dd {

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float v = s - a;
  e = (a - (s - v)) + (b - v);
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  e = b - (s - a);
}

__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
  p = a * b;
  e = fmaf(a, b, -p);
}

// (hi, lo) += (bh, bl), renormalised.
__device__ __forceinline__ void add(float &hi, float &lo, float bh, float bl) {
  float s, e;
  two_sum(hi, bh, s, e);
  e += lo + bl;
  fast_two_sum(s, e, hi, lo);
}

// (hi, lo) * f  (f a float), renormalised.
__device__ __forceinline__ void mul_f(float hi, float lo, float f, float &rh, float &rl) {
  float p, e;
  two_prod(hi, f, p, e);
  e = fmaf(lo, f, e);
  fast_two_sum(p, e, rh, rl);
}

// Complex dd stored as float4 (re_hi, re_lo, im_hi, im_lo).
__device__ __forceinline__ float4 cadd(float4 a, float4 b) {
  add(a.x, a.y, b.x, b.y);
  add(a.z, a.w, b.z, b.w);
  return a;
}
__device__ __forceinline__ float4 cneg(float4 a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }

// a * c for a complex dd and c a complex float.
__device__ __forceinline__ float4 cmul_f(float4 a, float2 c) {
  // re = a.re*c.x - a.im*c.y ; im = a.re*c.y + a.im*c.x
  float p1, e1, p2, e2, s, e;
  two_prod(a.x, c.x, p1, e1);
  e1 = fmaf(a.y, c.x, e1);
  two_prod(a.z, -c.y, p2, e2);
  e2 = fmaf(a.w, -c.y, e2);
  two_sum(p1, p2, s, e);
  e += e1 + e2;
  float4 r;
  fast_two_sum(s, e, r.x, r.y);
  two_prod(a.x, c.y, p1, e1);
  e1 = fmaf(a.y, c.y, e1);
  two_prod(a.z, c.x, p2, e2);
  e2 = fmaf(a.w, c.x, e2);
  two_sum(p1, p2, s, e);
  e += e1 + e2;
  fast_two_sum(s, e, r.z, r.w);
  return r;
}

// a + c * b for complex dd a, b and complex float c.
__device__ __forceinline__ float4 cfma_f(float4 a, float2 c, float4 b) { return cadd(a, cmul_f(b, c)); }

// Split a double into a dd pair.
__device__ __forceinline__ void split(double v, float &hi, float &lo) {
  hi = static_cast<float>(v);
  lo = static_cast<float>(v - static_cast<double>(hi));
}
__device__ __forceinline__ double join(float hi, float lo) {
  return static_cast<double>(hi) + static_cast<double>(lo);
}

// Product of two dd values as an unnormalised pair (p, e): p + e equals
// (ah + al)(bh + bl) up to the al*bl term and the rounding of e.
__device__ __forceinline__ void prod(float ah, float al, float bh, float bl, float &p, float &e) {
  two_prod(ah, bh, p, e);
  e = fmaf(ah, bl, fmaf(al, bh, e));
}

// a * b for complex dd a and b.
__device__ __forceinline__ float4 cmul(float4 a, float4 b) {
  float p1, e1, p2, e2, s, e;
  float4 r;
  prod(a.x, a.y, b.x, b.y, p1, e1);
  prod(a.z, a.w, b.z, b.w, p2, e2);
  two_sum(p1, -p2, s, e);
  e += e1 - e2;
  fast_two_sum(s, e, r.x, r.y);
  prod(a.x, a.y, b.z, b.w, p1, e1);
  prod(a.z, a.w, b.x, b.y, p2, e2);
  two_sum(p1, p2, s, e);
  e += e1 + e2;
  fast_two_sum(s, e, r.z, r.w);
  return r;
}

// Running sum of dd terms: the high word is an exact running TwoSum, the
// errors and low words collect in lo (renormalise with value()).  Enough
// for the short sums here (a matrix row, 16 rows of a dot product).
struct Acc {
  float hi, lo;
  __device__ __forceinline__ void zero() { hi = lo = 0.f; }
  __device__ __forceinline__ void add(float p, float e) {
    float s, t;
    two_sum(hi, p, s, t);
    hi = s;
    lo += t + e;
  }
  // += (ah + al)(bh + bl)
  __device__ __forceinline__ void add_prod(float ah, float al, float bh, float bl) {
    float p, e;
    prod(ah, al, bh, bl, p, e);
    add(p, e);
  }
  __device__ __forceinline__ double to_double() const { return static_cast<double>(hi) + static_cast<double>(lo); }
};

// Complex dd from two renormalised accumulators.
__device__ __forceinline__ float4 from_acc(const Acc &re, const Acc &im) {
  float4 r;
  fast_two_sum(re.hi, re.lo, r.x, r.y);
  fast_two_sum(im.hi, im.lo, r.z, r.w);
  return r;
}

// Unconjugated complex product a^T b of complex dd a, b added to (re, im).
__device__ __forceinline__ void dot_add(Acc &re, Acc &im, float4 a, float4 b) {
  re.add_prod(a.x, a.y, b.x, b.y);
  re.add_prod(-a.z, -a.w, b.z, b.w);
  im.add_prod(a.x, a.y, b.z, b.w);
  im.add_prod(a.z, a.w, b.x, b.y);
}

__device__ __forceinline__ float4 csplit(double re, double im) {
  float4 r;
  split(re, r.x, r.y);
  split(im, r.z, r.w);
  return r;
}
__device__ __forceinline__ double2 cjoin(float4 a) { return make_double2(join(a.x, a.y), join(a.z, a.w)); }

}  // namespace efg_dd
