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
//
// A complex dd number is stored as float4 (re_hi, im_hi, re_lo, im_lo): the
// high words of the real and imaginary parts form one float2 and the low
// words another, so every step of the complex arithmetic runs on both parts
// at once with the packed two-lane FP32 instructions of sm_100+ (FFMA2,
// FADD2, FMUL2: one instruction, two correctly rounded FP32 operations).
// Each packed operation rounds every lane exactly as its scalar form does,
// so the error-free transformations hold lane by lane.
#pragma once

#include <cuda_runtime.h>

namespace efg_dd {

// ------------------------------------------------------------ scalar forms
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

// Product of two dd values as an unnormalised pair (p, e): p + e equals
// (ah + al)(bh + bl) up to the al*bl term and the rounding of e.
__device__ __forceinline__ void prod(float ah, float al, float bh, float bl, float &p, float &e) {
  two_prod(ah, bh, p, e);
  e = fmaf(ah, bl, fmaf(al, bh, e));
}

// ------------------------------------------------------------ packed forms
// Subtractions are written as fused multiply-adds with -1 (a - b =
// fma(b, -1, a): the product is exact, so the single rounding is that of
// a - b), so no sign flip of a packed operand is ever needed.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 m1() { return make_float2(-1.f, -1.f); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, m1(), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 swap2(float2 a) { return make_float2(a.y, a.x); }

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2 &s, float2 &e) {
  s = add2(a, b);
  const float2 v = sub2(s, a);
  e = add2(sub2(a, sub2(s, v)), sub2(b, v));
}
__device__ __forceinline__ void fast_two_sum2(float2 a, float2 b, float2 &s, float2 &e) {
  s = add2(a, b);
  e = sub2(b, sub2(s, a));
}
// (ah + al)(bh + bl) lane by lane as an unnormalised pair (p, e); ahn = -ah
// (exact), so that -p comes out of one multiply: pn = -ah*bh rounded is
// exactly -p, and fma(ah, bh, pn) is the exact error of p.
__device__ __forceinline__ void prod2n(float2 ahn, float2 ah, float2 al, float2 bh, float2 bl, float2 &pn,
                                       float2 &e) {
  pn = mul2(ahn, bh);
  e = fma2(ah, bh, pn);
  e = fma2(ah, bl, fma2(al, bh, e));
}
__device__ __forceinline__ void prod2(float2 ah, float2 al, float2 bh, float2 bl, float2 &p, float2 &e) {
  float2 pn;
  prod2n(make_float2(-ah.x, -ah.y), ah, al, bh, bl, pn, e);
  p = make_float2(-pn.x, -pn.y);
}

// Running sums of dd terms for the real and imaginary lanes together: the
// high words are an exact running TwoSum, the errors and low words collect
// in lo (renormalise with value()).  Enough for the short sums here (a
// matrix row).
struct Acc2 {
  float2 hi, lo;
  __device__ __forceinline__ void zero() { hi = lo = make_float2(0.f, 0.f); }
  __device__ __forceinline__ void add(float2 p, float2 e) {
    float2 s, t;
    two_sum2(hi, p, s, t);
    hi = s;
    lo = add2(lo, add2(t, e));
  }
  // += -pn + e, with TwoSum(hi, -pn) written on pn directly
  __device__ __forceinline__ void sub(float2 pn, float2 e) {
    const float2 s = sub2(hi, pn);   // hi + p
    const float2 v = sub2(s, hi);    // s - hi
    const float2 t2 = sub2(hi, sub2(s, v));
    const float2 t3n = add2(pn, v);  // -(p - v)
    lo = add2(lo, add2(sub2(t2, t3n), e));
    hi = s;
  }
  // += (ah + al)(bh + bl) lane by lane; ahn = -ah
  __device__ __forceinline__ void add_prod(float2 ahn, float2 ah, float2 al, float2 bh, float2 bl) {
    float2 pn, e;
    prod2n(ahn, ah, al, bh, bl, pn, e);
    sub(pn, e);
  }
  __device__ __forceinline__ void add_prod(float2 ah, float2 al, float2 bh, float2 bl) {
    add_prod(make_float2(-ah.x, -ah.y), ah, al, bh, bl);
  }
  // renormalised complex dd (float4 layout)
  __device__ __forceinline__ float4 value() const {
    float2 h, l;
    fast_two_sum2(hi, lo, h, l);
    return make_float4(h.x, h.y, l.x, l.y);
  }
};

// ------------------------------------------------------- complex dd values
__device__ __forceinline__ float2 hi2(float4 a) { return make_float2(a.x, a.y); }
__device__ __forceinline__ float2 lo2(float4 a) { return make_float2(a.z, a.w); }
__device__ __forceinline__ float4 pack(float2 h, float2 l) { return make_float4(h.x, h.y, l.x, l.y); }

__device__ __forceinline__ float4 cadd(float4 a, float4 b) {
  float2 s, e, h, l;
  two_sum2(hi2(a), hi2(b), s, e);
  e = add2(e, add2(lo2(a), lo2(b)));
  fast_two_sum2(s, e, h, l);
  return pack(h, l);
}
__device__ __forceinline__ float4 cneg(float4 a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }

// a * c for a complex dd a and a complex float c:
// (re, im) = (c.x, c.x)(a.re, a.im) + (-c.y, c.y)(a.im, a.re).
__device__ __forceinline__ float4 cmul_f(float4 a, float2 c) {
  const float2 ah = hi2(a), al = lo2(a);
  const float2 c1 = f2(c.x), c2 = make_float2(-c.y, c.y);
  const float2 p1 = mul2(c1, ah);
  float2 e1 = fma2(c1, ah, mul2(p1, m1()));
  e1 = fma2(c1, al, e1);
  const float2 sh = swap2(ah), sl = swap2(al);
  const float2 p2 = mul2(c2, sh);
  float2 e2 = fma2(c2, sh, mul2(p2, m1()));
  e2 = fma2(c2, sl, e2);
  float2 s, e, h, l;
  two_sum2(p1, p2, s, e);
  e = add2(e, add2(e1, e2));
  fast_two_sum2(s, e, h, l);
  return pack(h, l);
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

// a * b for complex dd a and b:
// (re, im) = (a.re, a.re)(b.re, b.im) + (-a.im, a.im)(b.im, b.re).
__device__ __forceinline__ float4 cmul(float4 a, float4 b) {
  const float2 bh = hi2(b), bl = lo2(b), sh = swap2(bh), sl = swap2(bl);
  float2 p1, e1, p2, e2;
  prod2(f2(a.x), f2(a.z), bh, bl, p1, e1);
  prod2(make_float2(-a.y, a.y), make_float2(-a.w, a.w), sh, sl, p2, e2);
  float2 s, e, h, l;
  two_sum2(p1, p2, s, e);
  e = add2(e, add2(e1, e2));
  fast_two_sum2(s, e, h, l);
  return pack(h, l);
}

// (h + l) * a for a real dd (h, l) and a complex dd a.
__device__ __forceinline__ float4 rmul(float4 a, float h, float l) {
  float2 p, e, rh, rl;
  prod2(hi2(a), lo2(a), f2(h), f2(l), p, e);
  fast_two_sum2(p, e, rh, rl);
  return pack(rh, rl);
}

// Running sum of dd terms (one real quantity): the high word is an exact
// running TwoSum, the errors and low words collect in lo.  Enough for the
// short sums here (a matrix row, 16 rows of a dot product).
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

// Complex dd from the renormalised real and imaginary accumulators.
__device__ __forceinline__ float4 from_acc(const Acc &re, const Acc &im) {
  float4 r;
  fast_two_sum(re.hi, re.lo, r.x, r.z);
  fast_two_sum(im.hi, im.lo, r.y, r.w);
  return r;
}

// Unconjugated complex product a^T b of complex dd a, b added to (re, im).
__device__ __forceinline__ void dot_add(Acc &re, Acc &im, float4 a, float4 b) {
  re.add_prod(a.x, a.z, b.x, b.z);
  re.add_prod(-a.y, -a.w, b.y, b.w);
  im.add_prod(a.x, a.z, b.y, b.w);
  im.add_prod(a.y, a.w, b.x, b.z);
}

__device__ __forceinline__ float4 csplit(double re, double im) {
  float4 r;
  split(re, r.x, r.z);
  split(im, r.y, r.w);
  return r;
}
__device__ __forceinline__ double2 cjoin(float4 a) { return make_double2(join(a.x, a.z), join(a.y, a.w)); }

// |a|^2 from the high words (a magnitude for convergence tests).
__device__ __forceinline__ float cabs2_hi(float4 a) { return a.x * a.x + a.y * a.y; }

}  // namespace efg_dd
