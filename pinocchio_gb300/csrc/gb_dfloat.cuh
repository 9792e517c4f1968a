// Double-float scalar: an unevaluated sum hi + lo of two FP32 values, with
// error-free transformations (Knuth's TwoSum; TwoProduct through a fused
// multiply-add), giving about 48 significand bits from FP32 instructions.
// On GB300 FP32 issues at many times the FP64 rate, so the FP32 derivative
// passes use it where plain FP32 rounding, amplified by the conditioning of
// the mass matrix, would exceed the 1e-5 mixed-precision bar.
//
// The operations follow Dekker (1971) and Knuth (TAOCP vol. 2, 4.2.2);
// division is one Newton-style correction of the FP32 quotient.
#pragma once

#include "gb_spatial.cuh"

namespace gb {

GB_HD float gb_fmaf(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

// 8-byte aligned, so that a value moves with one 64-bit load or store
struct alignas(8) dfloat {
  float hi, lo;
  GB_HD dfloat(const dfloat&) = default;
  GB_HD dfloat& operator=(const dfloat&) = default;
  GB_HD dfloat() : hi(0.f), lo(0.f) {}
  GB_HD dfloat(float x) : hi(x), lo(0.f) {}  // NOLINT: implicit from float / literals
  GB_HD dfloat(int x) : hi(float(x)), lo(0.f) {}  // NOLINT
  GB_HD explicit dfloat(double x) : hi(narrow(x)), lo(narrow(x - widen(hi))) {}
  GB_HD dfloat(float h, float l, int) : hi(h), lo(l) {}
  GB_HD explicit operator float() const { return hi + lo; }
  GB_HD explicit operator double() const { return widen(hi) + widen(lo); }
};

// s + e = a + b exactly (Knuth TwoSum)
GB_HD void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// s + e = a + b exactly, |a| >= |b| (Dekker FastTwoSum)
GB_HD void fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}

// Sum with one TwoSum of the leading parts, the trailing parts added in FP32
// and one renormalisation (Dekker's add; the "sloppy" variant of the QD
// library): error below ~4u^2 (|a| + |b|), u = 2^-24.
GB_HD dfloat operator+(dfloat a, dfloat b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  fast_two_sum(s, e, s, e);
  return dfloat(s, e, 0);
}
GB_HD dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo, 0); }
GB_HD dfloat operator-(dfloat a, dfloat b) { return a + (-b); }
GB_HD dfloat operator*(dfloat a, dfloat b) {
  const float p = a.hi * b.hi;
  float e = gb_fmaf(a.hi, b.hi, -p);
  e = gb_fmaf(a.hi, b.lo, e);
  e = gb_fmaf(a.lo, b.hi, e);
  float s;
  fast_two_sum(p, e, s, e);
  return dfloat(s, e, 0);
}
GB_HD dfloat operator/(dfloat a, dfloat b) {
  const float q1 = a.hi / b.hi;
  const dfloat r = a - b * dfloat(q1);
  const float q2 = r.hi / b.hi;
  float s, e;
  fast_two_sum(q1, q2, s, e);
  return dfloat(s, e, 0);
}
// Compensated dot products (the Dot2 scheme of Ogita, Rump and Oishi, 2005,
// on double-float operands): every product is split exactly by an FMA
// (TwoProduct, with the cross terms of the trailing parts), the leading parts
// are summed with TwoSum and all error terms accumulate in one FP32 value,
// renormalised once at the end.  About 12 FP32 operations per term instead of
// a normalised multiply and add (about 18).
struct dacc {
  float s, e;
  GB_HD void first(dfloat a, dfloat b) {
    s = a.hi * b.hi;
    e = gb_fmaf(a.hi, b.hi, -s);
    e = gb_fmaf(a.hi, b.lo, e);
    e = gb_fmaf(a.lo, b.hi, e);
  }
  GB_HD void add(dfloat a, dfloat b) {
    const float p = a.hi * b.hi;
    float pe = gb_fmaf(a.hi, b.hi, -p);
    pe = gb_fmaf(a.hi, b.lo, pe);
    pe = gb_fmaf(a.lo, b.hi, pe);
    float t;
    two_sum(s, p, s, t);
    e += t + pe;
  }
  GB_HD dfloat result() const {
    float hi, lo;
    two_sum(s, e, hi, lo);
    return dfloat(hi, lo, 0);
  }
};
GB_HD dfloat dot2(dfloat a0, dfloat b0, dfloat a1, dfloat b1) {
  dacc d;
  d.first(a0, b0);
  d.add(a1, b1);
  return d.result();
}
GB_HD dfloat dot3(dfloat a0, dfloat b0, dfloat a1, dfloat b1, dfloat a2, dfloat b2) {
  dacc d;
  d.first(a0, b0);
  d.add(a1, b1);
  d.add(a2, b2);
  return d.result();
}
GB_HD dfloat dot6(const dfloat* a, const dfloat* b) {
  dacc d;
  d.first(a[0], b[0]);
#pragma unroll
  for (int k = 1; k < 6; ++k) d.add(a[k], b[k]);
  return d.result();
}
GB_HD dfloat& operator+=(dfloat& a, dfloat b) { a = a + b; return a; }
GB_HD dfloat& operator-=(dfloat& a, dfloat b) { a = a - b; return a; }
GB_HD dfloat& operator*=(dfloat& a, dfloat b) { a = a * b; return a; }
GB_HD bool operator>(dfloat a, dfloat b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
GB_HD bool operator<(dfloat a, dfloat b) { return b > a; }

}  // namespace gb
