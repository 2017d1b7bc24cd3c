// Double-float arithmetic for the FP64 form's transforms on sm_103a.
//
// GB300 issues FP32 at about 64 times its FP64 rate, so the FP64 form's FFT
// butterflies and twiddle products run on pairs of FP32 numbers: a value is
// hi + lo with |lo| <= ulp(hi) / 2, about 48 significant bits (unit
// roundoff 2^-48 ~ 3.6e-15).  The building blocks are the error-free
// transformations of Knuth (TwoSum: a + b = s + e exactly, six FP32
// operations), Dekker's FastTwoSum (for |a| >= |b|, three operations) and
// the FMA form of Dekker's TwoProduct (a b = p + e exactly with
// e = fma(a, b, -p)); the sum and product of two double-floats follow the
// "sloppy" addition and the product of Dekker (1971) as analysed by Joldes,
// Muller and Popescu (ACM TOMS 44, 2017): relative error of the sum bounded
// by about 2^-46 of |a| + |b| (an FFT's error is judged against the norm of
// its input, so cancellation does not matter), of the product by about
// 2^-45.  Data enter and leave in FP64 (hi = (float)x, lo = (float)(x - hi));
// the pointwise functional stays in FP64.
//
// Range: FP32's exponent (|x| below 3.4e38, lo underflows below about
// 1e-38 * 2^24), ample for densities, weighted densities and gradients.
#pragma once

#include <cuda_runtime.h>

namespace deft {

struct dfl {
  float hi, lo;
  dfl() = default;
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  // exact for integers up to 2^24, as for any float
  __host__ __device__ constexpr dfl(int v) : hi((float)v), lo(0.f) {}
  // the nearest double-float to d (two roundings, error below 2^-48 |d|)
  __host__ __device__ constexpr dfl(double d)
      : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return dfl(s, (a - (s - bb)) + (b - bb));
}
// Dekker's FastTwoSum (|a| >= |b| or a == 0): s + e == a + b exactly.
__device__ __forceinline__ dfl df_fast_two_sum(float a, float b) {
  const float s = a + b;
  return dfl(s, b - (s - a));
}
__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  const dfl s = df_two_sum(a.hi, b.hi);
  return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
// Dekker's product with the FMA TwoProduct for hi * hi; the cross terms
// enter the error word.  The rounded product is taken with __fmul_rn so the
// compiler cannot contract it into the following addition.
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return df_fast_two_sum(p, e);
}
__device__ __forceinline__ dfl &operator+=(dfl &a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl &operator-=(dfl &a, dfl b) { return a = a - b; }
__device__ __forceinline__ dfl &operator*=(dfl &a, dfl b) { return a = a * b; }
__device__ __forceinline__ bool operator==(dfl a, dfl b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator<(dfl a, dfl b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__device__ __forceinline__ dfl fabs(dfl a) { return a.hi < 0.f ? -a : a; }
// Quotient by one correction step (the long division of Dekker 1971):
// q1 = a.hi / b.hi in FP32, the remainder r = a - q1 b in double-float,
// q = q1 + r.hi / b.hi; relative error about 2^-44.
__device__ __forceinline__ dfl operator/(dfl a, dfl b) {
  const float rb = 1.0f / b.hi;
  const float q1 = a.hi * rb;
  const dfl r = a - dfl(q1, 0.f) * b;
  const float q2 = r.hi * rb;
  const dfl q = df_fast_two_sum(q1, q2);
  // a second correction for the last bits
  const dfl r2 = a - q * b;
  return q + dfl(r2.hi * rb, 0.f);
}
__host__ __device__ __forceinline__ double to_double(dfl a) { return (double)a.hi + (double)a.lo; }

// Complex double-float: 16 bytes, the size of a double2, so the FP64 form's
// tiles and spectra keep their shapes.
struct __align__(16) dfc {
  dfl x, y;
};

}  // namespace deft
