// Float-float ("double-single") arithmetic: a value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits.  Products use the exact FMA error term (Dekker/Knuth-style TwoProduct and TwoSum, as in
// the double-double literature, e.g. Hida, Li & Bailey's QD library and Joldes, Muller & Popescu 2017), with the
// low-order cross terms folded into the error word.
//
// Used by the B200_F64X kernel family: operands live in HBM as FP64, every contraction and pointwise product runs on
// the FP32 pipes in float-float, results go back as FP64.  On this GPU FP32 issues ~60x faster than FP64, so a
// float-float multiply-add (about 15 FP32 operations) is several times cheaper than one native FP64 FMA, while the
// apply stays within ~1e-13 of the FP64 reference (the parity bar is 1e-12).
#pragma once

namespace b200 {

struct dfloat {
  float hi, lo;
  __host__ __device__ dfloat() : hi(0.f), lo(0.f) {}
  __host__ __device__ explicit dfloat(int x) : hi((float)x), lo(0.f) {}
  __host__ __device__ explicit dfloat(double x) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
  }
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

template <typename T>
struct Store {
  using type = T;  // element type of the arrays in HBM
};
template <>
struct Store<dfloat> {
  using type = double;
};

__device__ __forceinline__ dfloat df_fast_two_sum(float a, float b) {
  dfloat r;
  r.hi = a + b;
  r.lo = b - (r.hi - a);
  return r;
}

// c + a*b in each arithmetic; the kernels call mad() so that every element type picks its own (never an implicit
// conversion to another type).
__device__ __forceinline__ double mad(double a, double b, double c) { return ::fma(a, b, c); }
__device__ __forceinline__ float  mad(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ dfloat mad(const dfloat &a, const dfloat &b, const dfloat &c) {
  const float p  = a.hi * b.hi;
  float       e  = __fmaf_rn(a.hi, b.hi, -p);
  e              = __fmaf_rn(a.hi, b.lo, e);
  e              = __fmaf_rn(a.lo, b.hi, e);
  const float s  = c.hi + p;
  const float bb = s - c.hi;
  float       t  = (c.hi - (s - bb)) + (p - bb);
  t += c.lo + e;
  return df_fast_two_sum(s, t);
}

__device__ __forceinline__ dfloat operator*(const dfloat &a, const dfloat &b) {
  const float p = a.hi * b.hi;
  float       e = __fmaf_rn(a.hi, b.hi, -p);
  e             = __fmaf_rn(a.hi, b.lo, e);
  e             = __fmaf_rn(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}

__device__ __forceinline__ dfloat operator+(const dfloat &a, const dfloat &b) {
  const float s  = a.hi + b.hi;
  const float bb = s - a.hi;
  float       t  = (a.hi - (s - bb)) + (b.hi - bb);
  t += a.lo + b.lo;
  return df_fast_two_sum(s, t);
}

__device__ __forceinline__ dfloat operator-(const dfloat &a) {
  dfloat r;
  r.hi = -a.hi;
  r.lo = -a.lo;
  return r;
}
__device__ __forceinline__ dfloat operator-(const dfloat &a, const dfloat &b) { return a + (-b); }
__device__ __forceinline__ dfloat &operator+=(dfloat &a, const dfloat &b) { return a = a + b; }
__device__ __forceinline__ dfloat &operator*=(dfloat &a, const dfloat &b) { return a = a * b; }

}  // namespace b200
