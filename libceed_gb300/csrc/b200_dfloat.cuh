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

__host__ __device__ inline unsigned df_bits_f(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  unsigned u;
  __builtin_memcpy(&u, &f, 4);
  return u;
#endif
}
__host__ __device__ inline float df_f_bits(unsigned u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  __builtin_memcpy(&f, &u, 4);
  return f;
#endif
}

// Split a double into a float-float pair with integer and FP32 operations only (no FP64 pipe: on this GPU the
// double<->float conversions issue on the slow FP64 pipe and would bound the float-float kernels).  hi keeps the
// leading 24 significant bits of x (truncated), lo = x - hi rounded to float: |lo| < ulp(hi) and hi + lo = x to a
// relative 2^-47.  Values outside [2^-74, 2^128) in magnitude take the conversion route (zero directly).
__host__ __device__ inline void df_split(double x, float &hi, float &lo) {
  unsigned long long b;
#ifdef __CUDA_ARCH__
  b = (unsigned long long)__double_as_longlong(x);
#else
  __builtin_memcpy(&b, &x, 8);
#endif
  const unsigned h32 = (unsigned)(b >> 32), l32 = (unsigned)b;
  const int      E   = (int)((h32 >> 20) & 0x7FFu);  // biased exponent
  if (E >= 949 && E <= 1150) {
    const unsigned sign = h32 & 0x80000000u;
    hi                  = df_f_bits(sign | ((unsigned)(E - 896) << 23) | ((h32 & 0xFFFFFu) << 3) | (l32 >> 29));
    const unsigned r    = l32 & 0x1FFFFFFFu;  // the 29 low significand bits, weight 2^(E - 1075)
    const float    rh   = df_f_bits(0x4B000000u | (r >> 6)) - 8388608.0f;  // exact: r >> 6 < 2^23
    const float    rl   = df_f_bits(0x4B000000u | (r & 63u)) - 8388608.0f;
    const float    rv   = rh * 64.0f + rl;                                  // r, rounded once to 24 bits
    lo                  = df_f_bits(df_bits_f(rv * df_f_bits((unsigned)(E - 948) << 23)) | sign);
  } else if ((b << 1) == 0) {
    hi = lo = 0.0f;
  } else {
    hi = (float)x;
    lo = (float)(x - (double)hi);
  }
}

struct dfloat {
  float hi, lo;
  __host__ __device__ dfloat() : hi(0.f), lo(0.f) {}
  __host__ __device__ explicit dfloat(int x) : hi((float)x), lo(0.f) {}
  __host__ __device__ explicit dfloat(double x) { df_split(x, hi, lo); }
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

// Dot-product accumulator.  The generic form is a chain of fused multiply-adds; the float-float form follows Ogita,
// Rump & Oishi's Dot2 ("Accurate sum and dot product", SIAM J. Sci. Comput. 2005): each product's error term (exact
// FMA residual plus the cross terms) and each TwoSum error of the running high sum collect in one float, and the pair
// is normalised once at the end (12 FP32 operations per term instead of 15 for a normalised multiply-add).
template <typename T>
struct Dot {
  T                                 s;
  __device__ __forceinline__ void   first(const T &a, const T &b) { s = a * b; }
  __device__ __forceinline__ void   add(const T &a, const T &b) { s = mad(a, b, s); }
  __device__ __forceinline__ T      value() const { return s; }
};

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

template <>
struct Dot<dfloat> {
  float                             s, c;
  __device__ __forceinline__ void   first(const dfloat &a, const dfloat &b) {
    s = a.hi * b.hi;
    c = __fmaf_rn(a.hi, b.hi, -s);
    c = __fmaf_rn(a.hi, b.lo, c);
    c = __fmaf_rn(a.lo, b.hi, c);
  }
  __device__ __forceinline__ void add(const dfloat &a, const dfloat &b) {
    const float p  = a.hi * b.hi;
    float       e  = __fmaf_rn(a.hi, b.hi, -p);
    e              = __fmaf_rn(a.hi, b.lo, e);
    e              = __fmaf_rn(a.lo, b.hi, e);
    const float s2 = s + p;
    const float bb = s2 - s;
    c += ((s - (s2 - bb)) + (p - bb)) + e;
    s = s2;
  }
  __device__ __forceinline__ dfloat value() const { return df_fast_two_sum(s, c); }
};

__device__ __forceinline__ dfloat operator-(const dfloat &a) {
  dfloat r;
  r.hi = -a.hi;
  r.lo = -a.lo;
  return r;
}
__device__ __forceinline__ dfloat operator-(const dfloat &a, const dfloat &b) { return a + (-b); }

// Running sum of FP32 terms in float-float (about 48 bits): each addition's rounding error from Knuth's TwoSum and
// each product's from an FMA (the product itself by __fmul_rn, so that it is not contracted into the sum) are
// collected in the low word.  Used by sums and dot products over FP32 vectors.
struct F2Acc {
  float                           hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float s = __fadd_rn(hi, v), bb = __fsub_rn(s, hi);
    lo            = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(v, bb)));
    hi            = s;
  }
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    lo            = __fadd_rn(lo, __fmaf_rn(a, b, -p));
    add(p);
  }
  __device__ __forceinline__ double value() const { return isfinite(hi) ? (double)hi + (double)lo : (double)hi; }
};
__device__ __forceinline__ dfloat &operator+=(dfloat &a, const dfloat &b) { return a = a + b; }
__device__ __forceinline__ dfloat &operator*=(dfloat &a, const dfloat &b) { return a = a * b; }

}  // namespace b200
