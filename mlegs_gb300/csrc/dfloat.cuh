// dfloat.cuh — double-float arithmetic and the typed load/store helpers shared by the radial
// contractions (radial.cu) and their transposes (adjoint.cu).
#pragma once
#include "common.cuh"

namespace mlg {

// ---- double-float: an unevaluated sum h + l of two FP32 values (about 44 significant bits), every
// operation on the FP32 pipe through error-free transformations (Knuth's two-sum, Dekker/Kahan's FMA
// product error; Dekker 1971, Hida-Li-Bailey 2001).  GB300 issues about 2 FP64 FMAs per clock per SM
// against 128 FP32 FMAs, so the work that needs more than FP32 in the mixed form runs in double-float.
// The intrinsics (__fadd_rn, ...) are never contracted into FMAs, which the transformations rely on.
struct dfl {
  float h, l;
  dfl() = default;
  __device__ __forceinline__ dfl(int v) : h((float)v), l(0.f) {}   // small integers are exact
  __host__ __device__ __forceinline__ dfl(float a, float b) : h(a), l(b) {}
  __device__ __forceinline__ explicit dfl(double x);
};
__device__ __forceinline__ dfl df_quick(float a, float b) {   // |a| >= |b|
  float s = __fadd_rn(a, b);
  return dfl(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  float s = __fadd_rn(a.h, b.h), v = __fsub_rn(s, a.h);
  float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, v)), __fsub_rn(b.h, v));
  return df_quick(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.h, -a.l); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return df_quick(p, e);
}
struct dfl2 { dfl x, y; };
__device__ __forceinline__ dfl df_shfl_xor(dfl v, int o) {   // a butterfly step of a warp reduction
  return dfl(__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o));
}

// multiply-accumulate in the kernel's arithmetic
__device__ __forceinline__ double tmac(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float tmac(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ dfl tmac(dfl a, dfl b, dfl c) { return a * b + c; }

template <typename T> struct V2;
template <> struct V2<double> { typedef double2 t; };
template <> struct V2<float> { typedef float2 t; };
template <> struct V2<dfl> { typedef dfl2 t; };

// x = hi + lo with hi the 24-bit truncation of x and lo the next bits rounded to FP32 (about 47 bits
// in all), split on the integer pipe; values below 2^-126 (and their lo below 2^-75) flush to zero
__device__ __forceinline__ float2 d2ff(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  unsigned sign = hi & 0x80000000u;
  int e = (int)((hi >> 20) & 0x7FFu);
  int e32 = e - 1023 + 127;
  if (e == 0x7FF) return make_float2(__uint_as_float(sign | 0x7F800000u | (((hi & 0xFFFFFu) | lo) ? 0x400000u : 0u)), 0.f);
  if (e32 <= 0) return make_float2(__uint_as_float(sign), 0.f);
  if (e32 >= 255) return make_float2(__uint_as_float(sign | 0x7F800000u), 0.f);
  float h = __uint_as_float(sign | ((unsigned)e32 << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
  int el = e - 1075 + 127;   // exponent of the unit of the 29 remaining bits
  float l = 0.f;
  if (el > 0) {
    l = __uint2float_rn(lo & 0x1FFFFFFFu) * __uint_as_float((unsigned)el << 23);
    if (sign) l = -l;
  }
  return make_float2(h, l);
}
__device__ __forceinline__ dfl::dfl(double x) { float2 v = d2ff(x); h = v.x; l = v.y; }

// field loads / stores: FP64 as is for the plain form; for the mixed form the conversions run on
// the integer pipe (d2f_fast / f2d_fast), keeping these kernels off GB300's narrow FP64 pipe
template <typename T> __device__ __forceinline__ typename V2<T>::t ldc(const double2* p);
template <> __device__ __forceinline__ double2 ldc<double>(const double2* p) { return *p; }
template <> __device__ __forceinline__ float2 ldc<float>(const double2* p) { return ld_c32(p); }
template <> __device__ __forceinline__ dfl2 ldc<dfl>(const double2* p) {
  double2 v = *p;
  dfl2 r; r.x = dfl(v.x); r.y = dfl(v.y); return r;
}
template <typename T> __device__ __forceinline__ double2 to_d2(T re, T im);
template <> __device__ __forceinline__ double2 to_d2<double>(double re, double im) { return make_double2(re, im); }
template <> __device__ __forceinline__ double2 to_d2<float>(float re, float im) {
  return make_double2(f2d_fast(re), f2d_fast(im));
}
template <> __device__ __forceinline__ double2 to_d2<dfl>(dfl re, dfl im) {
  return make_double2(f2d_fast(re.h) + f2d_fast(re.l), f2d_fast(im.h) + f2d_fast(im.l));
}
template <typename T> __device__ __forceinline__ T wsel(const double* w, const float* w32, int i);
template <> __device__ __forceinline__ double wsel<double>(const double* w, const float* w32, int i) { (void)w32; return w[i]; }
template <> __device__ __forceinline__ float wsel<float>(const double* w, const float* w32, int i) { (void)w; return w32[i]; }
template <> __device__ __forceinline__ dfl wsel<dfl>(const double* w, const float* w32, int i) { (void)w32; return dfl(w[i]); }
// table entries: stored as T (FP64 or FP32); double-float reads the FP64 table and splits it
template <typename T> struct TabT { typedef T t; };
template <> struct TabT<dfl> { typedef double t; };
template <typename T> __device__ __forceinline__ T tab(const typename TabT<T>::t* p, size_t o) { return (T)p[o]; }

}  // namespace mlg
